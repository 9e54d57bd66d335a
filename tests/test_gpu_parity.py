"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Bit-exact: the traced lines (entry, exit, direction, step count), every staircase, the
plain-method counts and the curl indicator.  Floating point: p after the iterations
within a stated relative L2 of the oracle's FP64 evaluation of the same discrete method
(the FP32 GPU path differs only in the order and precision of sums).
"""
import bf16_ref
import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu

# tolerances (relative L2 after removing the mean)
TOL_P_PLAIN = 2e-5     # FP32 + Kahan line scans vs FP64, a few iterations
TOL_P_SELECT = 1e-4    # curl-weighted averages amplify rounding a little
TOL_PN = 1e-5          # one sweep, accumulated sums


def _field(dims, seed=0, noise=0.05, sphere=None):
    n = max(dims)
    f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 5.0), noise=noise, seed=seed, spacing=1e-3,
                        sphere_radius=sphere)
    return f


def _pinit(dims, seed=1):
    """Bernoulli-like nonzero j = 0 face, exercising the first-iteration seeding (K:8811)."""
    nx, ny, nz = dims
    rng = np.random.default_rng(seed)
    p = np.zeros((nz, ny, nx), np.float32)
    p[:, 0, :] = rng.normal(0, 0.5, (nz, nx)).astype(np.float32)
    return p


def _lines_oracle(orc, dims, ls, dirs):
    """Valid lines in (direction, lattice point) order: table rows and, per line, the
    (entry/exit, offset) the oracle walk needs."""
    rows, geo = [], []
    for d in range(len(dirs)):
        valid, inout, nsteps, xyz = orc.trace_direction(dims, ls, dirs[d])
        X, Y, Z = dims
        for pt in np.nonzero(valid)[0]:
            i = inout[pt]
            e = i[0] + i[1] * X + i[2] * X * Y
            x = i[3] + i[4] * X + i[5] * X * Y
            rows.append((e, x, d, nsteps[pt]))
            geo.append((inout[pt].copy(), xyz[pt].copy()))
    return np.array(rows, np.int64).reshape(-1, 4), geo


@pytest.mark.parametrize("dims,ls,level", [((20, 17, 13), 1.0, 3), ((16, 16, 16), 0.7, 3), ((12, 9, 15), 1.0, 2)])
def test_line_table_bit_exact(omni, orc, match_lines, dims, ls, level):
    dirs = omni.icosphere(level)
    with omni.Omni3D(dims, 1e-3, dirs, line_spacing=ls, max_iter=1) as s:
        info = s.geometry_info()
        assert info["walk_errors"] == 0
        got = s.line_table().astype(np.int64)
        got[:, 0] &= 0xFFFFFFFF
        got[:, 1] &= 0xFFFFFFFF
        exp, geo = _lines_oracle(orc, dims, ls, dirs)
        at = match_lines(got, exp)  # the same rows, in the library's own order
        assert info["n_units"] == int((exp[:, 3] + 1).sum())
        # staircases of a sample of lines (where lines share a key, one of them walks alike)
        for k in range(0, len(exp), max(1, len(exp) // 60)):
            io, xyz = geo[k]
            ax = orc.walk(dims, io, xyz, dirs[exp[k, 2]])
            assert any(np.array_equal(s.line_steps(i), ax) for i in at[k]), k


@pytest.mark.parametrize("tile_width,dir_group", [(4, 1), (16, 8), (8, 4)])
def test_line_order_options(omni, orc, match_lines, tile_width, dir_group):
    """Other line orders (tile width, directions per group) hold the same lines and
    staircases and give the same solve up to the order of sums.  The default order: 8-wide
    tiles, groups of 32 directions on grids of up to 2^24 voxels (4 above)."""
    dims = (21, 18, 15)
    f = _field(dims, seed=14, sphere=3.5)
    dirs = omni.icosphere(3)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 85))
    res = {}
    for tw, dg in ((0, 0), (tile_width, dir_group)):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=4, method="select", threshold=thr, tile_width=tw,
                         dir_group=dg) as s:
            r = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
            assert (r.stats["tile_width"], r.stats["dir_group"]) == (tw or 8, dg or (32 if np.prod(dims) <= 2 ** 24 else 4))
            res[tw] = r
            if tw:
                got = s.line_table().astype(np.int64)
                got[:, 0] &= 0xFFFFFFFF
                got[:, 1] &= 0xFFFFFFFF
                exp, geo = _lines_oracle(orc, dims, 1.0, dirs)
                at = match_lines(got, exp)
                for k in range(0, len(exp), max(1, len(exp) // 40)):
                    io, xyz = geo[k]
                    ax = orc.walk(dims, io, xyz, dirs[exp[k, 2]])
                    assert any(np.array_equal(s.line_steps(i), ax) for i in at[k]), k
    np.testing.assert_array_equal(res[0].count > 0, res[tile_width].count > 0)
    assert synthetic.relative_l2(res[tile_width].count, res[0].count, gauge="none") < 1e-6
    assert synthetic.relative_l2(res[tile_width].p, res[0].p, gauge="none") < 1e-6


def test_autotune_picks_a_candidate_and_solves_alike(omni):
    """params.autotune times a few line orders at creation and keeps the fastest per size
    class; the result is the same solve."""
    dims = (40, 36, 33)
    f = _field(dims, seed=15, sphere=4.0)
    dirs = omni.icosphere(3)
    out = []
    for tune in (True, True, False):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=4, autotune=tune) as s:
            out.append(s.solve(f["ax"], f["ay"], f["az"]))
    pairs = [(r.stats["tile_width"], r.stats["dir_group"]) for r in out]
    assert pairs[0] in {(8, 4), (4, 4), (16, 4), (8, 2), (8, 8)}
    assert pairs[1] == pairs[0]  # the same size class reuses the choice
    assert pairs[2] == (8, 32)  # the default order at this size
    np.testing.assert_array_equal(out[0].count, out[2].count)
    assert synthetic.relative_l2(out[0].p, out[2].p, gauge="none") < 1e-6


def test_curl_bit_exact(omni, orc):
    dims = (14, 11, 9)
    f = _field(dims, sphere=3.0)
    dirs = omni.icosphere(2)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1) as s:
        got = s.curl(f["ax"], f["ay"], f["az"], f["mask"]).reshape(-1)
    exp = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    np.testing.assert_array_equal(got.view(np.uint32), exp.view(np.uint32))


def test_plain_sweep_matches_oracle(omni, orc):
    dims = (18, 15, 12)
    f = _field(dims, seed=3)
    dirs = omni.icosphere(3)
    p = _pinit(dims)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1) as s:
        pn, cnt = s.sweep(f["ax"], f["ay"], f["az"], p)
    epn, ecnt = orc.sweep(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p, precision="f64")
    np.testing.assert_array_equal(cnt.reshape(-1), ecnt.astype(np.float32))
    assert synthetic.relative_l2(pn, epn, gauge="none") < TOL_PN


@pytest.mark.parametrize("solver", ["sweep", "anchor"])
@pytest.mark.parametrize("niter", [1, 2, 5])
def test_plain_solve_matches_oracle(omni, orc, solver, niter):
    dims = (20, 16, 14)
    f = _field(dims, seed=4)
    dirs = omni.icosphere(3)
    p0 = _pinit(dims)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=niter, solver=solver) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], p_init=p0)
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, niter, precision="f64")
    np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
    assert r.stats["iterations"] == niter
    assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_PLAIN
    # also against the reference's own float arithmetic
    fp, fcnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, niter, precision="f32")
    np.testing.assert_array_equal(r.count.reshape(-1), fcnt)
    assert synthetic.relative_l2(r.p, fp, gauge="none") < TOL_P_PLAIN


@pytest.mark.parametrize("solver", ["sweep", "anchor"])
def test_select_solve_matches_oracle(omni, orc, solver):
    dims = (20, 18, 16)
    f = _field(dims, seed=5, noise=0.1, sphere=4.0)
    dirs = omni.icosphere(3)
    p0 = _pinit(dims, seed=2)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 85))
    niter = 4
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=niter, solver=solver, method="select", threshold=thr) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"], p_init=p0)
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, niter, mode=1, thr=thr, curl=curl,
                         precision="f64")
    # weights are curl-dependent floats: compare within tolerance, zero pattern exactly
    np.testing.assert_array_equal(r.count.reshape(-1) > 0, ecnt > 0)
    assert synthetic.relative_l2(r.count, ecnt, gauge="none") < 1e-5
    assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_SELECT


@pytest.mark.parametrize("method,mode", [("select", 1), ("weighted", 2)])
def test_anchor_fill_with_signed_zero_curl(omni, orc, method, mode):
    """The filling pass flags the anchors in the sign bit of the packed curl; a curl array
    with a sign bit already set (here -0.0) makes it keep the bitmap instead.  Both forms
    give the oracle's result, and the same field with +0.0 gives the same iterate."""
    dims = (19, 16, 14)
    f = _field(dims, seed=8, noise=0.1, sphere=3.5)
    dirs = omni.icosphere(3)
    p0 = _pinit(dims, seed=4)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    zero = np.nonzero(curl == 0)[0]
    assert len(zero) > 10
    signed = curl.copy()
    signed[zero[::3]] = -0.0
    assert (np.signbit(signed) & (signed == 0)).sum() > 0
    thr = float(np.percentile(curl[curl > 0], 85)) if mode == 1 else 0.0
    niter = 4
    out = {}
    for name, c in (("plus", curl), ("minus", signed)):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=niter, method=method, threshold=thr) as s:
            out[name] = s.solve(f["ax"], f["ay"], f["az"], curl=c, p_init=p0)
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, niter, mode=mode, thr=thr,
                         curl=signed, precision="f64")
    for r in out.values():
        np.testing.assert_array_equal(r.count.reshape(-1) > 0, ecnt > 0)
        assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_SELECT
    assert synthetic.relative_l2(out["minus"].p, out["plus"].p, gauge="none") < 1e-6


def test_weighted_sweep_matches_oracle(omni, orc):
    """One weighted sweep (K:1993-2135): the entry receives nothing, a step's weight is
    n / sum(curl/1e4) once that sum is nonzero; voxels inside the masked sphere have curl 0."""
    dims = (18, 15, 12)
    f = _field(dims, seed=21, sphere=3.5)
    dirs = omni.icosphere(3)
    p = _pinit(dims, seed=3)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1, method="weighted") as s:
        pn, cnt = s.sweep(f["ax"], f["ay"], f["az"], p, curl=curl)
    epn, ecnt = orc.sweep(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p, mode=2, curl=curl, precision="f64")
    _, fcnt = orc.sweep(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p, mode=2, curl=curl)
    np.testing.assert_array_equal(cnt.reshape(-1) > 0, fcnt > 0)  # which voxels receive: exact
    assert synthetic.relative_l2(cnt, ecnt, gauge="none") < TOL_PN
    assert synthetic.relative_l2(pn, epn, gauge="none") < TOL_PN


@pytest.mark.parametrize("solver", ["sweep", "anchor"])
@pytest.mark.parametrize("niter", [1, 4])
def test_weighted_solve_matches_oracle(omni, orc, solver, niter):
    dims = (20, 17, 15)
    f = _field(dims, seed=22, noise=0.1, sphere=4.0)
    dirs = omni.icosphere(3)
    p0 = _pinit(dims, seed=4)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=niter, solver=solver, method="weighted") as s:
        r = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"], p_init=p0)  # curl computed on the device
    assert r.stats["solver_used"] == (0 if solver == "anchor" else 1)
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, niter, mode=2, curl=curl,
                         precision="f64")
    fp, fcnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, niter, mode=2, curl=curl)
    np.testing.assert_array_equal(r.count.reshape(-1) > 0, fcnt > 0)
    assert synthetic.relative_l2(r.count, ecnt, gauge="none") < 1e-5
    assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_SELECT
    assert synthetic.relative_l2(r.p, fp, gauge="none") < TOL_P_SELECT


def test_weighted_tolerance_bf16_and_zero_curl(omni, orc):
    """Weighted method: the tolerance stop agrees between the solvers, BF16 storage stays
    close to FP32, and a zero-curl field gives no contribution at all."""
    dims = (16, 16, 16)
    f = _field(dims, seed=23, sphere=4.0)
    dirs = omni.icosphere(3)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    its = []
    for solver in ("sweep", "anchor"):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=200, tol=1e-4, gauge="point", solver=solver,
                         method="weighted") as s:
            r = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
            its.append(r.stats["iterations"])
            assert r.stats["rel_change"] < 1e-4
    assert abs(its[0] - its[1]) <= 1
    out = {}
    for g in ("f32", "bf16"):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=4, grad=g, method="weighted") as s:
            out[g] = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
    # BF16 storage rounds the curl too, so the weights (and counts) move by its rounding
    assert 0 < synthetic.relative_l2(out["bf16"].count, out["f32"].count, gauge="none") < 1e-2
    assert 0 < synthetic.relative_l2(out["bf16"].p, out["f32"].p) < 1e-2
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2, method="weighted") as s:
        p0 = _pinit(dims)
        r = s.solve(f["ax"], f["ay"], f["az"], curl=np.zeros_like(curl), p_init=p0)
    assert (r.count == 0).all()
    np.testing.assert_array_equal(r.p.reshape(-1), p0.reshape(-1))


def test_select_without_threshold_splits_at_mask(omni, orc):
    """Config-3 form: threshold above every curl, so only the masked voxels are excluded."""
    dims = (18, 18, 18)
    f = _field(dims, seed=6, sphere=5.0)
    dirs = omni.icosphere(2)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.finfo(np.float32).max)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=3, method="select", threshold=thr) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], np.zeros(curl.size, np.float32), 3,
                         mode=1, thr=thr, curl=curl, precision="f64")
    inside = (f["mask"].reshape(-1) == 0)
    assert (r.count.reshape(-1)[inside] == 0).all()
    assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_SELECT


def test_iteration_edge_cases(omni, orc):
    dims = (10, 9, 8)
    f = _field(dims, seed=7)
    dirs = omni.icosphere(2)
    p0 = _pinit(dims)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=0) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], p_init=p0)
        np.testing.assert_array_equal(r.p.reshape(-1), p0.reshape(-1))
        assert (r.count == 0).all()
    # seeding off: the first sweep starts from zero
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1, seed_first_iteration=False) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], p_init=p0)
    pn, cnt = orc.sweep(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, precision="f64")
    exp = np.where(cnt > 0, pn / np.maximum(cnt, 1), p0.reshape(-1))
    assert synthetic.relative_l2(r.p, exp, gauge="none") < TOL_P_PLAIN


def test_minimal_grid_and_pole_directions(omni, orc):
    """2x2x2 grid and a direction set holding only the poles and the axes."""
    dirs = np.array([[0, 0, 1], [0, 0, -1], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0]], np.float32)
    for dims in [(2, 2, 2), (3, 5, 4)]:
        f = _field(dims, seed=8)
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2) as s:
            r = s.solve(f["ax"], f["ay"], f["az"])
        ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], np.zeros(np.prod(dims), np.float32),
                             2, precision="f64")
        np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
        assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_PLAIN


def test_large_direction_set_matches_oracle(omni, orc):
    """2562 vertices (icosphere level 5): many direction groups and a long serpentine order
    over the sphere; counts exact, p against the FP64 oracle."""
    dims = (13, 11, 9)
    f = _field(dims, seed=17)
    dirs = omni.icosphere(5)
    assert len(dirs) == 2562
    p0 = _pinit(dims, seed=6)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], p_init=p0)
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2, precision="f64")
    np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
    assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_PLAIN


def test_gauges_and_tolerance(omni, orc):
    dims = (16, 16, 16)
    f = _field(dims, seed=9)
    dirs = omni.icosphere(3)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=6) as s:
        r0 = s.solve(f["ax"], f["ay"], f["az"])
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=6, gauge="point", ref=(0, 0, 0)) as s:
        r1 = s.solve(f["ax"], f["ay"], f["az"])
    assert r1.p.reshape(-1)[0] == 0.0
    np.testing.assert_allclose(r1.p, r0.p - r0.p.reshape(-1)[0], atol=1e-5 * np.abs(r0.p).max())
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=6, gauge="mean") as s:
        r2 = s.solve(f["ax"], f["ay"], f["az"])
    sel = r2.count > 0
    assert abs(float(r2.p[sel].mean())) < 1e-5 * np.abs(r2.p).max()
    # tolerance-driven stop: both solvers stop at the same iteration
    its = []
    for solver in ("sweep", "anchor"):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=200, tol=1e-4, gauge="point", solver=solver) as s:
            r = s.solve(f["ax"], f["ay"], f["az"])
            its.append(r.stats["iterations"])
            assert r.stats["rel_change"] < 1e-4
    assert abs(its[0] - its[1]) <= 1


@pytest.mark.parametrize("gauge,method", [("mean", "plain"), ("point", "select"), ("mean", "weighted")])
def test_tolerance_chunks_match_fixed_iterations(omni, orc, gauge, method):
    """A tolerance stop runs the anchor iterations in graph-captured chunks with a device-side
    stop word; the iterate and the count must be those of the same number of iterations run
    one by one (up to the order of the FP32 atomic sums of the operator's right-hand side and
    the final sweep, which differ between any two solves)."""
    dims = (30, 26, 22)
    f = _field(dims, seed=16, sphere=4.0)
    dirs = omni.icosphere(3)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"]) if method != "plain" else None
    thr = float(np.percentile(curl[curl > 0], 85)) if method == "select" else 0.0
    kw = dict(method=method, threshold=thr, gauge=gauge, ref=(3, 0, 2))
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1000, tol=1e-6, **kw) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
        r2 = s.solve(f["ax"], f["ay"], f["az"], curl=curl)  # the captured chunk relaunched
    K = r.stats["iterations"]
    assert 20 < K < 1000 and r.stats["rel_change"] < 1e-6
    # the plain operator is cached per context; the others are rebuilt per solve, their
    # rows filled in atomic slot order
    tol_p = 1e-6 if method == "plain" else 1e-5
    assert abs(r2.stats["iterations"] - K) <= 1
    assert synthetic.relative_l2(r2.p, r.p, gauge="none") < tol_p
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=K, **kw) as s:
        q = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
    if method == "plain":
        np.testing.assert_array_equal(q.count, r.count)
    else:
        assert synthetic.relative_l2(q.count, r.count, gauge="none") < 1e-6
    assert synthetic.relative_l2(q.p, r.p, gauge="none") < tol_p


def test_bf16_gradient_storage(omni):
    dims = (24, 24, 24)
    f = _field(dims, seed=10)
    dirs = omni.icosphere(3)
    out = {}
    for g in ("f32", "bf16"):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=4, grad=g) as s:
            out[g] = s.solve(f["ax"], f["ay"], f["az"])
    np.testing.assert_array_equal(out["f32"].count, out["bf16"].count)
    err = synthetic.relative_l2(out["bf16"].p, out["f32"].p)
    assert 0 < err < 1e-2


@pytest.mark.parametrize("method", ["plain", "weighted", "select"])
def test_bf16_anchor_solver_matches_sweep_solver(omni, orc, method):
    """With BF16 storage the filling pass finds the anchors from bit 31 of each gathered
    entry; the anchor solver must then give the sweep solver's iterate (same BF16 field,
    same arithmetic up to the order of sums)."""
    dims = (22, 19, 17)
    f = _field(dims, seed=12, noise=0.1, sphere=4.0)
    dirs = omni.icosphere(3)
    p0 = _pinit(dims, seed=5)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 85)) if method == "select" else 0.0
    out = {}
    for solver in ("sweep", "anchor"):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=5, grad="bf16", method=method, threshold=thr,
                         solver=solver) as s:
            out[solver] = s.solve(f["ax"], f["ay"], f["az"], curl=None if method == "plain" else curl, p_init=p0)
    np.testing.assert_array_equal(out["anchor"].count > 0, out["sweep"].count > 0)
    assert synthetic.relative_l2(out["anchor"].count, out["sweep"].count, gauge="none") < 1e-6
    assert synthetic.relative_l2(out["anchor"].p, out["sweep"].p, gauge="none") < 1e-5


@pytest.mark.parametrize("method,mode", [("plain", 0), ("weighted", 2), ("select", 1)])
def test_bf16_storage_matches_oracle_on_the_rounded_field(omni, orc, method, mode):
    """BF16 storage packs (ax, ay, az, curl) into one 8-byte record.  Given the FP32 field, the
    BF16 solve must equal the FP64 oracle fed the same field and curl rounded to BF16 (the
    curl and, for the selected method, the threshold as k_pack stores them; up to the order
    of the sums: the FP32 parity bars).  Because the stored curl keeps every threshold
    decision, the BF16 solve visits the same segments as the FP32 one, and its distance from
    the FP64 oracle on the unrounded field -- the storage's own error -- stays small."""
    dims = (22, 19, 17)
    f = _field(dims, seed=31, noise=0.05, sphere=4.0)
    dirs = omni.icosphere(3)
    p0 = _pinit(dims, seed=6)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 85)) if method == "select" else 0.0
    K = 5
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=K, grad="bf16", method=method, threshold=thr) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], curl=None if method == "plain" else curl, p_init=p0)
    rb = {k: bf16_ref.round_bf16(f[k]) for k in ("ax", "ay", "az")}
    cb, thr_b = bf16_ref.curl_bf16(curl, thr if method == "select" else None)
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, rb["ax"], rb["ay"], rb["az"], p0, K, mode=mode, thr=thr_b,
                         curl=cb, precision="f64", nthreads=4)
    if method == "plain":
        np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
    else:
        np.testing.assert_array_equal(r.count.reshape(-1) > 0, ecnt > 0)
        assert synthetic.relative_l2(r.count, ecnt, gauge="none") < 1e-5
    tol = 2e-5 if method == "plain" else 1e-4
    assert synthetic.relative_l2(r.p, ep, gauge="none", weights=ecnt > 0) < tol
    # the storage's own error against the FP64 oracle on the FP32 field
    fp, fcnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, K, mode=mode, thr=thr, curl=curl,
                         precision="f64", nthreads=4)
    err = synthetic.relative_l2(r.p, fp, gauge="none", weights=fcnt > 0)
    assert err < 5e-3, err


def test_device_pointers_match_host(omni):
    torch = pytest.importorskip("torch")
    dims = (16, 14, 12)
    f = _field(dims, seed=11)
    dirs = omni.icosphere(3)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=3) as s:
        rh = s.solve(f["ax"], f["ay"], f["az"])
        t = [torch.from_numpy(f[k].reshape(-1)).cuda() for k in ("ax", "ay", "az")]
        rd = s.solve(*t)
    np.testing.assert_array_equal(rd.count.cpu().numpy(), rh.count)
    assert synthetic.relative_l2(rd.p.cpu().numpy(), rh.p, gauge="none") < 1e-6


def test_solve_into_caller_buffers(omni):
    """out=(p, count): pinned host arrays for host inputs, CUDA tensors for device inputs."""
    torch = pytest.importorskip("torch")
    dims = (15, 13, 11)
    f = _field(dims, seed=14)
    dirs = omni.icosphere(2)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=3) as s:
        ref = s.solve(f["ax"], f["ay"], f["az"])
        host = [torch.empty(s.V, dtype=torch.float32).pin_memory().numpy() for _ in range(2)]
        r = s.solve(f["ax"], f["ay"], f["az"], out=host)
        assert r.p.base is not None or r.p.size == s.V
        np.testing.assert_array_equal(host[1], ref.count.reshape(-1))
        assert synthetic.relative_l2(host[0], ref.p, gauge="none") < 1e-6
        t = [torch.from_numpy(f[k].reshape(-1)).cuda() for k in ("ax", "ay", "az")]
        dev = [torch.empty(s.V, device="cuda") for _ in range(2)]
        s.solve(*t, out=dev)
        np.testing.assert_array_equal(dev[1].cpu().numpy(), ref.count.reshape(-1))
        with pytest.raises(ValueError):
            s.solve(f["ax"], f["ay"], f["az"], out=[np.empty(3, np.float32)] * 2)


@pytest.mark.parametrize("method", ["plain", "select"])
def test_fp64_defect_correction_sweep(omni, orc, method):
    """sweep_fp64: the full sweep accumulates in FP64.  With one iteration the solve is that
    sweep alone, so its distance to the FP64 oracle drops below the FP32-accumulated one's."""
    dims = (26, 22, 19)
    f = _field(dims, seed=15, sphere=4.0)
    dirs = omni.icosphere(4)  # 642 directions: about a thousand contributions per voxel
    p0 = _pinit(dims)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.finfo(np.float32).max)
    mode = 0 if method == "plain" else 1
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 1, mode=mode, thr=thr, curl=curl,
                         precision="f64", nthreads=8)
    err = {}
    for fp64 in (False, True):
        for solver in ("anchor", "sweep"):
            with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1, method=method, threshold=thr, solver=solver,
                             sweep_fp64=fp64) as s:
                r = s.solve(f["ax"], f["ay"], f["az"], curl=curl if method == "select" else None, p_init=p0)
            err[(fp64, solver)] = synthetic.relative_l2(r.p, ep, gauge="none")
            if method == "plain":
                np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
    for solver in ("anchor", "sweep"):
        assert err[(True, solver)] < err[(False, solver)] < TOL_PN, err
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1, sweep_fp64=True, engine="bricks") as s:
        with pytest.raises(omni.Omni3DError):
            s.solve(f["ax"], f["ay"], f["az"])


def test_counts_deterministic(omni):
    dims = (20, 20, 20)
    f = _field(dims, seed=12)
    dirs = omni.icosphere(3)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2) as s:
        a = s.solve(f["ax"], f["ay"], f["az"])
        b = s.solve(f["ax"], f["ay"], f["az"])
    np.testing.assert_array_equal(a.count, b.count)
    assert synthetic.relative_l2(a.p, b.p, gauge="none") < 1e-6


def test_select_scattered_bad_voxels_and_fallback(omni, orc):
    """With half of the voxels above the threshold, segment starts are everywhere: the
    anchor operator is large but still exact; with a small anchor_max_links the solve runs
    the sweep form instead.  Both match the oracle."""
    dims = (16, 14, 12)
    f = _field(dims, seed=13, noise=0.3)
    dirs = omni.icosphere(2)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 50))
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], np.zeros(curl.size, np.float32), 3,
                         mode=1, thr=thr, curl=curl, precision="f64")
    for limit, used in ((0, 0), (1000, 1)):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=3, method="select", threshold=thr,
                         anchor_max_links=limit) as s:
            r = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
        assert r.stats["solver_used"] == used
        assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_SELECT


def test_batch_graph_matches_single_solves(omni, orc):
    """Snapshots of different sizes in one CUDA-graph launch give the same results as one
    solve each, and match the oracle."""
    torch = pytest.importorskip("torch")
    dirs = omni.icosphere(2)
    dims_list = [(12, 10, 8), (9, 14, 11), (16, 12, 10)]
    fields = [_field(d, seed=20 + i) for i, d in enumerate(dims_list)]
    solvers = [omni.Omni3D(d, f["spacing"], dirs, max_iter=4) for d, f in zip(dims_list, fields)]
    singles = [s.solve(f["ax"], f["ay"], f["az"]) for s, f in zip(solvers, fields)]
    dev = [tuple(torch.from_numpy(f[k].reshape(-1)).cuda() for k in ("ax", "ay", "az")) for f in fields]
    out = [(torch.empty(s.V, device="cuda"), torch.empty(s.V, device="cuda")) for s in solvers]
    with omni.Batch(solvers) as b:
        for _ in range(2):  # the second call relaunches the captured graph
            ps, cs, st = b.solve(dev, out=out)
            for i, (d, f) in enumerate(zip(dims_list, fields)):
                np.testing.assert_array_equal(cs[i].cpu().numpy(), singles[i].count)
                assert synthetic.relative_l2(ps[i].cpu().numpy(), singles[i].p, gauge="none") < 1e-6
        assert st["kernel_launches"] > 0
        hp, hc, _ = b.solve([(f["ax"], f["ay"], f["az"]) for f in fields])
    for i, (d, f) in enumerate(zip(dims_list, fields)):
        ep, ecnt = orc.solve(d, f["spacing"], dirs, f["ax"], f["ay"], f["az"], np.zeros(np.prod(d), np.float32), 4,
                             precision="f64")
        assert synthetic.relative_l2(hp[i], ep, gauge="none") < TOL_P_PLAIN
        np.testing.assert_array_equal(hc[i].reshape(-1), ecnt.astype(np.float32))
    for s in solvers:
        s.close()
