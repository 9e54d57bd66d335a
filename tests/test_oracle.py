"""The oracle pinned against the reference: its own functions compiled from source
(oracle/_ref, where the sources are staged) and the committed golden fixtures made from
them (tests/golden/make_golden.py).  CPU only."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_small.npz")


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _dims(g, c):
    return tuple(int(x) for x in g[c + "_dims"])


def _sp(g, c):
    return tuple(float(x) for x in g[c + "_spacing"])


def test_golden_plain_bit_exact(orc, gold):
    g = gold
    p, c = orc.solve(_dims(g, "plain"), _sp(g, "plain"), g["dirs"], g["plain_ax"], g["plain_ay"], g["plain_az"],
                     g["plain_p0"], 2)
    np.testing.assert_array_equal(_bits(c), _bits(g["plain_count"]))
    np.testing.assert_array_equal(_bits(p), _bits(g["plain_p"]))


def test_golden_select_bit_exact(orc, gold):
    g = gold
    d = _dims(g, "select")
    curl = orc.curl(d, _sp(g, "select"), g["select_ax"], g["select_ay"], g["select_az"], g["select_mask"])
    np.testing.assert_array_equal(_bits(curl), _bits(g["select_curl"]))
    p, c = orc.solve(d, _sp(g, "select"), g["dirs"], g["select_ax"], g["select_ay"], g["select_az"], g["select_p0"], 3,
                     mode=1, thr=float(g["select_thr"]), curl=curl)
    np.testing.assert_array_equal(_bits(c), _bits(g["select_count"]))
    np.testing.assert_array_equal(_bits(p), _bits(g["select_p"]))


def test_golden_weighted_bit_exact(orc, gold):
    g = gold
    d = _dims(g, "weighted")
    curl = orc.curl(d, _sp(g, "weighted"), g["weighted_ax"], g["weighted_ay"], g["weighted_az"], g["weighted_mask"])
    np.testing.assert_array_equal(_bits(curl), _bits(g["weighted_curl"]))
    p, c = orc.solve(d, _sp(g, "weighted"), g["dirs"], g["weighted_ax"], g["weighted_ay"], g["weighted_az"],
                     g["weighted_p0"], 3, mode=2, curl=curl)
    np.testing.assert_array_equal(_bits(c), _bits(g["weighted_count"]))
    np.testing.assert_array_equal(_bits(p), _bits(g["weighted_p"]))


@pytest.mark.parametrize("mode", [3, 4, 5, 6])
def test_golden_variant_walks_bit_exact(orc, gold, mode):
    """Fixed-boundary walks (modes 3, 4) and minimum-curl walks (modes 5, 6)."""
    g = gold
    d = _dims(g, "variants")
    p, c = orc.solve(d, _sp(g, "variants"), g["dirs"], g["variants_ax"], g["variants_ay"], g["variants_az"],
                     g["variants_p0"], 2, mode=mode, thr=float(g["variants_thr"]), curl=g["variants_curl"])
    np.testing.assert_array_equal(_bits(c), _bits(g["variants_count_mode%d" % mode]))
    np.testing.assert_array_equal(_bits(p), _bits(g["variants_p_mode%d" % mode]))


def test_golden_centre_integration_bit_exact(orc, gold):
    """initialIntegration.cpp: FP64 p integrated outward from the centre voxel."""
    g = gold
    p = orc.centre_integration(_dims(g, "centre"), _sp(g, "centre"), g["centre_ax"], g["centre_ay"], g["centre_az"],
                               rho=1.25, pref=2.5)
    np.testing.assert_array_equal(p.view(np.uint64), g["centre_p"].view(np.uint64))


def test_centre_integration_matches_reference(orc, reflib):
    from omni3d import synthetic

    for dims in [(12, 10, 8), (7, 9, 11), (2, 3, 2), (16, 5, 13)]:
        f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=sum(dims))
        a = orc.centre_integration(dims, f["spacing"], f["ax"], f["ay"], f["az"], rho=1.2, pref=3.5)
        b = reflib.initial_integration(dims, f["spacing"], f["ax"], f["ay"], f["az"], rho=1.2, pref=3.5)
        np.testing.assert_array_equal(a.view(np.uint64), b.view(np.uint64))


def test_golden_line_spacing(orc, gold):
    g = gold
    d = _dims(g, "ls07")
    p, c = orc.solve(d, _sp(g, "ls07"), g["dirs"], g["ls07_ax"], g["ls07_ay"], g["ls07_az"],
                     np.zeros(np.prod(d), np.float32), 2, ls=0.7)
    np.testing.assert_array_equal(_bits(c), _bits(g["ls07_count"]))
    np.testing.assert_array_equal(_bits(p), _bits(g["ls07_p"]))


def test_golden_cpu_twin_loop(orc, gold):
    """The reference's own CPU loop: no pole guard (poles give NaN offsets and are skipped),
    lattice without the line-spacing division, normalisation where count > 1."""
    g = gold
    d = _dims(g, "cputwin")
    V = int(np.prod(d))
    p = np.zeros(V, np.float32)
    pn = np.zeros(V, np.float32)
    cnt = np.zeros(V, np.float32)
    for _ in range(2):
        cnt[:] = 0
        spn, scnt = orc.sweep(d, _sp(g, "cputwin"), g["dirs"], g["cputwin_ax"], g["cputwin_ay"], g["cputwin_az"], p,
                              cpu_twin=True)
        pn += spn
        cnt += scnt
        m = cnt > 1
        p[m] = (pn[m] / cnt[m]).astype(np.float32)
        pn[m] = 0
    np.testing.assert_array_equal(_bits(cnt), _bits(g["cputwin_count"]))
    np.testing.assert_array_equal(_bits(p), _bits(g["cputwin_p"]))


def test_oracle_matches_reference_functions(orc, reflib):
    """Direct comparison with the reference functions on a non-cubic grid, all three methods."""
    from omni3d import synthetic
    from omni3d.solver import icosphere

    dims = (17, 13, 11)
    dirs = icosphere(3)
    f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=11, sphere_radius=3.0)
    p0 = np.zeros(np.prod(dims), np.float32)
    p0[: dims[0]] = 0.25
    a, ca = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2)
    b, cb = reflib.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2)
    np.testing.assert_array_equal(_bits(ca), _bits(cb))
    np.testing.assert_array_equal(_bits(a), _bits(b))
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 70))
    a, ca = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2, mode=1, thr=thr, curl=curl)
    b, cb = reflib.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2, mode=1, thr=thr, curl=curl)
    np.testing.assert_array_equal(_bits(ca), _bits(cb))
    np.testing.assert_array_equal(_bits(a), _bits(b))
    a, ca = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2, mode=2, curl=curl)
    b, cb = reflib.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2, mode=2, curl=curl)
    np.testing.assert_array_equal(_bits(ca), _bits(cb))
    np.testing.assert_array_equal(_bits(a), _bits(b))


def test_cross2point_matches_reference(orc, reflib):
    """Random offsets and directions, including exact-zero components (cases 1-6)."""
    rng = np.random.default_rng(0)
    dims = (13, 9, 11)
    dirs = [rng.normal(size=3) for _ in range(60)]
    dirs += [np.array(v, float) for v in ([0, 1, 1], [1, 0, 1], [1, 1, 0], [0, 0, 1], [0, 1, 0], [1, 0, 0],
                                          [0, -1, 2], [-2, 0, 1], [3, -1, 0], [0, 0, -1], [0, -1, 0], [-1, 0, 0])]
    n = 0
    for k in dirs:
        k = (k / np.linalg.norm(k)).astype(np.float32)
        for _ in range(40):
            xyz = rng.uniform(-9, 9, 3).astype(np.float32)
            i = np.zeros(3, np.int32)
            o = np.zeros(3, np.int32)
            import ctypes as C

            ra = orc.lib.orc_cross2point(*dims, float(xyz[0]), float(xyz[1]), float(xyz[2]), float(k[0]),
                                         float(k[1]), float(k[2]), i.ctypes.data_as(C.POINTER(C.c_int)),
                                         o.ctypes.data_as(C.POINTER(C.c_int)))
            rb, io = reflib.cross2point(dims, xyz, k)
            assert ra == rb
            np.testing.assert_array_equal(np.concatenate([i, o]), io)
            n += 1
    assert n == len(dirs) * 40


def test_calindex_is_bijection_on_boundary(orc, reflib):
    """The reference's boundary numbering is a bijection on the boundary voxels, so its
    `nin != nout` test equals `entry voxel != exit voxel`."""
    for dims in [(12, 10, 8), (5, 7, 3), (32, 32, 32)]:
        a = orc.calindex(dims)
        b = reflib.calindex(dims)
        np.testing.assert_array_equal(a, b)
        X, Y, Z = dims
        v = np.arange(X * Y * Z)
        i, j, k = v % X, (v // X) % Y, v // (X * Y)
        surf = (i == 0) | (i == X - 1) | (j == 0) | (j == Y - 1) | (k == 0) | (k == Z - 1)
        assert len(np.unique(a[surf])) == surf.sum()
        assert (a[~surf] == -1).all()


def test_fp64_oracle_close_to_fp32(orc, gold):
    """The FP64 oracle follows the same discrete geometry: counts equal, values close."""
    g = gold
    d = _dims(g, "plain")
    p32, c32 = orc.solve(d, _sp(g, "plain"), g["dirs"], g["plain_ax"], g["plain_ay"], g["plain_az"], g["plain_p0"], 2)
    p64, c64 = orc.solve(d, _sp(g, "plain"), g["dirs"], g["plain_ax"], g["plain_ay"], g["plain_az"], g["plain_p0"], 2,
                         precision="f64")
    np.testing.assert_array_equal(c32, c64.astype(np.float32))
    assert np.linalg.norm(p32 - p64) / np.linalg.norm(p64) < 1e-5


def test_oracle_threads_change_only_sum_order(orc, gold):
    g = gold
    d = _dims(g, "plain")
    a, ca = orc.solve(d, _sp(g, "plain"), g["dirs"], g["plain_ax"], g["plain_ay"], g["plain_az"], g["plain_p0"], 2)
    b, cb = orc.solve(d, _sp(g, "plain"), g["dirs"], g["plain_ax"], g["plain_ay"], g["plain_az"], g["plain_p0"], 2,
                      nthreads=3)
    np.testing.assert_array_equal(ca, cb)
    assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-5


def test_oracle_converges_toward_analytic(orc):
    """Config-1 shape at reduced size: the iteration approaches the analytic field."""
    from omni3d import synthetic
    from omni3d.solver import icosphere

    f = synthetic.gaussian(n=16, sigma_cells=3.0, noise=0.0)
    dirs = icosphere(3)
    errs = []
    for k in (1, 4):
        p, c = orc.solve(f["dims"], f["spacing"], dirs, f["ax"], f["ay"], f["az"], np.zeros(16 ** 3, np.float32), k,
                         precision="f64")
        errs.append(synthetic.relative_l2(p, f["p_true"]))
    assert errs[1] < errs[0] and errs[1] < 0.1


@pytest.mark.parametrize("case,mode", [("plain", 0), ("select", 1), ("weighted", 2), ("variants", 4),
                                       ("variants", 6)])
def test_cached_fp64_solve_equals_fp64_solve(orc, gold, case, mode):
    """The FP64 solve with the lines traced once (the fixed-point oracle of the full-size
    parity tests) is the re-tracing FP64 solve up to the order of its sums, and it stops at
    the first iteration whose gauged relative change is below tol."""
    g = gold
    d = _dims(g, case)
    ax, ay, az = g[case + "_ax"], g[case + "_ay"], g[case + "_az"]
    curl = g[case + "_curl"] if case + "_curl" in g else None
    thr = float(g[case + "_thr"]) if case + "_thr" in g else 0.0
    p0 = g[case + "_p0"]
    a, ca = orc.solve(d, _sp(g, case), g["dirs"], ax, ay, az, p0, 3, mode=mode, thr=thr, curl=curl, precision="f64")
    b, cb, its, rel, saved = orc.solve_cached(d, _sp(g, case), g["dirs"], ax, ay, az, p0, 3, mode=mode, thr=thr,
                                              curl=curl, nthreads=3, save_at=(1, 3))
    assert its == 3
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()
    assert np.abs(ca - cb).max() <= 1e-12 * np.abs(ca).max()
    np.testing.assert_array_equal(saved[3], b)
    a1, _ = orc.solve(d, _sp(g, case), g["dirs"], ax, ay, az, p0, 1, mode=mode, thr=thr, curl=curl, precision="f64")
    assert np.abs(a1 - saved[1]).max() <= 1e-12 * np.abs(a1).max()
    _, _, its_tol, rel_tol = orc.solve_cached(d, _sp(g, case), g["dirs"], ax, ay, az, p0, 200, mode=mode, thr=thr,
                                              curl=curl, tol=1e-3)
    assert rel_tol < 1e-3 and its_tol < 200


def test_golden_sor_restatement_bit_exact(orc, gold):
    """The restated sor3D iteration (used to count the reference baseline's steps at sizes
    where the reference itself would run for hours) equals sor3D bit for bit, from the
    golden right-hand side of calRHS."""
    g = gold
    d = _dims(g, "sor")
    rhs = g["sor_rhs"]
    assert np.count_nonzero(rhs) > 0.9 * rhs.size  # calRHS returns its output (line 10 left out)
    for k in (2, 10):
        p = orc.sor_steps(d, rhs, np.zeros(rhs.size), k, nthreads=2)
        np.testing.assert_array_equal(p.view(np.uint64), np.ascontiguousarray(g["sor_p%d" % k]).view(np.uint64))


def test_sor_reference_calrhs_and_residual(orc, reflib):
    """The staged calRHS returns a nonzero right-hand side, and sor3D moves toward its fixed
    point: the distance from the conjugate-gradient solution of the same discrete problem
    falls with the step count, and the step count the restatement reports is where the
    reference code itself first meets 1e-3."""
    from omni3d import synthetic

    f = synthetic.blobs(n=16, count=3, sigma_range=(1.0, 3.0), noise=0.05, seed=3, spacing=1e-3 * 16)
    d = f["dims"]
    rhs = reflib.calrhs(d, f["spacing"], f["ax"], f["ay"], f["az"])
    assert np.count_nonzero(rhs) > 0.9 * rhs.size
    conv, cg = orc.sor_converged(d, rhs, tol=1e-13)
    assert cg > 10
    errs = [synthetic.relative_l2(reflib.sor(d, f["spacing"], f["ax"], f["ay"], f["az"], k, 0.0), conv, gauge="mean")
            for k in (10, 100, 400)]
    assert errs[0] > errs[1] > errs[2]
    n, err = orc.sor_steps_to(d, rhs, conv, 1e-3, check=8)
    assert n > 0 and n % 2 == 0 and err <= 1e-3
    at = synthetic.relative_l2(reflib.sor(d, f["spacing"], f["ax"], f["ay"], f["az"], n, 0.0), conv, gauge="mean")
    short = synthetic.relative_l2(reflib.sor(d, f["spacing"], f["ax"], f["ay"], f["az"], n - 2, 0.0), conv,
                                  gauge="mean")
    assert at <= 1e-3 < short


def test_anderson_fixed_point_is_the_iteration_limit(orc, gold):
    """The accelerated FP64 fixed point (the bench's FP64 reference) is where the plain FP64
    iteration goes: the same voxels, the same mean-gauged field.  As in the bench, the
    threshold lies above every curl, so segments split only at the mask and the iteration
    couples every receiving voxel (one free constant).  (A threshold that cuts the domain
    into islands leaves one free constant per island, set by the transient, and the
    accelerated limit need not equal the plain iteration's.)"""
    from omni3d import synthetic

    g = gold
    d = _dims(g, "select")
    args = (d, _sp(g, "select"), g["dirs"], g["select_ax"], g["select_ay"], g["select_az"])
    kw = dict(mode=1, thr=float(np.finfo(np.float32).max), curl=g["select_curl"])
    p, c, its, rel = orc.solve_cached(*args, np.zeros(int(np.prod(d)), np.float32), 2000, tol=1e-12, **kw)
    q, cq, ev, res = orc.fixed_point(*args, tol=1e-12, **kw)
    assert rel < 1e-12 and res < 1e-12 and ev < its
    np.testing.assert_array_equal(c > 0, cq > 0)
    assert synthetic.relative_l2(q, p, gauge="mean", weights=c > 0) < 1e-9


@pytest.mark.parametrize("mode", [0, 1, 2, 4, 6])
def test_fp64_adjoint_of_every_mode_is_the_transpose(orc, gold, mode):
    """orc_adjoint_modes_f64 (curl held fixed) is the transpose of the FP64 iteration: the
    plain mode equals the plain adjoint, and <g, J h> = <J^T g, h> with J h the FP64 solve's
    response to h (the map is affine in the field for a fixed curl)."""
    g_ = gold
    d = _dims(g_, "select")
    sp = _sp(g_, "select")
    ax, ay, az = (g_["select_" + k] for k in ("ax", "ay", "az"))
    curl = g_["select_curl"]
    thr = float(g_["select_thr"]) if mode in (1, 4) else 0.0
    V = int(np.prod(d))
    rng = np.random.default_rng(11)
    g = rng.normal(size=V)
    K = 3
    ga = orc.adjoint_modes(d, sp, g_["dirs"], K, g, mode=mode, thr=thr, curl=curl)
    if mode == 0:
        ref = orc.adjoint(d, sp, g_["dirs"], K, g)
        for a, b in zip(ga, ref):
            assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    p0 = np.zeros(V, np.float32)
    h = [(rng.normal(size=V) * np.abs(c).max()).astype(np.float32) for c in (ax, ay, az)]
    pp, _ = orc.solve(d, sp, g_["dirs"], ax + h[0], ay + h[1], az + h[2], p0, K, mode=mode, thr=thr, curl=curl,
                      precision="f64")
    pm, _ = orc.solve(d, sp, g_["dirs"], ax - h[0], ay - h[1], az - h[2], p0, K, mode=mode, thr=thr, curl=curl,
                      precision="f64")
    lhs = float(np.dot(g, (pp - pm) / 2))
    rhs = float(sum(np.dot(a, b.astype(np.float64)) for a, b in zip(ga, h)))
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)
