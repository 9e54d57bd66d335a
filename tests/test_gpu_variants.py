"""The variants the reference keeps beside its three methods, on the GPU against the oracle
(itself pinned bit for bit to the reference functions, tests/test_oracle.py):

  weighted_fixed_bc   bodyIntegralInnerWeightedFixedBC (K:2136-2279), walk rule 1
  select_fixed_bc     bodyIntegralInnerSelectFixedBC (K:2538-2796), walk rule 2
  mini_curl           bodyIntegralInnerMiniCurl (K:2797-2936), walk rule 3
  weighted_mini_curl  bodyIntegralInnerWeightedMiniCurl (K:2937-3085), walk rule 3

The staircases are bit-exact (the minimum-curl ones after a solve: they follow the field);
sums agree with the FP64 oracle within the selected method's bound."""
import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu

TOL_P = 1e-4
VARIANTS = [("weighted_fixed_bc", 3, 1), ("select_fixed_bc", 4, 2), ("mini_curl", 5, 3), ("weighted_mini_curl", 6, 3)]


def _field(dims, seed, sphere=None, noise=0.05):
    return synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 5.0), noise=noise, seed=seed, spacing=1e-3,
                           sphere_radius=sphere)


def _pinit(dims, seed=1):
    nx, ny, nz = dims
    rng = np.random.default_rng(seed)
    p = np.zeros((nz, ny, nx), np.float32)
    p[:, 0, :] = rng.normal(0, 0.5, (nz, nx)).astype(np.float32)
    return p


@pytest.mark.parametrize("method,mode,rule", VARIANTS)
def test_variant_staircases_bit_exact(omni, orc, match_lines, method, mode, rule):
    dims = (17, 14, 12)
    f = _field(dims, seed=50 + mode, sphere=3.0)
    dirs = omni.icosphere(3)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 75))
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1, method=method, threshold=thr) as s:
        s.solve(f["ax"], f["ay"], f["az"], curl=curl)
        got = s.line_table().astype(np.int64)
        got[:, 0] &= 0xFFFFFFFF
        got[:, 1] &= 0xFFFFFFFF
        X, Y, Z = dims
        exp, walks = [], []
        stopped = 0
        for d in range(len(dirs)):
            valid, inout, nsteps, xyz = orc.trace_direction(dims, 1.0, dirs[d])
            for pt in np.nonzero(valid)[0]:
                io = inout[pt]
                e = io[0] + io[1] * X + io[2] * X * Y
                x = io[3] + io[4] * X + io[5] * X * Y
                ax = orc.walk(dims, io, xyz[pt], dirs[d], rule=rule, curl=curl, allow_early_stop=True)
                exp.append((e, x, d, len(ax)))
                walks.append(ax)
                stopped += len(ax) < abs(io[3] - io[0]) + abs(io[4] - io[1]) + abs(io[5] - io[2])
        # the same (entry, exit, direction, steps) rows, in the library's own order
        at = match_lines(got, np.array(exp, np.int64).reshape(-1, 4))
        for k in range(0, len(exp), 7):
            assert any(np.array_equal(s.line_steps(i), walks[k]) for i in at[k]), k
        if rule in (1, 2):
            assert stopped > 0  # lines that would enter the j = 0 face stop before it


@pytest.mark.parametrize("solver", ["sweep", "anchor"])
@pytest.mark.parametrize("method,mode,rule", VARIANTS)
def test_variant_solve_matches_oracle(omni, orc, method, mode, rule, solver):
    dims = (19, 16, 13)
    f = _field(dims, seed=60 + mode, sphere=3.5, noise=0.1)
    dirs = omni.icosphere(3)
    p0 = _pinit(dims, seed=mode)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 80))
    niter = 3
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=niter, method=method, threshold=thr, solver=solver) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"], p_init=p0)  # curl computed on the device
        assert r.stats["walk_errors"] == 0
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, niter, mode=mode, thr=thr, curl=curl,
                         precision="f64")
    assert np.isfinite(r.p).all()
    if mode == 5:  # unit weights: integer counts
        np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
    else:
        np.testing.assert_array_equal(r.count.reshape(-1) > 0, ecnt > 0)
        assert synthetic.relative_l2(r.count, ecnt, gauge="none") < 1e-5
    assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P
    if rule in (1, 2):  # the fixed boundary: the j = 0 face keeps p_init wherever nothing reaches it
        face = r.count[:, 0, :] == 0
        np.testing.assert_array_equal(r.p[:, 0, :][face], p0[:, 0, :][face])


def test_minimum_curl_paths_follow_the_field(omni, orc):
    """Two fields solved by one context: the staircases are re-walked for each."""
    dims = (15, 13, 12)
    dirs = omni.icosphere(2)
    with omni.Omni3D(dims, 1e-3, dirs, max_iter=2, method="mini_curl") as s:
        for seed in (70, 71):
            f = _field(dims, seed=seed)
            curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
            r = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
            ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], np.zeros(np.prod(dims), np.float32),
                                 2, mode=5, curl=curl, precision="f64")
            np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
            assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P
            assert r.stats["n_units"] == s.geometry_info()["n_units"]


def test_variant_rejections(omni):
    dims = (12, 12, 12)
    f = _field(dims, seed=72)
    dirs = omni.icosphere(2)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2, method="mini_curl", engine="bricks") as s:
        with pytest.raises(omni.Omni3DError):
            s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2, method="select_fixed_bc", threshold=1e30,
                     engine="bricks") as s:
        r = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])
        assert r.stats["engine_used"] == 2
    # the adjoint takes every method (curl held fixed; checked against the FP64 oracle in
    # tests/test_gpu_adjoint.py)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2, method="weighted_fixed_bc") as s:
        s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])
        assert all(np.isfinite(g).all() for g in s.adjoint(np.ones(s.V, np.float32)))
