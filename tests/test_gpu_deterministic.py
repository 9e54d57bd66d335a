"""The bit-reproducible mode (params.deterministic): the sums the GPU would take in an
arbitrary order are taken in 64-bit fixed point, so that two solves of the same inputs give
the same bits -- for the anchor solver (its operator's rows, their iterations, the final
sweep), the tolerance-driven graph chunks and the sweep solver -- while the result stays
within the FP64 oracle's bars."""
import os

import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu

FLT_MAX = float(np.finfo(np.float32).max)
MODES = {"plain": 0, "select": 1, "weighted": 2}


def _bits(a):
    return np.ascontiguousarray(np.asarray(a, np.float32)).view(np.uint32)


@pytest.mark.parametrize("method,solver,tol", [("select", "anchor", 0.0), ("plain", "anchor", 1e-6),
                                               ("weighted", "anchor", 0.0), ("select", "sweep", 0.0)])
def test_deterministic_solves_give_identical_bits(omni, method, solver, tol):
    f = synthetic.blobs(n=96, count=6, sigma_range=(3.0, 9.0), noise=0.05, seed=80, sphere_radius=15.0)
    dims = f["dims"]
    dirs = omni.icosphere(4 if solver == "anchor" else 3)
    runs = []
    for _ in range(2):  # two contexts: nothing carried over between the solves
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=200 if tol else 8, tol=tol, method=method,
                         threshold=FLT_MAX, solver=solver, gauge="mean", deterministic=True) as s:
            runs.append(s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"]))
            again = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])  # and a second solve on one context
            np.testing.assert_array_equal(_bits(again.p), _bits(runs[-1].p))
    a, b = runs
    assert a.stats["iterations"] == b.stats["iterations"]
    np.testing.assert_array_equal(_bits(a.p), _bits(b.p))
    np.testing.assert_array_equal(_bits(a.count), _bits(b.count))
    # the same solve in the default mode agrees to its FP32 rounding
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=200 if tol else 8, tol=tol, method=method, threshold=FLT_MAX,
                     solver=solver, gauge="mean") as s:
        c = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])
    assert synthetic.relative_l2(c.p, a.p) < 1e-5


@pytest.mark.parametrize("method", ["plain", "select", "weighted"])
def test_deterministic_solve_matches_fp64_oracle(omni, orc, method):
    dims = (20, 18, 16)
    f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 5.0), noise=0.05, seed=81, sphere_radius=4.0)
    dirs = omni.icosphere(3)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 85)) if method == "select" else 0.0
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=4, method=method, threshold=thr, deterministic=True) as s:
        r = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], np.zeros(int(np.prod(dims)), np.float32),
                         4, mode=MODES[method], thr=thr, curl=curl, precision="f64", nthreads=os.cpu_count() or 1)
    if method == "plain":
        np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
    else:
        assert synthetic.relative_l2(r.count, ecnt, gauge="none") < 1e-6
    assert synthetic.relative_l2(r.p, ep, gauge="none", weights=ecnt > 0) < 2e-5


def test_deterministic_rejects_the_brick_engine(omni):
    with pytest.raises(omni.Omni3DError):
        omni.Omni3D((8, 8, 8), 1e-3, omni.icosphere(2), engine="bricks", deterministic=True)
