"""Batches whose members the one-graph form cannot run: the selected method (what the
reference's main runs; its operator is rebuilt for every field), per-member tolerances and
mask columns.  They run in the concurrent form (omni3d_batch_solve: each member by
omni3d_solve on its own stream, from a pool of host threads) and must give each member's
own solve, and the FP64 oracle's iterate for the members with a fixed iteration count."""
import os

import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu

MODES = {"plain": 0, "select": 1, "weighted": 2}


def test_batch_of_mixed_methods_and_tolerances(omni, orc):
    rng = np.random.default_rng(40)
    dirs = omni.icosphere(3)
    # (method, tolerance, iterations): the fixed-count selected members split their lines at
    # a threshold inside the curl's range; the members with a tolerance use a threshold above
    # every curl (lines split only at the mask) and the mean gauge, so that one constant is
    # free and the gauged change converges
    specs = [("select", 0.0, 4), ("select", 0.0, 6), ("select", 1e-5, 200), ("plain", 1e-5, 200), ("plain", 0.0, 5),
             ("weighted", 1e-4, 200)]
    members, fields, curls, thrs, gauges = [], [], [], [], []
    for m, (method, tol, K) in enumerate(specs):
        dims = tuple(int(d) for d in rng.integers(14, 27, 3))
        f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=41 + m,
                            sphere_radius=3.0)
        curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
        thr = 0.0
        if method == "select":
            thr = float(np.percentile(curl[curl > 0], 85)) if tol == 0.0 else float(np.finfo(np.float32).max)
        gauge = "mean" if tol > 0.0 else "none"
        fields.append(f)
        curls.append(curl)
        thrs.append(thr)
        gauges.append(gauge)
        members.append(omni.Omni3D(dims, f["spacing"], dirs, max_iter=K, tol=tol, method=method, threshold=thr,
                                   gauge=gauge))
    try:
        with omni.Batch(members) as b:
            args = [(f["ax"], f["ay"], f["az"]) for f in fields]
            masks = [f["mask"] for f in fields]
            ps, cs, st = b.solve(args, mask=masks)
            ps2, cs2, _ = b.solve(args, mask=masks)  # a second batch on the same contexts
        assert st["kernel_launches"] > 0 and st["iterations"] > 1
        for i, ((method, tol, K), f) in enumerate(zip(specs, fields)):
            dims = f["dims"]
            with omni.Omni3D(dims, f["spacing"], dirs, max_iter=K, tol=tol, method=method, threshold=thrs[i],
                             gauge=gauges[i]) as s:
                r = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])
            np.testing.assert_array_equal(np.asarray(cs[i]).reshape(-1) > 0, r.count.reshape(-1) > 0)
            assert synthetic.relative_l2(ps[i], r.p, gauge="none") < 1e-5, i
            assert synthetic.relative_l2(ps2[i], ps[i], gauge="none") < 1e-5, i
            if tol == 0.0:  # a fixed iteration count: the FP64 oracle's iterate
                ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"],
                                     np.zeros(int(np.prod(dims)), np.float32), K, mode=MODES[method], thr=thrs[i],
                                     curl=curls[i], precision="f64", nthreads=os.cpu_count() or 1)
                assert synthetic.relative_l2(np.asarray(ps[i]).reshape(-1), ep, gauge="none", weights=ecnt > 0) < 1e-4
            else:
                assert r.stats["rel_change"] < tol
    finally:
        for s in members:
            s.close()


def test_config4_batch_of_64_snapshots_selected_method(omni, orc):
    """Config 4's 64 snapshots (each dimension 32-160, vortex rings, 162 vertices, 20
    iterations) with the selected method, each member's threshold at the 90th percentile of
    its curl (lines split at the ring's core): the batch equals per-snapshot solves."""
    snaps = synthetic.batch_snapshots(count=64, lo=32, hi=160, seed=4)
    dirs = omni.icosphere(3)
    K = 20
    thrs = []
    for s in snaps:
        c = orc.curl(s["dims"], s["spacing"], s["ax"], s["ay"], s["az"], s["mask"])
        thrs.append(float(np.percentile(c[c > 0], 90)))
    solvers = [omni.Omni3D(s["dims"], s["spacing"], dirs, max_iter=K, method="select", threshold=t)
               for s, t in zip(snaps, thrs)]
    try:
        with omni.Batch(solvers) as b:
            ps, cs, st = b.solve([(s["ax"], s["ay"], s["az"]) for s in snaps])
        assert st["kernel_launches"] > 0
        for i in range(64):
            assert np.isfinite(ps[i]).all()
        for i in (0, 17, 40, 63):
            r = solvers[i].solve(snaps[i]["ax"], snaps[i]["ay"], snaps[i]["az"])
            np.testing.assert_array_equal(np.asarray(cs[i]).reshape(-1) > 0, r.count.reshape(-1) > 0)
            assert synthetic.relative_l2(ps[i], r.p, gauge="none") < 1e-5
    finally:
        for s in solvers:
            s.close()
