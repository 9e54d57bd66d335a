"""The benchmark configurations at their full grid sizes against the FP64 oracle.

The FP64 oracle cannot sweep all 642 vertices at 256^3 in test time, but the cost of an
iteration is proportional to the directions swept, and every property that depends on the
grid size -- 442-voxel lines, the masked sphere's segment splits, about a thousand
contributions per voxel, long compensated scans -- is there with any subset of them.  So
the GPU solve and the oracle (orc.solve_cached: the reference iteration in FP64 with the
lines traced once) run the same evenly spaced subset of the 642 vertices on the full grid:

  config 3  256^3, 8 seeded Gaussian blobs, 5 % noise, sphere of radius 40 cells masked
            out, the selected method with a threshold above every curl (lines split only
            at the mask), 16 of the 642 vertices
  config 2  128^3 Taylor-Green on [0, 2pi)^3, 10 % noise, the plain method, 32 of the 642
            vertices

after K = 8 iterations (the benchmark's count) and K = 16, starting from zero with the
reference's seeded first sweep (K:8811).  Bars: the same voxels receive contributions,
counts within 1e-5 relative L2 (exact integers for the plain method), p within 1e-4
relative L2 over those voxels (no gauge: both sides run the same iteration).
"""
import os

import bf16_ref
import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu

FLT_MAX = float(np.finfo(np.float32).max)
TOL_P = 1e-4
TOL_COUNT = 1e-5


def _subset(dirs, n):
    idx = np.linspace(0, len(dirs) - 1, n).round().astype(int)
    return np.ascontiguousarray(dirs[idx])


def _check(r, ep, ecnt, exact_counts):
    cnt = r.count.reshape(-1)
    sel = ecnt > 0
    np.testing.assert_array_equal(cnt > 0, sel)
    if exact_counts:
        np.testing.assert_array_equal(cnt, ecnt.astype(np.float32))
    else:
        assert synthetic.relative_l2(cnt, ecnt, gauge="none") < TOL_COUNT
    err = synthetic.relative_l2(r.p.reshape(-1), ep, gauge="none", weights=sel)
    assert err < TOL_P, err
    return err


def test_config3_blobs256_select_vs_fp64_oracle_on_a_direction_subset(omni, orc):
    f = synthetic.blobs(n=256, count=8, sigma_range=(8.0, 24.0), noise=0.05, seed=0, spacing=1e-3,
                        sphere_radius=40.0)
    dims = f["dims"]
    sub = _subset(omni.icosphere(4), 16)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    p0 = np.zeros(int(np.prod(dims)), np.float32)
    _, ecnt, its, _, saved = orc.solve_cached(dims, f["spacing"], sub, f["ax"], f["ay"], f["az"], p0, 16, mode=1,
                                              thr=FLT_MAX, curl=curl, nthreads=os.cpu_count() or 1, save_at=(8, 16))
    assert its == 16
    # the mask splits lines: voxels inside the sphere receive nothing
    assert (ecnt[f["mask"].reshape(-1) == 0] == 0).all() and (ecnt > 0).mean() > 0.9
    for K in (8, 16):
        with omni.Omni3D(dims, f["spacing"], sub, max_iter=K, method="select", threshold=FLT_MAX) as s:
            r = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])
        assert r.stats["iterations"] == K
        _check(r, saved[K], ecnt, exact_counts=False)


def test_config3_blobs256_select_bf16_storage_vs_fp64_oracle_on_the_stored_field(omni, orc):
    """The same configuration with BF16 storage (one 8-byte record per voxel): K = 8 against the
    FP64 oracle fed the field and curl as stored (tests/bf16_ref.py), and against the FP64
    oracle on the FP32 field (the storage's own error at this size)."""
    f = synthetic.blobs(n=256, count=8, sigma_range=(8.0, 24.0), noise=0.05, seed=0, spacing=1e-3,
                        sphere_radius=40.0)
    dims = f["dims"]
    sub = _subset(omni.icosphere(4), 16)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    p0 = np.zeros(int(np.prod(dims)), np.float32)
    K = 8
    with omni.Omni3D(dims, f["spacing"], sub, max_iter=K, method="select", threshold=FLT_MAX, grad="bf16") as s:
        r = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])
    rb = {k: bf16_ref.round_bf16(f[k]) for k in ("ax", "ay", "az")}
    cb, thr_b = bf16_ref.curl_bf16(curl, FLT_MAX)
    ep, ecnt, _, _ = orc.solve_cached(dims, f["spacing"], sub, rb["ax"], rb["ay"], rb["az"], p0, K, mode=1, thr=thr_b,
                                      curl=cb, nthreads=os.cpu_count() or 1)
    _check(r, ep, ecnt, exact_counts=False)
    fp, fcnt, _, _ = orc.solve_cached(dims, f["spacing"], sub, f["ax"], f["ay"], f["az"], p0, K, mode=1, thr=FLT_MAX,
                                      curl=curl, nthreads=os.cpu_count() or 1)
    np.testing.assert_array_equal(fcnt > 0, ecnt > 0)
    err = synthetic.relative_l2(r.p.reshape(-1), fp, gauge="mean", weights=fcnt > 0)
    assert err < 2e-3, err


def test_config2_taylor_green128_plain_vs_fp64_oracle_on_a_direction_subset(omni, orc):
    f = synthetic.taylor_green(n=128, noise=0.10, seed=2)
    dims = f["dims"]
    sub = _subset(omni.icosphere(4), 32)
    p0 = np.zeros(int(np.prod(dims)), np.float32)
    _, ecnt, its, _, saved = orc.solve_cached(dims, f["spacing"], sub, f["ax"], f["ay"], f["az"], p0, 16, mode=0,
                                              nthreads=os.cpu_count() or 1, save_at=(8, 16))
    assert its == 16
    for K in (8, 16):
        with omni.Omni3D(dims, f["spacing"], sub, max_iter=K) as s:
            r = s.solve(f["ax"], f["ay"], f["az"])
        _check(r, saved[K], ecnt, exact_counts=True)
