"""The survey's benchmark configurations at their stated shapes (seeded synthetic inputs in
place of measured fields), run through the C ABI on the GPU.

  config 1  32^3 Gaussian, 5 % noise, 162 vertices, plain, corner reference point,
            relative-change tolerance 1e-6, at most 500 iterations
  config 2  128^3 Taylor-Green on [0, 2pi)^3, 10 % noise, 642 vertices, tolerance 1e-6,
            at most 1000 iterations
  config 3  256^3 Gaussian blobs, 5 % noise, sphere of radius 40 masked out, 642 vertices,
            the selected method split only at the mask, 8 iterations (the benchmark workload)
  config 4  64 snapshots of uneven sizes (each dimension 32-160), vortex rings, 162
            vertices, solved in one CUDA-graph launch
  config 5  the adjoint at 96^3, 642 vertices, exactly 200 iterations, loss
            ||P(g) - p_target||^2 + a surface-force integral over a sphere of radius 20

Where the FP64 oracle finishes in seconds it is the reference (config 1 at full size;
configs 2 and 5 at reduced size); at full size the checks are properties that do not
depend on size: both solver forms reach the same fixed point, the fixed point satisfies one
more reference iteration, the batch equals per-snapshot solves, the gradient matches
central differences.
"""
import os

import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu


def test_config1_gaussian32_plain_to_tolerance(omni, orc):
    f = synthetic.gaussian(n=32, sigma_cells=6.0, noise=0.05, seed=1)
    dims = f["dims"]
    dirs = omni.icosphere(3)  # 162 vertices, the vertex set of GridIcosahedronDivide3.dat
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=500, tol=1e-6, gauge="point", ref=(0, 0, 0)) as s:
        r = s.solve(f["ax"], f["ay"], f["az"])
    K = r.stats["iterations"]
    assert 1 < K < 500 and r.stats["rel_change"] < 1e-6
    p = r.p.reshape(-1)
    assert p[0] == 0.0
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], np.zeros(np.prod(dims), np.float32), K,
                         precision="f64", nthreads=os.cpu_count() or 1)
    np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
    assert synthetic.relative_l2(p, ep, gauge="point", ref=0) < 1e-4
    # the reconstruction approaches the analytic field (the noise bounds how closely)
    err = synthetic.relative_l2(p, f["p_true"], gauge="point", ref=0)
    assert err < 0.1, err


def test_config2_taylor_green128_fixed_point(omni, orc):
    f = synthetic.taylor_green(n=128, noise=0.10, seed=2)
    dims = f["dims"]
    dirs = omni.icosphere(4)  # 642 vertices
    res = {}
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1000, tol=1e-6, gauge="mean") as s:
        res["anchor"] = s.solve(f["ax"], f["ay"], f["az"])
    K = res["anchor"].stats["iterations"]
    assert res["anchor"].stats["rel_change"] < 1e-6 and K < 1000
    # the reference loop form (one full sweep per iteration, FP32 atomic sums whose rounding
    # floor lies near this tolerance) run for the same number of iterations
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=K, gauge="mean", solver="sweep") as s:
        res["sweep"] = s.solve(f["ax"], f["ay"], f["az"])
    assert synthetic.relative_l2(res["anchor"].p, res["sweep"].p) < 1e-5
    # the fixed point: one more reference iteration from it changes p by about the tolerance
    p = res["anchor"].p.reshape(-1)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1, gauge="mean", seed_first_iteration=False) as s:
        p1 = s.solve(f["ax"], f["ay"], f["az"], p_init=p).p
    assert synthetic.relative_l2(p1, p) < 1e-5
    err = synthetic.relative_l2(p, f["p_true"])
    assert err < 0.2, err
    # the same field at reduced size against the FP64 oracle
    g = synthetic.taylor_green(n=32, noise=0.10, seed=2)
    d3 = omni.icosphere(3)
    with omni.Omni3D(g["dims"], g["spacing"], d3, max_iter=3) as s:
        r = s.solve(g["ax"], g["ay"], g["az"])
    ep, ecnt = orc.solve(g["dims"], g["spacing"], d3, g["ax"], g["ay"], g["az"], np.zeros(32 ** 3, np.float32), 3,
                         precision="f64", nthreads=os.cpu_count() or 1)
    np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
    assert synthetic.relative_l2(r.p, ep, gauge="none") < 2e-5


def test_config3_blobs256_masked_select(omni):
    """The benchmark workload at full size: 256^3, 642 vertices, the selected method with a
    threshold above every curl (lines split only at the masked sphere of radius 40), 8
    iterations.  Properties that hold at any size: the anchor solver gives the reference
    loop's iterate (8 full sweeps), the masked sphere receives nothing, both storage forms
    see the same lines, and the result approaches the analytic field."""
    f = synthetic.blobs(n=256, count=8, sigma_range=(8.0, 24.0), noise=0.05, seed=3, spacing=1e-3,
                        sphere_radius=40.0)
    dims = f["dims"]
    dirs = omni.icosphere(4)
    thr = float(np.finfo(np.float32).max)
    out = {}
    for solver in ("anchor", "sweep"):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=8, method="select", threshold=thr, gauge="mean",
                         solver=solver) as s:
            out[solver] = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])
    a, b = out["anchor"], out["sweep"]
    np.testing.assert_array_equal(a.count > 0, b.count > 0)
    assert synthetic.relative_l2(a.count, b.count, gauge="none") < 1e-5
    assert synthetic.relative_l2(a.p, b.p) < 1e-5
    inside = f["mask"].reshape(-1) == 0
    assert inside.sum() > 200_000 and (a.count.reshape(-1)[inside] == 0).all()
    outside = ~inside
    err = synthetic.relative_l2(a.p.reshape(-1)[outside], f["p_true"].reshape(-1)[outside])
    assert err < 0.05, err
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=8, method="select", threshold=thr, gauge="mean",
                     grad="bf16") as s:
        c = s.solve(f["ax"], f["ay"], f["az"], mask=f["mask"])
    np.testing.assert_array_equal(c.count > 0, a.count > 0)
    assert synthetic.relative_l2(c.p, a.p) < 1e-2


def test_config4_batch_of_64_uneven_snapshots(omni):
    snaps = synthetic.batch_snapshots(count=64, lo=32, hi=160, seed=4)
    dirs = omni.icosphere(3)  # 162 vertices
    K = 20
    solvers = [omni.Omni3D(s["dims"], s["spacing"], dirs, max_iter=K) for s in snaps]
    try:
        with omni.Batch(solvers) as b:
            ps, cs, st = b.solve([(s["ax"], s["ay"], s["az"]) for s in snaps])
            ps2, cs2, _ = b.solve([(s["ax"], s["ay"], s["az"]) for s in snaps])  # relaunch of the graph
        assert st["kernel_launches"] > 0
        for i in range(64):
            assert np.isfinite(ps[i]).all()
            np.testing.assert_array_equal(cs2[i], cs[i])
        # a sample of members solved one by one
        for i in (0, 17, 40, 63):
            r = solvers[i].solve(snaps[i]["ax"], snaps[i]["ay"], snaps[i]["az"])
            np.testing.assert_array_equal(np.asarray(cs[i]).reshape(-1), r.count.reshape(-1))
            assert synthetic.relative_l2(ps[i], r.p, gauge="none") < 1e-6
            assert synthetic.relative_l2(ps[i], snaps[i]["p_true"]) < 0.3
    finally:
        for s in solvers:
            s.close()


@pytest.mark.parametrize("method", ["plain", "select"])
def test_config5_adjoint96_matches_finite_differences(omni, orc, method):
    """Config 5 for the plain method and for the selected method (the one the reference's
    main runs), the latter with a sphere of radius 20 cells masked out, a threshold above
    every curl (lines split at the mask, weighted by the curl along them) and the curl held
    fixed.  (A threshold inside the curl's range cuts the domain into islands whose free
    constants drift over 200 iterations, so that FP32 finite differences of the loss lose
    their digits; the adjoint for such thresholds is checked against the FP64 oracle in
    tests/test_gpu_adjoint.py.)"""
    torch = pytest.importorskip("torch")
    from omni3d.autograd import omni_solve

    f = synthetic.blobs(n=96, count=8, sigma_range=(3.0, 9.0), noise=0.05, seed=5,
                        sphere_radius=20.0 if method == "select" else None)
    dims = f["dims"]
    dirs = omni.icosphere(4)  # 642 vertices
    dev = "cuda"
    a = [torch.tensor(f[k], device=dev, requires_grad=True) for k in ("ax", "ay", "az")]
    target = torch.tensor(f["p_true"], dtype=torch.float32, device=dev)
    target = target - target.mean()
    # surface-force integral over a sphere of radius 20 cells: sum of p * n_x * dA over the
    # voxels within half a cell of the sphere
    nz, ny, nx = dims[::-1]
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    c = (np.array(dims) - 1) / 2.0
    rx, ry, rz = i - c[0], j - c[1], k - c[2]
    r = np.sqrt(rx * rx + ry * ry + rz * rz)
    shell = np.abs(r - 20.0) < 0.5
    dA = f["spacing"][0] ** 2
    w = torch.tensor(np.where(shell, rx / np.maximum(r, 1e-9) * dA, 0.0).astype(np.float32), device=dev)
    curl, thr = None, 0.0
    if method == "select":
        cn = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
        thr = float(np.finfo(np.float32).max)
        curl = torch.tensor(cn.reshape(dims[::-1]), device=dev)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=200, gauge="mean", method=method, threshold=thr) as s:
        def loss_of(ax, ay, az):
            p = omni_solve(s, ax, ay, az, curl=curl)
            return ((p - target) ** 2).sum() + 1e6 * (p * w).sum()

        L = loss_of(*a)
        L.backward()
        grads = [t.grad.detach().clone() for t in a]
        assert all(torch.isfinite(gg).all() for gg in grads)
        rng = np.random.default_rng(6)
        worst = 0.0
        for _ in range(64):
            h = [torch.tensor(rng.normal(size=dims[::-1]).astype(np.float32), device=dev) for _ in range(3)]
            eps = 20.0
            with torch.no_grad():
                lp = loss_of(*[x + eps * d for x, d in zip(a, h)]).item()
                lm = loss_of(*[x - eps * d for x, d in zip(a, h)]).item()
            fd = (lp - lm) / (2 * eps)
            an = sum(float((gg.double() * d.double()).sum()) for gg, d in zip(grads, h))
            worst = max(worst, abs(fd - an) / max(abs(an), 1e-9))
        assert worst < 5e-3, worst
