"""The adjoint of the solve (omni3d_adjoint) against the FP64 oracle's transpose of the
reference iteration -- the plain method's (orc_adjoint_f64) and, with the curl held fixed,
every method's (orc_adjoint_modes_f64) -- and against finite differences, and the
torch.autograd binding."""
import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu

TOL_GRAD = 5e-5  # relative L2 of the gradient field vs the FP64 adjoint


def _field(dims, seed):
    return synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=seed)


@pytest.mark.parametrize("niter", [1, 3, 6])
@pytest.mark.parametrize("solver", ["anchor", "sweep"])
def test_adjoint_matches_fp64_oracle(omni, orc, niter, solver):
    dims = (12, 10, 9)
    f = _field(dims, 30)
    dirs = omni.icosphere(2)
    g = np.random.default_rng(1).normal(size=np.prod(dims)).astype(np.float32)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=niter, solver=solver) as s:
        s.solve(f["ax"], f["ay"], f["az"])
        got = s.adjoint(g)
    exp = orc.adjoint(dims, f["spacing"], dirs, niter, g)
    for a, b in zip(got, exp):
        assert synthetic.relative_l2(a, b, gauge="none") < TOL_GRAD


def test_adjoint_with_mean_gauge_is_a_transpose(omni):
    """<g, J h> = <J^T g, h> for the gauged map (the solve is affine in the field, so
    J h = P(a + h) - P(a))."""
    dims = (11, 10, 12)
    f = _field(dims, 31)
    dirs = omni.icosphere(2)
    rng = np.random.default_rng(2)
    g = rng.normal(size=np.prod(dims)).astype(np.float32)
    h = [rng.normal(size=np.prod(dims)).astype(np.float32) * 50 for _ in range(3)]
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=4, gauge="mean") as s:
        p1 = s.solve(*[f[k].reshape(-1) + hh for k, hh in zip(("ax", "ay", "az"), h)]).p.reshape(-1).astype(np.float64)
        p0 = s.solve(f["ax"], f["ay"], f["az"]).p.reshape(-1).astype(np.float64)
        gt = s.adjoint(g)
    lhs = float(np.dot(g, p1 - p0))
    rhs = float(sum(np.dot(a.reshape(-1).astype(np.float64), b) for a, b in zip(gt, h)))
    assert abs(lhs - rhs) <= 1e-4 * max(abs(lhs), 1e-12)


def test_autograd_matches_finite_differences(omni):
    torch = pytest.importorskip("torch")
    from omni3d.autograd import omni_solve

    dims = (12, 12, 12)
    f = _field(dims, 32)
    dirs = omni.icosphere(2)
    dev = "cuda"
    a = [torch.tensor(f[k], device=dev, requires_grad=True) for k in ("ax", "ay", "az")]
    target = torch.tensor(f["p_true"], dtype=torch.float32, device=dev)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=5, gauge="mean") as s:
        def loss_of(ax, ay, az):
            p = omni_solve(s, ax, ay, az)
            return ((p - (target - target.mean())) ** 2).sum() + p[2:5, 3:7, 4:9].sum()

        L = loss_of(*a)
        L.backward()
        grads = [t.grad.detach().clone() for t in a]
        rng = np.random.default_rng(3)
        for _ in range(4):
            h = [torch.tensor(rng.normal(size=dims[::-1]).astype(np.float32), device=dev) for _ in range(3)]
            eps = 20.0
            with torch.no_grad():
                lp = loss_of(*[x + eps * d for x, d in zip(a, h)]).item()
                lm = loss_of(*[x - eps * d for x, d in zip(a, h)]).item()
            fd = (lp - lm) / (2 * eps)
            an = sum(float((gg * d).sum()) for gg, d in zip(grads, h))
            assert abs(fd - an) <= 2e-3 * max(abs(an), 1e-9), (fd, an)


METHODS = [("select", 1), ("weighted", 2), ("weighted_fixed_bc", 3), ("select_fixed_bc", 4), ("mini_curl", 5),
           ("weighted_mini_curl", 6)]


@pytest.mark.parametrize("niter", [1, 4])
@pytest.mark.parametrize("solver", ["anchor", "sweep"])
@pytest.mark.parametrize("method,mode", METHODS)
def test_adjoint_of_every_method_matches_fp64_oracle(omni, orc, method, mode, solver, niter):
    """With the curl held fixed every method's solve is affine in the field; its adjoint must
    equal the FP64 oracle's transpose of the full-voxel reference iteration
    (orc_adjoint_modes_f64, no anchor operator).  After a sweep-form solve the adjoint builds
    the operator itself."""
    dims = (13, 11, 10)
    f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=34, sphere_radius=2.5)
    dirs = omni.icosphere(2)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 80)) if "select" in method else 0.0
    g = np.random.default_rng(7).normal(size=np.prod(dims)).astype(np.float32)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=niter, method=method, threshold=thr, solver=solver) as s:
        s.solve(f["ax"], f["ay"], f["az"], curl=curl)
        got = s.adjoint(g)
    exp = orc.adjoint_modes(dims, f["spacing"], dirs, niter, g, mode=mode, thr=thr, curl=curl)
    for a, b in zip(got, exp):
        assert synthetic.relative_l2(a, b, gauge="none") < 1e-4


def test_adjoint_bf16_storage_uses_the_stored_curl(omni, orc):
    """With BF16 storage the adjoint holds fixed the curl the solve stored (tests/bf16_ref.py)."""
    import bf16_ref

    dims = (13, 11, 10)
    f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=35, sphere_radius=2.5)
    dirs = omni.icosphere(2)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 80))
    g = np.random.default_rng(8).normal(size=np.prod(dims)).astype(np.float32)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=3, method="select", threshold=thr, grad="bf16") as s:
        s.solve(f["ax"], f["ay"], f["az"], curl=curl)
        got = s.adjoint(g)
    cb, thr_b = bf16_ref.curl_bf16(curl, thr)
    exp = orc.adjoint_modes(dims, f["spacing"], dirs, 3, g, mode=1, thr=thr_b, curl=cb)
    for a, b in zip(got, exp):
        assert synthetic.relative_l2(a, b, gauge="none") < 1e-4


@pytest.mark.parametrize("method", ["select", "weighted"])
def test_autograd_select_and_weighted_match_finite_differences(omni, orc, method):
    """Central differences of a loss through omni_solve with the curl given (held fixed)."""
    torch = pytest.importorskip("torch")
    from omni3d.autograd import omni_solve

    dims = (12, 12, 12)
    f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=36, sphere_radius=3.0)
    dirs = omni.icosphere(2)
    curl_np = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl_np[curl_np > 0], 85)) if method == "select" else 0.0
    dev = "cuda"
    curl = torch.tensor(curl_np.reshape(dims[::-1]), device=dev)
    a = [torch.tensor(f[k], device=dev, requires_grad=True) for k in ("ax", "ay", "az")]
    target = torch.tensor(f["p_true"], dtype=torch.float32, device=dev)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=5, gauge="mean", method=method, threshold=thr) as s:
        def loss_of(ax, ay, az):
            p = omni_solve(s, ax, ay, az, curl=curl)
            return ((p - (target - target.mean())) ** 2).sum() + p[2:5, 3:7, 4:9].sum()

        L = loss_of(*a)
        L.backward()
        grads = [t.grad.detach().clone() for t in a]
        rng = np.random.default_rng(9)
        for _ in range(4):
            h = [torch.tensor(rng.normal(size=dims[::-1]).astype(np.float32), device=dev) for _ in range(3)]
            eps = 20.0
            with torch.no_grad():
                lp = loss_of(*[x + eps * d for x, d in zip(a, h)]).item()
                lm = loss_of(*[x - eps * d for x, d in zip(a, h)]).item()
            fd = (lp - lm) / (2 * eps)
            an = sum(float((gg.double() * d.double()).sum()) for gg, d in zip(grads, h))
            assert abs(fd - an) <= 2e-3 * max(abs(an), 1e-9), (fd, an)
