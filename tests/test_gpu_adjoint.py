"""The adjoint of the plain-method solve (omni3d_adjoint) against the FP64 oracle's
transpose of the reference iteration and against finite differences, and the
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


def test_adjoint_rejects_select_method(omni):
    dims = (8, 8, 8)
    f = _field(dims, 33)
    with omni.Omni3D(dims, f["spacing"], omni.icosphere(2), max_iter=2, method="select", threshold=1e30) as s:
        s.solve(f["ax"], f["ay"], f["az"])
        with pytest.raises(omni.Omni3DError) as e:
            s.adjoint(np.ones(512, np.float32))
        assert e.value.code == -5
