"""The reference's initial guess by integration outward from the centre voxel
(initialIntegration.cpp:9-407) on the GPU: FP64 wavefronts, bit-identical to the oracle's
double result rounded to float; and the solve option that starts from it."""
import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(12, 10, 8), (7, 9, 11), (2, 3, 2), (33, 20, 17)])
def test_centre_integration_bit_exact(omni, orc, dims):
    f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 5.0), noise=0.05, seed=sum(dims))
    with omni.Omni3D(dims, f["spacing"], omni.icosphere(2), max_iter=1, density=1.2) as s:
        got = s.centre_integration(f["ax"], f["ay"], f["az"], pref=3.5).reshape(-1)
        torch = pytest.importorskip("torch")
        dev = s.centre_integration(*[torch.from_numpy(f[k].reshape(-1)).cuda() for k in ("ax", "ay", "az")])
    # the library holds spacing and density as float: the oracle gets the same values
    sp32 = tuple(float(np.float32(x)) for x in f["spacing"])
    exp = orc.centre_integration(dims, sp32, f["ax"], f["ay"], f["az"], rho=float(np.float32(1.2)),
                                 pref=3.5).astype(np.float32)
    np.testing.assert_array_equal(got.view(np.uint32), exp.view(np.uint32))
    np.testing.assert_array_equal(dev.cpu().numpy().reshape(-1).view(np.uint32), exp.view(np.uint32))
    c = (dims[0] // 2) + (dims[1] // 2) * dims[0] + (dims[2] // 2) * dims[0] * dims[1]
    assert got[c] == 0.0


def test_solve_from_centre_integration(omni, orc):
    """initial_guess="centre" starts the iteration from the centre integration when no
    p_init is given; both starts reach the same gauged fixed point."""
    f = synthetic.gaussian(n=32, sigma_cells=6.0, noise=0.05, seed=1)
    dims = f["dims"]
    dirs = omni.icosphere(3)
    out = {}
    for init in ("zero", "centre"):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=500, tol=1e-6, gauge="mean", initial_guess=init) as s:
            out[init] = s.solve(f["ax"], f["ay"], f["az"])
        assert out[init].stats["rel_change"] < 1e-6
    assert synthetic.relative_l2(out["centre"].p, out["zero"].p) < 1e-4
    # one iteration from the guess equals the oracle's first iteration from the same guess
    sp32 = tuple(float(np.float32(x)) for x in f["spacing"])
    g = orc.centre_integration(dims, sp32, f["ax"], f["ay"], f["az"]).astype(np.float32)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1, initial_guess="centre") as s:
        r = s.solve(f["ax"], f["ay"], f["az"])
    ep, _ = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], g, 1, precision="f64")
    assert synthetic.relative_l2(r.p, ep, gauge="none") < 2e-5
