"""omni3d_sweep_noalloc, the sweep for callers that cannot allocate device memory (inside a
CUDA-graph capture, under a framework-owned memory pool, in a real-time loop): called
through the C ABI, its (pn, count) must equal omni3d_sweep's on the same inputs, on two
calls in a row (the static scratch it shares between calls must not leak the first call's
sums into the second), and it must refuse grids larger than its static scratch."""
import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu

TOL_PN = 1e-5  # the same bound as the sweep parity test: relative L2 of pn


def _noalloc(omni, solver, arrays, curl):
    """Call omni3d_sweep_noalloc through the C ABI with CUDA tensors; returns (pn, count)."""
    import torch

    pn = torch.zeros(solver.V, dtype=torch.float32, device="cuda")
    cnt = torch.zeros_like(pn)
    torch.cuda.synchronize()
    rc = omni.lib().omni3d_sweep_noalloc(solver.handle, arrays[0].data_ptr(), arrays[1].data_ptr(),
                                         arrays[2].data_ptr(), None if curl is None else curl.data_ptr(),
                                         arrays[3].data_ptr(), pn.data_ptr(), cnt.data_ptr(), None)
    assert rc == 0, omni.lib().omni3d_last_error(solver.handle)
    torch.cuda.synchronize()
    return pn.cpu().numpy(), cnt.cpu().numpy()


@pytest.mark.parametrize("method", ["plain", "select"])
def test_noalloc_sweep_matches_sweep_twice(omni, orc, method):
    torch = pytest.importorskip("torch")
    dims = (20, 16, 12)
    dirs = omni.icosphere(3)
    with omni.Omni3D(dims, 1e-3, dirs, max_iter=1, method=method, threshold=1e30) as s:
        for call, seed in enumerate((50, 51)):
            f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=seed, sphere_radius=3.0)
            p = np.random.default_rng(seed).normal(0, 0.3, np.prod(dims)).astype(np.float32)
            curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"]) if method == "select" else None
            epn, ecnt = s.sweep(f["ax"], f["ay"], f["az"], p, curl=curl)
            dev = [torch.from_numpy(np.ascontiguousarray(f[k].reshape(-1))).cuda() for k in ("ax", "ay", "az")]
            dev.append(torch.from_numpy(p).cuda())
            curl_t = None if curl is None else torch.from_numpy(curl).cuda()
            pn, cnt = _noalloc(omni, s, dev, curl_t)
            if method == "plain":
                np.testing.assert_array_equal(cnt, ecnt.reshape(-1))
            else:
                assert synthetic.relative_l2(cnt, ecnt, gauge="none") < TOL_PN
            assert synthetic.relative_l2(pn, epn, gauge="none") < TOL_PN, "call %d" % call


def test_noalloc_sweep_rejects_grids_beyond_its_scratch(omni):
    torch = pytest.importorskip("torch")
    dims = (65, 64, 64)  # one plane more than 64^3
    with omni.Omni3D(dims, 1e-3, omni.icosphere(2), max_iter=1) as s:
        z = torch.zeros(s.V, dtype=torch.float32, device="cuda")
        out = [torch.zeros_like(z), torch.zeros_like(z)]
        rc = omni.lib().omni3d_sweep_noalloc(s.handle, z.data_ptr(), z.data_ptr(), z.data_ptr(), None, z.data_ptr(),
                                             out[0].data_ptr(), out[1].data_ptr(), None)
        assert rc == -6
        assert b"OMNI3D_NOALLOC_MAX_VOXELS" in omni.lib().omni3d_last_error(s.handle)
