"""omni3d_sweep_noalloc, the sweep for callers that cannot allocate device memory at the
point where they sweep (a framework whose own pool owns the device, a plugin with a fixed
device memory budget, a real-time loop that cannot take cudaMalloc's synchronisation).

Called through the C ABI, on two calls in a row (the static scratch it shares between calls
must not leak the first call's sums into the second), its (pn, count) must equal
omni3d_sweep's on the same inputs and the FP64 oracle's sweep within the sweep parity
tolerance; its device memory use must not change from call to call; a grid of exactly
OMNI3D_NOALLOC_MAX_VOXELS voxels must be accepted and one plane more refused.  This file
sorts last so that a run stopping at the first failure has run every other test first."""
import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu

TOL_PN = 1e-5  # the same bound as the sweep parity test: relative L2 of pn
MODES = {"plain": 0, "select": 1}


def _noalloc(omni, solver, arrays, curl, out=None):
    """Call omni3d_sweep_noalloc through the C ABI with CUDA tensors; returns (pn, count)."""
    import torch

    if out is None:
        out = (torch.zeros(solver.V, dtype=torch.float32, device="cuda"),
               torch.zeros(solver.V, dtype=torch.float32, device="cuda"))
    pn, cnt = out
    torch.cuda.synchronize()
    rc = omni.lib().omni3d_sweep_noalloc(solver.handle, arrays[0].data_ptr(), arrays[1].data_ptr(),
                                         arrays[2].data_ptr(), None if curl is None else curl.data_ptr(),
                                         arrays[3].data_ptr(), pn.data_ptr(), cnt.data_ptr(), None)
    assert rc == 0, omni.lib().omni3d_last_error(solver.handle)
    torch.cuda.synchronize()
    return pn.cpu().numpy(), cnt.cpu().numpy()


@pytest.mark.parametrize("method", ["plain", "select"])
def test_noalloc_sweep_matches_sweep_and_oracle_twice(omni, orc, method):
    torch = pytest.importorskip("torch")
    dims = (20, 16, 12)
    dirs = omni.icosphere(3)
    with omni.Omni3D(dims, 1e-3, dirs, max_iter=1, method=method, threshold=1e30) as s:
        for call, seed in enumerate((50, 51)):
            f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=seed, sphere_radius=3.0)
            p = np.random.default_rng(seed).normal(0, 0.3, np.prod(dims)).astype(np.float32)
            curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"]) if method == "select" else None
            epn, ecnt = s.sweep(f["ax"], f["ay"], f["az"], p, curl=curl)
            opn, ocnt = orc.sweep(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p, mode=MODES[method],
                                  thr=1e30, curl=curl, precision="f64", nthreads=4)
            dev = [torch.from_numpy(np.ascontiguousarray(f[k].reshape(-1))).cuda() for k in ("ax", "ay", "az")]
            dev.append(torch.from_numpy(p).cuda())
            curl_t = None if curl is None else torch.from_numpy(curl).cuda()
            pn, cnt = _noalloc(omni, s, dev, curl_t)
            if method == "plain":
                np.testing.assert_array_equal(cnt, ecnt.reshape(-1))
                np.testing.assert_array_equal(cnt, ocnt.astype(np.float32))
            else:
                assert synthetic.relative_l2(cnt, ecnt, gauge="none") < TOL_PN
                assert synthetic.relative_l2(cnt, ocnt, gauge="none") < TOL_PN
            assert synthetic.relative_l2(pn, epn, gauge="none") < TOL_PN, "call %d vs omni3d_sweep" % call
            assert synthetic.relative_l2(pn, opn, gauge="none") < TOL_PN, "call %d vs the FP64 oracle" % call


def test_noalloc_sweep_takes_no_device_memory_and_keeps_the_current_device(omni):
    """Calls after the first (which looks up the static arrays) leave the device's free
    memory exactly as it was, and the caller's current device is unchanged."""
    torch = pytest.importorskip("torch")
    dims = (24, 20, 16)
    f = synthetic.blobs(dims=dims, count=2, sigma_range=(2.0, 4.0), noise=0.05, seed=3)
    with omni.Omni3D(dims, 1e-3, omni.icosphere(2), max_iter=1) as s:
        dev = [torch.from_numpy(np.ascontiguousarray(f[k].reshape(-1))).cuda() for k in ("ax", "ay", "az")]
        dev.append(torch.zeros(s.V, dtype=torch.float32, device="cuda"))
        out = (torch.zeros(s.V, dtype=torch.float32, device="cuda"), torch.zeros(s.V, dtype=torch.float32,
                                                                                 device="cuda"))
        first = _noalloc(omni, s, dev, None, out)
        cur = torch.cuda.current_device()
        free0 = torch.cuda.mem_get_info()[0]
        for _ in range(2):
            out[0].zero_()
            out[1].zero_()
            again = _noalloc(omni, s, dev, None, out)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        assert torch.cuda.current_device() == cur
        np.testing.assert_array_equal(again[1], first[1])
        assert synthetic.relative_l2(again[0], first[0], gauge="none") < TOL_PN


def test_noalloc_sweep_accepts_its_maximum_and_rejects_one_plane_more(omni):
    torch = pytest.importorskip("torch")
    dirs = omni.icosphere(2)
    dims = (64, 64, 64)  # exactly OMNI3D_NOALLOC_MAX_VOXELS
    f = synthetic.blobs(dims=dims, count=2, sigma_range=(4.0, 8.0), noise=0.05, seed=7)
    with omni.Omni3D(dims, 1e-3, dirs, max_iter=1) as s:
        p = np.zeros(s.V, np.float32)
        epn, ecnt = s.sweep(f["ax"], f["ay"], f["az"], p)
        dev = [torch.from_numpy(np.ascontiguousarray(f[k].reshape(-1))).cuda() for k in ("ax", "ay", "az")]
        dev.append(torch.from_numpy(p).cuda())
        pn, cnt = _noalloc(omni, s, dev, None)
        np.testing.assert_array_equal(cnt, ecnt.reshape(-1))
        assert synthetic.relative_l2(pn, epn, gauge="none") < TOL_PN
    dims = (65, 64, 64)  # one plane more
    with omni.Omni3D(dims, 1e-3, dirs, max_iter=1) as s:
        z = torch.zeros(s.V, dtype=torch.float32, device="cuda")
        out = [torch.zeros_like(z), torch.zeros_like(z)]
        rc = omni.lib().omni3d_sweep_noalloc(s.handle, z.data_ptr(), z.data_ptr(), z.data_ptr(), None, z.data_ptr(),
                                             out[0].data_ptr(), out[1].data_ptr(), None)
        assert rc == -6
        assert b"OMNI3D_NOALLOC_MAX_VOXELS" in omni.lib().omni3d_last_error(s.handle)
