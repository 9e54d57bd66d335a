"""Python mirror of the C ABI: a solver object over one context, and the file helpers.

Arrays may be numpy arrays (host memory) or torch tensors; CUDA tensors are passed to the
library as device pointers, everything else is copied through host memory.  Volumes are
float32 and x-fastest: shape (nz, ny, nx) in C order.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from ._lib import check, lib

_METHODS = {"plain": L.METHOD_PLAIN, "select": L.METHOD_SELECT, "weighted": L.METHOD_WEIGHTED,
            "weighted_fixed_bc": L.METHOD_WEIGHTED_FIXED_BC, "select_fixed_bc": L.METHOD_SELECT_FIXED_BC,
            "mini_curl": L.METHOD_MINI_CURL, "weighted_mini_curl": L.METHOD_WEIGHTED_MINI_CURL}
_SOLVERS = {"anchor": L.SOLVER_ANCHOR, "sweep": L.SOLVER_SWEEP}
_ENGINES = {"auto": L.ENGINE_AUTO, "lines": L.ENGINE_LINES, "bricks": L.ENGINE_BRICKS}
_INITS = {"zero": 0, "centre": 1}
_GRADS = {"f32": L.GRAD_F32, "bf16": L.GRAD_BF16}
_GAUGES = {"none": L.GAUGE_NONE, "point": L.GAUGE_POINT, "mean": L.GAUGE_MEAN}


def _is_cuda_tensor(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def _as_host(a, n: int) -> np.ndarray:
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))
    if a.size != n:
        raise ValueError("volume has %d values, expected %d" % (a.size, n))
    return a


@dataclass
class SolveResult:
    p: object
    count: object
    stats: dict = field(default_factory=dict)


class Omni3D:
    """One solver context: grid, directions and options fixed; solve many fields."""

    def __init__(self, dims, spacing, dirs, *, density=1.0, line_spacing=1.0, max_iter=4, threshold=0.0,
                 method="plain", solver="anchor", grad="f32", tol=0.0, gauge="none", ref=(0, 0, 0),
                 seed_first_iteration=True, device=0, anchor_max_links=0, engine="auto", initial_guess="zero",
                 sweep_fp64=False, tile_width=0, dir_group=0, autotune=False, deterministic=False):
        nx, ny, nz = (int(d) for d in dims)
        self.dims = (nx, ny, nz)
        self.V = nx * ny * nz
        self._dirs = np.ascontiguousarray(np.asarray(dirs, np.float32).reshape(-1, 3))
        P = L.Params()
        lib().omni3d_default_params(C.byref(P))
        P.nx, P.ny, P.nz = nx, ny, nz
        sp = spacing if hasattr(spacing, "__len__") else (spacing, spacing, spacing)
        P.dx, P.dy, P.dz = (float(s) for s in sp)
        P.density = float(density)
        P.line_spacing = float(line_spacing)
        P.n_dirs = int(self._dirs.shape[0])
        P.dirs = self._dirs.ctypes.data_as(C.POINTER(C.c_float))
        P.max_iter = int(max_iter)
        P.threshold = float(threshold)
        P.method = _METHODS[method]
        P.solver = _SOLVERS[solver]
        P.grad_storage = _GRADS[grad]
        P.tol = float(tol)
        P.gauge = _GAUGES[gauge]
        P.ref_i, P.ref_j, P.ref_k = (int(r) for r in ref)
        P.seed_first_iteration = int(bool(seed_first_iteration))
        P.device = int(device)
        P.anchor_max_links = int(anchor_max_links)
        P.engine = _ENGINES[engine]
        P.initial_guess = _INITS[initial_guess]
        P.sweep_fp64 = int(bool(sweep_fp64))
        P.tile_width = int(tile_width)
        P.dir_group = int(dir_group)
        P.autotune = int(bool(autotune))
        P.deterministic = int(bool(deterministic))
        self.params = P
        self.method = method
        self.solve_count = 0
        h = C.c_void_p()
        check(lib().omni3d_create(C.byref(P), C.byref(h)))
        self._h = h

    # ------------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_h", None):
            lib().omni3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int):
        check(lib().omni3d_set_stream(self._h, C.c_void_p(stream_ptr)), self._h)

    # ------------------------------------------------------------------ geometry
    def geometry_info(self) -> dict:
        a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong()
        check(lib().omni3d_geometry_info(self._h, C.byref(a), C.byref(b), C.byref(c)), self._h)
        return {"n_lines": a.value, "n_units": b.value, "walk_errors": c.value}

    def line_table(self) -> np.ndarray:
        n = self.geometry_info()["n_lines"]
        rows = np.zeros((n, 4), np.int32)
        check(lib().omni3d_line_table(self._h, rows.ctypes.data, n), self._h)
        return rows

    def line_steps(self, line: int) -> np.ndarray:
        cap = sum(self.dims) + 4
        ax = np.zeros(cap, np.int8)
        n = check(lib().omni3d_line_steps(self._h, int(line), ax.ctypes.data, cap), self._h)
        return ax[:n].copy()

    # ------------------------------------------------------------------ compute
    def _ptrs(self, arrays):
        """Device pointers when every given array is a CUDA tensor, else host copies."""
        given = [a for a in arrays if a is not None]
        dev = bool(given) and all(_is_cuda_tensor(a) for a in given)
        if dev:
            import torch

            out = []
            for a in arrays:
                if a is None:
                    out.append(None)
                    continue
                if a.dtype != torch.float32 or not a.is_contiguous() or a.numel() != self.V:
                    raise ValueError("CUDA volumes must be contiguous float32 with %d values" % self.V)
                out.append(a)
            torch.cuda.current_stream().synchronize()
            return True, out, [None if a is None else a.data_ptr() for a in out]
        hosts = [None if a is None else _as_host(a, self.V) for a in arrays]
        return False, hosts, [None if a is None else a.ctypes.data for a in hosts]

    def solve(self, ax, ay, az, *, curl=None, mask=None, p_init=None, out=None) -> SolveResult:
        """out: optional (p, count) output arrays of V float32 each, CUDA tensors for device
        inputs or contiguous host arrays otherwise (e.g. views of pinned memory, which the
        device-to-host copy reaches without a bounce buffer)."""
        dev, keep, ptrs = self._ptrs([ax, ay, az, curl, mask, p_init])
        st = L.Stats()
        if out is not None:
            p, cnt = out
            if dev:
                if not (_is_cuda_tensor(p) and _is_cuda_tensor(cnt) and p.numel() == self.V and cnt.numel() == self.V):
                    raise ValueError("out must be two CUDA tensors of V elements for device inputs")
                pp, cp = p.data_ptr(), cnt.data_ptr()
            else:
                for a in (p, cnt):
                    if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.size == self.V
                            and a.flags.c_contiguous):
                        raise ValueError("out must be two contiguous float32 arrays of V elements")
                pp, cp = p.ctypes.data, cnt.ctypes.data
        elif dev:
            import torch

            p = torch.empty(self.V, dtype=torch.float32, device=keep[0].device)
            cnt = torch.empty_like(p)
            pp, cp = p.data_ptr(), cnt.data_ptr()
        else:
            p = np.empty(self.V, np.float32)
            cnt = np.empty(self.V, np.float32)
            pp, cp = p.ctypes.data, cnt.ctypes.data
        check(lib().omni3d_solve(self._h, ptrs[0], ptrs[1], ptrs[2], ptrs[3], ptrs[4], ptrs[5], pp, cp, int(dev),
                                 C.byref(st)), self._h)
        self.solve_count += 1
        shape = self.dims[::-1]
        return SolveResult(p.reshape(shape), cnt.reshape(shape), st.as_dict())

    def sweep(self, ax, ay, az, p, *, curl=None):
        """One omni sweep from p: returns (pn, count) without normalisation."""
        dev, keep, ptrs = self._ptrs([ax, ay, az, curl, p])
        if dev:
            import torch

            pn = torch.zeros(self.V, dtype=torch.float32, device=keep[0].device)
            cnt = torch.zeros_like(pn)
            a, b = pn.data_ptr(), cnt.data_ptr()
        else:
            pn = np.zeros(self.V, np.float32)
            cnt = np.zeros(self.V, np.float32)
            a, b = pn.ctypes.data, cnt.ctypes.data
        check(lib().omni3d_sweep(self._h, ptrs[0], ptrs[1], ptrs[2], ptrs[3], ptrs[4], a, b, int(dev)), self._h)
        shape = self.dims[::-1]
        return pn.reshape(shape), cnt.reshape(shape)

    def adjoint(self, grad_p):
        """Gradient of <grad_p, p> with respect to (ax, ay, az) for the last solve on this
        context, with its curl held fixed: the transpose of the solve's affine map."""
        if _is_cuda_tensor(grad_p):
            import torch

            g = grad_p.reshape(-1).to(torch.float32).contiguous()
            out = [torch.empty(self.V, dtype=torch.float32, device=g.device) for _ in range(3)]
            torch.cuda.current_stream().synchronize()
            check(lib().omni3d_adjoint(self._h, g.data_ptr(), *[o.data_ptr() for o in out], 1), self._h)
        else:
            g = _as_host(grad_p, self.V)
            out = [np.empty(self.V, np.float32) for _ in range(3)]
            check(lib().omni3d_adjoint(self._h, g.ctypes.data, *[o.ctypes.data for o in out], 0), self._h)
        return [o.reshape(self.dims[::-1]) for o in out]

    def gauge(self, p, count=None, mode="mean", ref=0):
        """Remove the constant mode of p (returns a gauged copy): p - p[ref] or p - mean(p)
        over count > 0."""
        if _is_cuda_tensor(p):
            out = p.reshape(-1).clone().contiguous()
            c = None if count is None else count.reshape(-1).contiguous()
            import torch

            torch.cuda.current_stream().synchronize()
            check(lib().omni3d_gauge(self._h, out.data_ptr(), None if c is None else c.data_ptr(), self.V,
                                     _GAUGES[mode], int(ref), 1), self._h)
        else:
            out = _as_host(p, self.V).copy()
            c = None if count is None else _as_host(count, self.V)
            check(lib().omni3d_gauge(self._h, out.ctypes.data, None if c is None else c.ctypes.data, self.V,
                                     _GAUGES[mode], int(ref), 0), self._h)
        return out.reshape(self.dims[::-1])

    def curl(self, ax, ay, az, mask=None):
        dev, keep, ptrs = self._ptrs([ax, ay, az, mask])
        if dev:
            import torch

            out = torch.empty(self.V, dtype=torch.float32, device=keep[0].device)
            o = out.data_ptr()
        else:
            out = np.empty(self.V, np.float32)
            o = out.ctypes.data
        check(lib().omni3d_curl(self._h, ptrs[0], ptrs[1], ptrs[2], ptrs[3], o, int(dev)), self._h)
        return out.reshape(self.dims[::-1])

    def centre_integration(self, ax, ay, az, pref=0.0):
        """The reference's initial guess (initialIntegration.cpp): p integrated outward from
        the centre voxel, FP64 on the device, returned as float32."""
        dev, keep, ptrs = self._ptrs([ax, ay, az])
        if dev:
            import torch

            out = torch.empty(self.V, dtype=torch.float32, device=keep[0].device)
            o = out.data_ptr()
        else:
            out = np.empty(self.V, np.float32)
            o = out.ctypes.data
        check(lib().omni3d_centre_integration(self._h, ptrs[0], ptrs[1], ptrs[2], float(pref), o, int(dev)), self._h)
        return out.reshape(self.dims[::-1])


# ---------------------------------------------------------------------- host helpers
def icosphere(level: int) -> np.ndarray:
    """Direction set of GridIcosahedronDivide<level>.dat (42, 162, 642, ... vertices)."""
    n = check(lib().omni3d_icosphere(int(level), None, 0))
    out = np.zeros((n, 3), np.float32)
    check(lib().omni3d_icosphere(int(level), out.ctypes.data, n))
    return out


def read_directions(path: str, n: int) -> np.ndarray:
    out = np.zeros((n, 3), np.float32)
    check(lib().omni3d_read_directions(path.encode(), int(n), out.ctypes.data))
    return out


def read_params(path: str) -> L.FileParams:
    fp = L.FileParams()
    check(lib().omni3d_read_params(path.encode(), C.byref(fp)))
    return fp


def read_tecplot(path: str, fp: L.FileParams) -> dict:
    nx = fp.roi[1] - fp.roi[0] + 1
    ny = fp.roi[3] - fp.roi[2] + 1
    nz = fp.roi[5] - fp.roi[4] + 1
    names = ["x", "y", "z", "u", "v", "w", "ax", "ay", "az", "mask"]
    arrs = {k: np.zeros(nx * ny * nz, np.float32) for k in names}
    ncol = check(lib().omni3d_read_tecplot(path.encode(), C.byref(fp), *[arrs[k].ctypes.data for k in names]))
    arrs["ncol"] = ncol
    return arrs


def bernoulli_face(dims, pref, density, u, v, w) -> np.ndarray:
    nx, ny, nz = dims
    out = np.zeros(nx * ny * nz, np.float32)
    u, v, w = (np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1)) for a in (u, v, w))
    check(lib().omni3d_bernoulli_face(nx, ny, nz, float(pref), float(density), u.ctypes.data, v.ctypes.data,
                                      w.ctypes.data, out.ctypes.data))
    return out


def write_pressure(path, dims, x, y, z, p, count):
    nx, ny, nz = dims
    f = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
    x, y, z, p, count = f(x), f(y), f(z), f(p), f(count)
    check(lib().omni3d_write_pressure(str(path).encode(), nx, ny, nz, x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                      p.ctypes.data, count.ctypes.data))


def write_curl(path, dims, x, y, z, curl):
    nx, ny, nz = dims
    f = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
    x, y, z, curl = f(x), f(y), f(z), f(curl)
    check(lib().omni3d_write_curl(str(path).encode(), nx, ny, nz, x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                  curl.ctypes.data))


class Batch:
    """Several snapshots, one context each (grid sizes, methods and tolerances may differ),
    solved together (omni3d_batch_*): in one CUDA-graph launch when every member has the
    plain method, the anchor solver and tol = 0, else concurrently, each member on its own
    stream from a pool of host threads."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.handle for s in self.solvers])
        h = C.c_void_p()
        check(lib().omni3d_batch_create(arr, len(self.solvers), C.byref(h)))
        self._h = h
        self._keep = arr

    def close(self):
        if getattr(self, "_h", None):
            lib().omni3d_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def solve(self, fields, p_init=None, out=None, mask=None):
        """fields: list of (ax, ay, az) per member (all CUDA tensors, or all host arrays).
        mask: optional list of per-member mask columns (the curl of the methods that read it
        is computed from the field and the mask).  out: optional list of (p, count) output
        buffers (reused between calls so that the captured graph is relaunched).  Returns
        ([p], [count], stats)."""
        n = len(self.solvers)
        if len(fields) != n:
            raise ValueError("one field per member")
        dev = _is_cuda_tensor(fields[0][0])
        keep = []

        def ptr(a, V):
            if a is None:
                return None
            if dev:
                if not (_is_cuda_tensor(a) and a.is_contiguous() and a.numel() == V):
                    raise ValueError("batch inputs must all be contiguous CUDA tensors")
                keep.append(a)
                return a.data_ptr()
            h = _as_host(a, V)
            keep.append(h)
            return h.ctypes.data

        outs = []
        for i, s in enumerate(self.solvers):
            if out is not None:
                outs.append(out[i])
            elif dev:
                import torch

                p = torch.empty(s.V, dtype=torch.float32, device=fields[i][0].device)
                outs.append((p, torch.empty_like(p)))
            else:
                outs.append((np.empty(s.V, np.float32), np.empty(s.V, np.float32)))
        arrs = []
        for k in range(3):
            arrs.append((C.c_void_p * n)(*[ptr(fields[i][k], s.V) for i, s in enumerate(self.solvers)]))
        mk = None
        if mask is not None:
            mk = (C.c_void_p * n)(*[ptr(mask[i], s.V) for i, s in enumerate(self.solvers)])
        p0 = None
        if p_init is not None:
            p0 = (C.c_void_p * n)(*[ptr(p_init[i], s.V) for i, s in enumerate(self.solvers)])
        po = (C.c_void_p * n)(*[ptr(outs[i][0], s.V) for i, s in enumerate(self.solvers)])
        co = (C.c_void_p * n)(*[ptr(outs[i][1], s.V) for i, s in enumerate(self.solvers)])
        if dev:
            import torch

            torch.cuda.current_stream().synchronize()
        st = L.Stats()
        rc = lib().omni3d_batch_solve(self._h, arrs[0], arrs[1], arrs[2], mk, p0, po, co, int(dev), C.byref(st))
        if rc < 0:
            msg = (lib().omni3d_batch_last_error(self._h) or b"").decode(errors="replace")
            raise L.Omni3DError(rc, msg)
        ps = [o[0].reshape(s.dims[::-1]) for o, s in zip(outs, self.solvers)]
        cs = [o[1].reshape(s.dims[::-1]) for o, s in zip(outs, self.solvers)]
        return ps, cs, st.as_dict()
