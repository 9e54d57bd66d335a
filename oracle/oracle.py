"""ctypes bindings of the CPU oracle and of the reference's own CPU functions.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline / reference arm, always as the checker or the timed CPU baseline, never by
the product package.

* ``Oracle`` wraps oracle/omni_oracle.c (built into oracle/_build/liborc.so), the plain-C
  restatement of the reference's omni path (Omni3D_8.0/Omni3D_8.0/kernel.cu), with an
  FP32 mode that reproduces the reference's float arithmetic and an FP64 mode on the same
  discrete line geometry.
* ``RefLib`` wraps oracle/_ref/libomni_ref.so: the reference's own functions
  (cross2point, bodyIntegralInner, bodyIntegralInnerSelect, calIndex,
  omni3dparallellinesESInnerCPU, devidecountInnerCPU, calCurlofMaterialAccCPU, sor3D,
  calRHS) compiled from its sources by oracle/build_ref.sh.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
ORC_SO = os.path.join(BUILD, "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libomni_ref.so")
REF_STAGED = os.path.join(HERE, "_ref", "src", "ref_kernel_extract.cpp")
# The reference checkout is located only through this variable; without it the staged copy
# under oracle/_ref/src (made by an earlier `build_ref.sh stage`) is used, if present.
REFERENCE_ROOT = os.environ.get("OMNI3D_REFERENCE_ROOT") or None

_f = C.c_float
_d = C.c_double
_i = C.c_int
_l = C.c_long
_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)
_bp = C.POINTER(C.c_byte)


def build_oracle(force: bool = False) -> str:
    """Compile the C restatement (one rounding per float operation: no contraction)."""
    src = os.path.join(HERE, "omni_oracle.c")
    if force or not os.path.exists(ORC_SO) or os.path.getmtime(ORC_SO) < os.path.getmtime(src):
        os.makedirs(BUILD, exist_ok=True)
        tmp = ORC_SO + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fopenmp", "-fPIC",
                               "-shared", "-o", tmp, src, "-lm"])
        os.replace(tmp, ORC_SO)
    return ORC_SO


def build_ref(force: bool = False) -> str | None:
    """Stage the reference sources (when the reference tree is present) and compile them.

    The reference tree is found through OMNI3D_REFERENCE_ROOT only.  Returns the library
    path, or None when neither the tree (variable unset or pointing elsewhere) nor a staged
    copy exists on this machine."""
    script = os.path.join(HERE, "build_ref.sh")
    have_tree = REFERENCE_ROOT is not None and os.path.exists(
        os.path.join(REFERENCE_ROOT, "Omni3D_8.0", "Omni3D_8.0", "kernel.cu"))
    if have_tree and (force or not os.path.exists(REF_STAGED)):
        subprocess.check_call(["bash", script, "stage"], env=dict(os.environ, REF_ROOT=REFERENCE_ROOT),
                              stdout=subprocess.DEVNULL)
    if not os.path.exists(REF_STAGED):
        return None
    deps = [REF_STAGED, os.path.join(HERE, "ref_driver.cpp")]
    if force or not os.path.exists(REF_SO) or any(os.path.getmtime(REF_SO) < os.path.getmtime(d) for d in deps):
        subprocess.check_call(["bash", script, "build"], stdout=subprocess.DEVNULL)
    return REF_SO


def _ptr(a: np.ndarray, ct):
    assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
    return a.ctypes.data_as(C.POINTER(ct))


class OrcProblem(C.Structure):
    _fields_ = [("X", _l), ("Y", _l), ("Z", _l), ("dx", _f), ("dy", _f), ("dz", _f), ("rho", _f),
                ("ls", _f), ("thr", _f), ("nv", _i), ("k1", _fp), ("k2", _fp), ("k3", _fp),
                ("mode", _i), ("geom_cpu_twin", _i)]


class Oracle:
    """The C restatement.  Arrays are numpy, x-fastest ([Z][Y][X] C order)."""

    def __init__(self, path: str | None = None):
        self.lib = C.CDLL(path or build_oracle())
        L = self.lib
        L.orc_nogrid.restype = _i
        L.orc_nogrid.argtypes = [_l, _l, _l, _f, _i]
        L.orc_dir_coeffs.argtypes = [_f, _f, _f, _i, _fp]
        L.orc_line_offset.argtypes = [_i, _i, _f, _fp, _fp]
        L.orc_cross2point.restype = _i
        L.orc_cross2point.argtypes = [_l, _l, _l, _f, _f, _f, _f, _f, _f, _ip, _ip]
        L.orc_line_valid.restype = _i
        L.orc_line_valid.argtypes = [_l, _l, _l, _ip, _ip]
        L.orc_walk.restype = _i
        L.orc_walk.argtypes = [_l, _l, _l, _ip, _ip, _f, _f, _f, _f, _f, _f, _bp, _i]
        L.orc_walk_rule.restype = _i
        L.orc_walk_rule.argtypes = [_l, _l, _l, _ip, _ip, _f, _f, _f, _f, _f, _f, _i, _fp, _bp, _i]
        L.orc_trace_direction.restype = _l
        L.orc_trace_direction.argtypes = [_l, _l, _l, _f, _f, _f, _f, _i, _ip, _ip, _ip, _fp]
        for s, ptr in (("f32", _fp), ("f64", _dp)):
            fn = getattr(L, "orc_sweep_" + s)
            fn.restype = _l
            fn.argtypes = [C.POINTER(OrcProblem), _fp, _fp, _fp, _fp, ptr, ptr, ptr, _i]
            fn = getattr(L, "orc_solve_" + s)
            fn.restype = _l
            fn.argtypes = [C.POINTER(OrcProblem), _fp, _fp, _fp, _fp, _fp, _i, ptr, ptr, _i]
            fn = getattr(L, "orc_divide_" + s)
            fn.argtypes = [_l, ptr, ptr, ptr, _i]
        L.orc_solve_cached_f64.restype = _l
        L.orc_solve_cached_f64.argtypes = [C.POINTER(OrcProblem), _fp, _fp, _fp, _fp, _fp, _i, _d, _dp, _dp, _i,
                                           _ip, _dp, _ip, _i, _dp]
        L.orc_sor_steps_f64.argtypes = [_l, _l, _l, _dp, _dp, _l, _i]
        L.orc_sor_converged_f64.restype = _l
        L.orc_sor_converged_f64.argtypes = [_l, _l, _l, _dp, _d, _l, _dp, _i]
        L.orc_sor_steps_to_f64.restype = _l
        L.orc_sor_steps_to_f64.argtypes = [_l, _l, _l, _dp, _dp, _d, _l, _l, _i, _dp]
        L.orc_cache_build.restype = C.c_void_p
        L.orc_cache_build.argtypes = [C.POINTER(OrcProblem), _fp, _i]
        L.orc_cache_errors.restype = _l
        L.orc_cache_errors.argtypes = [C.c_void_p]
        L.orc_cache_free.argtypes = [C.c_void_p]
        L.orc_cache_sweep_f64.argtypes = [C.c_void_p, _fp, _fp, _fp, _fp, _dp, _dp, _dp]
        L.orc_adjoint_modes_f64.argtypes = [C.POINTER(OrcProblem), _fp, _i, _dp, _dp, _dp, _dp]
        L.orc_adjoint_f64.argtypes = [C.POINTER(OrcProblem), _i, _dp, _dp, _dp, _dp]
        L.orc_calindex.argtypes = [_l, _l, _l, _lp]
        L.orc_curl.argtypes = [_l, _l, _l, _f, _f, _f, _fp, _fp, _fp, _fp, _fp]
        L.orc_num_threads.restype = _i
        L.orc_centre_integration.argtypes = [_l, _l, _l, C.c_double, C.c_double, C.c_double, C.c_double, _dp, _dp,
                                             _dp, C.c_double, _dp]

    # -- geometry ----------------------------------------------------------------------
    def nogrid(self, dims, ls, cpu_twin=False) -> int:
        X, Y, Z = dims
        return self.lib.orc_nogrid(X, Y, Z, ls, int(cpu_twin))

    def dir_coeffs(self, k, cpu_twin=False) -> np.ndarray:
        k = np.asarray(k, np.float32)
        out = np.zeros((len(k), 4), np.float32)
        for d in range(len(k)):
            self.lib.orc_dir_coeffs(float(k[d, 0]), float(k[d, 1]), float(k[d, 2]), int(cpu_twin),
                                    _ptr(out[d], C.c_float))
        return out

    def trace_direction(self, dims, ls, kd, cpu_twin=False):
        """Per lattice point: valid flag, (in ijk, out ijk), walk length, offset xyz."""
        X, Y, Z = dims
        ng = self.nogrid(dims, ls, cpu_twin)
        n = ng * ng
        valid = np.zeros(n, np.int32)
        inout = np.zeros((n, 6), np.int32)
        nsteps = np.zeros(n, np.int32)
        xyz = np.zeros((n, 3), np.float32)
        self.lib.orc_trace_direction(X, Y, Z, ls, float(kd[0]), float(kd[1]), float(kd[2]), int(cpu_twin),
                                     _ptr(valid, C.c_int), _ptr(inout, C.c_int), _ptr(nsteps, C.c_int),
                                     _ptr(xyz, C.c_float))
        return valid, inout, nsteps, xyz

    def walk(self, dims, inout, xyz, kd, rule=0, curl=None, allow_early_stop=False) -> np.ndarray:
        """Staircase of one line under walk rule `rule` (orc_walk_rule; rule 3 reads curl).
        A walk that stops early raises unless allow_early_stop (the variant rules stop by
        design)."""
        X, Y, Z = dims
        cap = X + Y + Z + 4
        ax = np.zeros(cap, np.int8)
        i = np.ascontiguousarray(inout[:3], np.int32)
        o = np.ascontiguousarray(inout[3:], np.int32)
        c = None if curl is None else np.ascontiguousarray(np.asarray(curl, np.float32).reshape(-1))
        n = self.lib.orc_walk_rule(X, Y, Z, _ptr(i, C.c_int), _ptr(o, C.c_int), float(xyz[0]), float(xyz[1]),
                                   float(xyz[2]), float(kd[0]), float(kd[1]), float(kd[2]), int(rule),
                                   None if c is None else _ptr(c, C.c_float), _ptr(ax, C.c_byte), cap)
        if n < 0:
            if not allow_early_stop:
                raise RuntimeError("walk failed")
            n = -n - 1
        return ax[:n].copy()

    # -- sweeps ------------------------------------------------------------------------
    def _problem(self, dims, spacing, rho, ls, thr, k, mode, cpu_twin):
        k = np.ascontiguousarray(np.asarray(k, np.float32))
        ks = [np.ascontiguousarray(k[:, a]) for a in range(3)]
        P = OrcProblem(dims[0], dims[1], dims[2], spacing[0], spacing[1], spacing[2], rho, ls, thr,
                       len(k), _ptr(ks[0], C.c_float), _ptr(ks[1], C.c_float), _ptr(ks[2], C.c_float),
                       int(mode), int(cpu_twin))
        return P, ks

    def solve(self, dims, spacing, k, au, av, aw, p_init, niter, *, rho=1.0, ls=1.0, mode=0, thr=0.0,
              curl=None, precision="f32", nthreads=1, cpu_twin=False):
        """The reference iteration: p = pn = p_init, niter x {sweep, p = pn/count}."""
        P, keep = self._problem(dims, spacing, rho, ls, thr, k, mode, cpu_twin)
        dt = np.float32 if precision == "f32" else np.float64
        ct = C.c_float if precision == "f32" else C.c_double
        V = dims[0] * dims[1] * dims[2]
        f = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
        au, av, aw, p_init = f(au), f(av), f(aw), f(p_init)
        curl = f(curl) if curl is not None else np.zeros(V, np.float32)
        p = np.zeros(V, dt)
        cnt = np.zeros(V, dt)
        fn = getattr(self.lib, "orc_solve_" + precision)
        err = fn(C.byref(P), _ptr(au, C.c_float), _ptr(av, C.c_float), _ptr(aw, C.c_float),
                 _ptr(curl, C.c_float), _ptr(p_init, C.c_float), int(niter), _ptr(p, ct), _ptr(cnt, ct),
                 int(nthreads))
        if err:
            raise RuntimeError("oracle: %d lines hit the wrong-point branch" % err)
        return p, cnt

    def solve_cached(self, dims, spacing, k, au, av, aw, p_init, niter, *, rho=1.0, ls=1.0, mode=0, thr=0.0,
                     curl=None, tol=0.0, nthreads=1, cpu_twin=False, save_at=()):
        """The FP64 reference iteration of ``solve(precision="f64")`` with the lines traced
        and walked once (orc_solve_cached_f64): up to niter iterations, stopping early once
        the mean-gauged relative change is below tol (tol > 0).  Returns (p, count,
        iterations, last relative change), plus a dict {k: p after k iterations} when
        save_at lists iteration counts."""
        P, keep = self._problem(dims, spacing, rho, ls, thr, k, mode, cpu_twin)
        V = dims[0] * dims[1] * dims[2]
        f = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
        au, av, aw, p_init = f(au), f(av), f(aw), f(p_init)
        curl = f(curl) if curl is not None else np.zeros(V, np.float32)
        p = np.zeros(V, np.float64)
        cnt = np.zeros(V, np.float64)
        its = C.c_int(0)
        rel = C.c_double(0.0)
        at = np.ascontiguousarray(sorted(int(x) for x in save_at), dtype=np.int32)
        saves = np.zeros((max(len(at), 1), V), np.float64)
        err = self.lib.orc_solve_cached_f64(C.byref(P), _ptr(au, C.c_float), _ptr(av, C.c_float),
                                            _ptr(aw, C.c_float), _ptr(curl, C.c_float), _ptr(p_init, C.c_float),
                                            int(niter), float(tol), _ptr(p, C.c_double), _ptr(cnt, C.c_double),
                                            int(nthreads), C.byref(its), C.byref(rel),
                                            _ptr(at, C.c_int) if len(at) else None, len(at), _ptr(saves, C.c_double))
        if err:
            raise RuntimeError("oracle: %d lines hit the wrong-point branch" % err)
        if len(at):
            return p, cnt, its.value, rel.value, {int(a): saves[j] for j, a in enumerate(at)}
        return p, cnt, its.value, rel.value

    def fixed_point(self, dims, spacing, k, au, av, aw, *, rho=1.0, ls=1.0, mode=0, thr=0.0, curl=None, tol=1e-10,
                    max_iter=500, memory=6, nthreads=1, p_init=None):
        """The fixed point of the FP64 reference iteration, mean-gauged over the voxels with
        count > 0, found by Anderson acceleration (type II, `memory` differences) of the map
        G(p) = (sweep of p) / count where count > 0, else p_init, with the mean over those
        voxels removed.  G is one iteration of ``solve(precision="f64")`` (lines traced once,
        orc_cache_*); the seeding of the reference's first sweep changes only the transient.
        Stops when ||G(p) - p|| <= tol ||G(p)|| over those voxels.  Returns (p, count,
        G evaluations, final residual).  The fixed point is unique (up to the removed
        constant) when the iteration couples all receiving voxels, e.g. the selected method
        with a threshold above every curl; where it splits them into islands, each island
        keeps a free constant that the transient of the plain iteration sets, and
        solve_cached is the reference."""
        P, keep = self._problem(dims, spacing, rho, ls, thr, k, mode, False)
        V = dims[0] * dims[1] * dims[2]
        f = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
        au, av, aw = f(au), f(av), f(aw)
        curl = f(curl) if curl is not None else np.zeros(V, np.float32)
        p_init = np.zeros(V, np.float64) if p_init is None else np.asarray(p_init, np.float64).reshape(-1)
        h = self.lib.orc_cache_build(C.byref(P), _ptr(curl, C.c_float), int(nthreads))
        try:
            if self.lib.orc_cache_errors(h):
                raise RuntimeError("oracle: lines hit the wrong-point branch")
            pn = np.zeros(V, np.float64)
            cnt = np.zeros(V, np.float64)
            full = p_init.copy()

            def sweep_into(vol):
                pn.fill(0.0)
                cnt.fill(0.0)
                self.lib.orc_cache_sweep_f64(h, _ptr(au, C.c_float), _ptr(av, C.c_float), _ptr(aw, C.c_float),
                                             _ptr(curl, C.c_float), _ptr(vol, C.c_double), _ptr(pn, C.c_double),
                                             _ptr(cnt, C.c_double))

            def G(x):
                full[sel] = x
                sweep_into(full)
                y = pn[sel]
                y /= cnt[sel]
                y -= y.mean()
                return y

            # the voxels that receive contributions depend on the field only: one sweep finds them
            sweep_into(full)
            sel = cnt > 0
            x = np.zeros(int(sel.sum()), np.float64)
            g = G(x)
            fx = g - x
            evals, dF, dG = 1, [], []
            res = np.linalg.norm(fx) / max(np.linalg.norm(g), 1e-300)
            while res > tol and evals < max_iter:
                xn = g.copy()
                if dF:  # least squares min ||fx - dF gamma|| by its normal equations (m x m)
                    M = np.array([[np.dot(a, b) for b in dF] for a in dF])
                    r = np.array([np.dot(a, fx) for a in dF])
                    gamma = np.linalg.lstsq(M, r, rcond=None)[0]
                    for gm, d in zip(gamma, dG):
                        xn -= gm * d
                gn = G(xn)
                fn = gn - xn
                evals += 1
                dF.append(fn - fx)
                dG.append(gn - g)
                if len(dF) > memory:
                    dF.pop(0)
                    dG.pop(0)
                x, g, fx = xn, gn, fn
                res = np.linalg.norm(fx) / max(np.linalg.norm(g), 1e-300)
            out = p_init.copy()
            out[sel] = g
            return out, cnt.copy(), evals, float(res)
        finally:
            self.lib.orc_cache_free(h)

    def sweep(self, dims, spacing, k, au, av, aw, p, *, rho=1.0, ls=1.0, mode=0, thr=0.0, curl=None,
              precision="f32", nthreads=1, cpu_twin=False):
        """One sweep from p: returns (pn, count) without normalisation."""
        P, keep = self._problem(dims, spacing, rho, ls, thr, k, mode, cpu_twin)
        dt = np.float32 if precision == "f32" else np.float64
        ct = C.c_float if precision == "f32" else C.c_double
        V = dims[0] * dims[1] * dims[2]
        f = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
        au, av, aw = f(au), f(av), f(aw)
        curl = f(curl) if curl is not None else np.zeros(V, np.float32)
        p = np.ascontiguousarray(np.asarray(p, dt).reshape(-1))
        pn = np.zeros(V, dt)
        cnt = np.zeros(V, dt)
        fn = getattr(self.lib, "orc_sweep_" + precision)
        err = fn(C.byref(P), _ptr(au, C.c_float), _ptr(av, C.c_float), _ptr(aw, C.c_float),
                 _ptr(curl, C.c_float), _ptr(p, ct), _ptr(pn, ct), _ptr(cnt, ct), int(nthreads))
        if err:
            raise RuntimeError("oracle: %d lines hit the wrong-point branch" % err)
        return pn, cnt

    def adjoint(self, dims, spacing, k, niter, g, *, rho=1.0, ls=1.0):
        """FP64 gradient of <g, p_niter> with respect to (au, av, aw), plain method."""
        P, keep = self._problem(dims, spacing, rho, ls, 0.0, k, 0, False)
        V = dims[0] * dims[1] * dims[2]
        g = np.ascontiguousarray(np.asarray(g, np.float64).reshape(-1))
        out = [np.zeros(V, np.float64) for _ in range(3)]
        self.lib.orc_adjoint_f64(C.byref(P), int(niter), _ptr(g, C.c_double), *[_ptr(o, C.c_double) for o in out])
        return out

    def adjoint_modes(self, dims, spacing, k, niter, g, *, rho=1.0, ls=1.0, mode=0, thr=0.0, curl=None):
        """FP64 gradient of <g, p_niter> with respect to (au, av, aw) for any mode, curl held
        fixed (orc_adjoint_modes_f64: the full-voxel iteration, no anchor operator)."""
        P, keep = self._problem(dims, spacing, rho, ls, thr, k, mode, False)
        V = dims[0] * dims[1] * dims[2]
        g = np.ascontiguousarray(np.asarray(g, np.float64).reshape(-1))
        curl = np.ascontiguousarray(np.asarray(curl, np.float32).reshape(-1)) if curl is not None else np.zeros(
            V, np.float32)
        out = [np.zeros(V, np.float64) for _ in range(3)]
        self.lib.orc_adjoint_modes_f64(C.byref(P), _ptr(curl, C.c_float), int(niter), _ptr(g, C.c_double),
                                       *[_ptr(o, C.c_double) for o in out])
        return out

    def calindex(self, dims) -> np.ndarray:
        X, Y, Z = dims
        idx = np.full(X * Y * Z, -1, np.int64)
        self.lib.orc_calindex(X, Y, Z, _ptr(idx, C.c_long))
        return idx

    def curl(self, dims, spacing, au, av, aw, mask) -> np.ndarray:
        X, Y, Z = dims
        f = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
        au, av, aw, mask = f(au), f(av), f(aw), f(mask)
        out = np.zeros(X * Y * Z, np.float32)
        self.lib.orc_curl(X, Y, Z, spacing[0], spacing[1], spacing[2], _ptr(au, C.c_float),
                          _ptr(av, C.c_float), _ptr(aw, C.c_float), _ptr(mask, C.c_float),
                          _ptr(out, C.c_float))
        return out

    def centre_integration(self, dims, spacing, au, av, aw, *, rho=1.0, pref=0.0) -> np.ndarray:
        """initialIntegration.cpp restated: FP64 p integrated outward from the centre voxel."""
        X, Y, Z = dims
        f = lambda a: np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1))
        au, av, aw = f(au), f(av), f(aw)
        out = np.zeros(X * Y * Z, np.float64)
        self.lib.orc_centre_integration(X, Y, Z, float(spacing[0]), float(spacing[1]), float(spacing[2]), float(rho),
                                        _ptr(au, C.c_double), _ptr(av, C.c_double), _ptr(aw, C.c_double),
                                        float(pref), _ptr(out, C.c_double))
        return out

    # -- the reference's CPU Poisson baseline (sor3D), restated for counting its steps ------
    def sor_steps(self, dims, rhs, p, nsteps, nthreads=1):
        """nsteps steps of sor3D's weighted Jacobi iteration (orc_sor_steps_f64) from p."""
        X, Y, Z = dims
        rhs = np.ascontiguousarray(np.asarray(rhs, np.float64).reshape(-1))
        p = np.array(np.asarray(p, np.float64).reshape(-1), copy=True)
        self.lib.orc_sor_steps_f64(X, Y, Z, _ptr(rhs, C.c_double), _ptr(p, C.c_double), int(nsteps), int(nthreads))
        return p

    def sor_converged(self, dims, rhs, tol=1e-12, max_iter=1000000, nthreads=1):
        """Mean-free fixed point of sor3D's iteration by conjugate gradients; (p, CG iterations)."""
        X, Y, Z = dims
        rhs = np.ascontiguousarray(np.asarray(rhs, np.float64).reshape(-1))
        p = np.zeros(X * Y * Z, np.float64)
        its = self.lib.orc_sor_converged_f64(X, Y, Z, _ptr(rhs, C.c_double), float(tol), int(max_iter),
                                             _ptr(p, C.c_double), int(nthreads))
        return p, int(its)

    def sor_steps_to(self, dims, rhs, ref, target=1e-3, max_steps=10 ** 8, check=64, nthreads=1):
        """Even number of sor3D steps from zero after which the mean-gauged relative L2
        distance from ref (mean-free) is at most target; (steps or -1, distance)."""
        X, Y, Z = dims
        rhs = np.ascontiguousarray(np.asarray(rhs, np.float64).reshape(-1))
        ref = np.ascontiguousarray(np.asarray(ref, np.float64).reshape(-1))
        err = C.c_double(0.0)
        n = self.lib.orc_sor_steps_to_f64(X, Y, Z, _ptr(rhs, C.c_double), _ptr(ref, C.c_double), float(target),
                                          int(max_steps), int(check), int(nthreads), C.byref(err))
        return int(n), err.value

    def num_threads(self) -> int:
        return self.lib.orc_num_threads()


class RefLib:
    """The reference's own functions (see oracle/build_ref.sh)."""

    def __init__(self, path: str | None = None):
        path = path or build_ref()
        if path is None:
            raise FileNotFoundError("reference sources are not staged on this machine")
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_calindex.argtypes = [_l, _l, _l, _lp]
        L.ref_cross2point.restype = _i
        L.ref_cross2point.argtypes = [_l, _l, _l, _f, _f, _f, _f, _f, _f, _ip]
        common = [_l, _l, _l, _f, _f, _f, _f, _f, _f]
        L.ref_sweep.restype = C.c_longlong
        L.ref_sweep.argtypes = common + [_i, _fp, _fp, _fp, _i, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _i]
        L.ref_sweep_dirs.argtypes = common + [_i, _i, _fp, _fp, _fp, _i, _fp, _fp, _fp, _fp, _fp, _fp, _fp]
        L.ref_solve.argtypes = common + [_i, _fp, _fp, _fp, _i, _fp, _fp, _fp, _fp, _fp, _i, _fp, _fp, _i]
        L.ref_cpu_twin_solve.argtypes = [_l, _l, _l, _f, _f, _f, _f, _f, _i, _fp, _fp, _fp, _fp, _fp, _fp,
                                         _fp, _i, _fp, _fp]
        L.ref_curl.argtypes = [_l, _l, _l, _f, _f, _f, _fp, _fp, _fp, _fp, _fp]
        L.ref_sor.argtypes = [_i, _i, _i, _d, _d, _d, _d, _dp, _dp, _dp, _i, _d, _dp]
        L.ref_calrhs.argtypes = [_i, _i, _i, _d, _d, _d, _d, _dp, _dp, _dp, _dp]
        L.ref_num_threads.restype = _i
        L.ref_initial_integration.argtypes = [C.c_long, C.c_long, C.c_long, _d, _d, _d, _d, _dp, _dp, _dp, _d, _dp]

    @staticmethod
    def _f(a):
        return np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))

    def calindex(self, dims):
        X, Y, Z = dims
        idx = np.full(X * Y * Z, -1, np.int64)
        self.lib.ref_calindex(X, Y, Z, _ptr(idx, C.c_long))
        return idx

    def cross2point(self, dims, xyz, kd):
        io = np.zeros(6, np.int32)
        ok = self.lib.ref_cross2point(dims[0], dims[1], dims[2], float(xyz[0]), float(xyz[1]), float(xyz[2]),
                                      float(kd[0]), float(kd[1]), float(kd[2]), _ptr(io, C.c_int))
        return ok, io

    def solve(self, dims, spacing, k, au, av, aw, p_init, niter, *, rho=1.0, ls=1.0, mode=0, thr=0.0,
              curl=None, nthreads=1):
        X, Y, Z = dims
        V = X * Y * Z
        k = np.asarray(k, np.float32)
        k1, k2, k3 = (np.ascontiguousarray(k[:, a]) for a in range(3))
        au, av, aw, p_init = self._f(au), self._f(av), self._f(aw), self._f(p_init)
        curl = self._f(curl) if curl is not None else np.zeros(V, np.float32)
        p = np.zeros(V, np.float32)
        cnt = np.zeros(V, np.float32)
        self.lib.ref_solve(X, Y, Z, spacing[0], spacing[1], spacing[2], rho, ls, thr, len(k),
                           _ptr(k1, C.c_float), _ptr(k2, C.c_float), _ptr(k3, C.c_float), int(mode),
                           _ptr(au, C.c_float), _ptr(av, C.c_float), _ptr(aw, C.c_float), _ptr(curl, C.c_float),
                           _ptr(p_init, C.c_float), int(niter), _ptr(p, C.c_float), _ptr(cnt, C.c_float),
                           int(nthreads))
        return p, cnt

    def sweep(self, dims, spacing, k, au, av, aw, p, *, rho=1.0, ls=1.0, mode=0, thr=0.0, curl=None, nthreads=1):
        """One full-coverage sweep over the given directions; returns (pn, count, units)."""
        X, Y, Z = dims
        V = X * Y * Z
        k = np.asarray(k, np.float32)
        k1, k2, k3 = (np.ascontiguousarray(k[:, a]) for a in range(3))
        au, av, aw, p = self._f(au), self._f(av), self._f(aw), self._f(p)
        curl = self._f(curl) if curl is not None else np.zeros(V, np.float32)
        pn = np.zeros(V, np.float32)
        cnt = np.zeros(V, np.float32)
        units = self.lib.ref_sweep(X, Y, Z, spacing[0], spacing[1], spacing[2], rho, ls, thr, len(k),
                                   _ptr(k1, C.c_float), _ptr(k2, C.c_float), _ptr(k3, C.c_float), int(mode),
                                   _ptr(au, C.c_float), _ptr(av, C.c_float), _ptr(aw, C.c_float),
                                   _ptr(curl, C.c_float), _ptr(p, C.c_float), _ptr(pn, C.c_float),
                                   _ptr(cnt, C.c_float), int(nthreads))
        return pn, cnt, int(units)

    def sweep_dirs(self, dims, spacing, k, d0, d1, au, av, aw, p, *, rho=1.0, ls=1.0, mode=0, thr=0.0,
                   curl=None, pn=None, cnt=None):
        X, Y, Z = dims
        V = X * Y * Z
        k = np.asarray(k, np.float32)
        k1, k2, k3 = (np.ascontiguousarray(k[:, a]) for a in range(3))
        curl = curl if curl is not None else np.zeros(V, np.float32)
        pn = pn if pn is not None else np.zeros(V, np.float32)
        cnt = cnt if cnt is not None else np.zeros(V, np.float32)
        self.lib.ref_sweep_dirs(X, Y, Z, spacing[0], spacing[1], spacing[2], rho, ls, thr, int(d0), int(d1),
                                _ptr(k1, C.c_float), _ptr(k2, C.c_float), _ptr(k3, C.c_float), int(mode),
                                _ptr(au, C.c_float), _ptr(av, C.c_float), _ptr(aw, C.c_float),
                                _ptr(curl, C.c_float), _ptr(p, C.c_float), _ptr(pn, C.c_float),
                                _ptr(cnt, C.c_float))
        return pn, cnt

    def cpu_twin_solve(self, dims, spacing, k, au, av, aw, p_init, niter, *, rho=1.0, ls=1.0):
        X, Y, Z = dims
        V = X * Y * Z
        k = np.asarray(k, np.float32)
        k1, k2, k3 = (np.ascontiguousarray(k[:, a]) for a in range(3))
        au, av, aw, p_init = self._f(au), self._f(av), self._f(aw), self._f(p_init)
        p = np.zeros(V, np.float32)
        cnt = np.zeros(V, np.float32)
        self.lib.ref_cpu_twin_solve(X, Y, Z, spacing[0], spacing[1], spacing[2], rho, ls, len(k),
                                    _ptr(k1, C.c_float), _ptr(k2, C.c_float), _ptr(k3, C.c_float),
                                    _ptr(au, C.c_float), _ptr(av, C.c_float), _ptr(aw, C.c_float),
                                    _ptr(p_init, C.c_float), int(niter), _ptr(p, C.c_float), _ptr(cnt, C.c_float))
        return p, cnt

    def curl(self, dims, spacing, au, av, aw, mask):
        X, Y, Z = dims
        au, av, aw, mask = self._f(au), self._f(av), self._f(aw), self._f(mask)
        out = np.zeros(X * Y * Z, np.float32)
        self.lib.ref_curl(X, Y, Z, spacing[0], spacing[1], spacing[2], _ptr(au, C.c_float), _ptr(av, C.c_float),
                          _ptr(aw, C.c_float), _ptr(mask, C.c_float), _ptr(out, C.c_float))
        return out

    def calrhs(self, dims, spacing, au, av, aw, *, rho=1.0):
        """calRHS (with its output-dropping line 10 left out of the staged copy)."""
        X, Y, Z = dims
        g = lambda a: np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1))
        au, av, aw = g(au), g(av), g(aw)
        rhs = np.zeros(X * Y * Z, np.float64)
        self.lib.ref_calrhs(X, Y, Z, spacing[0], spacing[1], spacing[2], rho, _ptr(au, C.c_double),
                            _ptr(av, C.c_double), _ptr(aw, C.c_double), _ptr(rhs, C.c_double))
        return rhs

    def sor(self, dims, spacing, au, av, aw, niter, eps, *, rho=1.0, p0=None):
        """sor3D from p0 (zero by default) for niter steps (run in pairs) or until its mean
        |residual| is below eps."""
        X, Y, Z = dims
        g = lambda a: np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1))
        au, av, aw = g(au), g(av), g(aw)
        p = np.zeros(X * Y * Z, np.float64) if p0 is None else np.array(g(p0), copy=True)
        self.lib.ref_sor(X, Y, Z, spacing[0], spacing[1], spacing[2], rho, _ptr(au, C.c_double),
                         _ptr(av, C.c_double), _ptr(aw, C.c_double), int(niter), float(eps), _ptr(p, C.c_double))
        return p

    def initial_integration(self, dims, spacing, au, av, aw, *, rho=1.0, pref=0.0) -> np.ndarray:
        """The reference's initialIntegration (initialIntegration.cpp) on zeroed buffers."""
        X, Y, Z = dims
        g = lambda a: np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1))
        au, av, aw = g(au), g(av), g(aw)
        p = np.zeros(X * Y * Z, np.float64)
        self.lib.ref_initial_integration(X, Y, Z, spacing[0], spacing[1], spacing[2], rho, _ptr(au, C.c_double),
                                         _ptr(av, C.c_double), _ptr(aw, C.c_double), float(pref), _ptr(p, C.c_double))
        return p

    def num_threads(self) -> int:
        return self.lib.ref_num_threads()


def load_reference_directions(level_file: str) -> np.ndarray | None:
    """Direction file of the reference tree (OMNI3D_REFERENCE_ROOT), or of the staged copy
    that build_ref.sh keeps beside the staged sources; None when neither is present."""
    cands = [os.path.join(HERE, "_ref", "src", level_file)]
    if REFERENCE_ROOT is not None:
        cands.insert(0, os.path.join(REFERENCE_ROOT, "Omni3D_8.0", "Executable", level_file))
    path = next((c for c in cands if os.path.exists(c)), None)
    if path is None:
        return None
    rows = open(path).read().replace("\r", "").strip().split("\n")
    return np.array([[float(x) for x in r.split()] for r in rows[:-1]], np.float32)


def icosphere(level: int) -> np.ndarray:
    """Direction vertices of the shipped GridIcosahedronDivide<level>.dat sets (12, 42, 162,
    642, ... vertices), restated in numpy for the CPU arms: recursive midpoint subdivision of
    the icosahedron with poles at +-z, the lower ring at z = -1/sqrt(5) and the upper ring,
    rotated by pi/5, at z = 0.46000602 (the shipped files' value), printed with six decimals
    and read back as the reference reads its direction file, sorted lexicographically."""
    zl, rl = -1.0 / np.sqrt(5.0), 2.0 / np.sqrt(5.0)
    zu = 0.46000602
    ru = np.sqrt(1.0 - zu * zu)
    verts = [(0.0, 0.0, 1.0), (0.0, 0.0, -1.0)]
    verts += [(rl * np.cos(2 * np.pi * k / 5), rl * np.sin(2 * np.pi * k / 5), zl) for k in range(5)]
    verts += [(ru * np.cos(2 * np.pi * k / 5 + np.pi / 5), ru * np.sin(2 * np.pi * k / 5 + np.pi / 5), zu)
              for k in range(5)]
    faces = []
    for k in range(5):
        a, b, ua, ub = 2 + k, 2 + (k + 1) % 5, 7 + k, 7 + (k + 1) % 5
        faces += [(1, b, a), (0, ua, ub), (a, b, ua), (b, ub, ua)]
    for _ in range(1, level):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = np.add(verts[a], verts[b])
                verts.append(tuple(m / np.sqrt(float(np.dot(m, m)))))
                mid[key] = len(verts) - 1
            return mid[key]

        nxt = []
        for t in faces:
            ab, bc, ca = midpoint(t[0], t[1]), midpoint(t[1], t[2]), midpoint(t[2], t[0])
            nxt += [(t[0], ab, ca), (t[1], bc, ab), (t[2], ca, bc), (ab, bc, ca)]
        faces = nxt
    rows = sorted(tuple(float(s) for s in ("%f %f %f" % v).split()) for v in verts)
    return np.array(rows, np.float32)
