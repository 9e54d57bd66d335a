"""Generate tests/golden/reference_small.npz from the reference's own CPU functions.

Run in a tree where the reference sources are available (oracle/build_ref.sh stages and
compiles them into oracle/_ref/libomni_ref.so):

    python tests/golden/make_golden.py

Each case stores its inputs (so the fixture does not depend on the generator) and the
outputs of the reference functions:
  plain    12x10x8 grid, 42 directions, 2 iterations of cross2point + bodyIntegralInner
           over every (direction, lattice point) pair with the GPU kernel's geometry, then
           the GPU normalisation (count > 0), starting from a nonzero j = 0 face
  select   14x12x10 grid with a masked sphere, 42 directions, 3 iterations of
           bodyIntegralInnerSelect, threshold at the 80th percentile of the curl
  weighted 13x11x9 grid with a masked sphere, 42 directions, 3 iterations of
           bodyIntegralInnerWeighted (curl-weighted, no entry contribution; voxels outside
           the mask have curl 0, so lines that start there skip their first steps)
  variants 12x11x9 grid with a masked sphere, 42 directions, 2 iterations of each variant
           the reference keeps beside its three methods: bodyIntegralInnerWeightedFixedBC
           (mode 3), bodyIntegralInnerSelectFixedBC (mode 4, threshold at the 75th
           percentile of the curl), bodyIntegralInnerMiniCurl (mode 5) and
           bodyIntegralInnerWeightedMiniCurl (mode 6)
  centre   11x8x9 grid: initialIntegration.cpp (FP64, outward from the centre voxel, pref 2.5)
  ls07     10x9x8 grid, 42 directions, line spacing 0.7, 2 plain iterations
  cputwin  10x10x10 grid, 42 directions, 2 iterations of the reference's own CPU loop
           omni3dparallellinesESInnerCPU + devidecountInnerCPU (no pole guard, count > 1)
  curl     the curl indicator calCurlofMaterialAccCPU of the select case
  sor      13x11x9 grid: calRHS.cpp's right-hand side (FP64; its output-dropping line 10 left
           out) and sor3D.cpp's iterate after 2 and 10 steps from zero (weighted Jacobi,
           omega 0.8, the reference's CPU Poisson baseline)
Directions are the 42-vertex icosphere (the vertex set of GridIcosahedronDivide2.dat).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "parallel-3d-pressure-reconstruction_gb300"))

import oracle  # noqa: E402
from omni3d import synthetic  # noqa: E402
from omni3d.solver import icosphere  # noqa: E402


def field(dims, seed, sphere=None):
    f = synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=seed, sphere_radius=sphere)
    return f


def pinit(dims, seed):
    nx, ny, nz = dims
    rng = np.random.default_rng(seed)
    p = np.zeros((nz, ny, nx), np.float32)
    p[:, 0, :] = rng.normal(0, 0.5, (nz, nx)).astype(np.float32)
    return p.reshape(-1)


def main():
    R = oracle.RefLib()
    dirs = icosphere(2)
    out = {"dirs": dirs}
    # plain
    d = (12, 10, 8)
    f = field(d, 1)
    p0 = pinit(d, 2)
    p, c = R.solve(d, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2)
    out.update({"plain_dims": np.array(d), "plain_spacing": np.array(f["spacing"], np.float32),
                "plain_ax": f["ax"].reshape(-1), "plain_ay": f["ay"].reshape(-1), "plain_az": f["az"].reshape(-1),
                "plain_p0": p0, "plain_p": p, "plain_count": c})
    # select
    d = (14, 12, 10)
    f = field(d, 3, sphere=3.0)
    p0 = pinit(d, 4)
    curl = R.curl(d, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = np.float32(np.percentile(curl[curl > 0], 80))
    p, c = R.solve(d, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 3, mode=1, thr=float(thr), curl=curl)
    out.update({"select_dims": np.array(d), "select_spacing": np.array(f["spacing"], np.float32),
                "select_ax": f["ax"].reshape(-1), "select_ay": f["ay"].reshape(-1), "select_az": f["az"].reshape(-1),
                "select_mask": f["mask"].reshape(-1), "select_curl": curl, "select_thr": np.array(thr),
                "select_p0": p0, "select_p": p, "select_count": c})
    # weighted
    d = (13, 11, 9)
    f = field(d, 7, sphere=3.0)
    p0 = pinit(d, 8)
    curl = R.curl(d, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    p, c = R.solve(d, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 3, mode=2, curl=curl)
    out.update({"weighted_dims": np.array(d), "weighted_spacing": np.array(f["spacing"], np.float32),
                "weighted_ax": f["ax"].reshape(-1), "weighted_ay": f["ay"].reshape(-1),
                "weighted_az": f["az"].reshape(-1), "weighted_mask": f["mask"].reshape(-1),
                "weighted_curl": curl, "weighted_p0": p0, "weighted_p": p, "weighted_count": c})
    # variants: fixed-boundary and minimum-curl walks
    d = (12, 11, 9)
    f = field(d, 9, sphere=2.5)
    p0 = pinit(d, 10)
    curl = R.curl(d, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = np.float32(np.percentile(curl[curl > 0], 75))
    out.update({"variants_dims": np.array(d), "variants_spacing": np.array(f["spacing"], np.float32),
                "variants_ax": f["ax"].reshape(-1), "variants_ay": f["ay"].reshape(-1),
                "variants_az": f["az"].reshape(-1), "variants_curl": curl, "variants_thr": np.array(thr),
                "variants_p0": p0})
    for mode in (3, 4, 5, 6):
        p, c = R.solve(d, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2, mode=mode, thr=float(thr), curl=curl)
        out.update({"variants_p_mode%d" % mode: p, "variants_count_mode%d" % mode: c})
    # centre integration
    d = (11, 8, 9)
    f = field(d, 11)
    sp32 = tuple(float(np.float32(x)) for x in f["spacing"])  # the spacing the library holds (float)
    pc = R.initial_integration(d, sp32, f["ax"], f["ay"], f["az"], rho=1.25, pref=2.5)
    out.update({"centre_dims": np.array(d), "centre_spacing": np.array(f["spacing"], np.float32),
                "centre_ax": f["ax"].reshape(-1), "centre_ay": f["ay"].reshape(-1), "centre_az": f["az"].reshape(-1),
                "centre_p": pc})
    # line spacing 0.7
    d = (10, 9, 8)
    f = field(d, 5)
    p0 = np.zeros(np.prod(d), np.float32)
    p, c = R.solve(d, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2, ls=0.7)
    out.update({"ls07_dims": np.array(d), "ls07_spacing": np.array(f["spacing"], np.float32),
                "ls07_ax": f["ax"].reshape(-1), "ls07_ay": f["ay"].reshape(-1), "ls07_az": f["az"].reshape(-1),
                "ls07_p": p, "ls07_count": c})
    # the reference's own CPU loop
    d = (10, 10, 10)
    f = field(d, 6)
    p0 = np.zeros(np.prod(d), np.float32)
    p, c = R.cpu_twin_solve(d, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, 2)
    out.update({"cputwin_dims": np.array(d), "cputwin_spacing": np.array(f["spacing"], np.float32),
                "cputwin_ax": f["ax"].reshape(-1), "cputwin_ay": f["ay"].reshape(-1),
                "cputwin_az": f["az"].reshape(-1), "cputwin_p": p, "cputwin_count": c})
    # the CPU Poisson baseline
    d = (13, 11, 9)
    f = field(d, 12)
    rhs = R.calrhs(d, f["spacing"], f["ax"], f["ay"], f["az"])
    out.update({"sor_dims": np.array(d), "sor_spacing": np.array(f["spacing"], np.float64),
                "sor_ax": f["ax"].reshape(-1), "sor_ay": f["ay"].reshape(-1), "sor_az": f["az"].reshape(-1),
                "sor_rhs": rhs})
    for k in (2, 10):
        out["sor_p%d" % k] = R.sor(d, f["spacing"], f["ax"], f["ay"], f["az"], k, 0.0)
    np.savez_compressed(os.path.join(HERE, "reference_small.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_small.npz"))


if __name__ == "__main__":
    main()
