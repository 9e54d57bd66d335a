"""The brick engine (lines cut into 16^3-brick segments, each brick's field staged in shared
memory by TMA, sums kept in shared memory) against the line engine and the FP64 oracle.

Plain-method counts are integers and must agree exactly; sums agree within the same
relative L2 bounds as the line engine's parity tests.  Grid sizes that are not multiples
of 16 exercise partial bricks and the zero-filled halo beyond the volume."""
import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu

TOL_PN = 1e-5
TOL_P_PLAIN = 2e-5
TOL_P_SELECT = 1e-4


def _field(dims, seed, noise=0.05, sphere=None):
    return synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 5.0), noise=noise, seed=seed, spacing=1e-3,
                           sphere_radius=sphere)


def _sweep(omni, dims, f, dirs, p, method, engine, curl=None, thr=0.0):
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=1, method=method, threshold=thr, engine=engine) as s:
        return s.sweep(f["ax"], f["ay"], f["az"], p, curl=curl)


@pytest.mark.parametrize("dims", [(20, 17, 13), (33, 16, 40), (3, 5, 4)])
@pytest.mark.parametrize("method", ["plain", "weighted", "select"])
def test_brick_sweep_matches_line_sweep(omni, orc, dims, method):
    f = _field(dims, seed=31, sphere=min(dims) / 4.0)
    dirs = omni.icosphere(3)
    p = np.random.default_rng(2).normal(0, 0.5, np.prod(dims)).astype(np.float32)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"]) if method != "plain" else None
    thr = float(np.percentile(curl[curl > 0], 75)) if method == "select" else 0.0
    pn_l, c_l = _sweep(omni, dims, f, dirs, p, method, "lines", curl, thr)
    pn_b, c_b = _sweep(omni, dims, f, dirs, p, method, "bricks", curl, thr)
    if method == "plain":
        np.testing.assert_array_equal(c_b, c_l)
    else:
        np.testing.assert_array_equal(c_b > 0, c_l > 0)
        assert synthetic.relative_l2(c_b, c_l, gauge="none") < TOL_PN
    assert synthetic.relative_l2(pn_b, pn_l, gauge="none") < TOL_PN


@pytest.mark.parametrize("method,solver", [("plain", "anchor"), ("plain", "sweep"), ("select", "anchor"),
                                           ("select", "sweep"), ("weighted", "anchor")])
def test_brick_solve_matches_oracle(omni, orc, method, solver):
    dims = (37, 29, 22)
    f = _field(dims, seed=32, noise=0.1, sphere=6.0)
    dirs = omni.icosphere(3)
    p0 = np.zeros(np.prod(dims), np.float32)
    p0[: dims[0] * 3] = 0.3
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.percentile(curl[curl > 0], 80)) if method == "select" else 0.0
    mode = {"plain": 0, "select": 1, "weighted": 2}[method]
    niter = 4
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=niter, method=method, threshold=thr, solver=solver,
                     engine="bricks") as s:
        r = s.solve(f["ax"], f["ay"], f["az"], curl=curl if method != "plain" else None, p_init=p0)
    assert r.stats["engine_used"] == 2
    ep, ecnt = orc.solve(dims, f["spacing"], dirs, f["ax"], f["ay"], f["az"], p0, niter, mode=mode, thr=thr, curl=curl,
                         precision="f64")
    if method == "plain":
        np.testing.assert_array_equal(r.count.reshape(-1), ecnt.astype(np.float32))
        assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_PLAIN
    else:
        assert synthetic.relative_l2(r.count, ecnt, gauge="none") < 1e-5
        assert synthetic.relative_l2(r.p, ep, gauge="none") < TOL_P_SELECT


def test_select_threshold_free_masked_sphere(omni, orc):
    """The bench's form: threshold above every curl, lines split only at the masked sphere,
    which spans many bricks (segments restart inside bricks and carry across them)."""
    dims = (48, 40, 36)
    f = _field(dims, seed=33, sphere=10.0)
    dirs = omni.icosphere(3)
    curl = orc.curl(dims, f["spacing"], f["ax"], f["ay"], f["az"], f["mask"])
    thr = float(np.finfo(np.float32).max)
    out = {}
    for engine in ("lines", "bricks"):
        with omni.Omni3D(dims, f["spacing"], dirs, max_iter=5, method="select", threshold=thr, engine=engine,
                         gauge="mean") as s:
            out[engine] = s.solve(f["ax"], f["ay"], f["az"], curl=curl)
            assert out[engine].stats["engine_used"] == (2 if engine == "bricks" else 1)
    np.testing.assert_array_equal(out["bricks"].count > 0, out["lines"].count > 0)
    assert synthetic.relative_l2(out["bricks"].p, out["lines"].p, gauge="none") < 1e-5


def test_engine_selection(omni):
    dims = (18, 18, 18)
    f = _field(dims, seed=34)
    dirs = omni.icosphere(2)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2) as s:
        assert s.solve(f["ax"], f["ay"], f["az"]).stats["engine_used"] == 1  # automatic: lines (faster)
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2, engine="bricks") as s:
        assert s.solve(f["ax"], f["ay"], f["az"]).stats["engine_used"] == 2
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2, grad="bf16") as s:
        assert s.solve(f["ax"], f["ay"], f["az"]).stats["engine_used"] == 1  # BF16 storage: lines
    with omni.Omni3D(dims, f["spacing"], dirs, max_iter=2, grad="bf16", engine="bricks") as s:
        with pytest.raises(omni.Omni3DError):
            s.solve(f["ax"], f["ay"], f["az"])


def test_brick_solves_repeat_and_change_method_fields(omni, orc):
    """The same context solving new fields: the brick summaries are rebuilt per field."""
    dims = (24, 20, 18)
    dirs = omni.icosphere(3)
    with omni.Omni3D(dims, 1e-3, dirs, max_iter=3, engine="bricks") as sb, \
            omni.Omni3D(dims, 1e-3, dirs, max_iter=3, engine="lines") as sl:
        for seed in (40, 41, 42):
            f = _field(dims, seed=seed)
            rb = sb.solve(f["ax"], f["ay"], f["az"])
            rl = sl.solve(f["ax"], f["ay"], f["az"])
            np.testing.assert_array_equal(rb.count, rl.count)
            assert synthetic.relative_l2(rb.p, rl.p, gauge="none") < 1e-6
