"""Host-side checks that need no GPU: the C-ABI library loads and exports every declared
symbol, the drop-in file formats (parameter file, direction file, Tecplot input, pressure
output), the icosphere direction sets, and the error paths."""
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "omni3d.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(omni3d_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(omni):
    L = omni.lib()
    names = declared_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    from omni3d._lib import SIGNATURES

    assert sorted(SIGNATURES) == names


def test_icosphere_counts_and_norms(omni):
    for level, n in [(1, 12), (2, 42), (3, 162), (4, 642), (5, 2562)]:
        d = omni.icosphere(level)
        assert d.shape == (n, 3)
        assert np.abs(np.linalg.norm(d.astype(np.float64), axis=1) - 1).max() < 2e-6
        # sorted by (x, y, z) as the reference files are
        assert (np.diff(d[:, 0]) >= 0).all()


def test_icosphere_matches_reference_vertex_sets(omni):
    import oracle

    for level in (2, 3, 4):
        ref = oracle.load_reference_directions("GridIcosahedronDivide%d.dat" % level)
        if ref is None:
            pytest.skip("reference direction files are not present on this machine")
        mine = omni.icosphere(level)
        assert set(map(tuple, mine.tolist())) == set(map(tuple, ref.tolist()))


def test_oracle_icosphere_equals_library(omni):
    """The CPU arms take their directions from the oracle's numpy icosphere, never from the
    library: the two must give the same arrays."""
    import oracle

    for level in (1, 2, 3, 4, 5):
        np.testing.assert_array_equal(oracle.icosphere(level), omni.icosphere(level))


def test_icosphere_is_stable(omni):
    h = {lv: hashlib.sha256(omni.icosphere(lv).tobytes()).hexdigest() for lv in (3, 4)}
    golden = os.path.join(REPO, "tests", "golden", "icosphere_sha256.txt")
    rows = dict(l.split() for l in open(golden).read().split("\n") if l.strip())
    for lv in (3, 4):
        assert h[lv] == rows[str(lv)]


def test_read_directions_reference_format(omni, tmp_path):
    d = omni.icosphere(2)
    p = tmp_path / "dirs.dat"
    with open(p, "wb") as fh:
        for v in d:
            fh.write(("%f %f %f\r\n" % tuple(v)).encode())
        fh.write(b"42\r\n")
    got = omni.read_directions(str(p), 42)
    np.testing.assert_array_equal(got, d)
    with pytest.raises(omni.Omni3DError) as e:
        omni.read_directions(str(p), 50)
    assert e.value.code == -3
    with pytest.raises(omni.Omni3DError):
        omni.read_directions(str(tmp_path / "missing.dat"), 4)


PARAMS = """64
48
32
0.00024
0.00025
0.00026
1000
1
0.7
162
GridIcosahedronDivide3.dat
.\\AccelerationFilesSample\\
.\\Pressure\\
10
52921780
{extra}




----------------------------------Omni3D Standard/Weighted/Selected-Weighted Method---------------
51
"""


def test_read_params_defaults_and_hidden_lines(omni, tmp_path):
    p = tmp_path / "Parameter_Omni3D.dat"
    p.write_bytes(PARAMS.format(extra="\n\n").replace("\n", "\r\n").encode())
    fp = omni.read_params(str(p))
    assert (fp.nx_org, fp.ny_org, fp.nz_org) == (64, 48, 32)
    assert fp.dx == np.float32(0.00024) and fp.dz == np.float32(0.00026)
    assert fp.density == 1000 and fp.line_spacing == np.float32(0.7) and fp.n_dirs == 162
    assert fp.dir_file == b"GridIcosahedronDivide3.dat"
    assert fp.accel_dir == b".\\AccelerationFilesSample\\"
    assert fp.n_iter == 10 and fp.threshold == np.float32(52921780)
    assert fp.pref == 0.0
    assert list(fp.roi) == [0, 63, 0, 47, 0, 31]
    # hidden pref and region of interest
    p.write_text(PARAMS.format(extra="101325\n2\n40\n1\n30\n0\n20"))
    fp = omni.read_params(str(p))
    assert fp.pref == 101325.0 and list(fp.roi) == [2, 40, 1, 30, 0, 20]
    p.write_text(PARAMS.format(extra="0\n0\n64\n\n\n\n"))
    with pytest.raises(omni.Omni3DError) as e:
        omni.read_params(str(p))
    assert e.value.code == -3
    with pytest.raises(omni.Omni3DError):
        omni.read_params(str(tmp_path / "nope.dat"))


def _write_tecplot(path, dims, cols, values, crlf=False):
    nx, ny, nz = dims
    eol = "\r\n" if crlf else "\n"
    with open(path, "w", newline="") as fh:
        fh.write('TITLE = "acc"' + eol + 'VARIABLES = "X","Y","Z"' + eol + "ZONE I=%d, J=%d, K=%d" % dims + eol)
        for r in range(nx * ny * nz):
            fh.write(" ".join("%.6f" % values[c][r] for c in range(cols)) + "  " + eol)


@pytest.mark.parametrize("cols", [10, 7])
def test_read_tecplot_with_roi(omni, tmp_path, cols):
    dims = (6, 5, 4)
    n = int(np.prod(dims))
    rng = np.random.default_rng(0)
    vals = [rng.normal(size=n).round(4) for _ in range(cols)]
    path = tmp_path / "acc.dat"
    _write_tecplot(path, dims, cols, vals, crlf=True)
    pf = tmp_path / "P.dat"
    pf.write_text(PARAMS.replace("64\n48\n32", "6\n5\n4").format(extra="\n1\n4\n0\n3\n1\n3"))
    fp = omni.read_params(str(pf))
    got = omni.read_tecplot(str(path), fp)
    assert got["ncol"] == cols
    full = np.stack(vals).reshape(cols, 4, 5, 6)[:, 1:4, 0:4, 1:5]  # k, j, i crop
    names = ["x", "y", "z", "u", "v", "w", "ax", "ay", "az", "mask"] if cols == 10 else ["x", "y", "z", "ax", "ay",
                                                                                          "az", "mask"]
    for c, nm in enumerate(names):
        np.testing.assert_allclose(got[nm], full[c].reshape(-1), rtol=0, atol=1e-6)
    if cols == 7:
        assert (got["u"] == 0).all()


def test_read_tecplot_errors(omni, tmp_path):
    dims = (3, 3, 3)
    pf = tmp_path / "P.dat"
    pf.write_text(PARAMS.replace("64\n48\n32", "3\n3\n3").format(extra="\n\n"))
    fp = omni.read_params(str(pf))
    short = tmp_path / "short.dat"
    _write_tecplot(short, (3, 3, 2), 10, [np.zeros(18)] * 10)
    with pytest.raises(omni.Omni3DError):
        omni.read_tecplot(str(short), fp)
    bad = tmp_path / "bad.dat"
    _write_tecplot(bad, dims, 5, [np.zeros(27)] * 5)
    with pytest.raises(omni.Omni3DError):
        omni.read_tecplot(str(bad), fp)
    with pytest.raises(omni.Omni3DError):
        omni.read_tecplot(str(tmp_path / "none.dat"), fp)


def test_read_tecplot_parallel_matches_serial_and_python(omni, tmp_path, monkeypatch):
    """The block-parallel reader: 1 and 7 threads give identical arrays, and every value is
    the float rounding of the correctly rounded double of its text (the reference's _wtof
    into float arrays), with blanks, tabs and commas as separators and CRLF line ends."""
    dims = (37, 23, 19)
    n = int(np.prod(dims))
    rng = np.random.default_rng(7)
    vals = [rng.normal(size=n) * 10.0 ** rng.integers(-8, 8, n) for _ in range(10)]
    seps = [" ", "\t", ", ", "  "]
    path = tmp_path / "acc.dat"
    with open(path, "w", newline="") as fh:
        fh.write('TITLE = "acc"\r\nVARIABLES = "X"\r\nZONE I=37, J=23, K=19\r\n')
        for r in range(n):
            sep = seps[r % 4]
            fh.write(sep.join(repr(float(vals[c][r])) if c % 3 else "%.9e" % vals[c][r] for c in range(10)) + "\r\n")
    pf = tmp_path / "P.dat"
    pf.write_text(PARAMS.replace("64\n48\n32", "37\n23\n19").format(extra="\n2\n30\n1\n20\n3\n18"))
    fp = omni.read_params(str(pf))
    monkeypatch.setenv("OMNI3D_IO_THREADS", "1")
    one = omni.read_tecplot(str(path), fp)
    monkeypatch.setenv("OMNI3D_IO_THREADS", "7")
    many = omni.read_tecplot(str(path), fp)
    monkeypatch.setenv("OMNI3D_IO_BLOCK", "97")  # lines and header lines span many blocks
    monkeypatch.setenv("OMNI3D_IO_THREADS", "2")
    small = omni.read_tecplot(str(path), fp)
    monkeypatch.delenv("OMNI3D_IO_BLOCK")
    names = ["x", "y", "z", "u", "v", "w", "ax", "ay", "az", "mask"]
    rows = [l for l in path.read_text().replace("\r", "").split("\n")[3:] if l]
    table = np.array([[float(t) for t in l.replace(",", " ").split()] for l in rows]).reshape(19, 23, 37, 10)
    crop = table[3:19, 1:21, 2:31]
    for c, nm in enumerate(names):
        np.testing.assert_array_equal(one[nm].view(np.uint32), many[nm].view(np.uint32))
        np.testing.assert_array_equal(one[nm].view(np.uint32), small[nm].view(np.uint32))
        np.testing.assert_array_equal(one[nm], crop[..., c].reshape(-1).astype(np.float32))


def test_writers_parallel_bytes_equal_serial(omni, tmp_path, monkeypatch):
    dims = (41, 30, 11)
    n = int(np.prod(dims))
    rng = np.random.default_rng(8)
    cols = [(rng.normal(size=n) * 10.0 ** rng.integers(-6, 6, n)).astype(np.float32) for _ in range(5)]
    cols[3][5] = np.float32(3e30)  # a row wider than the usual formatting buffer
    out = {}
    for t in ("1", "5"):
        monkeypatch.setenv("OMNI3D_IO_THREADS", t)
        path = tmp_path / ("p%s.dat" % t)
        omni.write_pressure(str(path), dims, *cols)
        out[t] = path.read_bytes()
        cpath = tmp_path / ("c%s.dat" % t)
        omni.write_curl(str(cpath), dims, *cols[:4])
        out["c" + t] = cpath.read_bytes()
    assert out["1"] == out["5"] and out["c1"] == out["c5"]
    lines = out["5"].decode().split("\n")
    for r in (0, 5, n - 1):
        assert lines[3 + r] == " ".join("%15.9f" % float(c[r]) for c in cols)


def test_bernoulli_face(omni):
    dims = (4, 3, 2)
    n = 24
    rng = np.random.default_rng(1)
    u, v, w = (rng.normal(size=n).astype(np.float32) for _ in range(3))
    p = omni.bernoulli_face(dims, 5.0, 2.0, u, v, w).reshape(2, 3, 4)
    exp = (5.0 - 0.5 * 2.0 * (u * u + v * v + w * w)).reshape(2, 3, 4)
    np.testing.assert_allclose(p[:, 0, :], exp[:, 0, :], rtol=1e-6)
    assert (p[:, 1:, :] == 0).all()


def test_write_pressure_format(omni, tmp_path):
    dims = (2, 2, 1)
    x = np.arange(4, dtype=np.float32)
    path = tmp_path / "PressureOmni3D_00000.dat"
    omni.write_pressure(str(path), dims, x, x + 1, x + 2, x * 0.5, x * 3)
    lines = path.read_text().split("\n")
    assert lines[0] == 'TITLE = "Pressure Integrated From GPU Based Omni 3D Method"'
    assert lines[1] == 'VARIABLES = "X","Y","Z","P","Count"'
    assert lines[2] == "ZONE I=2, J=2, K=1,F=POINT"
    assert lines[4] == "%15.9f %15.9f %15.9f %15.9f %15.9f" % (1, 2, 3, 0.5, 3)
    assert len([l for l in lines if l]) == 3 + 4


def test_create_rejects_bad_params_without_gpu(omni):
    d = omni.icosphere(2)
    with pytest.raises(omni.Omni3DError) as e:
        omni.Omni3D((1, 8, 8), 1e-3, d)
    assert e.value.code == -1
    with pytest.raises(omni.Omni3DError) as e:
        omni.Omni3D((8, 8, 8), 1e-3, d, line_spacing=0.0)
    assert e.value.code == -1
    with pytest.raises(omni.Omni3DError) as e:
        omni.Omni3D((8, 8, 8), 1e-3, d, gauge="point", ref=(8, 0, 0))
    assert e.value.code == -1
    for bad in ({"tile_width": 3}, {"tile_width": 32}, {"dir_group": 33}, {"dir_group": -1}):
        with pytest.raises(omni.Omni3DError) as e:
            omni.Omni3D((8, 8, 8), 1e-3, d, **bad)
        assert e.value.code == -1
    # voxel indices are 32-bit on the device: 2^32 voxels and more are refused up front
    with pytest.raises(omni.Omni3DError) as e:
        omni.Omni3D((2048, 2048, 1024), 1e-3, d)
    assert e.value.code == -6 and "32-bit" in str(e.value)  # OMNI3D_ERR_RANGE


def test_no_cpu_fallback(omni):
    """Without a usable GPU the solver refuses to run rather than computing on the host."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(omni.Omni3DError) as e:
        omni.Omni3D((8, 8, 8), 1e-3, omni.icosphere(2))
    assert e.value.code == -2


def test_cli_usage(omni):
    from omni3d.build import CLI

    r = subprocess.run([CLI, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
