"""The drop-in executable end to end: Parameter_Omni3D.dat, a direction file and a folder
of Tecplot acceleration files in, PressureOmni3D_%05d.dat (+ the curl sample and log.dat)
out, matching the library solve on the same inputs."""
import os
import subprocess

import numpy as np
import pytest

from omni3d import synthetic

pytestmark = pytest.mark.gpu


def _write_input(path, f, u):
    nx, ny, nz = f["dims"]
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cols = [i.reshape(-1) * 1e-3, j.reshape(-1) * 1e-3, k.reshape(-1) * 1e-3, u[0], u[1], u[2],
            f["ax"].reshape(-1), f["ay"].reshape(-1), f["az"].reshape(-1), f["mask"].reshape(-1)]
    with open(path, "w", newline="") as fh:
        fh.write('TITLE = "accelerations"\r\nVARIABLES = "X","Y","Z","U","V","W","Du","Dv","Dw","Mask"\r\n')
        fh.write("ZONE I=%d, J=%d, K=%d, F=POINT\r\n" % (nx, ny, nz))
        for r in range(nx * ny * nz):
            fh.write(" ".join("%.9g" % c[r] for c in cols) + "\r\n")


@pytest.mark.parametrize("extra", [[], ["--autotune"]])
def test_cli_matches_library(omni, tmp_path, extra):
    from omni3d.build import CLI

    dims = (14, 12, 10)
    dirs = omni.icosphere(2)
    thr = 5.0e5
    fields = [synthetic.blobs(dims=dims, count=3, sigma_range=(2.0, 4.0), noise=0.05, seed=40 + s, sphere_radius=2.5)
              for s in range(2)]
    rng = np.random.default_rng(5)
    vel = [[rng.normal(0, 0.3, np.prod(dims)).astype(np.float32) for _ in range(3)] for _ in fields]
    (tmp_path / "acc").mkdir()
    for s, (f, u) in enumerate(zip(fields, vel)):
        _write_input(tmp_path / "acc" / ("snap_%02d.dat" % s), f, u)
    with open(tmp_path / "dirs.dat", "w", newline="") as fh:
        for v in dirs:
            fh.write("%f %f %f\r\n" % tuple(v))
        fh.write("%d\r\n" % len(dirs))
    params = [str(dims[0]), str(dims[1]), str(dims[2]), "0.001", "0.001", "0.001", "1", "1", "1", str(len(dirs)),
              "dirs.dat", ".\\acc\\", ".\\out\\", "3", repr(thr), "0.5", "", "", "", "", "", ""]
    (tmp_path / "Parameter_Omni3D.dat").write_text("\r\n".join(params) + "\r\n")
    r = subprocess.run([CLI] + extra, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "log.dat").read_text().startswith("Processing Starts")
    assert (tmp_path / "CurlofMaterialAcc_Sample.dat").exists()
    for s, (f, u) in enumerate(zip(fields, vel)):
        out = (tmp_path / "out" / ("PressureOmni3D_%05d.dat" % s)).read_text().split("\n")
        assert out[0] == 'TITLE = "Pressure Integrated From GPU Based Omni 3D Method"'
        assert out[2] == "ZONE I=%d, J=%d, K=%d,F=POINT" % dims
        rows = np.array([[float(x) for x in l.split()] for l in out[3:] if l.strip()])
        assert rows.shape == (np.prod(dims), 5)
        # the same solve through the library: selected method, Bernoulli face, 3 iterations
        p0 = omni.bernoulli_face(dims, 0.5, 1.0, *u)
        with omni.Omni3D(dims, 1e-3, dirs, max_iter=3, method="select", threshold=thr) as sv:
            ref = sv.solve(f["ax"], f["ay"], f["az"], mask=f["mask"], p_init=p0)
        np.testing.assert_allclose(rows[:, 3], ref.p.reshape(-1), rtol=0, atol=2e-8 + 1e-5 * np.abs(ref.p).max())
        np.testing.assert_allclose(rows[:, 4], ref.count.reshape(-1), rtol=1e-6, atol=1e-6)
