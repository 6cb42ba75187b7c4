"""The C++ drop-in API (Solver3D / Solver2D, include/eikonalxx/) solving on the GPU,
checked against the oracle bit for bit."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_solver_api_matches_oracle(ctx, oracle, tmp_path):
    libdir = os.path.join(ROOT, "eikonalxx_gb300", "_build")
    exe = str(tmp_path / "solver_api")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "solver_api_main.cpp"), "-L" + libdir, "-leikx",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    nx, ny, nz, h = 21, 17, 13, 50.0
    pos = [333.0, 421.0, 222.0]
    cell = [min(n - 2, int(p / h)) for p, n in zip(pos, (nx, ny, nz))]
    for size, dt in ((4, np.float32), (8, np.float64)):
        v = np.fromfile(tmp_path / f"v3_{size}.bin", dtype=dt)
        s = np.fromfile(tmp_path / f"s3_{size}.bin", dtype=dt)
        assert np.array_equal(s, oracle.nodal_to_cell3d(v, nx, ny, nz, 0))
        t = np.fromfile(tmp_path / f"t3_{size}.bin", dtype=dt).reshape(nz, ny, nx)
        ref = oracle.solve3d(s, (nx, ny, nz, h, h, h), cell, pos, n_sweeps=2, radius=3, tol=0)
        assert np.array_equal(t, ref), (size, np.abs(t - ref).max())
    s2 = np.fromfile(tmp_path / "s2.bin", dtype=np.float64)
    t2 = np.fromfile(tmp_path / "t2.bin", dtype=np.float64).reshape(37, 61)
    ref2 = oracle.solve2d(s2, (61, 37, 10.0, 10.0), [25, 13], [250.0, 130.0], n_sweeps=2, radius=3, tol=0)
    assert np.array_equal(t2, ref2)
    # bilinear station time and the in-cell straight ray (src/solver2d.cpp:106-167)
    st = np.fromfile(tmp_path / "st2.bin", dtype=np.float64)
    x, z = 455.5, 301.25
    cx, cz = int(x / 10), int(z / 10)
    fx, fz = (x - cx * 10) / 10, (z - cz * 10) / 10
    f = t2[cz:cz + 2, cx:cx + 2]
    exp = (1 - fz) * ((1 - fx) * f[0, 0] + fx * f[0, 1]) + fz * ((1 - fx) * f[1, 0] + fx * f[1, 1])
    assert st[0] == pytest.approx(exp, rel=1e-12)
    assert st[1] == pytest.approx(np.hypot(1.0, 1.0) * s2[13 * 60 + 25], rel=1e-12)
    g = np.fromfile(tmp_path / "g2.bin", dtype=np.float64).reshape(37, 61, 2)
    assert g[10, 30, 0] == pytest.approx((t2[10, 31] - t2[10, 29]) / 20.0, rel=1e-12)
    # Solver2D::writeVTK: the field and its gradient, big-endian float32
    from test_vtk_cpp import Reader, _grid, _scalars
    r = Reader(tmp_path / "t2.vtk")
    assert r.title == "travel_time" and r.binary
    _grid(r, (61, 1, 37), 10.0 * np.arange(61), [0.0], -10.0 * np.arange(37))
    _scalars(r, "travel_time", t2.ravel().astype(np.float32), f"POINT_DATA {61 * 37}")
    assert r.line() == "VECTORS travel_time_gradient float"
    gv = r.floats(3 * 61 * 37).reshape(-1, 3)
    np.testing.assert_array_equal(gv[:, 0], g[..., 0].ravel().astype(np.float32))
    np.testing.assert_array_equal(gv[:, 2], g[..., 1].ravel().astype(np.float32))
    assert r.done()
