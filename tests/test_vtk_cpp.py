"""The C++ legacy-VTK writers (Model3D/Model2D::writeVTK, IO::VTKRectilinearGrid3D/2D,
IO::VTKLines2D), driven by tests/cpp/vtk_main.cpp on the CPU: every file is parsed back --
header, coordinates (z written as -depth), section keywords and the big-endian float32
payload -- and compared with the values written.  The layout follows the reference's
src/io/vtkRectilinearGrid3d.cpp, vtkRectilinearGrid2d.cpp and vtkLines2d.cpp."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(tmp_path):
    libdir = os.path.join(ROOT, "eikonalxx_gb300", "_build")
    exe = str(tmp_path / "vtk_main")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "vtk_main.cpp"), "-L" + libdir, "-leikx",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "vtk ok" in r.stdout, r.stdout + r.stderr


class Reader:
    """A legacy-VTK file: header lines and float blocks (binary big-endian or ASCII)."""

    def __init__(self, path):
        self.b = open(path, "rb").read()
        self.p = 0
        assert self.line() == "# vtk DataFile Version 3.0"
        self.title = self.line()
        self.binary = self.line() == "BINARY"

    def line(self):
        e = self.b.index(b"\n", self.p)
        s = self.b[self.p:e].decode()
        self.p = e + 1
        return s

    def floats(self, n):
        if self.binary:
            a = np.frombuffer(self.b[self.p:self.p + 4 * n], dtype=">f4").astype(np.float64)
            self.p += 4 * n
            assert self.b[self.p:self.p + 1] == b"\n"
            self.p += 1
            return a
        return np.array([float(self.line()) for _ in range(n)])

    def done(self):
        return self.p >= len(self.b)


def _grid(r, dims, x, y, z):
    assert r.line() == "DATASET RECTILINEAR_GRID"
    assert r.line() == "DIMENSIONS {} {} {}".format(*dims)
    for name, c in (("X", x), ("Y", y), ("Z", z)):
        assert r.line() == f"{name}_COORDINATES {len(c)} float"
        np.testing.assert_allclose(r.floats(len(c)), c, rtol=1e-6)


def _scalars(r, name, values, section=None):
    if section:
        assert r.line() == section
    assert r.line() == f"SCALARS {name} float 1"
    assert r.line() == "LOOKUP_TABLE default"
    np.testing.assert_allclose(r.floats(len(values)), values, rtol=1e-6)


def test_cpp_vtk_writers(lib, tmp_path):
    _run(tmp_path)
    nx, ny, nz = 5, 4, 3
    x, y, z = 100 + 10.0 * np.arange(nx), -50 + 20.0 * np.arange(ny), -(5 + 25.0 * np.arange(nz))
    nc3 = (nx - 1) * (ny - 1) * (nz - 1)
    vc = 3000 + 10.0 * np.arange(nc3)

    r = Reader(tmp_path / "sub" / "model3d.vtk")
    assert r.title == "velocity_m/s" and r.binary
    _grid(r, (nx, ny, nz), x, y, z)
    _scalars(r, "velocity_m/s", vc, f"CELL_DATA {nc3}")
    assert r.done()

    for name, binary in (("grid3d_bin.vtk", True), ("grid3d_ascii.vtk", False)):
        r = Reader(tmp_path / name)
        assert r.title == "vtk_dataset" and r.binary == binary
        _grid(r, (nx, ny, nz), x, y, z)
        n = nx * ny * nz
        _scalars(r, "index", np.arange(n), f"POINT_DATA {n}")      # XYZ input written in natural order
        _scalars(r, "twice", np.full(n, 2.5))
        _scalars(r, "cells", vc, f"CELL_DATA {nc3}")
        assert r.done()

    mx, mz = 6, 4
    x2, z2 = 1 + 5.0 * np.arange(mx), -(2 + 7.5 * np.arange(mz))
    nc2 = (mx - 1) * (mz - 1)
    r = Reader(tmp_path / "model2d.vtk")
    _grid(r, (mx, 1, mz), x2, [0.0], z2)
    _scalars(r, "velocity_m/s", 2000 + 100.0 * np.arange(nc2), f"CELL_DATA {nc2}")
    assert r.done()

    r = Reader(tmp_path / "grid2d.vtk")
    assert r.title == "two_d"
    _grid(r, (mx, 1, mz), x2, [0.0], z2)
    n = mx * mz
    _scalars(r, "t", 0.001 * np.arange(n), f"POINT_DATA {n}")
    assert r.line() == "VECTORS t_gradient float"
    g = r.floats(3 * n).reshape(n, 3)
    np.testing.assert_allclose(g[:, 0], 0.5 * np.arange(n), rtol=1e-6)
    assert np.all(g[:, 1] == 0)
    np.testing.assert_allclose(g[:, 2], -0.25 * np.arange(n), rtol=1e-6)
    _scalars(r, "v", 2000 + 100.0 * np.arange(nc2), f"CELL_DATA {nc2}")
    assert r.done()

    lines = open(tmp_path / "rays.vtk").read().split("\n")
    assert lines[:5] == ["# vtk DataFile Version 3.0", "ray_paths", "ASCII", "DATASET POLYDATA", "POINTS 5 float"]
    pts = np.array([[float(v) for v in s.split()] for s in lines[5:10]])
    np.testing.assert_allclose(pts, [[0, 0, -10], [5, 0, -12.5], [7.5, 0, -20], [1, 0, -2], [3, 0, -4]])
    assert lines[10:13] == ["LINES 2 7", "3 0 1 2", "2 3 4"]
    assert not os.path.exists(tmp_path / "never.vtk")
