"""The reference's Python interface (pyEikonalXX) mirrored by eikonalxx_gb300.pyEikonalXX:
the reference's own python/unit_tests.py runs against it (when the reference is present),
and the legacy-VTK files have the reference writer's layout."""
import importlib.util
import os
import sys

import numpy as np
import pytest

from eikonalxx_gb300 import pyEikonalXX, vtk

from oracle.build import reference_root

REFERENCE = reference_root()


def test_reference_python_unit_tests_pass():
    path = os.path.join(REFERENCE, "python", "unit_tests.py")
    if not os.path.exists(path):
        pytest.skip("reference sources not present")
    sys.modules["pyEikonalXX"] = pyEikonalXX
    try:
        spec = importlib.util.spec_from_file_location("reference_python_unit_tests", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        names = [n for n in dir(mod) if n.startswith("test_")]
        assert len(names) >= 9
        for n in names:
            getattr(mod, n)()
    finally:
        del sys.modules["pyEikonalXX"]


def test_value_types_validate_like_the_reference():
    g = pyEikonalXX.Geometry3D()
    with pytest.raises(ValueError):
        g.nx = 2
    with pytest.raises(ValueError):
        g.dx = 0
    g.nx, g.ny, g.nz, g.dx, g.dy, g.dz = 5, 6, 7, 10., 10., 10.
    s = pyEikonalXX.Source3D()
    s.geometry = g
    with pytest.raises(ValueError):
        s.x = 41.0                                   # beyond (nx - 1) * dx
    s.x, s.y, s.z = 40.0, 0.0, 12.5
    assert (s.x, s.y, s.z) == (40.0, 0.0, 12.5)
    o = pyEikonalXX.SolverOptions()
    assert (o.number_of_sweeps, o.tolerance, o.factored_eikonal_equation_solver_radius) == (5, 1e-5, 3)
    m = pyEikonalXX.VelocityModel3D()
    m.initialize(g)
    with pytest.raises(ValueError):
        m.set_nodal_velocities(np.ones(10))
    with pytest.raises(ValueError):
        m.set_nodal_velocities(-np.ones(5 * 6 * 7))


def test_vtk_binary_layout(tmp_path):
    nx, ny, nz = 4, 1, 3
    t = np.arange(nx * nz, dtype=np.float64) / 7
    path = tmp_path / "t.vtk"
    with vtk.RectilinearGridWriter(str(path), nx, ny, nz, 10., 1., 20., 5., 0., 2., title="travel time s") as w:
        w.nodal_scalars("travel time", t)
        w.nodal_vectors("grad", np.stack([t, -t], 1).ravel(), 2)
    data = path.read_bytes()
    expect = b"# vtk DataFile Version 3.0\ntravel_time_s\nBINARY\nDATASET RECTILINEAR_GRID\nDIMENSIONS 4 1 3\n"
    assert data.startswith(expect)
    pos = len(expect)

    def block(header, values):
        nonlocal pos
        h = (header + "\n").encode()
        assert data[pos:pos + len(h)] == h, (data[pos:pos + len(h)], h)
        pos += len(h)
        raw = np.asarray(values, np.float64).astype(">f4").tobytes()
        assert data[pos:pos + len(raw)] == raw
        pos += len(raw) + 1

    block("X_COORDINATES 4 float", 5. + 10. * np.arange(4))
    block("Y_COORDINATES 1 float", [0.])
    block("Z_COORDINATES 3 float", -(2. + 20. * np.arange(3)))
    h = b"POINT_DATA 12\n"
    assert data[pos:pos + len(h)] == h
    pos += len(h)
    block("SCALARS travel_time float 1\nLOOKUP_TABLE default", t)
    block("VECTORS grad float", np.stack([t, np.zeros_like(t), -t], 1).ravel())
    assert pos == len(data)


def test_vtk_ascii_values(tmp_path):
    path = tmp_path / "m.vtk"
    with vtk.RectilinearGridWriter(str(path), 3, 3, 3, 1., 1., 1., binary=False) as w:
        w.cell_scalars("velocity", np.full(8, 2500.))
    lines = path.read_text().splitlines()
    i = lines.index("CELL_DATA 8")
    assert lines[i + 1:i + 3] == ["SCALARS velocity float 1", "LOOKUP_TABLE default"]
    assert [float(v) for v in lines[i + 3:i + 11]] == [2500.] * 8
