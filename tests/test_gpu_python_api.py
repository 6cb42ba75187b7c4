"""pyEikonalXX Solver2D / Solver3D (the reference's Python interface) solve on the GPU and
agree bit for bit with the C-ABI context on the same inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402
from eikonalxx_gb300 import pyEikonalXX as pe  # noqa: E402


def test_solver3d_matches_context(tmp_path):
    rng = np.random.default_rng(91)
    g = pe.Geometry3D()
    g.nx, g.ny, g.nz, g.dx, g.dy, g.dz = 21, 17, 13, 50., 50., 50.
    g.x0, g.y0, g.z0 = 100., -50., 0.
    v = rng.uniform(2500, 5500, size=g.nx * g.ny * g.nz)
    m = pe.VelocityModel3D()
    m.initialize(g)
    m.set_nodal_velocities(v)
    o = pe.SolverOptions()
    o.number_of_sweeps = 4
    o.tolerance = 1e-9
    src = pe.Source3D()
    src.geometry = g
    src.x, src.y, src.z = 612., 233., 310.
    stations = []
    for x, y in ((150., -20.), (900., 600.), (612., 233.)):
        st = pe.Station3D()
        st.geometry = g
        st.x, st.y = x, y
        st.set_z_to_free_surface()
        stations.append(st)
    s = pe.Solver3D()
    s.initialize(o, g)
    s.velocity_model = m
    s.source = src
    s.stations = stations
    s.solve()
    assert s.have_travel_time_field and not s.have_travel_time_gradient_field
    s.compute_travel_time_gradient_field()

    ctx = ex.Context(0)
    ctx.set_grid3d(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.x0, g.y0, g.z0)
    ctx.set_nodal_velocity3d(v)
    t = ctx.solve3d([(612., 233., 310.)], ex.Options(n_sweeps=4, tolerance=1e-9, factored_radius=3), ex.F64)[0]
    assert np.array_equal(s.travel_time_field, t.ravel())
    assert np.array_equal(s.travel_time_gradient_field, ctx.gradient3d(0, ex.F64).ravel())
    st_t = ctx.station_times3d([(150., -20., 0.), (900., 600., 0.), (612., 233., 0.)])
    assert s.travel_times_at_stations == list(st_t)
    s.write_vtk(str(tmp_path / "t3.vtk"), write_gradient=True)
    assert (tmp_path / "t3.vtk").stat().st_size > 4 * 4 * g.nx * g.ny * g.nz


def test_solver2d_cellular_model_matches_context():
    rng = np.random.default_rng(92)
    g = pe.Geometry2D()
    g.nx, g.nz, g.dx, g.dz = 41, 23, 25., 25.
    vc = rng.uniform(2000, 6000, size=(g.nx - 1) * (g.nz - 1))
    m = pe.VelocityModel2D()
    m.initialize(g)
    m.set_cellular_velocities(vc)
    src = pe.Source2D()
    src.geometry = g
    src.x, src.z = 512.5, 130.
    s = pe.Solver2D()
    s.initialize(pe.SolverOptions(), g)
    s.velocity_model = m
    s.source = src
    s.solve()
    ctx = ex.Context(0)
    ctx.set_grid2d(g.nx, g.nz, g.dx, g.dz)
    ctx.set_slowness2d(1.0 / vc)
    t = ctx.solve2d([(512.5, 130.)], ex.Options(n_sweeps=5, tolerance=1e-5, factored_radius=3), ex.F64)[0]
    assert np.array_equal(s.travel_time_field, t.ravel())
