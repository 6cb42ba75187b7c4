"""GPU gradient and station times of solved fields against the oracle: bit-identical."""
import numpy as np
import pytest

from conftest import random_slowness

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402


def _cell(p, d, n):
    return min(n - 2, int(p / d))


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
def test_gradient_and_stations_3d(ctx, oracle, precision):
    rng = np.random.default_rng(41 + precision)
    nx, ny, nz, dx, dy, dz = 27, 22, 18, 40., 45., 35.
    dt = np.float32 if precision == ex.F32 else np.float64
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=dt)
    ctx.set_grid3d(nx, ny, nz, dx, dy, dz)
    ctx.set_slowness3d(s)
    srcs = [(rng.uniform(0, (nx - 1) * dx), rng.uniform(0, (ny - 1) * dy), rng.uniform(0, (nz - 1) * dz))
            for _ in range(2)]
    t = ctx.solve3d(srcs, ex.Options(n_sweeps=3, tolerance=-1), precision)
    st = rng.uniform(0, [(nx - 1) * dx, (ny - 1) * dy, (nz - 1) * dz], size=(40, 3))
    for f, p in enumerate(srcs):
        cell = [_cell(q, d, n) for q, d, n in zip(p, (dx, dy, dz), (nx, ny, nz))]
        slow0 = s.reshape(nz - 1, ny - 1, nx - 1)[cell[2], cell[1], cell[0]]
        g = ctx.gradient3d(f, precision)
        g_or = oracle.gradient3d(t[f], (nx, ny, nz, dx, dy, dz), cell, p, slow0)
        assert np.array_equal(g, g_or), f
        stations = np.vstack([st, [p]])                       # one station in the source cell
        cells = [[_cell(q, d, n) for q, d, n in zip(x, (dx, dy, dz), (nx, ny, nz))] for x in stations]
        got = ctx.station_times3d(stations, f)
        want = oracle.stations3d(t[f], (nx, ny, nz, dx, dy, dz), cell, p, float(slow0), cells, stations)
        assert np.array_equal(got, want), f


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
def test_gradient_and_stations_2d(ctx, oracle, precision):
    rng = np.random.default_rng(43 + precision)
    nx, nz, dx, dz = 61, 37, 20., 25.
    dt = np.float32 if precision == ex.F32 else np.float64
    s = random_slowness(rng, (nz - 1) * (nx - 1), dtype=dt)
    ctx.set_grid2d(nx, nz, dx, dz)
    ctx.set_slowness2d(s)
    src = (rng.uniform(0, (nx - 1) * dx), rng.uniform(0, (nz - 1) * dz))
    t = ctx.solve2d([src], ex.Options(n_sweeps=2, tolerance=-1), precision)[0]
    cell = [_cell(src[0], dx, nx), _cell(src[1], dz, nz)]
    slow0 = s.reshape(nz - 1, nx - 1)[cell[1], cell[0]]
    g = ctx.gradient2d(0, precision)
    assert np.array_equal(g, oracle.gradient2d(t, (nx, nz, dx, dz), cell, src, slow0))
    st = np.vstack([rng.uniform(0, [(nx - 1) * dx, (nz - 1) * dz], size=(30, 2)), [src]])
    cells = [[_cell(x[0], dx, nx), _cell(x[1], dz, nz)] for x in st]
    got = ctx.station_times2d(st, 0)
    assert np.array_equal(got, oracle.stations2d(t, (nx, nz, dx, dz), cell, src, float(slow0), cells, st))


def test_products_need_a_solve(ctx):
    c = ex.Context(0)
    with pytest.raises(ex.StateError):
        c.gradient3d(0)
    c.set_grid3d(5, 5, 5, 10., 10., 10.)
    c.set_slowness3d(np.full(64, 1 / 3000., np.float32))
    c.solve3d([(12., 13., 14.)], ex.Options(n_sweeps=1), ex.F32)
    with pytest.raises(ex.InvalidArgument):
        c.gradient3d(1)                                       # one field only
    with pytest.raises(ex.InvalidArgument):
        c.station_times3d([(100., 0., 0.)])                   # outside the grid


@pytest.mark.parametrize("v_top,v_bottom", [(4000.0, 4000.0), (3000.0, 6000.0)])
def test_analytic_fields_match_oracle(ctx, oracle, v_top, v_bottom):
    """Closed-form constant-velocity and linear-gradient times (the accuracy references):
    CUDA's acosh / sqrt / hypot against the C library's, a few ulps apart at most."""
    grid3 = (41, 33, 29, 50., 50., 50.)
    src3 = (812.5, 433.0, 610.0)
    ctx.set_grid3d(*grid3)
    g3 = ctx.analytic3d(src3, v_top, v_bottom)
    assert np.allclose(g3, oracle.linear_gradient3d(grid3, src3, v_top, v_bottom), rtol=1e-13, atol=1e-15)
    grid2 = (81, 43, 25., 25.)
    src2 = (1010.0, 320.0)
    ctx.set_grid2d(*grid2)
    g2 = ctx.analytic2d(src2, v_top, v_bottom)
    assert np.allclose(g2, oracle.linear_gradient2d(grid2, src2, v_top, v_bottom), rtol=1e-13, atol=1e-15)
