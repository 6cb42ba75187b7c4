"""Work the chunk-step kernel leaves out, checked against the oracle bit for bit.

The initialisation pass updates only the octant of each sweep that lies downstream of the
source; warp blocks wholly before it along y' or z' are left out and their rows are read
from the field by the blocks after them.  Sources in corners, on faces and in the middle
put the octant boundary in every position relative to the warp blocks.

The kernel evaluates the Cartesian (far-field) operators with lower-bound exits
(local_solver.cuh, fd3UniformFarBounded): it stops as soon as the rounded lower bounds of
the 2D and 8-point operators show that no operator can go below the node's current time,
and leaves out the 8-point operator when its bound shows it cannot be the one that does.
These exits fire on converged regions and on sweep orderings against the wave, so the
tests run smooth layered models for many iterations, random models past 256 sweeps, and
every warp-block shape, and compare with the oracle, which evaluates every operator as the
reference does (include/private/solver3d.hpp:186-243)."""
import numpy as np
import pytest

from conftest import random_slowness

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402
from eikonalxx_gb300 import synthetic  # noqa: E402


def _bits(a):
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def _cells(oracle, shape, seed, dt):
    nx, ny, nz, dx = shape[:4]
    v = synthetic.layered_grf_model(nx, ny, nz, dx, seed, corr_m=4 * dx, dtype=np.float64)
    return oracle.nodal_to_cell3d(v, nx, ny, nz).astype(dt)


def _sources(rng, shape, n):
    nx, ny, nz, dx, dy, dz = shape
    out = []
    for _ in range(n):
        pos = [float(rng.uniform(0, (k - 1) * h)) for k, h in zip((nx, ny, nz), (dx, dy, dz))]
        cell = [min(k - 2, int(p / h)) for p, k, h in zip(pos, (nx, ny, nz), (dx, dy, dz))]
        out.append((pos, cell))
    return out


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
@pytest.mark.parametrize("shape", [(44, 38, 30, 50., 50., 50.), (37, 30, 22, 45., 45., 45.)])
def test_many_iterations_exact_against_the_oracle(ctx, oracle, precision, shape):
    """Smooth layered model, 7 iterations without a tolerance: the late iterations run on
    converged fields, where the exits fire on most nodes."""
    dt = np.float32 if precision == ex.F32 else np.float64
    rng = np.random.default_rng(5 + precision)
    cells = _cells(oracle, shape, 21, dt)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(cells)
    srcs = _sources(rng, shape, 3)
    t = ctx.solve3d([p for p, _ in srcs], ex.Options(n_sweeps=7, tolerance=-1, factored_radius=3), precision)
    for (pos, cell), a in zip(srcs, t):
        ref = oracle.solve3d(cells, shape, cell, pos, n_sweeps=7, radius=3)
        assert np.array_equal(_bits(a), _bits(ref)), np.abs(a - ref).max()


@pytest.mark.parametrize("shape", [(24, 20, 18, 30., 30., 30.), (25, 17, 19, 20., 20., 20.)])
def test_random_model_past_256_sweeps(ctx, oracle, shape):
    """Random cell slowness keeps nodes changing for many sweeps; 40 iterations."""
    rng = np.random.default_rng(8)
    nx, ny, nz = shape[:3]
    cells = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(cells)
    srcs = _sources(rng, shape, 2)
    t = ctx.solve3d([p for p, _ in srcs], ex.Options(n_sweeps=40, tolerance=-1, factored_radius=2), ex.F32)
    for (pos, cell), a in zip(srcs, t):
        ref = oracle.solve3d(cells, shape, cell, pos, n_sweeps=40, radius=2)
        assert np.array_equal(_bits(a), _bits(ref)), np.abs(a - ref).max()


@pytest.mark.parametrize("block_shape", [1, 2, 3])
def test_every_warp_block_matches_the_node_step_kernel(ctx, oracle, block_shape):
    """The node-step kernel evaluates every operator (fd3UniformFar); the chunk-step kernel
    with the exits must give the same bits with each warp-block shape."""
    shape = (36, 34, 27, 50., 50., 50.)
    rng = np.random.default_rng(10 + block_shape)
    cells = _cells(oracle, shape, 6, np.float32)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(cells)
    srcs = [p for p, _ in _sources(rng, shape, 2)]
    base = dict(n_sweeps=6, tolerance=-1, factored_radius=3)
    t_chunk = ctx.solve3d(srcs, ex.Options(**base, sweep_kernel=2, block_shape=block_shape), ex.F32)
    t_node = ctx.solve3d(srcs, ex.Options(**base, sweep_kernel=1), ex.F32)
    for a, b in zip(t_chunk, t_node):
        assert np.array_equal(_bits(a), _bits(b)), np.abs(a - b).max()


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
def test_batch_of_smooth_models_exact(ctx, oracle, precision):
    dt = np.float32 if precision == ex.F32 else np.float64
    rng = np.random.default_rng(12)
    grids = [(30, 26, 20, 50., 50., 50.), (22, 35, 17, 40., 40., 40.), (19, 17, 23, 30., 30., 30.)]
    models, refs = [], []
    for k, g in enumerate(grids):
        cells = _cells(oracle, g, 30 + k, dt)
        srcs = _sources(rng, g, 2)
        models.append({"grid": g + (0., 0., 0.), "model": cells, "sources": [p for p, _ in srcs]})
        refs.append((cells, srcs))
    outs = ctx.solve3d_batch(models, ex.Options(n_sweeps=6, tolerance=-1, factored_radius=3), precision)
    for g, (cells, srcs), out in zip(grids, refs, outs):
        for j, (pos, cell) in enumerate(srcs):
            ref = oracle.solve3d(cells, g, cell, pos, n_sweeps=6, radius=3)
            assert np.array_equal(_bits(out[j]), _bits(ref)), (g, j)


CORNERS = [(0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (1.0, 0.0, 0.5), (0.0, 1.0, 1.0), (0.5, 0.5, 0.0), (0.37, 0.81, 0.66),
           (0.99, 0.02, 0.51), (0.12, 0.93, 0.97)]


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
@pytest.mark.parametrize("block_shape", [1, 2, 3])
def test_initialisation_pass_for_sources_anywhere(ctx, oracle, precision, block_shape):
    """n_sweeps = 0: the field after the 8 source-limited sweeps alone."""
    shape = (29, 35, 23, 40., 40., 40.)
    nx, ny, nz, dx, dy, dz = shape
    dt = np.float32 if precision == ex.F32 else np.float64
    cells = _cells(oracle, shape, 14, dt)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(cells)
    pos = [(fx * (nx - 1) * dx, fy * (ny - 1) * dy, fz * (nz - 1) * dz) for fx, fy, fz in CORNERS]
    for n_sweeps in (0, 1):
        opt = ex.Options(n_sweeps=n_sweeps, tolerance=-1, factored_radius=3, sweep_kernel=2,
                         block_shape=block_shape)
        t = ctx.solve3d(pos, opt, precision)
        for p, a in zip(pos, t):
            cell = [min(k - 2, int(q / h)) for q, k, h in zip(p, (nx, ny, nz), (dx, dy, dz))]
            ref = oracle.solve3d(cells, shape, cell, p, n_sweeps=n_sweeps, radius=3)
            assert np.array_equal(_bits(a), _bits(ref)), (p, n_sweeps, np.abs(a - ref).max())


def test_initialisation_pass_of_a_batch(ctx, oracle):
    grids = [(26, 33, 21, 50., 50., 50.), (40, 17, 30, 50., 50., 50.)]
    models, refs = [], []
    for k, g in enumerate(grids):
        nx, ny, nz, dx, dy, dz = g
        cells = _cells(oracle, g, 40 + k, np.float32)
        pos = [(fx * (nx - 1) * dx, fy * (ny - 1) * dy, fz * (nz - 1) * dz) for fx, fy, fz in CORNERS[:4]]
        models.append({"grid": g + (0., 0., 0.), "model": cells, "sources": pos})
        refs.append((cells, pos))
    outs = ctx.solve3d_batch(models, ex.Options(n_sweeps=0, tolerance=-1, factored_radius=3), ex.F32)
    for g, (cells, pos), out in zip(grids, refs, outs):
        nx, ny, nz, dx, dy, dz = g
        for j, p in enumerate(pos):
            cell = [min(k - 2, int(q / h)) for q, k, h in zip(p, (nx, ny, nz), (dx, dy, dz))]
            ref = oracle.solve3d(cells, g, cell, p, n_sweeps=0, radius=3)
            assert np.array_equal(_bits(out[j]), _bits(ref)), (g, j)


@pytest.mark.parametrize("block_shape", [1, 2, 3])
def test_mailbox_tags_after_a_longer_solve(ctx, oracle, block_shape):
    """A solve with fewer sweeps than the one before it must not meet that solve's mailbox
    words under its own tags, whatever the layout in between (precision, grid, warp block)."""
    rng = np.random.default_rng(50 + block_shape)
    long_shape, short_shape = (31, 27, 25, 40., 40., 40.), (29, 35, 23, 40., 40., 40.)
    cells = _cells(oracle, long_shape, 51, np.float64)
    ctx.set_grid3d(*long_shape)
    ctx.set_slowness3d(cells)
    ctx.solve3d([p for p, _ in _sources(rng, long_shape, 8)], ex.Options(n_sweeps=9, tolerance=-1), ex.F64)
    nx, ny, nz, dx, dy, dz = short_shape
    cells = _cells(oracle, short_shape, 52, np.float32)
    ctx.set_grid3d(*short_shape)
    ctx.set_slowness3d(cells)
    pos = [(fx * (nx - 1) * dx, fy * (ny - 1) * dy, fz * (nz - 1) * dz) for fx, fy, fz in CORNERS]
    for n_sweeps in (0, 1):
        t = ctx.solve3d(pos, ex.Options(n_sweeps=n_sweeps, tolerance=-1, sweep_kernel=2, block_shape=block_shape),
                        ex.F32)
        for p, a in zip(pos, t):
            cell = [min(k - 2, int(q / h)) for q, k, h in zip(p, (nx, ny, nz), (dx, dy, dz))]
            ref = oracle.solve3d(cells, short_shape, cell, p, n_sweeps=n_sweeps, radius=3)
            assert np.array_equal(_bits(a), _bits(ref)), (p, n_sweeps, np.abs(a - ref).max())


def test_batch_mailbox_tags_after_a_longer_batch(ctx, oracle):
    rng = np.random.default_rng(60)
    first = [{"grid": (30, 26, 20, 50., 50., 50., 0., 0., 0.), "model": _cells(oracle, (30, 26, 20, 50.), 61, np.float64),
              "sources": [p for p, _ in _sources(rng, (30, 26, 20, 50., 50., 50.), 3)]}]
    ctx.solve3d_batch(first, ex.Options(n_sweeps=8, tolerance=-1), ex.F64)
    g = (26, 33, 21, 50., 50., 50.)
    nx, ny, nz, dx, dy, dz = g
    cells = _cells(oracle, g, 62, np.float32)
    pos = [(fx * (nx - 1) * dx, fy * (ny - 1) * dy, fz * (nz - 1) * dz) for fx, fy, fz in CORNERS]
    out = ctx.solve3d_batch([{"grid": g + (0., 0., 0.), "model": cells, "sources": pos}],
                            ex.Options(n_sweeps=0, tolerance=-1), ex.F32)[0]
    for j, p in enumerate(pos):
        cell = [min(k - 2, int(q / h)) for q, k, h in zip(p, (nx, ny, nz), (dx, dy, dz))]
        ref = oracle.solve3d(cells, g, cell, p, n_sweeps=0, radius=3)
        assert np.array_equal(_bits(out[j]), _bits(ref)), j


def test_sweep_tags_across_the_32_bit_wrap_around(oracle):
    """Before a solve whose 32-bit sweep tags would wrap, the host clears the mailbox and
    restarts the tag base; solves on either side of the wrap stay exact."""
    c = ex.Context(0)
    try:
        shape = (29, 27, 23, 40., 40., 40.)
        nx, ny, nz, dx, dy, dz = shape
        cells = _cells(oracle, shape, 71, np.float32)
        c.set_grid3d(*shape)
        c.set_slowness3d(cells)
        pos = [(fx * (nx - 1) * dx, fy * (ny - 1) * dy, fz * (nz - 1) * dz) for fx, fy, fz in CORNERS]
        stride = 8 * (1 + 1) + 1               # tags one solve of one refinement iteration uses
        # the third solve would pass 2^32: it runs after the clear, with tags from 1
        opt = ex.Options(n_sweeps=1, tolerance=-1, test_tag_margin=2 * stride + 5)
        for rep in range(4):
            t = c.solve3d(pos, opt, ex.F32)
            for p, a in zip(pos, t):
                cell = [min(k - 2, int(q / h)) for q, k, h in zip(p, (nx, ny, nz), (dx, dy, dz))]
                ref = oracle.solve3d(cells, shape, cell, p, n_sweeps=1, radius=3)
                assert np.array_equal(_bits(a), _bits(ref)), (rep, p)
    finally:
        c.close()
