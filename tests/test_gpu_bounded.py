"""Many refinement iterations of the chunk-step kernel against the oracle, bit for bit.

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
