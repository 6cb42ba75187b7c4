"""A stream of sources through slots (eikx_options.max_in_flight).

With max_in_flight = S < n sources, eikx_solve3d keeps S fields in flight: a field that
converged (or ran n_sweeps iterations) is copied out at the next iteration boundary and its
slot takes the next source, whose initialisation sweeps then run inside the same launches as
the other slots' refinement sweeps.  Every field must still be the solve of its source alone,
bit for bit: against the same sources solved as one batch, against the oracle, with the same
iteration counts.  The cases cover FP32 and FP64, uniform and non-uniform spacing, the FP64
analytic factor, warp-block shapes, no initialisation pass, a fixed iteration count, host and
device output, one slot, and the bounded-wait timeout.  The sweep is the reference's
(include/private/solver3d.hpp:150-326).
"""
import numpy as np
import pytest

from conftest import random_slowness

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402


def _bits(a):
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def _sources(rng, n, grid):
    nx, ny, nz, dx, dy, dz = grid
    return np.column_stack([rng.uniform(0, (nx - 1) * dx, n), rng.uniform(0, (ny - 1) * dy, n),
                            rng.uniform(0, (nz - 1) * dz, n)])


def _cell(p, grid):
    return [min(k - 2, int(q / h)) for q, k, h in zip(p, grid[:3], grid[3:])]


# (grid, precision, sources, slots, options)
CASES = [
    ((40, 36, 28, 50.0, 50.0, 50.0), ex.F32, 11, 4, dict()),
    ((40, 36, 28, 50.0, 50.0, 50.0), ex.F32, 9, 3, dict(near_fp64=True)),
    ((33, 29, 21, 40.0, 40.0, 40.0), ex.F64, 7, 2, dict()),
    ((30, 26, 22, 50.0, 45.0, 60.0), ex.F32, 8, 3, dict(near_fp64=True)),
    ((37, 25, 31, 30.0, 30.0, 30.0), ex.F32, 10, 4, dict(block_shape=2)),
    ((37, 25, 31, 30.0, 30.0, 30.0), ex.F32, 10, 4, dict(block_shape=3, factored_radius=0)),
    ((29, 31, 23, 50.0, 50.0, 50.0), ex.F32, 6, 2, dict(init_sweeps=False)),
    ((29, 31, 23, 50.0, 50.0, 50.0), ex.F32, 6, 1, dict(tolerance=-1, n_sweeps=2)),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_stream_equals_batch_and_oracle(ctx, oracle, case):
    grid, precision, n, slots, kw = CASES[case]
    rng = np.random.default_rng(700 + case)
    nx, ny, nz = grid[:3]
    dt = np.float32 if precision == ex.F32 else np.float64
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), vmin=1500.0, vmax=7000.0, dtype=dt)
    srcs = _sources(rng, n, grid)
    ctx.set_grid3d(*grid)
    ctx.set_slowness3d(s)
    base = dict(n_sweeps=6, tolerance=1e-6, factored_radius=3)
    base.update(kw)
    t_batch = ctx.solve3d(srcs, ex.Options(**base), precision)
    st_batch = ctx.stats()
    t_stream = ctx.solve3d(srcs, ex.Options(max_in_flight=slots, **base), precision)
    st_stream = ctx.stats()
    assert np.array_equal(_bits(t_stream), _bits(t_batch)), np.abs(t_stream - t_batch).max()
    for key in ("iterations_min", "iterations_max", "refine_node_updates"):
        assert st_stream[key] == st_batch[key], key
    for i in (0, n - 1):
        t_or = oracle.solve3d(s, grid, _cell(srcs[i], grid), srcs[i], n_sweeps=base["n_sweeps"],
                              radius=base["factored_radius"], tol=base["tolerance"],
                              init_sweeps=base.get("init_sweeps", True), near_fp64=base.get("near_fp64", False))
        assert np.array_equal(_bits(t_stream[i]), _bits(t_or)), (i, np.abs(t_stream[i] - t_or).max())


def test_stream_device_output_and_repeat(ctx):
    """Device output, and a second stream on the same context (buffers, tags and slot state
    reused) giving the same fields."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(790)
    grid = (48, 40, 32, 50.0, 50.0, 50.0)
    nx, ny, nz = grid[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), vmin=1500.0, vmax=7000.0, dtype=np.float32)
    srcs = _sources(rng, 13, grid)
    ctx.set_grid3d(*grid)
    ctx.set_slowness3d(s)
    opt = ex.Options(n_sweeps=10, tolerance=1e-5, factored_radius=3, near_fp64=True)
    t_batch = ctx.solve3d(srcs, opt, ex.F32)
    out = torch.full((len(srcs), nz, ny, nx), -1.0, dtype=torch.float32, device="cuda")
    sopt = ex.Options(n_sweeps=10, tolerance=1e-5, factored_radius=3, near_fp64=True, max_in_flight=5)
    for _ in range(2):
        out.fill_(-1.0)
        ctx.solve3d(srcs, sopt, ex.F32, out=out)
        assert np.array_equal(_bits(out.cpu().numpy()), _bits(t_batch))


def test_stream_bounded_wait_times_out_then_solves(ctx, oracle):
    """The first warp blocks of every launch's queue are left out: the blocks that wait on
    them give up after 2^12 polls and the stream returns EIKX_ERR_TIMEOUT; the next stream on
    the context is correct."""
    rng = np.random.default_rng(791)
    grid = (24, 20, 16, 50.0, 50.0, 50.0)
    nx, ny, nz = grid[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    srcs = _sources(rng, 5, grid)
    ctx.set_grid3d(*grid)
    ctx.set_slowness3d(s)
    with pytest.raises(ex.TimeoutError_):
        ctx.solve3d(srcs, ex.Options(n_sweeps=2, tolerance=-1, spin_limit_log2=12, test_drop_blocks=1,
                                     max_in_flight=2), ex.F32)
    t = ctx.solve3d(srcs, ex.Options(n_sweeps=2, tolerance=-1, max_in_flight=2), ex.F32)
    t_or = oracle.solve3d(s, grid, _cell(srcs[4], grid), srcs[4], n_sweeps=2, radius=3)
    assert np.array_equal(_bits(t[4]), _bits(t_or))


def test_stream_rejects_negative_slots(ctx):
    ctx.set_grid3d(12, 10, 9, 50.0, 50.0, 50.0)
    ctx.set_slowness3d(np.full(11 * 9 * 8, 1 / 3000.0))
    with pytest.raises(ex.InvalidArgument):
        ctx.solve3d([[100.0, 100.0, 100.0]] * 3, ex.Options(max_in_flight=-1), ex.F32)
