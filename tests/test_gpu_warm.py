"""Warm-started solves (eikx_solve3d_warm)."""
import numpy as np
import pytest

from conftest import random_slowness

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402


def _setup(ctx, rng, shape):
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    src = (rng.uniform(0, (nx - 1) * shape[3]), rng.uniform(0, (ny - 1) * shape[4]), rng.uniform(0, (nz - 1) * shape[5]))
    cell = [min(n - 2, int(p / d)) for p, d, n in zip(src, shape[3:], shape[:3])]
    return s, src, cell


def test_all_huge_start_equals_a_solve_without_init_pass(ctx, oracle):
    rng = np.random.default_rng(61)
    shape = (23, 19, 15, 40., 40., 40.)
    s, src, cell = _setup(ctx, rng, shape)
    init = np.full((1, 15, 19, 23), 1e10, np.float32)
    t = ctx.solve3d_warm([src], init, ex.Options(n_sweeps=4, tolerance=-1, factored_radius=2), ex.F32)[0]
    assert ctx.stats()["reset_nodes"] == 0
    ref = oracle.solve3d(s, shape, cell, src, n_sweeps=4, radius=2, init_sweeps=False)
    assert np.array_equal(t.view(np.uint32), ref.view(np.uint32))


def test_underestimated_nodes_are_reset_and_recomputed(ctx):
    rng = np.random.default_rng(62)
    shape = (31, 27, 21, 50., 50., 50.)
    s, src, cell = _setup(ctx, rng, shape)
    opt = ex.Options(n_sweeps=20, tolerance=1e-7, factored_radius=0)
    cold = ctx.solve3d([src], opt, ex.F32)
    cold_iters = ctx.stats()["iterations_max"]
    init = cold.copy()
    init[0, 15, 20, 25] = 0.0                 # far from the source: far too small
    init[0, 5, 6, 7] *= 0.5
    warm = ctx.solve3d_warm([src], init, opt, ex.F32, gate_tol=1e-6)
    assert ctx.stats()["reset_nodes"] >= 2
    assert ctx.stats()["iterations_max"] <= cold_iters
    # The planted nodes are recomputed.  The rest of the field is not guaranteed to match
    # the cold start: the reference's local solver is not monotone in its neighbours, so a
    # restart can settle on a nearby fixed point (measured in bench.py --workload warmstart).
    assert abs(warm[0, 15, 20, 25] - cold[0, 15, 20, 25]) < 1e-5
    assert abs(warm[0, 5, 6, 7] - cold[0, 5, 6, 7]) < 1e-5
    assert np.isfinite(warm).all() and (warm < 1e9).all()


@pytest.mark.parametrize("seed", [0, 1])
def test_a_converged_field_is_a_fixed_point_of_the_warm_start(ctx, seed):
    """The cold start's sweeps can lower source-cell corners below their analytic start
    value; a warm start from the converged field keeps them, so it ends where it began."""
    rng = np.random.default_rng(seed)
    shape = (33, 29, 25, 50., 50., 50.)
    s, src, cell = _setup(ctx, rng, shape)
    opt = ex.Options(n_sweeps=20, tolerance=1e-5, factored_radius=3)
    cold = ctx.solve3d([src], opt, ex.F32)
    start = ctx.solve3d([src], ex.Options(n_sweeps=0, tolerance=-1, factored_radius=3, init_sweeps=False), ex.F32)
    lowered = sum(cold[0, cell[2] + (k >> 2), cell[1] + ((k >> 1) & 1), cell[0] + (k & 1)] <
                  start[0, cell[2] + (k >> 2), cell[1] + ((k >> 1) & 1), cell[0] + (k & 1)] for k in range(8))
    assert lowered >= 1          # the case this test is about
    warm = ctx.solve3d_warm([src], cold, opt, ex.F32, gate_tol=1e9)
    st = ctx.stats()
    assert st["reset_nodes"] == 0
    assert st["iterations_max"] <= 2
    assert np.max(np.abs(warm.astype(np.float64) - cold)) < 1e-4
