"""Parity at the benchmark configurations' full sizes, bit for bit against the oracle.

The other parity tests run small grids.  These run the configurations the benchmark
measures, so the persistent work queue, the tagged mailbox and the own-pencil prefetch
ring are checked at the occupancy the headline runs at (every SM full, thousands of warp
blocks in flight):
  * the plain 2D configuration: 501 x 251 nodes, 10 m, FP64, v(z) = 3000 + 0.5 z m/s,
    source (2500, 500) m, factored radius 3, 2 iterations, tolerance 1e-8 s -- one field,
    and a batch of 64 fields with seeded sources;
  * the plain 3D configuration: 256 x 256 x 128 nodes, 50 m, layered + GRF model from
    nodal velocities, FP32 sweeps, radius 3, one seeded source, one refinement iteration
    (16 sweeps);
  * the benchmark's batch: the same model with its 64 seeded sources, solved to tolerance
    1e-5 s (at most 10 iterations) in one schedule with host output, 8 seeded fields of
    it checked against the oracle (each stops at its own iteration).
The oracle runs its fields on host threads (the ctypes calls release the GIL).
Reference counterparts: the 3D sweep include/private/solver3d.hpp:150-326, the 2D solve
src/solver2d.cpp:462-565.
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402
from eikonalxx_gb300 import synthetic  # noqa: E402

NX3, NY3, NZ3, H3 = 256, 256, 128, 50.0
MODEL_SEED, SOURCE_SEED = 20240601, 7      # the benchmark's seeds


def _bits(a):
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def _cell(pos, n, d):
    return [min(k - 2, int(p / h)) for p, k, h in zip(pos, n, d)]


@pytest.fixture(scope="module")
def model3(oracle):
    """The benchmark's FP32 nodal velocities and their cell slowness (the reference's
    8 / sum of the 8 corner velocities, formed in the input's precision, FP32)."""
    v = synthetic.layered_grf_model(NX3, NY3, NZ3, H3, MODEL_SEED)
    s32 = oracle.nodal_to_cell3d(v.ravel(), NX3, NY3, NZ3, 0)
    assert s32.dtype == np.float32
    return v, s32


def _pool():
    return cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1))


def test_plain_2d_configuration(ctx, oracle):
    nx, nz, h = 501, 251, 10.0
    v = synthetic.linear_gradient_2d(nx, nz, h, 3000.0, 0.5)
    ctx.set_grid2d(nx, nz, h, h)
    ctx.set_nodal_velocity2d(v)
    s = oracle.nodal_to_cell2d(v.ravel(), nx, nz, 0)
    opt = ex.Options(n_sweeps=2, tolerance=1e-8, factored_radius=3)
    src = (2500.0, 500.0)
    t = ctx.solve2d([src], opt, ex.F64)[0]
    t_or = oracle.solve2d(s, (nx, nz, h, h), _cell(src, (nx, nz), (h, h)), src, n_sweeps=2, radius=3, tol=1e-8)
    assert np.array_equal(_bits(t), _bits(t_or)), np.abs(t - t_or).max()
    # 64 fields of the configuration in one launch schedule, seeded sources
    rng = np.random.default_rng(SOURCE_SEED)
    srcs = np.column_stack([rng.uniform(0, (nx - 1) * h, 64), rng.uniform(0, (nz - 1) * h, 64)])
    tb = ctx.solve2d(srcs, opt, ex.F64)
    with _pool() as pool:
        ors = list(pool.map(lambda p: oracle.solve2d(s, (nx, nz, h, h), _cell(p, (nx, nz), (h, h)), p, n_sweeps=2,
                                                     radius=3, tol=1e-8), srcs))
    for i, t_or in enumerate(ors):
        assert np.array_equal(_bits(tb[i]), _bits(t_or)), (i, np.abs(tb[i] - t_or).max())


def test_plain_3d_configuration_one_source(ctx, oracle, model3):
    v, s32 = model3
    ctx.set_grid3d(NX3, NY3, NZ3, H3, H3, H3)
    ctx.set_nodal_velocity3d(v)
    # the device's nodal -> cell slowness at full size
    assert np.array_equal(ctx.get_slowness3d(), s32.astype(np.float64))
    src = synthetic.uniform_sources(1, NX3, NY3, NZ3, H3, SOURCE_SEED + 1)[0]
    opt = ex.Options(n_sweeps=1, tolerance=-1, factored_radius=3)
    t = ctx.solve3d([src], opt, ex.F32)[0]
    t_or = oracle.solve3d(s32, (NX3, NY3, NZ3, H3, H3, H3), _cell(src, (NX3, NY3, NZ3), (H3,) * 3),
                          src, n_sweeps=1, radius=3)
    assert np.array_equal(_bits(t), _bits(t_or)), np.abs(t - t_or).max()


def test_benchmark_batch_fields_match_oracle(ctx, oracle, model3):
    v, s32 = model3
    ctx.set_grid3d(NX3, NY3, NZ3, H3, H3, H3)
    ctx.set_nodal_velocity3d(v)
    srcs = synthetic.uniform_sources(64, NX3, NY3, NZ3, H3, SOURCE_SEED)
    opt = ex.Options(n_sweeps=10, tolerance=1e-5, factored_radius=3)
    t = ctx.solve3d(srcs, opt, ex.F32)             # host output: fields copied out as they converge
    st = ctx.stats()
    assert st["iterations_min"] < st["iterations_max"] <= 10     # fields stop at different iterations
    pick = sorted(np.random.default_rng(3).choice(64, 8, replace=False))
    grid = (NX3, NY3, NZ3, H3, H3, H3)

    def one(i):
        return oracle.solve3d(s32, grid, _cell(srcs[i], grid[:3], grid[3:]), srcs[i], n_sweeps=10, radius=3, tol=1e-5)

    with _pool() as pool:
        ors = list(pool.map(one, pick))
    for i, t_or in zip(pick, ors):
        assert np.array_equal(_bits(t[i]), _bits(t_or)), (i, np.abs(t[i] - t_or).max())
