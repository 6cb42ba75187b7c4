"""GPU kernels against the oracle (bit-exact) through the C ABI."""
import numpy as np
import pytest

from conftest import random_slowness

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402


def _src(rng, n, d):
    """Absolute position, cell and offset of a random source (origin 0)."""
    pos = [float(rng.uniform(0, (k - 1) * h)) for k, h in zip(n, d)]
    cell = [min(k - 2, int(p / h)) for p, k, h in zip(pos, n, d)]
    return pos, cell, pos


def _bits(a):
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


SHAPES3 = [
    (9, 10, 11, 100., 100., 100.),
    (13, 7, 8, 100., 120., 90.),      # non-uniform spacing
    (3, 3, 3, 50., 50., 50.),          # smallest grid the reference allows
    (33, 17, 9, 25., 25., 25.),        # not multiples of the 8x4 warp block
    (21, 40, 18, 10., 10., 10.),
]


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
@pytest.mark.parametrize("radius", [0, 3, 1000])
@pytest.mark.parametrize("shape", SHAPES3)
def test_solve3d_bitexact_vs_oracle(ctx, oracle, precision, radius, shape):
    rng = np.random.default_rng(abs(hash((shape, radius, precision))) % 2**32)
    nx, ny, nz, dx, dy, dz = shape
    dt = np.float32 if precision == ex.F32 else np.float64
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=dt)
    pos, cell, off = _src(rng, (nx, ny, nz), (dx, dy, dz))
    ctx.set_grid3d(nx, ny, nz, dx, dy, dz)
    ctx.set_slowness3d(s)
    for init_fp64 in (True, False):
        opt = ex.Options(n_sweeps=2, tolerance=-1, factored_radius=radius, init_fp64=init_fp64)
        t_gpu = ctx.solve3d([pos], opt, precision)[0]
        t_or = oracle.solve3d(s, shape, cell, off, n_sweeps=2, radius=radius, init_fp64=init_fp64)
        assert np.array_equal(_bits(t_gpu), _bits(t_or)), np.abs(t_gpu - t_or).max()


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
def test_solve3d_batch_each_field_matches(ctx, oracle, precision):
    rng = np.random.default_rng(11)
    shape = (24, 19, 14, 50., 50., 50.)
    nx, ny, nz = shape[:3]
    dt = np.float32 if precision == ex.F32 else np.float64
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=dt)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    srcs = [_src(rng, (nx, ny, nz), shape[3:]) for _ in range(7)]
    opt = ex.Options(n_sweeps=1, tolerance=-1, factored_radius=3)
    t = ctx.solve3d([p for p, _, _ in srcs], opt, precision)
    for i, (_, cell, off) in enumerate(srcs):
        t_or = oracle.solve3d(s, shape, cell, off, n_sweeps=1, radius=3)
        assert np.array_equal(_bits(t[i]), _bits(t_or)), i


def test_solve3d_without_init_pass(ctx, oracle):
    rng = np.random.default_rng(12)
    shape = (17, 12, 10, 40., 40., 40.)
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    pos, cell, off = _src(rng, (nx, ny, nz), shape[3:])
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    opt = ex.Options(n_sweeps=3, tolerance=-1, factored_radius=2, init_sweeps=False)
    t = ctx.solve3d([pos], opt, ex.F32)[0]
    t_or = oracle.solve3d(s, shape, cell, off, n_sweeps=3, radius=2, init_sweeps=False)
    assert np.array_equal(_bits(t), _bits(t_or))


def test_convergence_stops_like_the_oracle(ctx, oracle):
    rng = np.random.default_rng(13)
    shape = (30, 26, 22, 100., 100., 100.)
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    pos, cell, off = _src(rng, (nx, ny, nz), shape[3:])
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    opt = ex.Options(n_sweeps=20, tolerance=1e-6, factored_radius=0)
    t = ctx.solve3d([pos], opt, ex.F32)[0]
    st = ctx.stats()
    t_or, res, it = oracle.solve3d(s, shape, cell, off, n_sweeps=20, radius=0, tol=1e-6, residuals=True)
    assert st["iterations_max"] == it < 20
    assert np.array_equal(_bits(t), _bits(t_or))
    # the field stops after the first run of 8 sweeps with decreases below tol; residual_last
    # is the largest decrease of that window
    r = res.ravel()
    quiet = np.convolve((r < 1e-6).astype(int), np.ones(8, int), "valid")
    stop = int(np.argmax(quiet == 8)) + 8
    assert (it - 1) * 8 < stop <= it * 8
    assert st["residual_last"] == pytest.approx(r[stop - 8:stop].max(), rel=0, abs=0)


def test_slowness_orderings_and_device_inputs(ctx, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(14)
    shape = (12, 9, 7, 30., 30., 30.)
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1, ny - 1, nx - 1), dtype=np.float32)
    pos, cell, off = _src(rng, (nx, ny, nz), shape[3:])
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(np.ascontiguousarray(s.transpose(2, 1, 0)).ravel(), ordering=ex.TRANSPOSED)
    opt = ex.Options(n_sweeps=2, tolerance=-1)
    t1 = ctx.solve3d([pos], opt, ex.F32)[0]
    ctx.set_slowness3d(torch.from_numpy(s.ravel()).cuda())
    out = torch.empty((1, nz, ny, nx), dtype=torch.float32, device="cuda")
    ctx.solve3d([pos], opt, ex.F32, out=out)
    t_or = oracle.solve3d(s.ravel(), shape, cell, off, n_sweeps=2, radius=3)
    assert np.array_equal(_bits(t1), _bits(t_or))
    assert np.array_equal(_bits(out[0].cpu().numpy()), _bits(t_or))


def test_nodal_velocity_model_matches_oracle(ctx, oracle):
    rng = np.random.default_rng(15)
    nx, ny, nz = 11, 10, 9
    v = rng.uniform(2500, 5500, nx * ny * nz)
    ctx.set_grid3d(nx, ny, nz, 20., 20., 20.)
    ctx.set_nodal_velocity3d(v)
    assert np.array_equal(ctx.get_slowness3d(), oracle.nodal_to_cell3d(v, nx, ny, nz, 0))
    vt = np.ascontiguousarray(v.reshape(nz, ny, nx).transpose(2, 1, 0)).ravel()
    ctx.set_nodal_velocity3d(vt, ordering=ex.TRANSPOSED)
    assert np.array_equal(ctx.get_slowness3d(), oracle.nodal_to_cell3d(vt, nx, ny, nz, 1))


SHAPES2 = [(31, 27, 10., 10.), (25, 33, 10., 12.5), (3, 3, 10., 10.), (70, 45, 5., 5.),
           (12, 530, 10., 10.)]   # more rows than one CTA holds: the warp-block kernel


@pytest.mark.parametrize("kernel", [0, 2])        # 0: warp blocks, 2: one CTA per field (<= 512 rows)
@pytest.mark.parametrize("precision", [ex.F64, ex.F32])
@pytest.mark.parametrize("radius", [0, 3, 1000])
@pytest.mark.parametrize("shape", SHAPES2)
def test_solve2d_bitexact_vs_oracle(ctx, oracle, precision, radius, shape, kernel):
    rng = np.random.default_rng(abs(hash((shape, radius, precision, 2))) % 2**32)
    nx, nz, dx, dz = shape
    dt = np.float32 if precision == ex.F32 else np.float64
    s = random_slowness(rng, (nz - 1) * (nx - 1), dtype=dt)
    pos, cell, off = _src(rng, (nx, nz), (dx, dz))
    ctx.set_grid2d(nx, nz, dx, dz)
    ctx.set_slowness2d(s)
    opt = ex.Options(n_sweeps=2, tolerance=-1, factored_radius=radius, sweep_kernel=kernel)
    t_gpu = ctx.solve2d([pos], opt, precision)[0]
    t_or = oracle.solve2d(s, shape, cell, off, n_sweeps=2, radius=radius, hypot_mode=1)
    assert np.array_equal(_bits(t_gpu), _bits(t_or)), np.abs(t_gpu - t_or).max()


def test_invalid_inputs_raise(ctx):
    with pytest.raises(ex.InvalidArgument):
        ctx.set_grid3d(2, 5, 5, 1., 1., 1.)
    ctx.set_grid3d(5, 5, 5, 10., 10., 10.)
    with pytest.raises(ex.InvalidArgument):
        ctx.set_slowness3d(-np.ones(64))
    ctx.set_slowness3d(np.full(64, 1 / 3000.))
    with pytest.raises(ex.InvalidArgument):
        ctx.solve3d([[100., 0., 0.]])          # outside [0, 40]
    t = ctx.solve3d([[40., 40., 40.]], ex.Options(tolerance=-1))   # far corner is allowed
    assert t[0, 4, 4, 4] == 0.0


def test_bounded_wait_times_out_and_context_survives(ctx, oracle):
    """Failure detection: blocks whose upstream never runs give up after the spin bound;
    the solve reports EIKX_ERR_TIMEOUT and the next solve on the context is correct."""
    rng = np.random.default_rng(16)
    shape = (20, 24, 16, 50., 50., 50.)
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    pos, cell, off = _src(rng, (nx, ny, nz), shape[3:])
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    with pytest.raises(ex.TimeoutError_):
        ctx.solve3d([pos], ex.Options(n_sweeps=1, tolerance=-1, spin_limit_log2=12, test_drop_blocks=1), ex.F32)
    t = ctx.solve3d([pos], ex.Options(n_sweeps=1, tolerance=-1), ex.F32)[0]
    t_or = oracle.solve3d(s, shape, cell, off, n_sweeps=1, radius=3)
    assert np.array_equal(_bits(t), _bits(t_or))


@pytest.mark.parametrize("n_src", [2, 5, 8])
def test_paired_fields_converge_independently(ctx, oracle, n_src):
    """Two fields per lane (FP32, uniform grid): fields of one pair converge at different
    iterations and each must still stop exactly where the oracle stops."""
    rng = np.random.default_rng(100 + n_src)
    shape = (37, 29, 21, 60., 60., 60.)
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    srcs = [_src(rng, (nx, ny, nz), shape[3:]) for _ in range(n_src)]
    pos = [p for p, _, _ in srcs]
    outs = {}
    for pair in (True, False):
        opt = ex.Options(n_sweeps=12, tolerance=1e-6, factored_radius=3, pair_fields=pair)
        outs[pair] = ctx.solve3d(pos, opt, ex.F32)
    for i, (_, cell, off) in enumerate(srcs):
        t_or = oracle.solve3d(s, shape, cell, off, n_sweeps=12, radius=3, tol=1e-6)
        assert np.array_equal(_bits(outs[True][i]), _bits(t_or)), i
        assert np.array_equal(_bits(outs[False][i]), _bits(t_or)), i


@pytest.mark.parametrize("variant,block", [(1, 0), (2, 1), (2, 2), (2, 3)])
@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
@pytest.mark.parametrize("shape", [(29, 23, 19, 40., 40., 40.), (18, 21, 13, 50., 45., 60.), (5, 4, 3, 10., 10., 10.)])
def test_sweep_kernel_variants_match_oracle(ctx, oracle, variant, block, precision, shape):
    """Node-step (one node per lane and step) and chunk-step (one 16-byte chunk per lane
    and step, warp blocks of 8x4, 4x8 and 16x2 pencils) kernels, uniform and non-uniform
    grids, near-source nodes included."""
    rng = np.random.default_rng(200 + variant)
    nx, ny, nz = shape[:3]
    dt = np.float32 if precision == ex.F32 else np.float64
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=dt)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    srcs = [_src(rng, (nx, ny, nz), shape[3:]) for _ in range(3)]
    opt = ex.Options(n_sweeps=3, tolerance=-1, factored_radius=2, sweep_kernel=variant, block_shape=block)
    t = ctx.solve3d([p for p, _, _ in srcs], opt, precision)
    for i, (_, cell, off) in enumerate(srcs):
        t_or = oracle.solve3d(s, shape, cell, off, n_sweeps=3, radius=2)
        assert np.array_equal(_bits(t[i]), _bits(t_or)), (i, np.abs(t[i] - t_or).max())


@pytest.mark.parametrize("kernel", [0, 2])
def test_solve2d_batch_converges_per_field(ctx, oracle, kernel):
    rng = np.random.default_rng(71)
    shape = (57, 41, 20., 20.)
    nx, nz, dx, dz = shape
    s = random_slowness(rng, (nz - 1) * (nx - 1), dtype=np.float64)
    ctx.set_grid2d(nx, nz, dx, dz)
    ctx.set_slowness2d(s)
    srcs = [_src(rng, (nx, nz), (dx, dz)) for _ in range(5)]
    opt = ex.Options(n_sweeps=15, tolerance=1e-7, factored_radius=3, sweep_kernel=kernel)
    t = ctx.solve2d([p for p, _, _ in srcs], opt, ex.F64)
    for i, (_, cell, off) in enumerate(srcs):
        t_or = oracle.solve2d(s, shape, cell, off, n_sweeps=15, radius=3, tol=1e-7, hypot_mode=1)
        assert np.array_equal(_bits(t[i]), _bits(t_or)), i


@pytest.mark.parametrize("block", [0, 2, 3])
@pytest.mark.parametrize("radius", [3, 1000])
@pytest.mark.parametrize("shape", [(29, 23, 19, 40., 40., 40.), (18, 21, 13, 50., 45., 60.)])
def test_near_fp64_matches_oracle(ctx, oracle, block, radius, shape):
    """near_fp64: FP32 sweeps whose nodes within the factored radius take the FP64
    operator (T0, its gradient, tau and the quadratic solves in double), uniform and
    non-uniform grids, every warp-block shape, the whole grid factored (radius 1000)."""
    rng = np.random.default_rng(300 + radius + block)
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    srcs = [_src(rng, (nx, ny, nz), shape[3:]) for _ in range(3)]
    opt = ex.Options(n_sweeps=4, tolerance=1e-6, factored_radius=radius, near_fp64=True, block_shape=block)
    t = ctx.solve3d([p for p, _, _ in srcs], opt, ex.F32)
    for i, (_, cell, off) in enumerate(srcs):
        t_or = oracle.solve3d(s, shape, cell, off, n_sweeps=4, radius=radius, tol=1e-6, near_fp64=True)
        assert np.array_equal(_bits(t[i]), _bits(t_or)), (i, np.abs(t[i] - t_or).max())
        t_32 = oracle.solve3d(s, shape, cell, off, n_sweeps=4, radius=radius, tol=1e-6)
        assert not np.array_equal(_bits(t_or), _bits(t_32))     # the mode changes the near field


def test_near_fp64_batch_and_pair_request(ctx, oracle):
    """near_fp64 in a multi-model batch, and with pair_fields requested (the FP64 branch
    runs on the chunk-step kernel, so the request falls back to one field per lane)."""
    rng = np.random.default_rng(17)
    shape = (24, 19, 14, 50., 50., 50.)
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    srcs = [_src(rng, (nx, ny, nz), shape[3:]) for _ in range(4)]
    opt = ex.Options(n_sweeps=3, tolerance=-1, factored_radius=3, near_fp64=True, pair_fields=True)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    t = ctx.solve3d([p for p, _, _ in srcs], opt, ex.F32)
    tb = ctx.solve3d_batch([{"grid": shape, "model": s, "sources": [p for p, _, _ in srcs]}], opt, ex.F32)[0]
    for i, (_, cell, off) in enumerate(srcs):
        t_or = oracle.solve3d(s, shape, cell, off, n_sweeps=3, radius=3, near_fp64=True)
        assert np.array_equal(_bits(t[i]), _bits(t_or)), i
        assert np.array_equal(_bits(tb[i]), _bits(t_or)), i


def test_near_fp64_rejects_a_factored_region_beyond_its_table(ctx):
    """The FP64 analytic factor is tabulated per solve (8 sweep orderings x the nodes within
    the radius, at most 2^18 entries per field): a larger factored region is refused."""
    rng = np.random.default_rng(18)
    shape = (70, 70, 70, 20., 20., 20.)
    nx, ny, nz = shape[:3]
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32))
    with pytest.raises(ex.EikxError) as e:
        ctx.solve3d([[690., 690., 690.]], ex.Options(n_sweeps=1, factored_radius=1000, near_fp64=True), ex.F32)
    assert e.value.code == ex.EIKX_ERR_UNSUPPORTED
    t = ctx.solve3d([[690., 690., 690.]], ex.Options(n_sweeps=1, factored_radius=3, near_fp64=True), ex.F32)
    assert np.isfinite(t).all()
