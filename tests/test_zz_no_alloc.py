"""eikx_solve3d_noalloc: the solve for callers that cannot allocate GPU memory.

Some hosts own every device allocation (their framework's memory pool) or forbid
allocation once running, so they cannot let the solver call cudaMalloc.  The
no-allocation entry point keeps all of its intermediate buffers in a fixed array
compiled into the library.  These tests call it through the C ABI and check that it
returns exactly what the regular entry point (eikx_solve3d) and the oracle return --
bit for bit, the tolerance every parity test here uses -- on calls in a row, on
different grids so that state left by an earlier call would show.  They also cover the
options it honours (convergence window, node-step kernel, warp-block shape), non-uniform
spacing, the model check, the bounded-wait timeout and the size limit.  This file is
collected last, so a stop at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import eikonalxx_gb300 as ex
    from eikonalxx_gb300 import build
    build.build()
    return ex, ex.load()


def _noalloc(lib):
    f = lib.eikx_solve3d_noalloc
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 6 + [ctypes.c_void_p] * 5
    f.restype = ctypes.c_int
    return f


def _case(rng, nx, ny, nz, dx, dy, dz):
    s = (1.0 / rng.uniform(2000, 6000, (nz - 1) * (ny - 1) * (nx - 1))).astype(np.float32)
    pos = [float(rng.uniform(0, (n - 1) * d)) for n, d in zip((nx, ny, nz), (dx, dy, dz))]
    return s, pos


def _regular(ex, s, grid, pos, opt):
    nx, ny, nz, dx, dy, dz = grid
    with ex.Context(0) as ctx:
        ctx.set_grid3d(nx, ny, nz, dx, dy, dz)
        ctx.set_slowness3d(s)
        return ctx.solve3d([pos], opt, ex.F32)[0]


def _no_alloc_solve(ex, f, s, grid, pos, opt):
    nx, ny, nz, dx, dy, dz = grid
    s_dev = torch.from_numpy(s).cuda()
    out = torch.full((nz, ny, nx), -1.0, dtype=torch.float32, device="cuda")
    src = ex._Src3(*pos)
    o = opt._c() if opt is not None else None
    torch.cuda.synchronize()
    rc = f(nx, ny, nz, dx, dy, dz, 0.0, 0.0, 0.0, ctypes.c_void_p(s_dev.data_ptr()), ctypes.byref(src),
           ctypes.byref(o) if o is not None else None, ctypes.c_void_p(out.data_ptr()), None)
    return rc, out.cpu().numpy()


def _oracle_solve(s, grid, pos, opt):
    from oracle import Oracle
    cell = [min(n - 2, int(p / d)) for p, n, d in zip(pos, grid[:3], grid[3:])]
    return Oracle().solve3d(s, grid, cell, pos, n_sweeps=opt.n_sweeps, radius=opt.factored_radius,
                            tol=opt.tolerance, near_fp64=opt.near_fp64)


def _bits(a):
    return a.view(np.uint32)


def test_no_alloc_matches_regular_solve_twice():
    ex, lib = _lib()
    f = _noalloc(lib)
    rng = np.random.default_rng(99)
    opt = ex.Options(n_sweeps=2, tolerance=-1, factored_radius=3)
    for grid in [(37, 29, 21, 25.0, 25.0, 25.0), (24, 33, 17, 40.0, 40.0, 40.0)]:
        s, pos = _case(rng, *grid)
        rc, t = _no_alloc_solve(ex, f, s, grid, pos, opt)
        assert rc == ex.EIKX_OK, lib.eikx_last_error()
        ref = _regular(ex, s, grid, pos, opt)
        assert np.array_equal(_bits(t), _bits(ref)), np.abs(t - ref).max()
        assert np.array_equal(_bits(t), _bits(_oracle_solve(s, grid, pos, opt)))


# (grid, options): the convergence window with a positive tolerance, the node-step kernel,
# the 4x8 warp block at two blocks per SM, non-uniform spacing (dx != dz), and the FP64
# factored branch
CASES = [
    ((30, 26, 22, 100.0, 100.0, 100.0), dict(n_sweeps=6, tolerance=1e-6, factored_radius=0)),
    ((29, 23, 19, 40.0, 40.0, 40.0), dict(n_sweeps=3, tolerance=-1, factored_radius=2, sweep_kernel=1)),
    ((33, 17, 25, 30.0, 30.0, 30.0), dict(n_sweeps=2, tolerance=-1, block_shape=2, blocks_per_sm=2)),
    ((18, 21, 13, 50.0, 45.0, 60.0), dict(n_sweeps=4, tolerance=1e-6, factored_radius=2)),
    ((21, 19, 17, 50.0, 50.0, 50.0), dict(n_sweeps=3, tolerance=-1, factored_radius=3, near_fp64=True)),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_no_alloc_options_match_regular_and_oracle(case):
    ex, lib = _lib()
    f = _noalloc(lib)
    grid, kw = CASES[case]
    rng = np.random.default_rng(1000 + case)
    opt = ex.Options(**kw)
    s, pos = _case(rng, *grid)
    for _ in range(2):   # two calls in a row on the same scratch
        rc, t = _no_alloc_solve(ex, f, s, grid, pos, opt)
        assert rc == ex.EIKX_OK, lib.eikx_last_error()
        assert np.array_equal(_bits(t), _bits(_regular(ex, s, grid, pos, opt)))
        assert np.array_equal(_bits(t), _bits(_oracle_solve(s, grid, pos, opt)))


def test_no_alloc_rejects_bad_models_and_options():
    ex, lib = _lib()
    f = _noalloc(lib)
    rng = np.random.default_rng(5)
    grid = (12, 10, 9, 50.0, 50.0, 50.0)
    s, pos = _case(rng, *grid)
    s[17] = -s[17]
    rc, _ = _no_alloc_solve(ex, f, s, grid, pos, ex.Options())
    assert rc == ex.EIKX_ERR_INVALID
    assert b"Non-positive" in lib.eikx_last_error()
    s[17] = -s[17]
    rc, _ = _no_alloc_solve(ex, f, s, grid, pos, ex.Options(block_shape=7))
    assert rc == ex.EIKX_ERR_INVALID
    rc, t = _no_alloc_solve(ex, f, s, grid, pos, None)     # NULL options: the defaults
    assert rc == ex.EIKX_OK
    assert np.array_equal(_bits(t), _bits(_regular(ex, s, grid, pos, ex.Options())))


def test_no_alloc_bounded_wait_times_out_then_solves():
    """Failure detection on the no-allocation path: the first warp block is left out of
    the queue, so the blocks that wait on it give up after 2^12 polls; the call returns
    EIKX_ERR_TIMEOUT and the next call on the shared scratch is correct."""
    ex, lib = _lib()
    f = _noalloc(lib)
    rng = np.random.default_rng(16)
    grid = (20, 24, 16, 50.0, 50.0, 50.0)
    s, pos = _case(rng, *grid)
    rc, _ = _no_alloc_solve(ex, f, s, grid, pos,
                            ex.Options(n_sweeps=1, tolerance=-1, spin_limit_log2=12, test_drop_blocks=1))
    assert rc == ex.EIKX_ERR_TIMEOUT
    opt = ex.Options(n_sweeps=1, tolerance=-1)
    rc, t = _no_alloc_solve(ex, f, s, grid, pos, opt)
    assert rc == ex.EIKX_OK, lib.eikx_last_error()
    assert np.array_equal(_bits(t), _bits(_oracle_solve(s, grid, pos, opt)))


def test_no_alloc_rejects_grids_beyond_its_scratch():
    ex, lib = _lib()
    f = _noalloc(lib)
    nx = ny = nz = 200          # 8M nodes: more than the 64 MiB array holds
    s_dev = torch.full(((nx - 1) * (ny - 1) * (nz - 1),), 1 / 3000.0, device="cuda")
    out = torch.empty(nx * ny * nz, device="cuda")
    src = ex._Src3(10.0, 10.0, 10.0)
    rc = f(nx, ny, nz, 10.0, 10.0, 10.0, 0.0, 0.0, 0.0, ctypes.c_void_p(s_dev.data_ptr()), ctypes.byref(src),
           None, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == ex.EIKX_ERR_INVALID
    assert b"64 MiB" in lib.eikx_last_error()
