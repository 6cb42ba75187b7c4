"""eikx_solve3d_noalloc: the solve for callers that cannot allocate GPU memory.

Some hosts own every device allocation (their framework's memory pool) or forbid
allocation once running, so they cannot let the solver call cudaMalloc.  The
no-allocation entry point keeps all of its intermediate buffers in a fixed array
compiled into the library.  These tests call it through the C ABI and check that it
returns exactly what the regular entry point (eikx_solve3d) returns -- bit for bit, the
tolerance every parity test here uses -- on two calls in a row, the second on a
different grid so that state left by the first call would show.  This file is
collected last, so a stop at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc(lib):
    f = lib.eikx_solve3d_noalloc
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 6 + [ctypes.c_void_p] * 5
    f.restype = ctypes.c_int
    return f


def _case(rng, nx, ny, nz, h):
    s = (1.0 / rng.uniform(2000, 6000, (nz - 1) * (ny - 1) * (nx - 1))).astype(np.float32)
    pos = [float(rng.uniform(0, (n - 1) * h)) for n in (nx, ny, nz)]
    return s, pos


def _regular(ex, s, grid, pos, opt):
    nx, ny, nz, h = grid
    with ex.Context(0) as ctx:
        ctx.set_grid3d(nx, ny, nz, h, h, h)
        ctx.set_slowness3d(s)
        return ctx.solve3d([pos], opt, ex.F32)[0]


def _no_alloc_solve(ex, f, s, grid, pos, opt):
    nx, ny, nz, h = grid
    s_dev = torch.from_numpy(s).cuda()
    out = torch.full((nz, ny, nx), -1.0, dtype=torch.float32, device="cuda")
    src = ex._Src3(*pos)
    o = opt._c()
    torch.cuda.synchronize()
    rc = f(nx, ny, nz, h, h, h, 0.0, 0.0, 0.0, ctypes.c_void_p(s_dev.data_ptr()), ctypes.byref(src),
           ctypes.byref(o), ctypes.c_void_p(out.data_ptr()), None)
    return rc, out.cpu().numpy()


def test_no_alloc_matches_regular_solve_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import eikonalxx_gb300 as ex
    from eikonalxx_gb300 import build
    build.build()
    lib = ex.load()
    f = _noalloc(lib)
    rng = np.random.default_rng(99)
    opt = ex.Options(n_sweeps=2, tolerance=-1, factored_radius=3)
    for grid in [(37, 29, 21, 25.0), (24, 33, 17, 40.0)]:
        s, pos = _case(rng, *grid)
        rc, t = _no_alloc_solve(ex, f, s, grid, pos, opt)
        assert rc == ex.EIKX_OK, lib.eikx_last_error()
        ref = _regular(ex, s, grid, pos, opt)
        assert np.array_equal(t.view(np.uint32), ref.view(np.uint32)), np.abs(t - ref).max()


def test_no_alloc_rejects_grids_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import eikonalxx_gb300 as ex
    lib = ex.load()
    f = _noalloc(lib)
    nx = ny = nz = 200          # 8M nodes: more than the 64 MiB array holds
    s_dev = torch.full(((nx - 1) * (ny - 1) * (nz - 1),), 1 / 3000.0, device="cuda")
    out = torch.empty(nx * ny * nz, device="cuda")
    src = ex._Src3(10.0, 10.0, 10.0)
    rc = f(nx, ny, nz, 10.0, 10.0, 10.0, 0.0, 0.0, 0.0, ctypes.c_void_p(s_dev.data_ptr()), ctypes.byref(src),
           None, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == ex.EIKX_ERR_INVALID
    assert b"64 MiB" in lib.eikx_last_error()
