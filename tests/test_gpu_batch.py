"""Multi-model batches (eikx_solve3d_batch): every field bit-identical to the oracle's
solve of its model alone, whatever the mix of grid sizes, spacings and inputs."""
import numpy as np
import pytest

from conftest import random_slowness

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402


def _bits(a):
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def _locate(p, x0, d, n):
    off = p - x0
    return min(n - 2, int(off / d)), off


MODELS = [
    # (nx, ny, nz, dx, dy, dz, x0, y0, z0), number of sources
    ((23, 17, 12, 100., 100., 100., 0., 0., 0.), 2),
    ((9, 31, 7, 100., 100., 100., 500., -200., 1000.), 1),     # origin away from zero
    ((40, 12, 19, 50., 50., 50., 0., 0., 0.), 3),
    ((3, 3, 3, 10., 10., 10., 0., 0., 0.), 1),                  # smallest grid
    ((14, 11, 16, 60., 80., 70., 0., 0., 0.), 2),               # non-uniform spacing
]


def _batch(rng, dt):
    models, ref = [], []
    for k, (g, ns) in enumerate(MODELS):
        nx, ny, nz, dx, dy, dz, x0, y0, z0 = g
        cells = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=dt)
        srcs = [(x0 + rng.uniform(0, (nx - 1) * dx), y0 + rng.uniform(0, (ny - 1) * dy),
                 z0 + rng.uniform(0, (nz - 1) * dz)) for _ in range(ns)]
        models.append({"grid": g, "model": cells, "sources": srcs})
        ref.append((cells, srcs))
    return models, ref


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
def test_batch_fields_match_the_oracle(ctx, oracle, precision):
    rng = np.random.default_rng(31 + precision)
    dt = np.float32 if precision == ex.F32 else np.float64
    models, ref = _batch(rng, dt)
    opt = ex.Options(n_sweeps=6, tolerance=1e-6, factored_radius=3)
    outs = ctx.solve3d_batch(models, opt, precision)
    st = ctx.stats()
    assert st["n_fields"] == sum(ns for _, ns in MODELS)
    for (g, ns), (cells, srcs), out in zip(MODELS, ref, outs):
        nx, ny, nz, dx, dy, dz, x0, y0, z0 = g
        for j, (x, y, z) in enumerate(srcs):
            cx, ox = _locate(x, x0, dx, nx)
            cy, oy = _locate(y, y0, dy, ny)
            cz, oz = _locate(z, z0, dz, nz)
            t_or = oracle.solve3d(cells, (nx, ny, nz, dx, dy, dz), (cx, cy, cz), (ox, oy, oz),
                                  n_sweeps=6, radius=3, tol=1e-6)
            assert np.array_equal(_bits(out[j]), _bits(t_or)), (g, j, np.abs(out[j] - t_or).max())


def test_batch_equals_single_model_solves_and_replays(ctx):
    """Nodal-velocity and transposed inputs; a second call replays the captured schedule."""
    rng = np.random.default_rng(77)
    specs = [((20, 15, 10, 40., 40., 40.), 2), ((12, 25, 9, 40., 40., 40.), 1)]
    models = []
    for g, ns in specs:
        nx, ny, nz = g[:3]
        v = rng.uniform(2000, 6000, size=(nz, ny, nx)).astype(np.float32)
        srcs = [(rng.uniform(0, (nx - 1) * g[3]), rng.uniform(0, (ny - 1) * g[4]), rng.uniform(0, (nz - 1) * g[5]))
                for _ in range(ns)]
        models.append({"grid": g, "model": np.ascontiguousarray(v.transpose(2, 1, 0)), "nodal": True,
                       "ordering": ex.TRANSPOSED, "sources": srcs, "v": v})
    opt = ex.Options(n_sweeps=4, tolerance=-1, factored_radius=2)
    first = [o.copy() for o in ctx.solve3d_batch(models, opt, ex.F32)]
    again = ctx.solve3d_batch(models, opt, ex.F32)
    for m, a, b in zip(models, first, again):
        assert np.array_equal(_bits(a), _bits(b))
        ctx.set_grid3d(*m["grid"])
        ctx.set_nodal_velocity3d(m["model"], ordering=ex.TRANSPOSED)   # same input, same summation order
        single = ctx.solve3d(m["sources"], opt, ex.F32)
        assert np.array_equal(_bits(a), _bits(single))


def test_batch_rejects_bad_models(ctx):
    good = {"grid": (5, 5, 5, 10., 10., 10.), "model": np.full(64, 1 / 3000, np.float32),
            "sources": [(10., 10., 10.)]}
    with pytest.raises(ex.InvalidArgument):
        ctx.solve3d_batch([good, dict(good, sources=[(100., 0., 0.)])])      # source outside its grid
    with pytest.raises(ex.InvalidArgument):
        ctx.solve3d_batch([dict(good, grid=(2, 5, 5, 10., 10., 10.))])     # too few grid points
    with pytest.raises(ex.InvalidArgument):
        ctx.solve3d_batch([dict(good, model=np.full(64, -1.0, np.float32))])   # non-positive slowness
    out = ctx.solve3d_batch([good])[0]                                       # context still usable
    assert np.isfinite(out).all()


def test_fields_copied_out_as_they_converge_equal_the_device_result(ctx):
    """Host output copies each field (each model, in a batch) at the end of the iteration in
    which it converged, while the others sweep on; the result must equal the device output."""
    import torch
    rng = np.random.default_rng(77)
    shape = (41, 37, 29, 50.0, 50.0, 50.0)
    nx, ny, nz = shape[:3]
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=np.float32)
    ctx.set_grid3d(*shape)
    ctx.set_slowness3d(s)
    src = np.column_stack([rng.uniform(0, (nx - 1) * 50, 6), rng.uniform(0, (ny - 1) * 50, 6),
                           rng.uniform(0, (nz - 1) * 50, 6)])
    opt = ex.Options(n_sweeps=12, tolerance=1e-5)
    host = ctx.solve3d(src, opt, ex.F32)
    st = ctx.stats()
    assert st["iterations_min"] < st["iterations_max"]      # fields converge at different iterations
    dev = torch.empty((6, nz, ny, nx), dtype=torch.float32, device="cuda")
    ctx.solve3d(src, opt, ex.F32, out=dev)
    assert np.array_equal(host.view(np.uint32), dev.cpu().numpy().view(np.uint32))
    # the same per model in a batch: one model with host output, one with device output
    models = []
    for k in range(3):
        g = (33 + 8 * k, 29, 25, 50.0, 50.0, 50.0)
        v = (3000 + 2000 * rng.random((g[2], g[1], g[0]))).astype(np.float32)
        p = [(rng.uniform(0, (g[0] - 1) * 50), rng.uniform(0, (g[1] - 1) * 50), rng.uniform(0, (g[2] - 1) * 50))
             for _ in range(2)]
        models.append({"grid": g, "model": v, "nodal": True, "sources": p})
    outs_host = ctx.solve3d_batch(models, opt, ex.F32)
    dev_models = [dict(m, out=torch.empty((2, m["grid"][2], m["grid"][1], m["grid"][0]), dtype=torch.float32,
                                          device="cuda")) for m in models]
    outs_dev = ctx.solve3d_batch(dev_models, opt, ex.F32)
    for a, b in zip(outs_host, outs_dev):
        assert np.array_equal(a.view(np.uint32), b.cpu().numpy().view(np.uint32))


def test_2d_fields_copied_out_as_they_converge_equal_the_device_result(ctx):
    import torch
    rng = np.random.default_rng(78)
    nx, nz, h = 61, 47, 25.0
    s = random_slowness(rng, (nz - 1) * (nx - 1), dtype=np.float64)
    ctx.set_grid2d(nx, nz, h, h)
    ctx.set_slowness2d(s)
    src = np.column_stack([rng.uniform(0, (nx - 1) * h, 5), rng.uniform(0, (nz - 1) * h, 5)])
    opt = ex.Options(n_sweeps=15, tolerance=1e-9)
    host = ctx.solve2d(src, opt, ex.F64)
    dev = torch.empty((5, nz, nx), dtype=torch.float64, device="cuda")
    ctx.solve2d(src, opt, ex.F64, out=dev)
    assert np.array_equal(host.view(np.uint64), dev.cpu().numpy().view(np.uint64))
