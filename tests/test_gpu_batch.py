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
