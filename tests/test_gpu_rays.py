"""2D gradient ray tracing on the GPU (eikx_trace_rays2d) against the oracle's restatement of
Ray::GradientTracer2D::trace (src/ray/gradientTracer2d.cpp:339-600), bit for bit: segment
counts, end points and slownesses, for analytic and solved gradient fields, FP32 and FP64."""
import os

import numpy as np
import pytest

from test_oracle_rays import DEFAULT_RADII, DEFAULT_SCALES, homogeneous_case, path_stats

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402


def _compare(oracle, ctx, grad, grid, origin, slow, source, stations, radius_scale=None, max_steps=0, capacity=None):
    nx, nz = grid[:2]
    cap = capacity or 4 * (nx + nz) + 16
    radii = [r for r, _ in radius_scale] if radius_scale else DEFAULT_RADII
    scales = [s for _, s in radius_scale] if radius_scale else DEFAULT_SCALES
    if radii[-1] < 2 ** 31 - 1:
        radii, scales = radii + [2 ** 31 - 1], scales + [scales[-1]]
    steps = max_steps or int(np.ceil(4.0 * (nx + nz) / min(scales))) + 16
    paths, counts = ctx.trace_rays2d(grad, slow, source, stations, radius_scale=radius_scale, max_steps=max_steps,
                                     capacity=cap, grid=grid + tuple(origin))
    seg, ocounts = oracle.trace_rays2d(grad, grid, origin, slow, source, stations, radii, scales, steps, cap)
    assert np.array_equal(counts, ocounts), (counts, ocounts)
    for i, p in enumerate(paths):
        if counts[i] > 0:
            assert np.array_equal(p.view(np.uint64), seg[i, :counts[i]].view(np.uint64)), i
    return paths, counts


def test_homogeneous_case_of_the_reference(ctx, oracle):
    c = homogeneous_case()
    paths, counts = _compare(oracle, ctx, c["grad"], c["grid"], c["origin"], c["slow"], c["source"], c["stations"])
    assert (counts > 0).all()
    xs, zs = c["source"]
    for (x, z), p in zip(c["stations"], paths):
        length, t = path_stats(p)
        d = np.hypot(x - xs, z - zs)
        assert abs(length - d) < 1.0 and abs(t - d / c["v"]) < 1e-3


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
def test_rays_through_a_solved_linear_gradient(ctx, oracle, precision):
    """Gradient of a 2D solve (eikx_gradient2d) in a v(z) = 3000 + 0.5 z model."""
    nx, nz, h = 161, 81, 25.0
    v = (3000.0 + 0.5 * np.arange(nz) * h)[:, None] * np.ones((1, nx))
    ctx.set_grid2d(nx, nz, h, h)
    ctx.set_nodal_velocity2d(np.ascontiguousarray(v, dtype=np.float64))
    src = (1512.5, 640.0)
    opt = ex.Options(n_sweeps=3, tolerance=-1, factored_radius=3)
    ctx.solve2d([src], opt, precision)
    grad = ctx.gradient2d(precision=precision)
    slow = np.ascontiguousarray(4.0 / (v[:-1, :-1] + v[:-1, 1:] + v[1:, :-1] + v[1:, 1:]), dtype=np.float64)
    rng = np.random.default_rng(3)
    stations = [(float(rng.uniform(0, (nx - 1) * h)), 0.0) for _ in range(20)]
    stations += [(float(rng.uniform(0, (nx - 1) * h)), float(rng.uniform(0, (nz - 1) * h))) for _ in range(20)]
    paths, counts = _compare(oracle, ctx, grad, (nx, nz, h, h), (0.0, 0.0), slow, src, stations)
    assert (counts > 0).mean() > 0.9, counts


def test_custom_steps_and_bounds(ctx, oracle):
    c = homogeneous_case()
    rs = [(0, 0.02), (4, 0.1), (10, 0.25)]
    _compare(oracle, ctx, c["grad"], c["grid"], c["origin"], c["slow"], c["source"], c["stations"], radius_scale=rs)
    _, counts = _compare(oracle, ctx, c["grad"], c["grid"], c["origin"], c["slow"], c["source"], c["stations"][1:3],
                         max_steps=10)
    assert (counts == -1).all()
    _, counts = _compare(oracle, ctx, c["grad"], c["grid"], c["origin"], c["slow"], c["source"], c["stations"][1:3],
                         capacity=3)
    assert (counts == -2).all()


@pytest.mark.parametrize("rs, message", [
    ([], "empty"),
    ([(-1, 0.1)], "non-negative"),
    ([(1, 1.0)], "less than 1"),
    ([(1, 0.0)], "non-negative"),
    ([(2, 0.1), (2, 0.2)], "Duplicate"),
])
def test_invalid_step_rules(ctx, rs, message):
    c = homogeneous_case()
    with pytest.raises(ex.InvalidArgument, match=message):
        ctx.trace_rays2d(c["grad"], c["slow"], c["source"], c["stations"][:2], radius_scale=rs,
                         grid=c["grid"] + c["origin"])


def test_stations_outside_the_grid(ctx):
    c = homogeneous_case()
    with pytest.raises(ex.InvalidArgument, match="outside the grid"):
        ctx.trace_rays2d(c["grad"], c["slow"], c["source"], [(-50.0, 10.0)], grid=c["grid"] + c["origin"])


def test_cpp_gradient_tracer(ctx, tmp_path):
    """GradientTracer2D of the C++ API on the GPU: the reference's homogeneous case through an
    analytic gradient, and rays through a solved field whose travel times match the field."""
    import subprocess
    from test_ray_api import build_ray_api
    r = subprocess.run([build_ray_api(tmp_path), "gpu"], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, RAY_VTK_DIR=str(tmp_path)))
    assert r.returncode == 0 and "ray_api ok" in r.stdout, r.stdout + r.stderr
