"""The network oracle's backward pass against finite differences of its forward pass
(float64, no BF16 rounding), per layer, on a small grid.  No GPU."""
import numpy as np
import pytest

from oracle import warmnet_oracle as wo

GRID = (16, 16, 8, 50.0, 50.0, 50.0, 0.0, 0.0, 0.0)


def _samples(seed, n=2):
    rng = np.random.default_rng(seed)
    nx, ny, nz = GRID[:3]
    out = []
    for _ in range(n):
        z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        vel = (3000 + 800 * np.sin(0.3 * x + rng.uniform(0, 6)) * np.cos(0.2 * y) + 40 * z).astype(np.float32)
        src = (rng.uniform(0, (nx - 1) * 50), rng.uniform(0, (ny - 1) * 50), rng.uniform(0, (nz - 1) * 50))
        t0 = wo.target(np.zeros(vel.size), vel.ravel(), src, GRID)[2]
        tt = (t0 * (1 + 0.2 * np.sin(0.25 * x + 0.1 * z))).astype(np.float32)
        out.append((vel.ravel(), tt.ravel(), src))
    return out


def _params(seed):
    rng = np.random.default_rng(seed)
    p = wo.init_params(seed)
    offs, head, total = wo.layout()
    for (cin, cout, _), (w, b) in zip(wo.SPEC, offs):
        p[b:b + cout] = rng.normal(0, 0.05, cout)
    p[head:head + 17] = rng.normal(0, 0.3, 17)
    return p


def test_layout_counts_the_documented_parameters():
    assert wo.layout()[2] == 1466065


def test_bf16_rounding_is_round_to_nearest_even():
    vals = np.array([1.0, 1.00390625, 1.005859375, 1.001953125, 1.0029296875, -2.5e-3, 3.0e38], np.float32)
    r = wo.bf16(vals)
    # 1 + 2^-8 is exactly halfway between 1 and 1 + 2^-7: ties to even (1.0)
    assert r[1] == 1.0
    assert r[0] == 1.0 and r[2] == 1.0078125
    assert np.all(np.abs(r - vals) <= np.abs(vals) * 2.0 ** -8 + 1e-45)


@pytest.mark.parametrize("layer", [0, 1, 4, 7, 8, 11, 12, 13])
def test_backward_matches_finite_differences(layer):
    samples = _samples(3)
    p = _params(5)
    loss, grad, _ = wo.loss_and_grads(p, samples, GRID, emulate=False)
    offs, head, total = wo.layout()
    wo_, bo = offs[layer]
    cout = wo.SPEC[layer][1]
    rng = np.random.default_rng(layer)
    d = np.zeros(total)
    d[wo_:bo + cout] = rng.standard_normal(bo + cout - wo_)
    if layer == 0:
        # only the six data-carrying input channels reach the loss
        w = d[wo_:bo].reshape(27, cout, 16)
        w[:, :, 6:] = 0
    # a small step: larger ones move a few pre-activations across the ReLU kink
    eps = 1e-8
    lp = wo.loss_and_grads(p + eps * d, samples, GRID, emulate=False)[0]
    lm = wo.loss_and_grads(p - eps * d, samples, GRID, emulate=False)[0]
    fd = (lp - lm) / (2 * eps)
    an = float(grad @ d)
    assert abs(fd - an) <= 1e-6 * abs(an) + 1e-9, (layer, fd, an)


def test_head_gradient_matches_finite_differences():
    samples = _samples(4, n=1)
    p = _params(6)
    loss, grad, _ = wo.loss_and_grads(p, samples, GRID, emulate=False)
    offs, head, total = wo.layout()
    for k in (head, head + 7, head + 16):
        e = np.zeros(total)
        e[k] = 1e-8
        fd = (wo.loss_and_grads(p + e, samples, GRID, emulate=False)[0] -
              wo.loss_and_grads(p - e, samples, GRID, emulate=False)[0]) / 2e-8
        assert abs(fd - grad[k]) <= 1e-6 * abs(grad[k]) + 1e-9, (k, fd, grad[k])


def test_untrained_prediction_is_the_homogeneous_field():
    samples = _samples(7, n=1)
    p = wo.init_params(1)   # zero head: tau = 1
    t = wo.predict(p, samples, GRID)[0]
    t0 = wo.target(np.zeros(16 * 16 * 8), samples[0][0], samples[0][2], GRID)[2]
    np.testing.assert_array_equal(t, t0)


def test_straight_ray_contrast_of_a_constant_model_is_zero_and_of_a_gradient_is_its_mean():
    nx, ny, nz = GRID[:3]
    vel = np.full(nx * ny * nz, 2500.0, np.float32)
    src = (100.0, 200.0, 50.0)
    s_src = wo.source_slowness(vel, src, GRID)
    np.testing.assert_array_equal(wo.straight_ray_contrast(vel, src, GRID, s_src), 0.0)
    # slowness linear in x: the mean over a segment is the value at its midpoint
    x = np.tile(np.arange(nx), ny * nz)
    vel = (1.0 / (4e-4 + 1e-5 * x)).astype(np.float32)
    src = (0.0, 0.0, 0.0)
    s_src = wo.source_slowness(vel, src, GRID)
    r = wo.straight_ray_contrast(vel, src, GRID, s_src).reshape(nz, ny, nx)
    mid = (4e-4 + 1e-5 * np.arange(nx) / 2) / s_src - 1
    np.testing.assert_allclose(r[3, 5, :], mid, rtol=0, atol=1e-5)
