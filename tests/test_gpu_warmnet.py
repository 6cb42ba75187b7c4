"""The learned warm start's network on the GPU: its forward pass and gradients against
the CPU oracle, training on solver-generated fields, and what its prediction gains as
the starting field of a warm-started solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import eikonalxx_gb300 as ex                       # noqa: E402
from eikonalxx_gb300 import warmstart as ws        # noqa: E402
from oracle import warmnet_oracle as wo            # noqa: E402

GRID = (16, 16, 8, 50.0, 50.0, 50.0, 0.0, 0.0, 0.0)
# x extent 128: the first level's convolutions run on the tcgen05 path
GRID128 = (128, 8, 8, 50.0, 50.0, 50.0, 0.0, 0.0, 0.0)


def _host_samples(seed, n=2, grid=GRID):
    rng = np.random.default_rng(seed)
    nx, ny, nz = grid[:3]
    out = []
    for _ in range(n):
        z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        vel = (3000 + 800 * np.sin(0.3 * x + rng.uniform(0, 6)) * np.cos(0.2 * y) + 40 * z).astype(np.float32)
        src = (rng.uniform(0, (nx - 1) * 50), rng.uniform(0, (ny - 1) * 50), rng.uniform(0, (nz - 1) * 50))
        t0 = wo.target(np.zeros(vel.size), vel.ravel(), src, grid)[2]
        tt = (t0 * (1 + 0.2 * np.sin(0.25 * x + 0.1 * z))).astype(np.float32)
        out.append((vel.ravel(), tt.ravel(), src))
    return out


def _device(samples):
    return [(torch.from_numpy(v).cuda(), torch.from_numpy(t).cuda() if t is not None else None, s)
            for v, t, s in samples]


def _params(seed):
    rng = np.random.default_rng(seed)
    p = wo.init_params(seed)
    offs, head, total = wo.layout()
    for (cin, cout, _), (w, b) in zip(wo.SPEC, offs):
        p[b:b + cout] = rng.normal(0, 0.05, cout)
    p[head:head + 17] = rng.normal(0, 0.3, 17)
    return p.astype(np.float32)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("n,grid", [(1, GRID), (2, GRID), (2, GRID128)])
def test_gradients_match_the_oracle(n, grid):
    host = _host_samples(11, n, grid)
    p = _params(5)
    with ws.WarmNet(grid, batch=2, seed=0) as net:
        assert net.num_params == wo.layout()[2]
        net.set_params(p)
        np.testing.assert_array_equal(net.get_params(), p)
        g, loss = net.gradients(_device(host))
    oloss, og, _ = wo.loss_and_grads(p, host, grid, emulate=True)
    f64 = wo.loss_and_grads(p, host, grid, emulate=False)[1]
    assert abs(loss - oloss) <= 1e-3 * oloss
    offs, head, _ = wo.layout()
    rows, bad = [], []
    for L, ((cin, cout, _), (w, b)) in enumerate(zip(wo.SPEC, offs)):
        for name, sl in ((wo.NAMES[L], slice(w, b)), (wo.NAMES[L] + ".b", slice(b, b + cout))):
            # the GPU against the oracle's BF16 emulation, and that emulation's own distance
            # from exact FP64 arithmetic: the BF16 rounding noise at this depth
            # the GPU (BF16 storage, FP32 accumulation) must be about as close to exact FP64
            # arithmetic as the oracle's BF16 emulation is: the rounding noise at this depth
            e, e64, noise = _rel(g[sl], og[sl]), _rel(g[sl], f64[sl]), _rel(og[sl], f64[sl])
            cos = float(g[sl] @ og[sl] / (np.linalg.norm(g[sl]) * np.linalg.norm(og[sl]) + 1e-30))
            rows.append(f"{name:6s} gpu-vs-oracle {e:.2e}  gpu-vs-fp64 {e64:.2e}  oracle-vs-fp64 {noise:.2e}  "
                        f"cos {cos:.6f}")
            if not (e64 < max(2e-2, 2 * noise) and cos > 0.99):
                bad.append(rows[-1])
    print("\n" + "\n".join(rows))
    assert not bad, bad
    assert _rel(g[head:], og[head:]) < 1e-3
    # the zero-padded input channels of the first convolution get no gradient
    assert not np.any(g[:27 * 16 * 16].reshape(27, 16, 16)[:, :, 6:])


@pytest.mark.parametrize("grid", [GRID, GRID128])
def test_prediction_matches_the_oracle(grid):
    host = _host_samples(12, 2, grid)
    p = _params(8)
    with ws.WarmNet(grid, batch=2, seed=0) as net:
        net.set_params(p)
        t, loss = net.predict(_device(host), inflate=1.03)
        td = torch.empty(2 * grid[0] * grid[1] * grid[2], dtype=torch.float32, device="cuda")
        net.predict(_device([(v, None, s) for v, _, s in host]), inflate=1.03, out=td)
    ot = wo.predict(p, host, grid, inflate=1.03)
    assert np.max(np.abs(t - ot)) <= 2e-3 * np.max(np.abs(ot))
    np.testing.assert_array_equal(td.cpu().numpy().reshape(t.shape), t)
    oloss = wo.loss_and_grads(p, host, grid)[0]
    assert abs(loss - oloss) <= 1e-2 * oloss


@pytest.mark.parametrize("late", [1, 2])
def test_tensor_core_wait_timeout_drains_and_recovers(late):
    """Failure detection of the tcgen05 convolutions without a GPU fault: the test hook
    makes the first input chunk's wait run out while its copies (late = 1) or MMAs
    (late = 2) still complete; the kernel drains them before it frees TMEM, the call
    returns EIKX_ERR_TIMEOUT, and the next call on the same network is correct: the
    forward pass exactly, the gradients to the order of their FP32 atomic sums."""
    host = _host_samples(14, 2, GRID128)
    p = _params(10)
    with ws.WarmNet(GRID128, batch=2, seed=0) as net:
        net.set_params(p)
        t_ref, _ = net.predict(_device(host), inflate=1.0)
        g_ref, _ = net.gradients(_device(host))
        net.set_test_hooks(spin_limit_log2=10, late=late)
        with pytest.raises(ex.TimeoutError_):
            net.predict(_device(host), inflate=1.0)
        with pytest.raises(ex.TimeoutError_):
            net.gradients(_device(host))
        net.set_test_hooks(0, 0)
        t, _ = net.predict(_device(host), inflate=1.0)
        g, _ = net.gradients(_device(host))
    np.testing.assert_array_equal(t, t_ref)
    assert _rel(g, g_ref) < 1e-5          # weight gradients sum with FP32 atomics, in any order


@pytest.mark.parametrize("grid", [GRID, GRID128])
def test_a_step_moves_against_the_gradient(grid):
    host = _device(_host_samples(13, 2, grid))
    with ws.WarmNet(grid, batch=2, seed=3) as net:
        net.set_params(_params(9))
        l0 = net.train_step(host, 1e-4)
        l1 = net.train_step(host, 1e-4)
        _, l2 = net.predict(host)
    assert l1 < l0 and l2 < l1


def test_invalid_arguments():
    with pytest.raises(ex.InvalidArgument):
        ws.WarmNet((20, 16, 8, 50.0, 50.0, 50.0), batch=1)
    with pytest.raises(ex.InvalidArgument):
        ws.WarmNet(GRID, batch=0)
    with pytest.raises(ex.InvalidArgument):
        ws.WarmNet(tuple(GRID[:3]) + (float("inf"), 50.0, 50.0), batch=1)
    with pytest.raises(ex.InvalidArgument):
        ws.WarmNet(tuple(GRID[:6]) + (0.0, float("nan"), 0.0), batch=1)
    host = _device(_host_samples(14, 2))
    with ws.WarmNet(GRID, batch=1) as net:
        with pytest.raises(ex.InvalidArgument):
            net.train_step(host, 1e-3)            # more samples than the batch
        with pytest.raises(ex.InvalidArgument):
            net.predict(host[:1], inflate=0.0)
        with pytest.raises(ex.InvalidArgument):
            net.train_step(host[:1], float("nan"))
        bad = net.get_params()
        bad[3] = np.nan
        with pytest.raises(ex.InvalidArgument):
            net.set_params(bad)
        with pytest.raises(ex.InvalidArgument):
            net.gradients([(host[0][0], None, host[0][2])])   # training needs a travel-time field


def test_profile_step_reports_every_kernel_class():
    host = _device(_host_samples(15, 2))
    with ws.WarmNet(GRID, batch=2) as net:
        r = net.profile_step(host, 1e-4)
    assert all(v > 0 for v in r["ms"].values())
    f = r["flops"]
    assert f["forward_conv"] == f["weight_grad"] > f["input_grad_conv"] > 0


LGRID = (64, 64, 32, 100.0, 100.0, 100.0)


@pytest.fixture(scope="module")
def trained():
    """A network trained on solver fields of random smooth models (64x64x32, h=100 m)."""
    ctx = ex.Context(0)
    data = ws.generate_fields(ctx, LGRID, n_models=10, sources_per_model=6, seed=21)
    n = data["travel_time"].shape[0]
    train_idx, test_idx = np.arange(0, n - 6), np.arange(n - 6, n)
    net = ws.WarmNet(LGRID, batch=6, seed=4)
    zero = np.zeros(net.num_params, np.float32)
    trained_p = net.get_params()
    net.set_params(zero)
    base = ws.evaluate_loss(net, data, test_idx)
    net.set_params(trained_p)
    losses = ws.train(net, data, steps=600, lr=1e-3, seed=5, fields=train_idx)
    yield {"ctx": ctx, "data": data, "net": net, "test": test_idx, "base": base, "losses": losses}
    net.close()
    ctx.close()


def _straight_ray_loss(data, fields):
    """Loss of the straight-ray estimate alone (input feature 5 as the prediction)."""
    tot = 0.0
    for i in fields:
        vel = data["velocity"][int(data["model"][i])].cpu().numpy()
        src = tuple(data["sources"][i])
        g = LGRID[:3] + (LGRID[3],) * 3 + (0.0, 0.0, 0.0)
        tgt, w, _ = wo.target(data["travel_time"][i].cpu().numpy(), vel, src, g)
        ray = wo.straight_ray_contrast(vel, src, g, np.float32(wo.source_slowness(vel, src, g)))
        tot += float((((ray - tgt) * w) ** 2).sum() / w.sum())
    return tot / len(fields)


def test_training_lowers_the_loss(trained):
    l = trained["losses"]
    first, last = np.mean(l[:20]), np.mean(l[-20:])
    held_out = ws.evaluate_loss(trained["net"], trained["data"], trained["test"])
    ray = _straight_ray_loss(trained["data"], trained["test"])
    print(f"\ntraining loss {first:.4e} -> {last:.4e}; held-out {held_out:.4e}; "
          f"tau = 1: {trained['base']:.4e}; straight ray: {ray:.4e}")
    assert last < 0.5 * first
    assert held_out < 0.5 * trained["base"]


def test_warm_start_from_the_prediction(trained):
    """What the trained network gains as a starting field, against the start without it
    (the untrained network, T = T0) and the cold start: how close the start is to the
    cold-start result, the refinement iterations, and where the warm solve settles."""
    ctx, data, net = trained["ctx"], trained["data"], trained["net"]
    idx = trained["test"]
    nx, ny, nz, h = LGRID[:4]
    m = int(data["model"][idx[0]])
    same = [i for i in idx if int(data["model"][i]) == m]
    ctx.set_grid3d(nx, ny, nz, h, h, h)
    ctx.set_nodal_velocity3d(data["velocity"][m])
    src = data["sources"][same]
    opt = ex.Options(n_sweeps=20, tolerance=1e-5)
    cold = ctx.solve3d(src, opt, ex.F32)
    it_cold = ctx.stats()["iterations_max"]
    rows = {}
    p_trained = net.get_params()
    for name, params in (("T0", np.zeros_like(p_trained)), ("network", p_trained)):
        net.set_params(params)
        start, _ = net.predict(ws.samples_of(data, same, with_target=False), inflate=1.0)
        err = start.astype(np.float64) - cold
        init, _ = net.predict(ws.samples_of(data, same, with_target=False), inflate=1.02)
        out = ctx.solve3d_warm(src, init, opt, ex.F32, gate_tol=1e-6)
        st = ctx.stats()
        rows[name] = {"start_rms_s": float(np.sqrt(np.mean(err ** 2))), "iterations": st["iterations_max"],
                      "max_dev_s": float(np.max(np.abs(out - cold))), "reset": st["reset_nodes"]}
    net.set_params(p_trained)
    print(f"\ncold: {it_cold} iterations; warm starts: {rows}")
    assert rows["network"]["start_rms_s"] < 0.5 * rows["T0"]["start_rms_s"]
    assert rows["network"]["iterations"] <= opt.n_sweeps
