"""Learned warm start: the travel-time predictor, its training data and its trainer.

No counterpart in the reference.  The predictor is the 3D U-Net behind the C entry
points eikx_warmnet_* (include/eikx/eikx_c.h): its forward and backward passes, the
loss and Adam run in the library's own CUDA kernels (BF16 tensor-core convolutions with
FP32 accumulation); this module only arranges the calls.

    net = WarmNet(grid, batch=4, seed=0)
    data = generate_fields(ctx, grid, n_models=64, sources_per_model=8, seed=1)
    history = train(net, data, steps=500, lr=1e-3, seed=2)
    t_init, _ = net.predict(samples_of(data, idx), inflate=1.05)
    t = ctx.solve3d_warm(sources, t_init, options)

A sample is (velocity, travel_time or None, (x, y, z)) with velocity and travel_time
contiguous float32 CUDA tensors of nx*ny*nz nodes in natural order.
"""
import ctypes
import math

import numpy as np

from . import DEVICE, F32, HOST, Options, _check, _NetConfig, _NetSample, load
from . import synthetic


class WarmNet:
    """The travel-time predictor on one GPU (eikx_warmnet)."""

    def __init__(self, grid, batch, seed=0, device=0):
        nx, ny, nz, dx, dy, dz = grid[:6]
        x0, y0, z0 = tuple(grid[6:9]) if len(grid) >= 9 else (0.0, 0.0, 0.0)
        self._lib = load()
        cfg = _NetConfig(int(nx), int(ny), int(nz), float(dx), float(dy), float(dz), float(x0), float(y0),
                         float(z0), int(batch), int(seed))
        h = ctypes.c_void_p()
        _check(self._lib.eikx_warmnet_create(int(device), ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.grid = (int(nx), int(ny), int(nz), float(dx), float(dy), float(dz), float(x0), float(y0), float(z0))
        self.batch = int(batch)
        n = ctypes.c_longlong()
        _check(self._lib.eikx_warmnet_num_params(self._h, ctypes.byref(n)))
        self.num_params = n.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.eikx_warmnet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def get_params(self):
        p = np.empty(self.num_params, np.float32)
        _check(self._lib.eikx_warmnet_get_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters, got {p.size}")
        _check(self._lib.eikx_warmnet_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def _samples(self, samples):
        nodes = self.grid[0] * self.grid[1] * self.grid[2]
        arr = (_NetSample * len(samples))()
        for i, (vel, tt, src) in enumerate(samples):
            for t in (vel, tt):
                if t is None:
                    continue
                if not (getattr(t, "is_cuda", False) and t.is_contiguous() and str(t.dtype) == "torch.float32"):
                    raise ValueError("velocity and travel_time must be contiguous float32 CUDA tensors")
                if t.numel() != nodes:
                    raise ValueError(f"expected {nodes} nodes, got {t.numel()}")
            arr[i] = _NetSample(vel.data_ptr(), tt.data_ptr() if tt is not None else None, *map(float, src))
        return arr, len(samples)

    def train_step(self, samples, lr):
        """One Adam step; returns the loss before it."""
        arr, n = self._samples(samples)
        loss = ctypes.c_double()
        _check(self._lib.eikx_warmnet_train_step(self._h, arr, n, ctypes.c_float(lr), ctypes.byref(loss)))
        return loss.value

    def gradients(self, samples):
        """(gradient of the loss w.r.t. the parameter vector, loss), without a step."""
        arr, n = self._samples(samples)
        g = np.empty(self.num_params, np.float32)
        loss = ctypes.c_double()
        _check(self._lib.eikx_warmnet_gradients(self._h, arr, n, g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                ctypes.byref(loss)))
        return g, loss.value

    def predict(self, samples, inflate=1.0, out=None):
        """(predicted travel times T0 (1 + tau) * inflate, loss or None).  `out`: a float32
        CUDA tensor or numpy array of len(samples) * nodes values (default: numpy)."""
        arr, n = self._samples(samples)
        nx, ny, nz = self.grid[:3]
        if out is None:
            out = np.empty((n, nz, ny, nx), np.float32)
        if isinstance(out, np.ndarray):
            p, where = ctypes.c_void_p(out.ctypes.data), HOST
        else:
            p, where = ctypes.c_void_p(out.data_ptr()), (DEVICE if out.is_cuda else HOST)
        loss = ctypes.c_double()
        _check(self._lib.eikx_warmnet_predict(self._h, arr, n, float(inflate), p, where, ctypes.byref(loss)))
        return out, (loss.value if loss.value >= 0 else None)

    def set_test_hooks(self, spin_limit_log2=0, late=0):
        """Test hook of the tensor-core convolutions' bounded waits (see
        eikx_warmnet_set_test_hooks); (0, 0) restores production behaviour."""
        _check(self._lib.eikx_warmnet_set_test_hooks(self._h, int(spin_limit_log2), int(late)))

    def profile_step(self, samples, lr):
        """One training step timed per kernel class: dict of ms and algorithmic FLOPs."""
        arr, n = self._samples(samples)
        ms = (ctypes.c_double * 4)()
        fl = (ctypes.c_double * 3)()
        _check(self._lib.eikx_warmnet_profile_step(self._h, arr, n, ctypes.c_float(lr), ms, fl))
        return {"ms": {"forward_conv": ms[0], "input_grad_conv": ms[1], "weight_grad": ms[2], "other": ms[3]},
                "flops": {"forward_conv": fl[0], "input_grad_conv": fl[1], "weight_grad": fl[2]}}


def random_smooth_model(nx, ny, nz, h, rng, vmin=1500.0, vmax=8000.0, corr_m=(500.0, 3000.0)):
    """Nodal velocities (nz, ny, nx) of a random smooth model: a Gaussian random field
    with a correlation length uniform in `corr_m`, around a mean velocity uniform in
    [vmin, vmax] with a relative amplitude uniform in [0.1, 0.5], clipped to [vmin, vmax]."""
    corr = rng.uniform(*corr_m)
    mean = rng.uniform(vmin, vmax)
    amp = rng.uniform(0.1, 0.5)
    p = synthetic.grf((nz, ny, nx), h, corr, rng)
    return np.clip(mean * (1.0 + amp * p), vmin, vmax).astype(np.float32)


def generate_fields(ctx, grid, n_models, sources_per_model, seed, options=None, device="cuda"):
    """Training data made by the solver: n_models random smooth models, each solved
    (cold start, FP32) for `sources_per_model` seeded sources uniform in the domain.
    Returns a dict of CUDA tensors ``velocity`` (n_models, nodes) and ``travel_time``
    (n_fields, nodes), ``sources`` (n_fields, 3) and ``model`` (n_fields,) indices."""
    import torch

    nx, ny, nz, h = grid[0], grid[1], grid[2], grid[3]
    rng = np.random.default_rng(seed)
    nodes = nx * ny * nz
    vel = torch.empty((n_models, nodes), dtype=torch.float32, device=device)
    tt = torch.empty((n_models * sources_per_model, nodes), dtype=torch.float32, device=device)
    srcs = np.empty((n_models * sources_per_model, 3))
    model = np.repeat(np.arange(n_models), sources_per_model)
    ctx.set_grid3d(nx, ny, nz, h, h, h)
    for m in range(n_models):
        v = random_smooth_model(nx, ny, nz, h, rng)
        vel[m].copy_(torch.from_numpy(v.ravel()))
        ctx.set_nodal_velocity3d(vel[m])
        s = synthetic.uniform_sources(sources_per_model, nx, ny, nz, h, int(rng.integers(1 << 31)))
        k = m * sources_per_model
        ctx.solve3d(s, options or Options(n_sweeps=20, tolerance=1e-5), F32,
                    out=tt[k:k + sources_per_model].view(sources_per_model, nz, ny, nx))
        srcs[k:k + sources_per_model] = s
    torch.cuda.synchronize()
    return {"velocity": vel, "travel_time": tt, "sources": srcs, "model": model}


def samples_of(data, idx, with_target=True):
    """Samples of the fields `idx` of `generate_fields` output."""
    return [(data["velocity"][int(data["model"][i])], data["travel_time"][i] if with_target else None,
             tuple(data["sources"][i])) for i in idx]


def learning_rate(k, steps, lr, warmup_frac=0.05, lr_min_frac=0.05):
    """Linear warm-up over the first `warmup_frac` of the steps, then cosine decay to
    lr * lr_min_frac."""
    w = max(1, int(warmup_frac * steps))
    if k < w:
        return lr * (k + 1) / w
    f = (k - w) / max(1, steps - w)
    return lr * (lr_min_frac + (1 - lr_min_frac) * 0.5 * (1 + math.cos(math.pi * f)))


def train(net, data, steps, lr=1e-3, seed=0, fields=None, log_every=0):
    """Adam on random minibatches of `net.batch` fields (from `fields`, default all) with
    the `learning_rate` schedule; returns the per-step losses."""
    rng = np.random.default_rng(seed)
    pool = np.arange(data["travel_time"].shape[0]) if fields is None else np.asarray(fields)
    losses = []
    for k in range(steps):
        idx = rng.choice(pool, size=min(net.batch, pool.size), replace=False)
        r = learning_rate(k, steps, lr)
        losses.append(net.train_step(samples_of(data, idx), r))
        if log_every and (k % log_every == 0 or k == steps - 1):
            print(f"step {k}: loss {losses[-1]:.4e} lr {r:.2e}", flush=True)
    return losses


def evaluate_loss(net, data, fields):
    """Mean loss of the network over `fields` (batches of net.batch fields)."""
    tot, n = 0.0, 0
    for i in range(0, len(fields), net.batch):
        idx = list(fields[i:i + net.batch])
        _, loss = net.predict(samples_of(data, idx))
        tot += loss * len(idx)
        n += len(idx)
    return tot / max(1, n)
