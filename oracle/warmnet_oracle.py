"""CPU oracle of the learned warm start's network (test infrastructure only).

A numpy restatement of the travel-time predictor behind eikx_warmnet_*
(include/eikx/eikx_c.h): features, the 3D U-Net's forward pass, the loss, and the
backward pass written out by hand.  It exists to check the GPU kernels' outputs and
gradients; nothing in the product calls it.  The reference has no learned component,
so nothing in the reference pins this oracle; its backward pass is pinned against
finite differences of its own forward pass in float64 (tests/test_oracle_warmnet.py).

With ``emulate=True`` it rounds to BF16 where the GPU path stores BF16 (convolution
weights, features, every activation and activation gradient) and keeps FP32/FP64
elsewhere, computing in float64; the GPU accumulates in FP32 in another order, so the
two agree to a tolerance, not bit for bit.
"""
import numpy as np

# (input channels, output channels, level) of E0a, E0b, E1a, E1b, E2a, E2b, Ba, Bb,
# D2a, D2b, D1a, D1b, D0a, D0b
SPEC = [(16, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (64, 128, 3),
        (128, 128, 3), (192, 64, 2), (64, 64, 2), (96, 32, 1), (32, 32, 1), (48, 16, 0), (16, 16, 0)]
NAMES = ["E0a", "E0b", "E1a", "E1b", "E2a", "E2b", "Ba", "Bb", "D2a", "D2b", "D1a", "D1b", "D0a", "D0b"]


def layout():
    """Offsets of (weights, biases) per layer and of the head in the parameter vector."""
    off, out = 0, []
    for cin, cout, _ in SPEC:
        w = off
        off += 27 * cin * cout
        out.append((w, off))
        off += cout
    return out, off, off + 17


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def _identity(a):
    return np.asarray(a, dtype=np.float64)


def unpack(params, emulate):
    """Per-layer (w [27][out][in], b [out]) and the head (w [16], b)."""
    params = np.asarray(params, dtype=np.float64)
    offs, head, _ = layout()
    rnd = bf16 if emulate else _identity
    layers = []
    for (cin, cout, _), (wo, bo) in zip(SPEC, offs):
        layers.append((rnd(params[wo:bo].reshape(27, cout, cin)), params[bo:bo + cout]))
    return layers, params[head:head + 16], params[head + 16]


def source_slowness(vel, src, g):
    """1/v (FP32) at the node nearest the source."""
    nx, ny, nz, dx, dy, dz, x0, y0, z0 = g
    ix = int(min(nx - 1, max(0, np.rint((src[0] - x0) / dx))))
    iy = int(min(ny - 1, max(0, np.rint((src[1] - y0) / dy))))
    iz = int(min(nz - 1, max(0, np.rint((src[2] - z0) / dz))))
    return np.float32(1) / np.float32(vel.reshape(nz, ny, nx)[iz, iy, ix])


def geometry_terms(src, g):
    """Per node (nz, ny, nx), FP32: the offsets from the source (FP64 differences rounded to
    FP32) and the distance."""
    nx, ny, nz, dx, dy, dz, x0, y0, z0 = g
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ddx = ((x0 + x * dx) - src[0]).astype(np.float32)
    ddy = ((y0 + y * dy) - src[1]).astype(np.float32)
    ddz = ((z0 + z * dz) - src[2]).astype(np.float32)
    return ddx, ddy, ddz, np.sqrt(ddx * ddx + ddy * ddy + ddz * ddz)


RAY_SAMPLES = 32


def straight_ray_contrast(vel, src, g, s_src):
    """Mean of s/s_src - 1 at RAY_SAMPLES midpoints of the segment from the source to
    each node, s trilinear in the nodal 1/v; float32 in the kernel's operation order."""
    nx, ny, nz, dx, dy, dz, x0, y0, z0 = g
    f32 = np.float32
    sl = (f32(1.0) / np.asarray(vel, dtype=f32)).reshape(nz, ny, nx)
    sx, sy, sz = f32((src[0] - x0) / dx), f32((src[1] - y0) / dy), f32((src[2] - z0) / dz)
    z, y, x = np.meshgrid(np.arange(nz, dtype=f32), np.arange(ny, dtype=f32), np.arange(nx, dtype=f32),
                          indexing="ij")
    ex, ey, ez = x - sx, y - sy, z - sz
    acc = np.zeros((nz, ny, nx), f32)
    ss = f32(s_src)
    for k in range(RAY_SAMPLES):
        t = (f32(k) + f32(0.5)) / f32(RAY_SAMPLES)
        px = np.minimum(np.maximum(sx + t * ex, f32(0)), f32(nx - 1))
        py = np.minimum(np.maximum(sy + t * ey, f32(0)), f32(ny - 1))
        pz = np.minimum(np.maximum(sz + t * ez, f32(0)), f32(nz - 1))
        ix = np.minimum(np.floor(px).astype(np.int64), nx - 2)
        iy = np.minimum(np.floor(py).astype(np.int64), ny - 2)
        iz = np.minimum(np.floor(pz).astype(np.int64), nz - 2)
        fx, fy, fz = px - ix.astype(f32), py - iy.astype(f32), pz - iz.astype(f32)
        c00 = sl[iz, iy, ix] + fx * (sl[iz, iy, ix + 1] - sl[iz, iy, ix])
        c10 = sl[iz, iy + 1, ix] + fx * (sl[iz, iy + 1, ix + 1] - sl[iz, iy + 1, ix])
        c01 = sl[iz + 1, iy, ix] + fx * (sl[iz + 1, iy, ix + 1] - sl[iz + 1, iy, ix])
        c11 = sl[iz + 1, iy + 1, ix] + fx * (sl[iz + 1, iy + 1, ix + 1] - sl[iz + 1, iy + 1, ix])
        c0 = c00 + fy * (c10 - c00)
        c1 = c01 + fy * (c11 - c01)
        c = c0 + fz * (c1 - c0)
        acc = acc + (c / ss - f32(1))
    return acc / f32(RAY_SAMPLES)


def features(vel, src, g, emulate=True):
    nx, ny, nz = g[:3]
    lx, ly, lz = (nx - 1) * g[3], (ny - 1) * g[4], (nz - 1) * g[5]
    inv_l = 1.0 / np.sqrt(lx * lx + ly * ly + lz * lz)
    s_src = source_slowness(vel, src, g)
    ddx, ddy, ddz, dist = geometry_terms(src, g)
    f32 = np.float32
    sl = f32(1) / np.asarray(vel, dtype=f32).reshape(nz, ny, nx)
    il = f32(inv_l)
    cols = [sl / s_src - f32(1), dist * il, ddx * il, ddy * il, ddz * il,
            straight_ray_contrast(vel, src, g, s_src)]
    f = np.zeros((nz, ny, nx, 16))
    for k, c in enumerate(cols):
        f[..., k] = bf16(c) if emulate else c.astype(np.float64)
    return f


def target(tt, vel, src, g):
    """(tau - 1, weight, T0): the regression target, 1 where T0 > 0, and T0, all FP32
    (returned as float64)."""
    nx, ny, nz = g[:3]
    t0 = source_slowness(vel, src, g) * geometry_terms(src, g)[3]
    t = np.asarray(tt, dtype=np.float32).reshape(nz, ny, nx)
    pos = t0 > 0
    tau = np.where(pos, t / np.where(pos, t0, np.float32(1)) - np.float32(1), np.float32(0))
    return tau.astype(np.float64), pos.astype(np.float64), t0.astype(np.float64)


def conv(x, w, b):
    """x [B, D, H, W, in], w [27][out][in] -> [B, D, H, W, out] (zero padding), float64."""
    B, D, H, W, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((B, D, H, W, w.shape[1]))
    for t in range(27):
        dz, dy, dx = t // 9, (t // 3) % 3, t % 3
        y += xp[:, dz:dz + D, dy:dy + H, dx:dx + W, :] @ w[t].T
    if b is not None:
        y += b
    return y


def conv_input_grad(dy, w):
    B, D, H, W, _ = dy.shape
    dxp = np.zeros((B, D + 2, H + 2, W + 2, w.shape[2]))
    for t in range(27):
        dz, dyy, dx = t // 9, (t // 3) % 3, t % 3
        dxp[:, dz:dz + D, dyy:dyy + H, dx:dx + W, :] += dy @ w[t]
    return dxp[:, 1:-1, 1:-1, 1:-1, :]


def conv_weight_grad(x, dy):
    B, D, H, W, cin = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    g = np.zeros((27, dy.shape[-1], cin))
    d2 = dy.reshape(-1, dy.shape[-1])
    for t in range(27):
        dz, dyy, dx = t // 9, (t // 3) % 3, t % 3
        g[t] = d2.T @ xp[:, dz:dz + D, dyy:dyy + H, dx:dx + W, :].reshape(-1, cin)
    return g, d2.sum(axis=0)


def pool(x):
    B, D, H, W, C = x.shape
    return x.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4, 6))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def up_sum(d):
    B, D, H, W, C = d.shape
    return d.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4, 6))


def forward(params, samples, g, emulate=True):
    """samples: list of (vel, tt or None, src).  Returns (state, head output [B, nz, ny, nx])."""
    rnd = bf16 if emulate else _identity
    layers, hw, hb = unpack(params, emulate)
    x = np.stack([features(v, s, g, emulate) for v, _, s in samples])
    act, cat, pools = {}, {}, {}

    def c(L, inp):
        w, b = layers[L]
        act[L] = rnd(np.maximum(conv(inp, w, b), 0.0))
        return act[L]

    c(0, x)
    pools[0] = rnd(pool(c(1, act[0])))
    c(2, pools[0])
    pools[1] = rnd(pool(c(3, act[2])))
    c(4, pools[1])
    pools[2] = rnd(pool(c(5, act[4])))
    c(6, pools[2])
    c(7, act[6])
    cat[2] = np.concatenate([up(act[7]), act[5]], axis=-1)
    c(8, cat[2])
    c(9, act[8])
    cat[1] = np.concatenate([up(act[9]), act[3]], axis=-1)
    c(10, cat[1])
    c(11, act[10])
    cat[0] = np.concatenate([up(act[11]), act[1]], axis=-1)
    c(12, cat[0])
    c(13, act[12])
    out = act[13] @ hw + hb
    return {"x": x, "act": act, "cat": cat, "pool": pools, "layers": layers, "hw": hw}, out


def loss_and_grads(params, samples, g, emulate=True):
    """(loss, gradient vector float64, head output)."""
    rnd = bf16 if emulate else _identity
    st, out = forward(params, samples, g, emulate)
    act, cat, pools, layers, hw = st["act"], st["cat"], st["pool"], st["layers"], st["hw"]
    tg = [target(tt, v, s, g) for v, tt, s in samples]
    tgt = np.stack([t[0] for t in tg])
    wgt = np.stack([t[1] for t in tg])
    n = wgt.sum()
    diff = (out - tgt) * wgt
    loss = float((diff * diff).sum() / n)
    dout = 2.0 * diff / n
    offs, head, total = layout()
    grad = np.zeros(total)
    h = act[13]
    grad[head:head + 16] = (dout[..., None] * h).reshape(-1, 16).sum(axis=0)
    grad[head + 16] = dout.sum()

    gpre = {13: rnd(np.where(h > 0, dout[..., None] * hw, 0.0))}

    def back(L, inp, mask=None, need_dx=True):
        w, _ = layers[L]
        gw, gb = conv_weight_grad(inp, gpre[L])
        wo, bo = offs[L]
        grad[wo:bo] = gw.ravel()
        grad[bo:bo + SPEC[L][1]] = gb
        if not need_dx:
            return None
        dx = conv_input_grad(gpre[L], w)
        if mask is not None:
            dx = np.where(mask > 0, dx, 0.0)
        return rnd(dx)

    def gate(d, a):
        return rnd(np.where(a > 0, d, 0.0))

    gpre[12] = back(13, act[12], act[12])
    gcat0 = back(12, cat[0])
    gpre[11] = gate(up_sum(gcat0[..., :32]), act[11])
    gpre[10] = back(11, act[10], act[10])
    gcat1 = back(10, cat[1])
    gpre[9] = gate(up_sum(gcat1[..., :64]), act[9])
    gpre[8] = back(9, act[8], act[8])
    gcat2 = back(8, cat[2])
    gpre[7] = gate(up_sum(gcat2[..., :128]), act[7])
    gpre[6] = back(7, act[6], act[6])
    gpool2 = back(6, pools[2])
    gpre[5] = gate(gcat2[..., 128:] + 0.125 * up(gpool2), act[5])
    gpre[4] = back(5, act[4], act[4])
    gpool1 = back(4, pools[1])
    gpre[3] = gate(gcat1[..., 64:] + 0.125 * up(gpool1), act[3])
    gpre[2] = back(3, act[2], act[2])
    gpool0 = back(2, pools[0])
    gpre[1] = gate(gcat0[..., 32:] + 0.125 * up(gpool0), act[1])
    gpre[0] = back(1, act[0], act[0])
    back(0, st["x"], need_dx=False)
    return loss, grad, out


def predict(params, samples, g, inflate=1.0, emulate=True):
    """Predicted travel times T0 (1 + out) * inflate, [B, nz, ny, nx]."""
    _, out = forward(params, samples, g, emulate)
    t0 = np.stack([target(np.zeros(g[0] * g[1] * g[2]), v, s, g)[2] for v, _, s in samples])
    return t0 * (1.0 + out) * inflate


def init_params(seed):
    """He-normal weights, zero biases and head (numpy stream; the library uses its own)."""
    rng = np.random.default_rng(seed)
    offs, head, total = layout()
    p = np.zeros(total)
    for L, ((cin, cout, _), (wo, bo)) in enumerate(zip(SPEC, offs)):
        fan = 27 * (6 if L == 0 else cin)
        p[wo:bo] = rng.standard_normal(bo - wo) * np.sqrt(2.0 / fan)
    return p
