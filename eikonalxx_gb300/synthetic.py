"""Seeded synthetic velocity models and source sets for the benchmark workloads.

The reference ships no benchmark data; the workloads are defined by their recipe:
  * layered + Gaussian-random-field models: ``n_layers`` horizontal layers of equal
    thickness with velocities drawn uniformly from [vmin, vmax] and sorted to increase
    with depth, multiplied by (1 + p) where p is white noise filtered with a Gaussian
    kernel (correlation length ``corr_m``), scaled to +-``pert`` and clipped;
  * sources drawn uniformly in the domain (or on its top surface, for station tables
    computed by reciprocity).
"""
import numpy as np


def grf(shape, spacing, corr_m, rng):
    """Zero-mean, unit-max Gaussian random field with a Gaussian correlation kernel."""
    noise = rng.standard_normal(shape)
    freqs = [np.fft.fftfreq(n, d=spacing) for n in shape[:-1]] + [np.fft.rfftfreq(shape[-1], d=spacing)]
    grids = np.meshgrid(*freqs, indexing="ij", sparse=True)
    k2 = sum(g ** 2 for g in grids)
    # Gaussian kernel exp(-r^2/corr^2) has spectrum ~ exp(-pi^2 corr^2 k^2)
    filt = np.exp(-(np.pi ** 2) * corr_m ** 2 * k2)
    axes = list(range(len(shape)))
    field = np.fft.irfftn(np.fft.rfftn(noise, axes=axes) * filt, s=shape, axes=axes)
    field -= field.mean()
    m = np.max(np.abs(field))
    return field / m if m > 0 else field


def layered_grf_model(nx, ny, nz, h, seed, n_layers=8, vmin=3000.0, vmax=7000.0, pert=0.05,
                      corr_m=1000.0, dtype=np.float32):
    """Nodal velocities (nz, ny, nx) of the layered + GRF recipe."""
    rng = np.random.default_rng(seed)
    layer_v = np.sort(rng.uniform(vmin, vmax, n_layers))
    iz = np.arange(nz)
    layer = np.minimum(iz * n_layers // nz, n_layers - 1)
    v = np.broadcast_to(layer_v[layer][:, None, None], (nz, ny, nx)).astype(np.float64)
    p = grf((nz, ny, nx), h, corr_m, rng) * pert
    v = v * (1.0 + np.clip(p, -pert, pert))
    return np.ascontiguousarray(v, dtype=dtype)


def uniform_sources(n, nx, ny, nz, h, seed, surface=False):
    """n source positions (x, y, z) in metres, uniform in the domain (or on z = 0)."""
    rng = np.random.default_rng(seed)
    xyz = np.column_stack([rng.uniform(0, (nx - 1) * h, n), rng.uniform(0, (ny - 1) * h, n),
                           np.zeros(n) if surface else rng.uniform(0, (nz - 1) * h, n)])
    return xyz


def uneven_models(n, seed, h=100.0, nxy=(64, 256), nz=(32, 128), dtype=np.float32):
    """n independent models of uneven size: nx, ny uniform in `nxy`, nz uniform in `nz`,
    spacing h, each a layered + GRF model with one source uniform in its domain.
    Returns a list of dicts with ``grid`` (nx, ny, nz, h, h, h), ``v`` (nodal, (nz, ny, nx))
    and ``source`` (x, y, z)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        gx, gy = (int(v) for v in rng.integers(nxy[0], nxy[1] + 1, 2))
        gz = int(rng.integers(nz[0], nz[1] + 1))
        v = layered_grf_model(gx, gy, gz, h, int(rng.integers(1 << 31)), dtype=dtype)
        src = uniform_sources(1, gx, gy, gz, h, int(rng.integers(1 << 31)))[0]
        out.append({"grid": (gx, gy, gz, h, h, h), "v": v, "source": tuple(float(c) for c in src)})
    return out


def slab_model(nx, ny, nz, h, seed, slab_v=8000.0, dip_deg=30.0, thickness_m=None, dtype=np.float32):
    """Layered + GRF model with a high-velocity slab: nodes within thickness/2 of a plane
    dipping `dip_deg` degrees along x (through a seeded point near the top centre) get
    `slab_v`.  Nodal velocities (nz, ny, nx)."""
    v = layered_grf_model(nx, ny, nz, h, seed, dtype=np.float64)
    rng = np.random.default_rng(seed + 1)
    x0 = rng.uniform(0.3, 0.5) * (nx - 1) * h
    z0 = rng.uniform(0.05, 0.15) * (nz - 1) * h
    thick = thickness_m if thickness_m is not None else 0.08 * (nz - 1) * h
    dip = np.deg2rad(dip_deg)
    z, _, x = np.meshgrid(np.arange(nz) * h, np.zeros(1), np.arange(nx) * h, indexing="ij", sparse=True)
    # signed distance to the plane through (x0, z0) dipping along +x
    d = (z - z0) * np.cos(dip) - (x - x0) * np.sin(dip)
    mask = np.abs(d) <= thick / 2
    v = np.where(np.broadcast_to(mask, v.shape), slab_v, v)
    return np.ascontiguousarray(v, dtype=dtype)


def linear_gradient_2d(nx, nz, h, v_top, gradient, dtype=np.float64):
    """Nodal velocities (nz, nx) of v(z) = v_top + gradient * z, z = iz * h."""
    z = np.arange(nz) * h
    v = v_top + gradient * z
    return np.ascontiguousarray(np.broadcast_to(v[:, None], (nz, nx)), dtype=dtype)
