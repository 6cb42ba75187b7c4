"""The oracle's gradient and station interpolation (test infrastructure) against the
properties the reference's own tests check: testing/gradient.cpp:14-60 compares the
central-difference gradient of a homogeneous 2D field with the analytic gradient within
5e-5; a linear field is reproduced exactly by bilinear / trilinear interpolation."""
import numpy as np


def _cell(p, d, n):
    return min(n - 2, int(p / d)), p


def test_gradient2d_of_homogeneous_field_matches_analytic(oracle):
    # the configuration of testing/gradient.cpp:14-60
    v, nx, nz, dx, dz = 2500.0, 201, 51, 10.0, 10.5
    xs = (nx - 1) / 4 * dx + 0.3 * dx
    zs = (nz - 1) / 3 * dz - 0.4 * dx
    x = np.arange(nx) * dx
    z = np.arange(nz) * dz
    X, Z = np.meshgrid(x, z)
    r = np.hypot(X - xs, Z - zs)
    t = r / v
    cx, _ = _cell(xs, dx, nx)
    cz, _ = _cell(zs, dz, nz)
    g = oracle.gradient2d(t, (nx, nz, dx, dz), (cx, cz), (xs, zs), 1 / v)
    with np.errstate(invalid="ignore", divide="ignore"):
        gx, gz = (X - xs) / (v * r), (Z - zs) / (v * r)
    assert np.abs(g[..., 0] - gx).max() < 5e-5
    assert np.abs(g[..., 1] - gz).max() < 5e-5


def test_gradient3d_of_homogeneous_field_matches_analytic(oracle):
    v, nx, ny, nz, h = 3000.0, 61, 47, 33, 10.0
    xs, ys, zs = 27.3 * h, 19.6 * h, 14.2 * h
    z, y, x = np.meshgrid(np.arange(nz) * h, np.arange(ny) * h, np.arange(nx) * h, indexing="ij")
    r = np.sqrt((x - xs) ** 2 + (y - ys) ** 2 + (z - zs) ** 2)
    t = r / v
    cell = [_cell(p, h, n)[0] for p, n in ((xs, nx), (ys, ny), (zs, nz))]
    g = oracle.gradient3d(t, (nx, ny, nz, h, h, h), cell, (xs, ys, zs), 1 / v)
    for k, c in enumerate((x, y, z)):
        exact = (c - (xs, ys, zs)[k]) / (v * r)
        assert np.abs(g[..., k] - exact).max() < 5e-5, k


def test_station_interpolation_reproduces_linear_fields(oracle):
    rng = np.random.default_rng(3)
    nx, ny, nz, h = 12, 9, 7, 25.0
    z, y, x = np.meshgrid(np.arange(nz) * h, np.arange(ny) * h, np.arange(nx) * h, indexing="ij")
    a = rng.uniform(1e-4, 4e-4, 3)
    t = 0.3 + a[0] * x + a[1] * y + a[2] * z
    src = (0.6 * h, 0.2 * h, 0.9 * h)
    st = rng.uniform([h, h, h], [(nx - 1) * h, (ny - 1) * h, (nz - 1) * h], size=(50, 3))
    cells = np.array([[_cell(p, h, n)[0] for p, n in zip(q, (nx, ny, nz))] for q in st])
    got = oracle.stations3d(t, (nx, ny, nz, h, h, h), (0, 0, 0), src, 1 / 3000., cells, st)
    want = 0.3 + st @ a
    assert np.allclose(got, want, rtol=0, atol=1e-12)
    # a station in the source cell gets the straight-ray time
    one = oracle.stations3d(t, (nx, ny, nz, h, h, h), (0, 0, 0), src, 1 / 3000., [[0, 0, 0]], [[h, h, h]])
    assert np.isclose(one[0], np.sqrt(0.4 ** 2 + 0.8 ** 2 + 0.1 ** 2) * h / 3000., rtol=1e-14, atol=0)
    # 2D: bilinear, same property
    t2 = 0.1 + a[0] * x[:, 0, :] + a[2] * z[:, 0, :]        # (nz, nx)
    st2 = st[:, [0, 2]]
    cells2 = cells[:, [0, 2]]
    got2 = oracle.stations2d(np.ascontiguousarray(t2), (nx, nz, h, h), (0, 0), (src[0], src[2]), 1 / 3000., cells2,
                             st2)
    assert np.allclose(got2, 0.1 + st2 @ a[[0, 2]], rtol=0, atol=1e-12)
