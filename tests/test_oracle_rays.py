"""The oracle's 2D gradient ray tracer (Ray::GradientTracer2D::trace, src/ray/gradientTracer2d.cpp)
on the reference's own homogeneous test case (testing/ray.cpp:337-411): every ray's length within
1 m of the straight-line distance and its travel time within 1 ms -- no GPU needed."""
import numpy as np

DEFAULT_RADII = [1, 2, 3, 5, 2 ** 31 - 1]
DEFAULT_SCALES = [0.05, 0.10, 0.20, 0.30, 0.45]


def homogeneous_case():
    """Grid, source, stations and the analytic gradient of the reference's test."""
    v, dx, dz, x0, z0, nx, nz = 4000.0, 100.0, 101.0, 1.0, 2.0, 201, 101
    xs, zs = x0 + nx // 2 * dx, z0 + nz // 2 * dz
    zz, xx = np.meshgrid(np.arange(nz) * dz, np.arange(nx) * dx, indexing="ij")
    r = np.hypot(xx - (xs - x0), zz - (zs - z0))
    r[r == 0] = 1
    grad = np.stack([(xx - (xs - x0)) / r / v, (zz - (zs - z0)) / r / v], axis=-1)
    slow = np.full((nz - 1) * (nx - 1), 1 / v)
    stations = [(xs + 0.001, zs + 0.001)] + [(x0 + i / 10 * (nx - 1) * dx, z0) for i in range(11)]
    for i in range(11):
        stations += [(x0, z0 + i / 10 * (nz - 1) * dz), (x0 + (nx - 1) * dx, z0 + i / 10 * (nz - 1) * dz)]
    return dict(v=v, grid=(nx, nz, dx, dz), origin=(x0, z0), source=(xs, zs), grad=grad, slow=slow,
                stations=stations)


def path_stats(seg):
    length = np.hypot(seg[:, 2] - seg[:, 0], seg[:, 3] - seg[:, 1])
    return length.sum(), (length * seg[:, 4]).sum()


def test_homogeneous_rays_are_straight(oracle):
    c = homogeneous_case()
    nx, nz = c["grid"][:2]
    seg, counts = oracle.trace_rays2d(c["grad"], c["grid"], c["origin"], c["slow"], c["source"], c["stations"],
                                      DEFAULT_RADII, DEFAULT_SCALES, 200000, 4 * (nx + nz) + 16)
    assert (counts > 0).all(), counts
    xs, zs = c["source"]
    for i, (x, z) in enumerate(c["stations"]):
        length, t = path_stats(seg[i, :counts[i]])
        d = np.hypot(x - xs, z - zs)
        assert abs(length - d) < 1.0, (i, length, d)
        assert abs(t - d / c["v"]) < 1e-3, (i, t, d / c["v"])
        # the path runs from the source to the station, segment after segment
        s = seg[i, :counts[i]]
        assert np.allclose(s[0, :2], c["source"]) and np.allclose(s[-1, 2:4], (x, z))
        assert np.array_equal(s[1:, :2], s[:-1, 2:4])


def test_station_in_the_source_cell_gets_one_segment(oracle):
    c = homogeneous_case()
    seg, counts = oracle.trace_rays2d(c["grad"], c["grid"], c["origin"], c["slow"], c["source"], c["stations"][:1],
                                      DEFAULT_RADII, DEFAULT_SCALES, 1000, 8)
    assert counts[0] == 1 and seg[0, 0, 5] >= 0


def test_bounds_are_reported(oracle):
    c = homogeneous_case()
    far = c["stations"][1:2]
    _, counts = oracle.trace_rays2d(c["grad"], c["grid"], c["origin"], c["slow"], c["source"], far,
                                    DEFAULT_RADII, DEFAULT_SCALES, 10, 1000)
    assert counts[0] == -1       # the march needs more than 10 steps
    _, counts = oracle.trace_rays2d(c["grad"], c["grid"], c["origin"], c["slow"], c["source"], far,
                                    DEFAULT_RADII, DEFAULT_SCALES, 200000, 3)
    assert counts[0] == -2       # the healed path needs more than 3 segments
