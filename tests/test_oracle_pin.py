"""The oracle pinned against the reference's own code and its golden vectors (CPU)."""
import json
import os

import numpy as np
import pytest

from conftest import random_slowness

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _case3(rng, nx, ny, nz, dx, dy, dz, dtype):
    s = random_slowness(rng, (nz - 1) * (ny - 1) * (nx - 1), dtype=dtype)
    cell = [int(rng.integers(0, n - 1)) for n in (nx, ny, nz)]
    off = [(c + rng.uniform()) * d for c, d in zip(cell, (dx, dy, dz))]
    return s, (nx, ny, nz, dx, dy, dz), cell, off


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("radius", [0, 3, 1000])
@pytest.mark.parametrize("shape", [(9, 10, 11, 100., 100., 100.), (13, 7, 8, 100., 120., 90.),
                                   (3, 3, 3, 50., 50., 50.), (6, 4, 12, 25., 25., 25.)])
def test_oracle_3d_matches_reference_bitwise(oracle, reference, dtype, radius, shape):
    rng = np.random.default_rng(hash((shape, radius)) % 2**32)
    s, g, cell, off = _case3(rng, *shape, dtype)
    t_ref = reference.solve3d(s, g, cell, off, n_sweeps=2, radius=radius)
    t_or = oracle.solve3d(s, g, cell, off, n_sweeps=2, radius=radius, init_fp64=False)
    assert np.array_equal(t_ref.view(np.uint8), t_or.view(np.uint8))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("radius", [0, 3, 1000])
@pytest.mark.parametrize("shape", [(31, 27, 10., 10.), (25, 33, 10., 12.5), (3, 3, 10., 10.)])
def test_oracle_2d_matches_reference_bitwise(oracle, reference, dtype, radius, shape):
    rng = np.random.default_rng(hash((shape, radius, 2)) % 2**32)
    nx, nz, dx, dz = shape
    s = random_slowness(rng, (nz - 1) * (nx - 1), dtype=dtype)
    cell = [int(rng.integers(0, nx - 1)), int(rng.integers(0, nz - 1))]
    off = [(cell[0] + rng.uniform()) * dx, (cell[1] + rng.uniform()) * dz]
    t_ref = reference.solve2d(s, shape, cell, off, n_sweeps=2, radius=radius)
    # hypot_mode 0: std::hypot, as the reference calls it
    t_or = oracle.solve2d(s, shape, cell, off, n_sweeps=2, radius=radius, init_fp64=False, hypot_mode=0)
    assert np.array_equal(t_ref.view(np.uint8), t_or.view(np.uint8))


def test_oracle_2d_own_hypot_within_an_ulp(oracle, reference):
    """The GPU's hypot (Borges 2019) differs from std::hypot by at most an ulp."""
    rng = np.random.default_rng(7)
    shape = (31, 27, 10., 10.)
    s = random_slowness(rng, 30 * 26)
    t_ref = reference.solve2d(s, shape, [11, 9], [115.0, 93.0], n_sweeps=2, radius=1000)
    t_or = oracle.solve2d(s, shape, [11, 9], [115.0, 93.0], n_sweeps=2, radius=1000, init_fp64=False,
                          hypot_mode=1)
    assert np.max(np.abs(t_ref - t_or)) <= 1e-15


def test_graph3d_golden(oracle):
    g = json.load(open(os.path.join(GOLDEN, "graph3d_4x3x5.json")))
    nx, ny, nz = g["nx"], g["ny"], g["nz"]
    for e in range(8):
        t = oracle.graph3d(e, nx, ny, nz)
        assert t["n_levels"] == g["n_levels"]
        assert t["max_level_size"] == g["max_level_size"]
        assert t["level_start"].tolist() == g["level_start"]
        assert t["node_to_index"].tolist() == g["node_in_level_to_index"][e]
        idx = t["node_to_index"]
        assert np.array_equal(t["to_x"], idx % nx)
        assert np.array_equal(t["to_y"], (idx // nx) % ny)
        assert np.array_equal(t["to_z"], idx // (nx * ny))


@pytest.mark.parametrize("shape", [(4, 3, 5), (5, 3, 7), (7, 6, 3), (11, 4, 9)])
def test_graph3d_oracle_matches_reference(oracle, reference, shape):
    for e in range(8):
        a, b = oracle.graph3d(e, *shape), reference.graph3d(e, *shape)
        for k in a:
            if isinstance(a[k], np.ndarray):
                assert np.array_equal(a[k], b[k]), (e, k)
            else:
                assert a[k] == b[k], (e, k)


def test_residual_and_convergence_rule(oracle):
    """A solve stops after the first refinement sweep that completes a run of 8 sweeps (a
    window that may span two iterations) each with largest decrease below tol."""
    rng = np.random.default_rng(3)
    s, g, cell, off = _case3(rng, 17, 15, 13, 100., 100., 100., np.float64)
    for tol in (1e-9, 1e-6, 1e-4):
        t, res, it = oracle.solve3d(s, g, cell, off, n_sweeps=12, radius=0, tol=tol, residuals=True)
        assert 1 <= it <= 12
        r = res.ravel()
        quiet = np.convolve((r < tol).astype(int), np.ones(8, int), "valid")   # run lengths over windows
        stop = int(np.argmax(quiet == 8)) + 8 if (quiet == 8).any() else len(r)
        assert (it - 1) * 8 < stop <= it * 8, (tol, it, stop)
        assert not (quiet[:max(0, stop - 8)] == 8).any()
        # the swept field equals the same sweeps run without a tolerance, stopped there
        t_full = oracle.solve3d(s, g, cell, off, n_sweeps=it, radius=0, tol=-1)
        if stop == it * 8:
            assert np.array_equal(t, t_full)


def test_stepped_cold_solve_equals_one_call(oracle):
    """The benchmark's CPU baselines run real cold-start solves a few sweeps at a time
    (oracle.ColdSolve3): stepped to the end, the field and the stopping sweep are those
    of the one-call solve."""
    from oracle import ColdSolve3
    rng = np.random.default_rng(4)
    s, g, cell, off = _case3(rng, 19, 16, 14, 100., 100., 100., np.float32)
    for tol, step in ((1e-6, 3), (1e-4, 8), (-1.0, 5)):
        t, res, it = oracle.solve3d(s, g, cell, off, n_sweeps=9, radius=3, tol=tol, residuals=True)
        cs = ColdSolve3(oracle, s, g, off, n_sweeps=9, radius=3, tol=tol)
        n = 0
        while not cs.advance(step):
            n += 1
            assert n < 100
        assert np.array_equal(cs.tt.reshape(t.shape).view(np.uint32), t.view(np.uint32))
        r = res.ravel()
        assert 8 + 8 * (it - 1) < cs.sweeps <= 8 + 8 * it
        if tol < 0:
            assert cs.sweeps == 8 * (1 + 9)


def test_near_fp64_mode_moves_fp32_towards_fp64(oracle):
    """The oracle's near_fp64 mode (FP32 sweeps whose factored branch forms its analytic
    factor T0 = s0 |x - xs|, its gradient and the differences tau in FP64): within the
    factored radius its field lies closer to the FP64 solve than plain FP32, on every one
    of a set of random cases (the FP32 differences t - T0 lose digits to cancellation)."""
    for seed in range(6):
        rng = np.random.default_rng(seed)
        s, g, cell, off = _case3(rng, 21, 18, 16, 50., 50., 50., np.float32)
        z, y, x = np.meshgrid(np.arange(16), np.arange(18), np.arange(21), indexing="ij")
        near = (np.abs(x - cell[0]) <= 3) & (np.abs(y - cell[1]) <= 3) & (np.abs(z - cell[2]) <= 3)
        kw = dict(n_sweeps=1, radius=3)
        t64 = oracle.solve3d(s.astype(np.float64), g, cell, off, **kw)
        e32 = np.abs(oracle.solve3d(s, g, cell, off, **kw) - t64)[near].sum()
        e_near = np.abs(oracle.solve3d(s, g, cell, off, near_fp64=True, **kw) - t64)[near].sum()
        assert e_near < e32, seed


def test_analytic_homogeneous_matches_closed_form(oracle):
    g = (21, 19, 17, 10., 11., 12.)
    t = oracle.linear_gradient3d(g, (53.0, 41.0, 77.0), 3000.0, 3000.0)
    z, y, x = np.meshgrid(np.arange(17) * 12., np.arange(19) * 11., np.arange(21) * 10., indexing="ij")
    exact = np.sqrt((x - 53.) ** 2 + (y - 41.) ** 2 + (z - 77.) ** 2) / 3000.
    assert np.max(np.abs(t - exact)) < 1e-15


def test_analytic_linear_gradient_satisfies_eikonal(oracle):
    """|grad T| = 1/v(z) for the linear-gradient solution (central differences)."""
    nx, nz, dx, dz = 201, 101, 5., 5.
    t = oracle.linear_gradient2d((nx, nz, dx, dz), (500., 250.), 3000., 4250.)
    gz, gx = np.gradient(t, dz, dx)
    zz = np.arange(nz)[:, None] * dz
    v = 3000. + (4250. - 3000.) * zz / ((nz - 1) * dz)
    err = np.abs(np.sqrt(gx ** 2 + gz ** 2) * v - 1.0)[5:-5, 5:-5]
    dist = np.hypot(np.arange(nx)[None, :] * dx - 500., zz - 250.)[5:-5, 5:-5]
    assert np.max(err[dist > 100]) < 1e-3


def test_nodal_to_cell_orderings_agree(oracle):
    rng = np.random.default_rng(5)
    nx, ny, nz = 6, 5, 4
    v = rng.uniform(2000, 5000, (nz, ny, nx))
    s_nat = oracle.nodal_to_cell3d(v.ravel(), nx, ny, nz, 0)
    s_tr = oracle.nodal_to_cell3d(np.ascontiguousarray(v.transpose(2, 1, 0)).ravel(), nx, ny, nz, 1)
    assert np.allclose(s_nat, s_tr, rtol=1e-14)  # pairwise sums differ in order
    mean = (v[:-1, :-1, :-1] + v[:-1, :-1, 1:] + v[:-1, 1:, :-1] + v[:-1, 1:, 1:] + v[1:, :-1, :-1] +
            v[1:, :-1, 1:] + v[1:, 1:, :-1] + v[1:, 1:, 1:]) / 8
    assert np.allclose(s_nat, (1 / mean).ravel(), rtol=1e-14)


def _ray_cases():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_oracle_rays import homogeneous_case
    c = homogeneous_case()
    cases = [("homogeneous", c)]
    # a linear gradient v(z) = 3000 + 0.6 z with its analytic travel-time gradient
    nx, nz, dx, dz = 161, 81, 25.0, 25.0
    v0, k = 3000.0, 0.6
    xs, zs = 2012.5, 812.5
    zz, xx = np.meshgrid(np.arange(nz) * dz, np.arange(nx) * dx, indexing="ij")
    vs, v = v0 + k * zs, v0 + k * zz
    r2 = (xx - xs) ** 2 + (zz - zs) ** 2
    arg = 1 + k * k * r2 / (2 * vs * v)
    denom = np.sqrt(np.maximum(arg * arg - 1, 1e-30)) * k
    dadx = k * k * (xx - xs) / (vs * v)
    dadz = k * k * (zz - zs) / (vs * v) - k * k * r2 / (2 * vs * v * v) * k
    grad = np.stack([dadx / denom, dadz / denom], axis=-1)
    grad[r2 == 0] = 0
    vc = v0 + k * (np.arange(nz - 1) + 0.5) * dz
    slow = np.repeat(1 / vc, nx - 1)
    rng = np.random.default_rng(4)
    stations = [(float(rng.uniform(0, (nx - 1) * dx)), float(rng.uniform(0, (nz - 1) * dz))) for _ in range(24)]
    cases.append(("linear", dict(grid=(nx, nz, dx, dz), origin=(0.0, 0.0), source=(xs, zs), grad=grad, slow=slow,
                                 stations=stations)))
    return cases


@pytest.mark.parametrize("precision", [np.float64, np.float32])
def test_ray_tracer_matches_the_reference(oracle, reference, precision):
    """The oracle's restatement of GradientTracer2D::trace against the reference's own tracer:
    the same segments, end points within 1e-6 m (the march uses eikxHypot where the reference
    uses std::hypot), the same slownesses; rays the reference does not converge (empty paths)
    are the oracle's count -1."""
    radii, scales = [1, 2, 3, 5, 2 ** 31 - 1], [0.05, 0.10, 0.20, 0.30, 0.45]
    for name, c in _ray_cases():
        nx, nz, dx, dz = c["grid"]
        cap = 4 * (nx + nz) + 16
        g = c["grad"].astype(precision)
        # A ray starting on the last node row makes the reference read past the end of its
        # gradient array (gradientTracer2d.cpp:452-455): those stations are left out here.
        zmax = c["origin"][1] + (nz - 1) * dz
        stations = [p for p in c["stations"] if p[1] < zmax - 1e-9]
        # a solver in T reports its slowness in T (ISolver2D<T>::getSlowness)
        slow = c["slow"].astype(precision).astype(np.float64)
        seg, counts = oracle.trace_rays2d(g, c["grid"], c["origin"], slow, c["source"], stations, radii,
                                          scales, 200000, cap)
        rseg, rcounts = reference.trace_rays2d(g, c["grid"], c["origin"], slow, c["source"], stations,
                                               radii, scales, cap)
        assert np.array_equal(np.where(counts < 0, 0, counts), rcounts), (name, counts, rcounts)
        for i in range(len(counts)):
            n = max(0, counts[i])
            assert np.allclose(seg[i, :n, :4], rseg[i, :n, :4], rtol=0, atol=1e-6), (name, i)
            assert np.array_equal(seg[i, :n, 4], rseg[i, :n, 4]), (name, i)
            assert np.array_equal(seg[i, :n, 5], rseg[i, :n, 5]), (name, i)
