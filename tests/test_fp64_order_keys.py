"""The integer-pipe comparisons of the FP64 sweeps (csrc/local_solver.cuh: pmin, pmax,
orderKey / atMostAll), restated on the host with numpy's int64 views of the same bit
patterns: for non-negative doubles the signed order of the bits is the IEEE order (so the
selected operand is fmin's / fmax's), a maximum that includes a positive floor is exact
whatever the sign of the other operands, and the order key is monotone with -0 and +0
equal, so `t0 <= min(...)` is decided exactly for every non-NaN input."""
import numpy as np


def _bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def _pmin(a, b):
    return np.where(_bits(a) < _bits(b), a, b)


def _pmax(a, b):
    return np.where(_bits(a) > _bits(b), a, b)


def _key(x):
    v = _bits(x)
    return np.where(v >= 0, v, -(v & np.int64(0x7FFFFFFFFFFFFFFF)))


def _samples(rng, n):
    """Positive doubles over many binades, with ties, +0 and the solver's huge value."""
    x = np.exp(rng.uniform(-700, 700, n)) * rng.choice([1.0, 1.0 + 2.0 ** -52], n)
    x[::97] = 0.0
    x[::89] = 1.0e10
    return x


def test_pmin_pmax_match_ieee_on_non_negative_values():
    rng = np.random.default_rng(5)
    a, b = _samples(rng, 200_000), _samples(rng, 200_000)
    b[::7] = a[::7]
    assert np.array_equal(_bits(_pmin(a, b)), _bits(np.fmin(a, b)))
    assert np.array_equal(_bits(_pmax(a, b)), _bits(np.fmax(a, b)))


def test_pmax_with_positive_floor_is_exact_for_any_sign():
    rng = np.random.default_rng(6)
    t = rng.standard_normal((7, 100_000)) * np.exp(rng.uniform(-50, 50, (7, 100_000)))
    t[:, ::13] = -0.0
    floor = 2.0 ** -100
    m = np.full(t.shape[1], floor)
    ref = np.full(t.shape[1], floor)
    for row in t:
        m = _pmax(m, row)
        ref = np.fmax(ref, row)
    assert np.array_equal(_bits(m), _bits(ref))


def test_order_key_decides_t0_at_most_all_exactly():
    rng = np.random.default_rng(7)
    n = 200_000
    vals = rng.standard_normal((6, n)) * np.exp(rng.uniform(-30, 30, (6, n)))
    vals[:, ::11] = 0.0
    vals[:, ::17] = -0.0
    vals[0, ::5] = vals[1, ::5]                      # ties between t0 and an operand
    t0, rest = vals[0], vals[1:]
    ref = t0 <= rest.min(axis=0)
    got = np.all(_key(t0)[None, :] <= _key(rest), axis=0)
    assert np.array_equal(got, ref)
    # the key is monotone and equal for the two zeros
    x = np.sort(vals.ravel())
    k = _key(x)
    assert np.all(np.diff(k) >= 0)
    assert _key(np.array([-0.0]))[0] == _key(np.array([0.0]))[0]
