"""The 3D sweep's operator shortcuts, exact at their edges.

The uniform-grid Cartesian operator of the sweep kernels (fd3UniformFarBounded) returns the
node's own time as soon as lower bounds show that no operator goes below it, evaluates each 2D
operator only where its own bound leaves it a chance, and bounds the 8-point operator by t6.
Parity of whole solves (test_gpu_parity.py, test_gpu_fullsize.py) exercises these on real
fields, where stencils rarely sit at a bound's edge.  Here the device evaluates the operator
with and without its shortcuts on seeded stencils built to sit at those edges -- node times a
few units in the last place from the operator's own value, neighbour differences at the 2D
windows' limits, homogeneous slowness, unreached neighbours -- and min(t0, result) must agree
bit for bit on every one.  The operator is the reference's (solverUtilities3d.hpp:258-558).
"""
import pytest

pytestmark = pytest.mark.gpu

import eikonalxx_gb300 as ex  # noqa: E402


@pytest.mark.parametrize("precision", [ex.F32, ex.F64])
@pytest.mark.parametrize("seed", [1, 2])
def test_operator_shortcuts_exact_at_their_edges(ctx, precision, seed):
    n = 50_000_000 if precision == ex.F32 else 10_000_000
    c = ex.selftest_operator3d(n, seed=seed, precision=precision)
    assert c["evaluated"] == n
    assert c["mismatches"] == 0, c
    # the stencils reach both sides of the shortcuts: some end at t0, some do not
    assert 0 < c["shortcut_t0"] < n
    assert c["t0_is_operator"] > n // 20


def test_selftest_rejects_bad_arguments(ctx):
    with pytest.raises(ex.EikxError):
        ex.selftest_operator3d(-1)
    with pytest.raises(ex.EikxError):
        ex.selftest_operator3d(10, precision=7)
