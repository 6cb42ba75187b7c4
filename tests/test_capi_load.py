"""The C-ABI library loads, exports every symbol eikx_c.h declares, and its host-only
entry points (level-set tables) reproduce the reference's goldens -- no GPU needed."""
import json
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _declared():
    text = open(os.path.join(ROOT, "include", "eikx", "eikx_c.h")).read()
    decl = r"^(?:eikx_status|int|void|const char \*)\s*(eikx_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(decl, text, flags=re.M)))


def test_every_declared_symbol_is_exported(lib):
    import eikonalxx_gb300 as ex
    declared = _declared()
    assert set(declared) == set(ex.EXPORTED), "binding list out of sync with eikx_c.h"
    for name in declared:
        assert hasattr(lib, name), name


def test_options_default_mirrors_solver_options(lib):
    import eikonalxx_gb300 as ex
    o = ex._Options()
    lib.eikx_options_default(o)
    assert (o.n_sweeps, o.tolerance, o.factored_radius) == (5, 1e-5, 3)


def test_graph3d_tables_golden(lib):
    import eikonalxx_gb300 as ex
    g = json.load(open(os.path.join(GOLDEN, "graph3d_4x3x5.json")))
    for e in range(8):
        t = ex.graph3d_tables(e, g["nx"], g["ny"], g["nz"])
        assert t["n_levels"] == g["n_levels"]
        assert t["max_level_size"] == g["max_level_size"]
        assert t["level_start"].tolist() == g["level_start"]
        assert t["node_to_index"].tolist() == g["node_in_level_to_index"][e]


@pytest.mark.parametrize("shape", [(4, 3, 5), (9, 7, 3), (16, 5, 11), (3, 3, 3)])
def test_graph3d_tables_match_oracle(lib, oracle, shape):
    import eikonalxx_gb300 as ex
    for e in range(8):
        a, b = ex.graph3d_tables(e, *shape), oracle.graph3d(e, *shape)
        for k in a:
            if isinstance(a[k], np.ndarray):
                assert np.array_equal(a[k], b[k]), (e, k)
            else:
                assert a[k] == b[k], (e, k)


def test_graph3d_rejects_small_grids(lib):
    import eikonalxx_gb300 as ex
    with pytest.raises(ex.InvalidArgument):
        ex.graph3d_tables(0, 2, 5, 5)


def test_levels2d_golden(lib):
    import eikonalxx_gb300 as ex
    g = json.load(open(os.path.join(GOLDEN, "levels2d.json")))
    for case in g["cases"]:
        nx, nz = case["nx"], case["nz"]
        ref = np.array(case["order_ix_iz"])
        for e in range(4):
            ls, ix, iz = ex.levels2d(e, nx, nz)
            ex_ix = ref[:, 0] if e in (0, 2) else nx - 1 - ref[:, 0]
            ex_iz = ref[:, 1] if e in (0, 1) else nz - 1 - ref[:, 1]
            assert np.array_equal(ix, ex_ix) and np.array_equal(iz, ex_iz)
            assert ls[0] == 0 and ls[-1] == nx * nz
