"""Regenerate the golden fixtures in this folder from the reference's own tests.

The reference (uofuseismo/eikonalxx) keeps its known answers inside its GoogleTest
sources.  This script reads those files AS TEXT (nothing of the reference is built or
run) and writes the integer tables they hold as JSON:

* graph3d_4x3x5.json   -- testing/graph.cpp:40-266 (Graph.Graph3D): node-in-level ->
                          grid index for all 8 sweeps, level start pointers, level
                          count and maximum level size on a 4x3x5 grid.
* levels2d.json        -- testing/solver2d.cpp:245-438 (Solver2D.levelSetIndices):
                          the (ix, iz) visiting order of the 2D level-set method for
                          3x5, 5x3 and 4x4 grids (sweep 1; the other sweeps mirror it).

Usage:  python tests/golden/make_golden.py [/path/to/reference]
The fixtures are committed; tests never read the reference at run time.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _strip_comments(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def _int_vector(text, name):
    m = re.search(r"std::vector<int>\s+" + re.escape(name) + r"\s*\{([^}]*)\}", text)
    if m is None:
        raise ValueError(f"{name} not found")
    return [int(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()]


def _int_scalar(text, name):
    m = re.search(r"int\s+" + re.escape(name) + r"\s*=\s*(-?\d+)\s*;", text)
    if m is None:
        raise ValueError(f"{name} not found")
    return int(m.group(1))


def graph_golden(ref):
    path = os.path.join(ref, "testing", "graph.cpp")
    raw = open(path).read()
    text = _strip_comments(raw)
    start = text.index("TEST(Graph, Graph3D)")
    body = text[start:]
    out = {
        "source": "testing/graph.cpp (TEST Graph.Graph3D)",
        "nx": _int_scalar(body, "nx"),
        "ny": _int_scalar(body, "ny"),
        "nz": _int_scalar(body, "nz"),
        "n_levels": _int_scalar(body, "nLevelsRef"),
        "max_level_size": _int_scalar(body, "maxLevelSizeRef"),
        "level_start": _int_vector(body, "levelStartPtrRef"),
        "node_in_level_to_index": [
            _int_vector(body, f"nodeInLevelToGridPointRef{e}") for e in range(1, 9)
        ],
    }
    # the test's own sanity checks, restated (testing/graph.cpp:134-149)
    n = out["nx"] * out["ny"] * out["nz"]
    assert all(len(v) == n for v in out["node_in_level_to_index"])
    assert len(out["level_start"]) == out["n_levels"] + 1
    # indexToGrid reference cases (testing/graph.cpp:8-38)
    out["index_to_grid_case"] = {"nx": 44, "ny": 53, "nz": 23}
    out["number_of_levels_case"] = {"nx": 5, "ny": 3, "nz": 7, "n_levels": 5 + 3 + 7 - 2}
    return out


def levels2d_golden(ref):
    path = os.path.join(ref, "testing", "solver2d.cpp")
    text = _strip_comments(open(path).read())
    start = text.index("TEST(Solver2D, levelSetIndices)")
    end = text.index("TEST(", start + 10)
    body = text[start:end]
    cases = []
    # each case: "nx = A; nz = B;" (or "int nx = A; int nz = B;") then a refLevels list
    for m in re.finditer(
        r"nx\s*=\s*(\d+)\s*;\s*(?:int\s+)?nz\s*=\s*(\d+)\s*;(.*?)refLevels\s*(?:=)?\s*\{(.*?)\};",
        body,
        flags=re.S,
    ):
        nx, nz = int(m.group(1)), int(m.group(2))
        pairs = [
            [int(a), int(b)]
            for a, b in re.findall(r"\{\s*(-?\d+)\s*,\s*(-?\d+)\s*\}", m.group(4))
        ]
        assert len(pairs) == nx * nz, (nx, nz, len(pairs))
        cases.append({"nx": nx, "nz": nz, "order_ix_iz": pairs})
    if len(cases) < 2:
        raise ValueError("expected the 3x5 and 5x3 cases")
    return {"source": "testing/solver2d.cpp (TEST Solver2D.levelSetIndices)", "cases": cases}


def main():
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle.build import reference_root
    ref = sys.argv[1] if len(sys.argv) > 1 else reference_root()
    with open(os.path.join(HERE, "graph3d_4x3x5.json"), "w") as f:
        json.dump(graph_golden(ref), f, indent=1)
    with open(os.path.join(HERE, "levels2d.json"), "w") as f:
        json.dump(levels2d_golden(ref), f, indent=1)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
