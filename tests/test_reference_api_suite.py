"""The reference's own unit tests, compiled unchanged against this library (CPU).

The reference keeps its API tests in GoogleTest sources (testing/*.cpp).  Those that
exercise the public API alone -- geometry, sources, stations, options, the Graph3D
level tables and the velocity models -- are compiled here, as they are, against
include/eikonalxx/ and libeikx.so with a GoogleTest-compatible shim (tests/cpp/gtest):
the drop-in must pass the reference's own checks.  Skipped where the reference
checkout is absent.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.build import reference_root  # noqa: E402

REF = reference_root()
SUITES = ["geometry", "source", "station", "solverOptions", "graph", "model"]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "testing")), reason="reference tests not available")
def test_reference_unit_tests_pass_against_dropin(lib, tmp_path):
    libdir = os.path.join(ROOT, "eikonalxx_gb300", "_build")
    objs = []
    for name in SUITES + ["main"]:
        src = (os.path.join(ROOT, "tests", "cpp", "gtest_main.cpp") if name == "main"
               else os.path.join(REF, "testing", name + ".cpp"))
        obj = str(tmp_path / (name + ".o"))
        # private/grid.hpp (index helpers the graph test uses) comes from the reference
        cmd = ["g++", "-std=c++17", "-w", "-I" + os.path.join(ROOT, "tests", "cpp"),
               "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(REF, "include"), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        objs.append(obj)
    exe = str(tmp_path / "reference_unit_tests")
    r = subprocess.run(["g++"] + objs + ["-L" + libdir, "-leikx", "-Wl,-rpath," + libdir, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "0 failed" in r.stdout
