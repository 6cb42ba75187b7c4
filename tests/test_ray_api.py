"""The C++ ray classes (include/eikonalxx/ray/: Point2D, Segment2D, Path2D,
GradientTracerOptions), driven by tests/cpp/ray_api_main.cpp in its CPU mode -- no GPU."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_ray_api(tmp_path):
    libdir = os.path.join(ROOT, "eikonalxx_gb300", "_build")
    exe = str(tmp_path / "ray_api")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "ray_api_main.cpp"), "-L" + libdir, "-leikx",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_ray_classes(lib, tmp_path):
    r = subprocess.run([build_ray_api(tmp_path), "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "ray_api ok" in r.stdout, r.stdout + r.stderr
