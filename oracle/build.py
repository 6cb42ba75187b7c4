"""Build the oracle libraries -- test infrastructure only.

* oracle/_build/libeikx_oracle.so : the project's CPU restatement (eikx_oracle.cpp).
* oracle/_ref/libeikx_ref.so      : the reference's OWN hot-path sources, compiled in
  place from the reference checkout (default /root/reference, or $EIKX_REFERENCE) with
  the host shim in oracle/shim/ and the drivers ref_driver.cpp and ref_trace.cpp.  Files
  compiled from the reference: src/graph3d.cpp, src/geometry3d.cpp, src/geometry2d.cpp,
  src/solverOptions.cpp, src/station2d.cpp, src/source2d.cpp, the 2D ray tracer
  src/ray/{gradientTracer2d,gradientTracerOptions,path2d,segment2d,point2d}.cpp and
  src/io/vtkLines2d.cpp, plus the headers include/private/solver{2,3}d.hpp and
  solverUtilities{2,3}d.hpp (through ref_driver.cpp).  Skipped, with a message, when
  the checkout is absent (it never travels to a GPU host).

Both are compiled with -ffp-contract=off so no multiply-add is fused: the CPU rounding
then matches the GPU kernels built with --fmad=false.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libeikx_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libeikx_ref.so")
FLAGS = ["-O2", "-ffp-contract=off", "-fPIC", "-shared"]
_REF_SKIP_SAID = False


def reference_root():
    """Where the reference checkout is read from: $EIKX_REFERENCE, else the read-only
    checkout this recipe was written against.  The tests and the golden-vector script
    ask this function, so the location is named in this recipe alone."""
    return os.environ.get("EIKX_REFERENCE", "/root/reference")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_oracle():
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    src = os.path.join(HERE, "eikx_oracle.cpp")
    if os.path.exists(ORACLE_LIB) and os.path.getmtime(ORACLE_LIB) > os.path.getmtime(src):
        return ORACLE_LIB
    _run(["g++", "-std=c++17"] + FLAGS + [src, "-o", ORACLE_LIB + ".tmp"])
    os.replace(ORACLE_LIB + ".tmp", ORACLE_LIB)
    return ORACLE_LIB


def build_ref():
    ref = reference_root()
    if not os.path.isdir(os.path.join(ref, "include", "private")):
        global _REF_SKIP_SAID
        if not _REF_SKIP_SAID:
            print(f"oracle/_ref: reference sources not found at {ref}; skipped", file=sys.stderr)
            _REF_SKIP_SAID = True
        return None
    os.makedirs(os.path.dirname(REF_LIB), exist_ok=True)
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "ref_trace.cpp")] + [
        os.path.join(ref, "src", f) for f in ("graph3d.cpp", "geometry3d.cpp", "geometry2d.cpp",
                                              "solverOptions.cpp", "station2d.cpp", "source2d.cpp",
                                              "ray/gradientTracer2d.cpp", "ray/gradientTracerOptions.cpp",
                                              "ray/path2d.cpp", "ray/segment2d.cpp", "ray/point2d.cpp",
                                              "io/vtkLines2d.cpp")]
    if os.path.exists(REF_LIB) and all(os.path.getmtime(REF_LIB) > os.path.getmtime(s) for s in srcs):
        return REF_LIB
    cmd = (["g++", "-std=c++20", "-w"] + FLAGS +
           ["-I" + os.path.join(HERE, "shim"), "-I" + os.path.join(ref, "include"), "-I" + ref] +
           srcs + ["-o", REF_LIB + ".tmp"])
    _run(cmd)
    os.replace(REF_LIB + ".tmp", REF_LIB)
    return REF_LIB


def build():
    build_oracle()
    build_ref()


if __name__ == "__main__":
    build()
    print("oracle built:", ORACLE_LIB, REF_LIB if os.path.exists(REF_LIB) else "(no _ref)")
    sys.exit(0)
