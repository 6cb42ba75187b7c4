"""Build the native library of the package in-tree.

Compiles the CUDA kernels and the host runtime for sm_103a with nvcc and links
eikonalxx_gb300/_build/libeikx.so (C ABI of include/eikx/eikx_c.h plus the C++ API
of include/eikonalxx/).  Translation units compile in parallel; an unchanged unit is
not rebuilt.

The sweep kernels compile with --fmad=false, -prec-sqrt=true and -prec-div=true so each
floating-point operation rounds as the reference's CPU code does (no contraction,
correctly rounded sqrt and division): that is what makes the GPU travel times
bit-identical to the reference's for the same inputs.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libeikx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-sqrt=true", "-prec-div=true",
    "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
    "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
             "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

CUDA_SOURCES = ["sweep.cu", "sweep_pair.cu", "sweep_chunk_8x4.cu", "sweep_chunk_4x8.cu", "sweep_chunk_16x2.cu", "fields.cu", "post.cu", "rays.cu", "capi.cu", "noalloc.cu",
                "warmnet_kernels.cu", "warmnet.cu"]
CXX_SOURCES = ["levels.cpp", "api/options.cpp", "api/geometry.cpp", "api/source.cpp", "api/model.cpp",
               "api/graph3d.cpp", "api/solver3d.cpp", "api/solver2d.cpp", "api/ray.cpp", "api/vtk.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build eikonalxx_gb300")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _digest(paths, flags):
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def _headers():
    out = []
    for d in (CSRC, os.path.join(ROOT, "include")):
        for base, _, files in os.walk(d):
            out += [os.path.join(base, f) for f in files if f.endswith((".h", ".hpp", ".cuh"))]
    return sorted(out)


def _compile(cmd, src, obj, stamp_paths, flags):
    stamp = obj + ".sha"
    dig = _digest([src] + stamp_paths, flags)
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == dig:
        return obj
    os.makedirs(os.path.dirname(obj), exist_ok=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(dig)
    return obj


def build(verbose=False):
    """Compile every translation unit for sm_103a and link libeikx.so; returns its path."""
    nvcc = _nvcc()
    cuda_home = _cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for s in CUDA_SOURCES:
            src = os.path.join(CSRC, s)
            obj = os.path.join(BUILD, s.replace("/", "_") + ".o")
            cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
            jobs.append(ex.submit(_compile, cmd, src, obj, headers, cmd))
        for s in CXX_SOURCES:
            src = os.path.join(CSRC, s)
            obj = os.path.join(BUILD, s.replace("/", "_") + ".o")
            cmd = ["g++"] + CXX_FLAGS + ["-I" + os.path.join(cuda_home, "include"), "-c", src, "-o", obj]
            jobs.append(ex.submit(_compile, cmd, src, obj, headers, cmd))
        objs = [j.result() for j in jobs]
    link = [nvcc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart_static", "-lrt", "-ldl",
                                                                   "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
