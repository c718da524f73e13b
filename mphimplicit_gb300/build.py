"""Build of the engine library (libmph_gb300.so) and the CLI, in-tree.

Every .cu translation unit is compiled by nvcc for sm_103a only; host C++ is
compiled without floating-point contraction (the derived constants and file
I/O must give the same bits on x86_64 and aarch64 hosts).  Objects go to
_lib/obj, the shared library and the CLI to _lib/.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "libmph_gb300.so")
CLI_PATH = os.path.join(LIB_DIR, "mph_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2"] + ARCH
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off"]
# tuning builds: -D definitions of the kernels' compile-time constants (MPH_PAIR_BLOCK,
# MPH_CTA_ROWS, ...) from the environment, e.g. MPH_NVCC_DEFINES="-DMPH_CLUSTER_CTAS=16"
NVCC_FLAGS += [f for f in os.environ.get("MPH_NVCC_DEFINES", "").split() if f.startswith("-D")]

LIB_SOURCES = ["k_particles.cu", "k_neighbor.cu", "k_explicit.cu", "k_assemble.cu", "k_multigrid.cu",
               "k_solver.cu", "k_mixed.cu", "k_assemble_cells.cu", "k_factored.cu", "k_resid_noalloc.cu", "mph_case.cu", "mph_export.cu",
               "mph_io.cpp", "mph_batch.cpp", "mph_capi.cpp"]
HEADERS = ["mph_internal.h", "mph_device.cuh", "mph_solver.cuh", os.path.join("..", "..", "include", "mph_gb300.h")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_lib_dir() -> str:
    root = os.path.dirname(os.path.dirname(_nvcc()))
    for sub in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"), os.path.join("targets", "x86_64-linux", "lib")):
        p = os.path.join(root, sub)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(root, "lib64")


def _digest(paths) -> str:
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()[:16]


def _compile(src: str) -> str:
    path = os.path.join(SRC, src)
    obj = os.path.join(OBJ_DIR, src + ".o")
    hdrs = [os.path.join(SRC, h) for h in HEADERS]
    stamp = obj + ".sha"
    dig = _digest([path] + hdrs)
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == dig:
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-c", path, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-I" + os.path.join(SRC), "-I" + os.path.join(os.path.dirname(_nvcc()), "..", "include"),
                                    "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(dig)
    return obj


def build(verbose: bool = False, jobs: int = 0) -> str:
    """Compile the engine library (and the CLI); returns the library path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    jobs = jobs or min(len(LIB_SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(_compile, LIB_SOURCES))
    dig = _digest(objs) + "-cudart-static"
    stamp = LIB_PATH + ".sha"
    if not (os.path.exists(LIB_PATH) and os.path.exists(stamp) and open(stamp).read() == dig):
        tmp = LIB_PATH + ".tmp"
        cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
        with open(stamp, "w") as f:
            f.write(dig)
    cli_src = os.path.join(SRC, "mph_cli.cpp")
    if os.path.exists(cli_src):
        cmd = ["g++"] + CXX_FLAGS + ["-I" + SRC, cli_src, "-o", CLI_PATH, "-L" + LIB_DIR, "-lmph_gb300",
                                     "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB_PATH}")
    return LIB_PATH


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
