"""Build libmpc_gpu.so (sm_103a) in-tree with nvcc: one object per translation unit,
compiled in parallel, linked with -shared.  No cmake, no torch extension machinery."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.environ.get("MPC_GPU_OBJ_DIR", os.path.join(HERE, "_build"))
LIB = os.environ.get("MPC_GPU_LIB_OUT", os.path.join(HERE, "libmpc_gpu.so"))
SOURCES = ["mpc_capi.cu", "mpc_shapes_a.cu", "mpc_shapes_b.cu", "mpc_shapes_c.cu", "mpc_shapes_d.cu",
           "mpc_noalloc.cu", "mpc_mlp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-diag-suppress", "177"]
# extra defines for tuning builds, e.g. MPC_NVCC_EXTRA="-DMPC_PENCIL_UNROLL=2"
FLAGS += os.environ.get("MPC_NVCC_EXTRA", "").split()


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "mpc_gpu.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append((s, o))

    def compile_one(job):
        s, o = job
        cmd = [nvcc(), *ARCH, *FLAGS, "-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {s}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return o

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(compile_one, jobs))
    if force or jobs or not _newer(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_driver(force)
    return LIB


DRIVER_SRC = os.path.join(HERE, "driver", "mpc_run.c")
DRIVER = os.path.join(os.path.dirname(LIB), "mpc_run")


def build_driver(force: bool = False) -> str:
    """The C run driver (driver/mpc_run.c), linked against the library beside it."""
    hdr = os.path.join(HERE, "..", "include", "mpc_gpu.h")
    if force or not _newer(DRIVER, [DRIVER_SRC, hdr, LIB]):
        libdir = os.path.dirname(os.path.abspath(LIB))
        libname = os.path.basename(LIB)
        cmd = [os.environ.get("CC", "gcc"), "-O2", "-std=c11", "-Wall", "-Wextra", "-o", DRIVER, DRIVER_SRC,
               f"-L{libdir}", f"-l:{libname}", "-Wl,-rpath,$ORIGIN", "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
