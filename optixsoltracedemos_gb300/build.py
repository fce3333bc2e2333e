"""Build the native library libcsp_gb300.so in-tree (optixsoltracedemos_gb300/_lib/).

Device code targets sm_103a only.  Flags that the parity contract depends on:
  -fmad=false, IEEE division/sqrt (no fast math)   device float arithmetic rounds as written
  -Xcompiler -ffp-contract=off                       host float/double arithmetic rounds as written
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB_NAME = "libcsp_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
# the bounds-check build (-DCSP_BOUNDS_CHECK): every launch checks its queue, record-row, flux-bin
# and grid indices against their buffers (csp_bounds_check_status); for tests on small cases
CHECK_LIB_PATH = os.path.join(OUT_DIR, "libcsp_gb300_check.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = [
    "csp_kernels.cu",
    "csp_sungrid.cu",
    "csp_scene.cpp",
    "csp_c_api.cpp",
    "csp_io.cpp",
    "csp_noalloc.cu",
    "csp_batch.cu",
    "csp_batch.cpp",
    "csp_server.cpp",
    "../cpp/src/dropin.cpp",
]
COMMON = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-fmad=false",
    "-prec-div=true",
    "-prec-sqrt=true",
    "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden,-fno-fast-math",
    "-I", os.path.join(ROOT, "include"),
    "-I", CSRC,
    "-I", os.path.join(PKG, "cpp", "include"),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcsp_gb300.so")


def _compile(src: str, verbose: bool, check: bool = False) -> str:
    obj = os.path.join(OUT_DIR, "obj_check" if check else "obj", os.path.basename(src) + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *(["-DCSP_BOUNDS_CHECK"] if check else []), "-c", os.path.join(CSRC, src),
           "-o", obj]
    if verbose and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        sys.stderr.write(r.stdout + r.stderr)
    return obj


def _stale(lib: str) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = []
    for d in (CSRC, os.path.join(ROOT, "include"), os.path.join(PKG, "cpp", "include"), os.path.join(PKG, "cpp", "src")):
        deps += [os.path.join(d, f) for f in os.listdir(d) if os.path.isfile(os.path.join(d, f))]
    return any(os.path.getmtime(d) > t for d in deps) or os.path.getmtime(__file__) > t


def build(force: bool = False, verbose: bool = False, bounds_check: bool = False) -> str:
    lib = CHECK_LIB_PATH if bounds_check else LIB_PATH
    if not force and not _stale(lib):
        return lib
    os.makedirs(os.path.join(OUT_DIR, "obj_check" if bounds_check else "obj"), exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, bounds_check), SOURCES))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, bounds_check="--bounds-check" in sys.argv))
