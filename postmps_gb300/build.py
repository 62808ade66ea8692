"""Builds libpms.so (and the VisGPU-compatible CLI) in-tree for sm_103a.

Every translation unit is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a), host C++ with the same nvcc driver,
and linked into postmps_gb300/_build/libpms.so.  The marching-cubes tables are
extracted from the reference tree first when it is present
(gen_mc_tables.py); otherwise mc_tables.cu derives them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpms.so")
CLI = os.path.join(OUT, "visgpu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = [
    "scan.cu", "k_grid.cu", "k_aniso.cu", "k_band.cu", "k_field.cu", "k_mc.cu", "k_diffuse.cu",
    "mc_tables.cu", "pms_api.cpp", "host_io.cpp", "scan_noalloc.cu", "k_learn.cu", "pms_learn.cpp", "pms_batch.cpp", "pms_tune.cpp",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(src: str) -> list[str]:
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC,-O2", "-I" + os.path.join(HERE, "..", "include")]
    if src.endswith(".cu"):
        return ARCH + ["-lineinfo", "-Xptxas", "-O3"] + common
    return ["-x", "c++"] + common


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in ("pms_internal.h", "k_common.cuh")] + \
        [os.path.join(HERE, "..", "include", "pms.h")]
    gen = os.path.join(OUT, "gen", "mc_tables.inc")
    if os.path.exists(gen):
        deps.append(gen)
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return obj
    cmd = [nvcc(), "-c", path, "-o", obj] + _flags(src)
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    subprocess.run([sys.executable, os.path.join(HERE, "gen_mc_tables.py")], check=True,
                   stdout=subprocess.DEVNULL if not verbose else None)
    jobs = jobs or min(len(SOURCES), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc(), "-shared", "-o", LIB + ".tmp"] + ARCH + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    cli_src = os.path.join(CSRC, "visgpu.cpp")
    if os.path.exists(cli_src) and (not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(LIB),
                                                                                            os.path.getmtime(cli_src))):
        cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(HERE, "..", "include"), cli_src, "-o", CLI,
               "-L" + OUT, "-lpms", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI link failed\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
