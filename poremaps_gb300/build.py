"""Build the poremaps_gb300 native library and CLI in-tree (sm_103a only).

Outputs (git-ignored) in ``poremaps_gb300/_build/``:
  libporemaps_gb300.so   C ABI of include/poremaps.h (CUDA kernels + host runtime)
  poremaps_gpu           drop-in command-line program (``poremaps_gpu file.inp``)

Translation units are compiled in parallel with nvcc; no cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libporemaps_gb300.so")
CLI = os.path.join(OUT, "poremaps_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr"]

# (source, extra flags).  pm_kernels.cu holds the exact-arithmetic kernels and
# must not contract multiply-adds (bitwise parity with the reference CPU code).
UNITS = [
    ("pm_kernels.cu", ["-fmad=false"]),
    ("pm_fast.cu", []),
    ("pm_compact.cu", []),
    ("pm_zmarch.cu", []),
    ("pm_brick.cu", []),
    ("pm_api.cpp", []),
    ("pm_io.cpp", []),
    ("pm_server.cpp", []),
    ("pm_batch.cu", []),
    ("pm_noalloc.cu", []),
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    units = [(s, f) for s, f in UNITS if os.path.exists(os.path.join(CSRC, s))]
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda a: _compile(*a), units))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    cli_src = os.path.join(CSRC, "pm_cli.cpp")
    if os.path.exists(cli_src):
        cmd = [nvcc(), *ARCH, "-O2", "-std=c++17", cli_src, "-o", CLI, "-L" + OUT,
               "-lporemaps_gb300", "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
