"""Build liblbm_gpu.so (sm_103a) in-tree: lbc_gb300/_build/liblbm_gpu.so.

Translation units are compiled in parallel with nvcc:
  kernels_exact.cu    --fmad=false (lbc's FP64 rounding sequence, bit for bit)
  kernels_shifted.cu  FP32/FP16 shifted-storage kernels (--fmad=false as well: FMAs
                      are written out, so every kernel rounds a node the same way)
  engine.cpp, dropin.cpp  host code (-ffp-contract=off: same host arithmetic on
                          x86-64 and aarch64)
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
LIB = os.path.join(OUT, "liblbm_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = [
    ("kernels_exact.cu", ["-O3", "-lineinfo", "--fmad=false"] + ARCH),
    ("kernels_shifted.cu", ["-O3", "-lineinfo", "--fmad=false"] + ARCH),
    ("engine.cpp", ["-O2"]),
    ("dropin.cpp", ["-O2"]),
    ("server.cpp", ["-O2"]),
    ("tune.cpp", ["-O2"]),
    ("io.cu", ["-O3", "-lineinfo"] + ARCH),
    ("noalloc.cu", ["-O3", "-lineinfo", "--fmad=false"] + ARCH),
]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _compile(unit, flags):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, unit + ".o")
    cmd = [nvcc(), "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC] + flags + \
          ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{r.stderr}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for n in os.listdir(d):
            if os.path.getmtime(os.path.join(d, n)) > t:
                return True
    return os.path.getmtime(__file__) > t


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-cudart", "static"] + ARCH + objs + ["-o", tmp, "-ldl", "-lpthread",
                                                                    "-Xlinker", "--no-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
