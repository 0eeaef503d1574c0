"""Build recipe of libfa2cuda.so (in-tree, for sm_103a only).

Each translation unit is compiled by nvcc in parallel, with the flags of its
precision, then linked into ``forceatlas2_rc_gb300/libfa2cuda.so`` with the
CUDA runtime linked statically (the library needs only the driver at run
time). Rebuilds only what changed. Usable as ``python -m
forceatlas2_rc_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfa2cuda.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                 "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off"]

# translation unit -> extra flags
UNITS = {
    "api.cu": [],
    "sort_tree.cu": [],
    # FP32 path: FMA contraction, approximate division and square root
    "inst_f32.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
    # FP64 path: no contraction, IEEE division / square root (parity with the
    # reference's src/forceatlas2.c)
    "inst_f64.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"],
    # the allocation-free Morton order (FP32 positions)
    "noalloc.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
    # the layout server (host threads over the layouts of both precisions)
    "server.cu": [],
    # graph preparation on the device (integer work and IEEE double
    # coefficients, as the reference's host code)
    "prep.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build "
                       "libfa2cuda.so")


def _deps_mtime() -> float:
    files = glob.glob(os.path.join(CSRC, "*")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h")) + [__file__]
    return max(os.path.getmtime(f) for f in files)


def _compile(unit: str, extra: list[str], verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OBJ, unit.replace(".cu", ".o"))
    cmd = [nvcc()] + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link libfa2cuda.so if it is missing or out of date;
    return its path."""
    os.makedirs(OBJ, exist_ok=True)
    newest = _deps_mtime()
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose),
                           UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"linking libfa2cuda.so failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
