"""Build the GB300 (sm_103a) solver library in-tree.

Compiles every translation unit under cfd__gb300/csrc with nvcc in parallel
and links cfd__gb300/_native/libcfdgb300.so.  No cmake, no torch extension
machinery: plain nvcc, one -gencode (compute_103a/sm_103a).

Every unit is built with -fmad=false and IEEE division and square root, so
each fp32 operation rounds where the source writes it: the lattice-Boltzmann
units then match the CPU oracle bit for bit, and the others (learned closure,
voxelizer, visualisation) fuse a multiply-add only where they call fmaf().
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
OUT_DIR = os.path.join(PKG, "_native")
LIB = os.path.join(OUT_DIR, "libcfdgb300.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BASE = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE,
               "--expt-relaxed-constexpr"]

# translation unit -> extra flags
UNITS = {
    "lbm_api.cu": ["-fmad=false"],
    "lbm_inst_f32.cu": ["-fmad=false"],
    "lbm_inst_f64.cu": ["-fmad=false"],
    "lbm_inst_f16s.cu": ["-fmad=false"],
    "lbm_inst_bf16s.cu": ["-fmad=false"],
    "lbm_inst_f16sr.cu": ["-fmad=false"],
    "lbm_inst_bf16sr.cu": ["-fmad=false"],
    "lbm_inst_f16sr_clo.cu": ["-fmad=false"],
    "lbm_inst_bf16sr_clo.cu": ["-fmad=false"],
    "lbm_inst_f32_clo.cu": ["-fmad=false"],
    "lbm_inst_f16s_clo.cu": ["-fmad=false"],
    "lbm_inst_bf16s_clo.cu": ["-fmad=false"],
    "vox.cu": ["-fmad=false"],
    "lbm_noalloc.cu": ["-fmad=false"],
    "lbm_batch.cu": ["-fmad=false"],
    "closure.cu": ["-fmad=false"],
    "vis.cu": ["-fmad=false"],
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the solver")
    return p


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit: str, flags, verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OBJ, unit.replace(".cu", ".o"))
    if not _stale(obj, [src] + _headers()):
        return obj
    cmd = [nvcc()] + BASE + flags + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile (when stale) and link the library; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    jobs = jobs or min(len(UNITS), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "--cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
