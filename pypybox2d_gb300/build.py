"""In-tree build of libgb2d.so for sm_103a (nvcc, no cmake).

Three translation units:
  gb_f64.cu  float64 step kernels, -fmad=false (bit-exact with the CPU restatement)
  gb_f32.cu  float32-bulk step kernels
  gb_api.cu  the C ABI (include/gb2d.h)
The two precision units are each compiled once per part (-DGB_PART=k, see
csrc/gb_kernels.cuh), so that 19 objects compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libgb2d.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-diag-suppress", "177,550"]
N_PARTS = 9
# (source, extra flags, object)
UNITS = [("gb_api.cu", [], "gb_api.o")] + [
    (src, [*flags, f"-DGB_PART={k}"], src.replace(".cu", f"_p{k}.o"))
    for src, flags in (("gb_f64.cu", ["-fmad=false"]), ("gb_f32.cu", []))
    for k in range(N_PARTS)
]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _sources() -> list[str]:
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))] + [
        os.path.join(os.path.dirname(PKG), "include", "gb2d.h")]


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libgb2d.so in-tree; returns its path."""
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()

    def compile_unit(item):
        src, extra, obj = item
        obj = os.path.join(OUT, obj)
        cmd = [nvcc, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(UNITS), max(2, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
