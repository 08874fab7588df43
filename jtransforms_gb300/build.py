"""Builds libjtgpu.so (the CUDA library behind include/jtgpu.h) in-tree.

nvcc -gencode arch=compute_103a,code=sm_103a, one shared library; the object
files compile in parallel.  Called by __graft_entry__.build() and on import
when the library is missing.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "libjtgpu.so")
BUILD = os.path.join(PKG, "_build")
SOURCES = ["jt_engine.cu", "jt_pow2_f32.cu", "jt_pow2_f64.cu", "jt_tc_f32.cu", "jt_peak.cu", "jt_r2r_f32.cu",
           "jt_r2r_f64.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "jtgpu.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def comp(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, len(SOURCES))) as ex:
        results = list(ex.map(comp, SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            print(err)
    tmp = OUT + ".tmp"
    subprocess.check_call([cc, *ARCH, "-shared", *objs, "-o", tmp, "-lcudart"])
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    import sys
    build(force=True, verbose="-v" in sys.argv)
    print(OUT)
