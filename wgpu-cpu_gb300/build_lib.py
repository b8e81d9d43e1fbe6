"""Builds libgbr.so (the CUDA library behind include/gbr.h) in-tree for sm_103a.

    python wgpu-cpu_gb300/build_lib.py [--force]

Translation units are compiled in parallel with nvcc and linked into
wgpu-cpu_gb300/wgpu_gb300/libgbr.so.  Every kernel is built with --fmad=false (no multiply-add
contraction: the path reproduces wgpu-cpu's IEEE binary32 arithmetic bit for bit) and host code
with -ffp-contract=off for the same reason.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "wgpu_gb300")
LIB = os.path.join(OUT_DIR, "libgbr.so")
BUILD = os.path.join(HERE, "_build")

SOURCES = ["kernels.cu", "kernels_edge.cu", "runtime.cu", "jit.cu", "wgsl.cpp"]
# headers compiled again at run time by NVRTC for WGSL programs (embedded in the library)
JIT_HEADERS = ["gbr_types.h", "exact.cuh", "srgb_tables.h", "sampling.cuh", "programs.cuh", "raster.cuh",
               "raster_vis.cuh", "raster_lines.cuh", "wgsl_rt.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    # --fmad=false for the front end and for ptxas: no multiply-add contraction of scalar code
    return ["-std=c++17", "-O3", *ARCH, "-lineinfo", "--fmad=false", "-Xptxas", "--fmad=false",
            "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", BUILD]


def write_jit_sources() -> str:
    """jit_sources.inc: the kernel headers as raw string literals, with their names."""
    out = os.path.join(BUILD, "jit_sources.inc")
    parts = ["// generated by build_lib.py from csrc/: the headers NVRTC compiles with each WGSL program",
             "static const char* const kJitHeaderNames[] = {" + ", ".join(f'"{h}"' for h in JIT_HEADERS) + "};",
             "static const char* const kJitHeaders[] = {"]
    for h in JIT_HEADERS:
        text = open(os.path.join(CSRC, h)).read()
        if ")GBRJIT\"" in text:
            raise RuntimeError(f"{h} contains the raw-string delimiter")
        # split into pieces below the compiler's string-literal limit
        chunks = [text[i:i + 12000] for i in range(0, len(text), 12000)] or [""]
        parts.append("    " + "\n".join(f'R"GBRJIT({c})GBRJIT"' for c in chunks) + ",")
    parts.append("};")
    data = "\n".join(parts) + "\n"
    if not os.path.exists(out) or open(out).read() != data:
        with open(out, "w") as f:
            f.write(data)
    return out


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    write_jit_sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "gbr.h"))
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append([nvcc(), *_flags(), "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread", "-ldl"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
