"""Build recipe of the CUDA library (liblsgb.so) for sm_103a.

Each translation unit under csrc/ is compiled in parallel with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``_build/liblsgb.so`` (git-ignored, in-tree).  f64_kernels.cu is compiled with
``--fmad=false`` so the FP64 path keeps the reference's rounding of every
multiply and add.  No torch, no cmake: one nvcc per file, then one link.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liblsgb.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]
# per-file extra flags
EXTRA = {
    "f64_kernels.cu": ["--fmad=false"],
    "sample_kernels.cu": ["--fmad=false"],
    "contour.cu": ["--fmad=false"],
    # host arithmetic of the forced velocity must not contract (aarch64 gcc would)
    "sample_api.cu": ["-Xcompiler", "-ffp-contract=off"],
}
SOURCES = ["api.cu", "f64_kernels.cu", "f32_kernels.cu", "reduce.cu", "synth.cu", "noalloc.cu", "stage3d_f32.cu",
           "stage2d_f32.cu", "adjoint.cu", "sample_kernels.cu", "sample_api.cu", "dump.cu", "diag.cu", "contour.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile csrc/*.cu and link _build/liblsgb.so; returns the library path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "lsgb.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [path, *headers]):
            cmd = [nvcc, *ARCH, *COMMON, *EXTRA.get(src, []), "-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
