"""Builds the in-tree CUDA library libom_gb300.so for sm_103a with nvcc.

Each translation unit under csrc/ is compiled in parallel with
`-gencode arch=compute_103a,code=sm_103a`, then linked with -shared.
Outputs stay in the package directory (git-ignored)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libom_gb300.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
# Per-file flags.  hydro_exact.cu must round every operation as the
# generated C++ does: no multiply-add contraction, IEEE division and sqrt.
FILE_FLAGS = {
    "hydro_exact.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"],
    # the production FP32 step: approximate division/sqrt, flush-to-zero
    "hydro_fast.cu": ["-use_fast_math"],
    "hydro_persist.cu": ["-use_fast_math"],
    # single-precision fast math only: the FP64 adjoint stays IEEE
    "adjoint.cu": ["-use_fast_math"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build paraiso_gb300")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "om_gb300.h"))
    flags = NVCC_FLAGS + (extra_flags or [])
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers + [__file__]):
            jobs.append([nvcc(), *ARCH, *flags, *FILE_FLAGS.get(os.path.basename(src), []),
                         "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or _stale(OUT, objs):
        run([nvcc(), *ARCH, "-shared", "-o", OUT, *objs, "-lcudart", "-lnvrtc"])
    return OUT


if __name__ == "__main__":
    print(build(verbose=True))
