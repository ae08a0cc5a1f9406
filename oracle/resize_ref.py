"""Resize the reference's pre-generated Life / Hydro classes to another
square mesh, and time them.

TEST INFRASTRUCTURE ONLY (part of the oracle): it reads the reference tree
and writes under oracle/_ref/ (git-ignored), never into the product.

The generator bakes the mesh into the emitted class (Native.localSize;
PlanTrans.hs:75-86, 167-215): the loop bounds over the cells and over the
memory array, the `% W` / `/ W` splits of a loop index, the row pitch of
`addr_origin`, every neighbour offset K = dy * ms0 + dx of a shifted read
(|dx|, |dy| <= the margin; PlanTrans.hs:468-484, 561-563), the LoadSize
literals and the size accessors of the header.  For a square resize these
values are all distinct in the source (n, ms0 = n + 2 lm, n^2, ms0^2 and the
offsets), so each integer literal is mapped by value:

  n -> n',  ms0 -> ms0',  n^2 -> n'^2,  ms0^2 -> ms0'^2,
  K = dy ms0 + dx (1 <= |dy| <= lm, |dx| <= lm) -> dy ms0' + dx,

and every other literal (the margins, small offsets, constants) is kept.
Checks: resizing to the original size reproduces the files byte for byte,
a round trip through another size does too, and tests/test_oracle.py runs
resized classes against the oracle at other sizes.

  python oracle/resize_ref.py --kind life --size 16384        # writes _ref/
  python oracle/resize_ref.py --time                          # builds, times
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")

# the pre-generated classes: directory under the reference tree, class
# name, mesh size and margin as generated
KINDS = {
    "life": ("examples-old/Life-exampled/dist", "Life", 128, 1),
    "hydro": ("examples-old/Hydro-exampled/dist", "Hydro", 1024, 3),
}

_INT = re.compile(r"(?<![\w.])(-?\d+)(?![\w.])")


def reference_tree() -> str:
    r = subprocess.run(["make", "-s", "-C", HERE, "ref-path"], capture_output=True, text=True,
                       check=True)
    return r.stdout.strip()


def literal_map(n: int, lm: int, n_new: int) -> dict[int, int]:
    ms, ms_new = n + 2 * lm, n_new + 2 * lm
    m = {n: n_new, ms: ms_new, n * n: n_new * n_new, ms * ms: ms_new * ms_new}
    for dy in range(-lm, lm + 1):
        if dy == 0:
            continue
        for dx in range(-lm, lm + 1):
            k = dy * ms + dx
            assert k not in m or m[k] == dy * ms_new + dx, "ambiguous literal"
            m[k] = dy * ms_new + dx
    return m


def resize_text(text: str, n: int, lm: int, n_new: int) -> str:
    m = literal_map(n, lm, n_new)

    def sub(mo):
        v = int(mo.group(1))
        return str(m[v]) if v in m else mo.group(1)
    return _INT.sub(sub, text)


def resize(kind: str, n_new: int, out_dir: str | None = None) -> str:
    """Write the resized .hpp/.cpp of `kind` into out_dir (default
    _ref/<kind>_<n_new>/); returns the directory."""
    sub, name, n, lm = KINDS[kind]
    src = os.path.join(reference_tree(), sub)
    out = out_dir or os.path.join(REF_OUT, f"{kind}_{n_new}")
    os.makedirs(out, exist_ok=True)
    for ext in ("hpp", "cpp"):
        with open(os.path.join(src, f"{name}.{ext}")) as f:
            text = f.read()
        with open(os.path.join(out, f"{name}.{ext}"), "w") as f:
            f.write(resize_text(text, n, lm, n_new))
    return out


def check_identity(kind: str, via: int) -> bool:
    """Resizing to the original size, and to `via` and back, reproduce the
    generated files byte for byte."""
    sub, name, n, lm = KINDS[kind]
    src = os.path.join(reference_tree(), sub)
    for ext in ("hpp", "cpp"):
        with open(os.path.join(src, f"{name}.{ext}")) as f:
            text = f.read()
        if resize_text(text, n, lm, n) != text:
            return False
        there = resize_text(text, n, lm, via)
        if resize_text(there, via, lm, n) != text:
            return False
    return True


def build(kind: str, n_new: int, openmp: bool = False) -> str:
    """Compile the resized class with its C driver into a shared library;
    returns its path.  OpenMP builds rewrite the generated loop headers
    `for(int i = 0; (i) < (N) ; (i) += (1))`, which GCC rejects under
    -fopenmp, to `for(int i = 0; i < N; i += 1)` (same iterations)."""
    sub, name, n, lm = KINDS[kind]
    d = resize(kind, n_new)
    cpp = os.path.join(d, f"{name}.cpp")
    if openmp:
        with open(cpp) as f:
            text = f.read()
        text = re.sub(r"for\(int (\w+) = 0; \(\1\) < \((\d+)\) ; \(\1\) \+= \(1\)\)",
                      r"for(int \1 = 0; \1 < \2; \1 += 1)", text)
        cpp = os.path.join(d, f"{name}_omp.cpp")
        with open(cpp, "w") as f:
            f.write(text)
    lib = os.path.join(d, f"libref_{kind}{'_omp' if openmp else ''}.so")
    drv = os.path.join(HERE, "ref_drivers", f"{kind}_ref.cpp")
    cmd = ["g++", "-O3", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-shared",
           f"-I{d}", "-o", lib, drv, cpp]
    if openmp:
        cmd.insert(1, "-fopenmp")
    subprocess.run(cmd, check=True)
    return lib


def time_life(lib: str, n: int, gens: int) -> float:
    """Seconds of `gens` proceed() of the resized Life from its init()."""
    import ctypes as C
    L = C.CDLL(lib)
    L.ref_life_run.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    out = (C.c_int32 * ((n + 2) * (n + 2)))()
    t0 = time.perf_counter()
    L.ref_life_run(None, gens, out, None)
    return time.perf_counter() - t0


def time_hydro(lib: str, n: int, steps: int) -> float:
    import ctypes as C
    L = C.CDLL(lib)
    L.ref_hydro_run.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_void_p]
    out = (C.c_float * (4 * (n + 6) * (n + 6)))()
    t0 = time.perf_counter()
    L.ref_hydro_run(None, steps, C.c_float(0.4), out, None)
    return time.perf_counter() - t0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--kind", choices=sorted(KINDS))
    ap.add_argument("--size", type=int)
    ap.add_argument("--time", action="store_true",
                    help="build and time Life 16384^2 and Hydro 4096^2 (1 thread and all threads)")
    a = ap.parse_args()
    if a.kind and a.size:
        print(resize(a.kind, a.size))
    if a.time:
        for kind, n, units in (("life", 16384, 4), ("hydro", 4096, 1)):
            assert check_identity(kind, n)
            for omp in (False, True):
                lib = build(kind, n, openmp=omp)
                env_threads = os.environ.get("OMP_NUM_THREADS")
                f = time_life if kind == "life" else time_hydro
                f(lib, n, 1)  # first touch of the arrays
                s = f(lib, n, units)
                rate = n * n * units / s
                print(f"{kind} {n}x{n} {'OpenMP' if omp else '1 thread'} "
                      f"({env_threads or os.cpu_count()} threads available): "
                      f"{rate / 1e6:.1f} Mcell-updates/s ({units} steps, {s:.2f} s)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
