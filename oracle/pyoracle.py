"""ctypes view of the CPU oracle (liboracle.so) and of the reference's own
pre-generated classes (_ref/libref_*.so, present only where the reference
tree was available at build time).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
the CPU-baseline leg of bench.py, as the checker.  The product never imports
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class HydroShape(C.Structure):
    _fields_ = [("n0", C.c_int), ("n1", C.c_int), ("cyclic", C.c_int),
                ("gamma", C.c_double)]


def build(ref: str | None = None) -> None:
    """Compile liboracle.so (and _ref/ when the reference tree exists)."""
    args = ["make", "-s", "-C", HERE]
    if ref is not None:
        args.append(f"REF={ref}")
    subprocess.run(args, check=True)


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.oracle_hash64.restype = C.c_uint64
        L.oracle_hash64.argtypes = [C.c_uint64, C.c_uint64]
        L.oracle_hash_uniform_f32.argtypes = [C.c_uint64, C.c_size_t, C.c_double, C.c_double, _f32p]
        L.oracle_life_fill_bernoulli.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_double, _i32p]
        L.oracle_life_step.restype = C.c_int32
        L.oracle_life_step.argtypes = [C.c_int, C.c_int, C.c_int, _i32p, _i32p]
        L.oracle_life_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p, C.c_void_p]
        for suf, fp, R in (("f64", _f64p, C.c_double), ("f32", _f32p, C.c_float)):
            f = getattr(L, f"oracle_hydro_step_{suf}")
            f.restype = R
            f.argtypes = [HydroShape, R, R, R, R, R, C.POINTER(R), fp, fp, fp, fp]
            f = getattr(L, f"oracle_hydro_init_jet_{suf}")
            f.argtypes = [HydroShape, R, R, R, R, fp, fp, fp, fp]
            f = getattr(L, f"oracle_hydro_init_kh_{suf}")
            f.argtypes = [C.c_int, C.c_int, C.c_uint64, fp, fp, fp, fp]
            f = getattr(L, f"oracle_hydro_totals_{suf}")
            f.argtypes = [HydroShape, fp, fp, fp, fp, _f64p]
        L.oracle_hydro_step_tl_f64.restype = C.c_double
        L.oracle_hydro_step_tl_f64.argtypes = [HydroShape, C.c_double, C.c_double, C.c_double,
                                               C.POINTER(C.c_double)] + [_f64p] * 8
        L.oracle_num_threads.restype = C.c_int
        _lib = L
    return _lib


def hash_uniform_f32(seed: int, shape, lo: float, hi: float) -> np.ndarray:
    out = np.empty(shape, np.float32)
    lib().oracle_hash_uniform_f32(seed, out.size, lo, hi, out)
    return out


# ---- Life -----------------------------------------------------------------

def life_memory_shape(n0: int, n1: int, cyclic: bool) -> tuple[int, int]:
    lm = 0 if cyclic else 1
    return (n1 + 2 * lm, n0 + 2 * lm)


def life_bernoulli(n0: int, n1: int, seed: int, p: float = 0.3, cyclic: bool = True) -> np.ndarray:
    a = np.zeros(life_memory_shape(n0, n1, cyclic), np.int32)
    lib().oracle_life_fill_bernoulli(n0, n1, int(cyclic), seed, p, a)
    return a


def life_run(cell: np.ndarray, steps: int, cyclic: bool = True):
    """Returns (final memory array, populations[steps])."""
    lm = 0 if cyclic else 1
    n1, n0 = cell.shape[0] - 2 * lm, cell.shape[1] - 2 * lm
    c = np.ascontiguousarray(cell, np.int32).copy()
    pops = np.zeros(max(steps, 1), np.int32)
    lib().oracle_life_run(n0, n1, int(cyclic), steps, c, pops.ctypes.data)
    return c, pops[:steps]


# ---- Hydro ----------------------------------------------------------------

def hydro_shape(n0: int, n1: int, cyclic: bool, gamma: float) -> HydroShape:
    return HydroShape(n0, n1, int(cyclic), gamma)


def hydro_run(state, steps: int, *, cyclic: bool, gamma: float, cfl: float,
              dR=(None, None), extent=(1.0, 1.0), time: float = 0.0,
              dtype=np.float64):
    """Advance (rho, vx, vy, p) memory arrays `steps` times.

    Returns (new state tuple, time, list of dt)."""
    ms1, ms0 = state[0].shape
    lm = 0 if cyclic else 3
    n0, n1 = ms0 - 2 * lm, ms1 - 2 * lm
    R = C.c_double if dtype == np.float64 else C.c_float
    suf = "f64" if dtype == np.float64 else "f32"
    d0 = dR[0] if dR[0] is not None else np.array(extent[0], dtype) / dtype(n0)
    d1 = dR[1] if dR[1] is not None else np.array(extent[1], dtype) / dtype(n1)
    arrs = [np.ascontiguousarray(a, dtype).copy() for a in state]
    t = R(time)
    dts = []
    f = getattr(lib(), f"oracle_hydro_step_{suf}")
    sh = hydro_shape(n0, n1, cyclic, gamma)
    for _ in range(steps):
        dts.append(f(sh, R(cfl), R(float(d0)), R(float(d1)), R(extent[0]), R(extent[1]),
                     C.byref(t), *arrs))
    return tuple(arrs), t.value, dts


def hydro_init_kh(n0: int, n1: int, seed: int, dtype=np.float64):
    arrs = [np.zeros((n1, n0), dtype) for _ in range(4)]
    suf = "f64" if dtype == np.float64 else "f32"
    getattr(lib(), f"oracle_hydro_init_kh_{suf}")(n0, n1, seed, *arrs)
    return tuple(arrs)


def hydro_init_jet(n0: int, n1: int, *, cyclic: bool, gamma: float, dtype=np.float32,
                   extent=(1.0, 1.0)):
    lm = 0 if cyclic else 3
    arrs = [np.zeros((n1 + 2 * lm, n0 + 2 * lm), dtype) for _ in range(4)]
    suf = "f64" if dtype == np.float64 else "f32"
    R = C.c_double if dtype == np.float64 else C.c_float
    d0 = np.array(extent[0], dtype) / dtype(n0)
    d1 = np.array(extent[1], dtype) / dtype(n1)
    getattr(lib(), f"oracle_hydro_init_jet_{suf}")(hydro_shape(n0, n1, cyclic, gamma),
                                                   R(float(d0)), R(float(d1)),
                                                   R(extent[0]), R(extent[1]), *arrs)
    return tuple(arrs)


def hydro_totals(state, *, cyclic: bool, gamma: float) -> np.ndarray:
    ms1, ms0 = state[0].shape
    lm = 0 if cyclic else 3
    out = np.zeros(4, np.float64)
    dt = state[0].dtype
    suf = "f64" if dt == np.float64 else "f32"
    arrs = [np.ascontiguousarray(a) for a in state]
    getattr(lib(), f"oracle_hydro_totals_{suf}")(hydro_shape(ms0 - 2 * lm, ms1 - 2 * lm, cyclic, gamma),
                                                 *arrs, out)
    return out


def hydro_tl_run(state, dstate, steps: int, *, gamma: float, cfl: float, time: float = 0.0):
    """Tangent-linear FP64 run (cyclic): returns (state, dstate, time)."""
    ms1, ms0 = state[0].shape
    arrs = [np.ascontiguousarray(a, np.float64).copy() for a in state]
    darrs = [np.ascontiguousarray(a, np.float64).copy() for a in dstate]
    t = C.c_double(time)
    sh = hydro_shape(ms0, ms1, True, gamma)
    for _ in range(steps):
        lib().oracle_hydro_step_tl_f64(sh, cfl, 1.0 / ms0, 1.0 / ms1, C.byref(t), *arrs, *darrs)
    return tuple(arrs), tuple(darrs), t.value


def hydro_count_ops(n0: int, n1: int, seed: int, *, gamma: float, cfl: float) -> dict:
    """Operations of one FP step of the periodic Kelvin-Helmholtz start,
    counted on the restatement, per cell-update."""
    out = (C.c_longlong * 6)()
    lib().oracle_hydro_count_ops(n0, n1, C.c_uint64(seed), C.c_double(gamma),
                                 C.c_double(cfl), out)
    cells = n0 * n1
    names = ("add", "mul", "div", "sqrt", "cmp", "absneg")
    return {k: out[i] / cells for i, k in enumerate(names)}


# ---- the reference's own pre-generated classes ----------------------------

def ref_available() -> bool:
    return (os.path.exists(os.path.join(REF_DIR, "libref_life.so"))
            and os.path.exists(os.path.join(REF_DIR, "libref_hydro.so")))


_ref_life = None
_ref_hydro = None


def ref_life():
    global _ref_life
    if _ref_life is None:
        L = C.CDLL(os.path.join(REF_DIR, "libref_life.so"))
        L.ref_life_run.argtypes = [C.c_void_p, C.c_int, _i32p, C.c_void_p]
        _ref_life = L
    return _ref_life


def ref_hydro():
    global _ref_hydro
    if _ref_hydro is None:
        L = C.CDLL(os.path.join(REF_DIR, "libref_hydro.so"))
        L.ref_hydro_run.argtypes = [C.c_void_p, C.c_int, C.c_float, _f32p, C.c_void_p]
        _ref_hydro = L
    return _ref_hydro


def ref_life_run(initial: np.ndarray | None, steps: int):
    """Reference Life (128x128 open, memory 130x130).  Returns (cells, pops)."""
    out = np.zeros((130, 130), np.int32)
    pops = np.zeros(max(steps, 1), np.int32)
    ini = None
    if initial is not None:
        initial = np.ascontiguousarray(initial, np.int32)
        ini = initial.ctypes.data
    ref_life().ref_life_run(ini, steps, out, pops.ctypes.data)
    return out, pops[:steps]


def ref_hydro_run(initial, steps: int, cfl: float = 0.5):
    """Reference Hydro (1024x1024 float open, memory 1030x1030)."""
    n = 1030
    out = np.zeros((4, n, n), np.float32)
    times = np.zeros(max(steps, 1), np.float32)
    ini = None
    if initial is not None:
        initial = np.ascontiguousarray(np.stack(initial), np.float32)
        ini = initial.ctypes.data
    ref_hydro().ref_hydro_run(ini, steps, cfl, out, times.ctypes.data)
    return (out[0], out[1], out[2], out[3]), times[:steps]
