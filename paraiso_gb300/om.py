"""Python host side of the GB300 Orthotope Machine runtime.

Mirrors the class Paraiso's generator prints per OM
(Language/Paraiso/Generator/PlanTrans.hs:51-277): a constructor taking the
mesh size, `om_size*` / `om_memory_size*` / margin accessors, one accessor
per static variable, and one method per kernel (`init`, `proceed`).  Every
call goes through the C ABI of include/om_gb300.h in libom_gb300.so; there
is no other compute path, and constructing an object fails loudly when the
library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libom_gb300.so")

OM_OK = 0
KIND_LIFE = 1
KIND_HYDRO = 2
KIND_GRAPH = 3
CYCLIC = 0
OPEN = 1

STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_UNSUPPORTED", 4: "ERR_NOMEM",
          5: "ERR_NONFINITE", 6: "ERR_TIMEOUT", 7: "ERR_STATE"}

# every entry point declared in include/om_gb300.h
EXPORTS = [
    "om_config_default", "om_last_error", "om_version", "om_create", "om_destroy",
    "om_size", "om_memory_size", "om_lower_margin", "om_upper_margin",
    "om_kernel_id", "om_run", "om_run_n", "om_scalar_ptr", "om_array_host",
    "om_array_host_const", "om_array_device", "om_array_read", "om_array_write",
    "om_life_fill_random", "om_life_population_history", "om_hydro_init_kh",
    "om_hydro_totals", "om_hydro_dt_history", "om_time_run", "om_last_launch_count",
    "om_profile_enable", "om_profile_query",
    "om_ensemble_create", "om_ensemble_destroy", "om_ensemble_info", "om_ensemble_init_kh",
    "om_ensemble_step", "om_ensemble_time_step", "om_ensemble_read", "om_ensemble_write",
    "om_ensemble_scalar", "om_ensemble_set_scalar", "om_ensemble_totals",
    "om_ensemble_last_launch_count", "om_life_proceed_noalloc", "om_autotune",
    "om_autotune_ensemble", "om_hydro_vjp", "om_hydro_adjoint_run", "om_hydro_time_vjp",
    "om_hydro_time_tape", "om_hydro_forward", "om_hydro_backward", "om_hydro_tape_free", "om_create_graph",
    "om_graph_source", "om_graph_check", "om_save", "om_load", "om_hydro_write_snapshot",
    "om_selftest_wait_bound",
]


class OMError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("boundary", C.c_int), ("precision", C.c_int), ("gamma", C.c_double),
                ("device", C.c_int), ("depth", C.c_int), ("tile_x", C.c_int),
                ("tile_y", C.c_int), ("use_graph", C.c_int), ("variant", C.c_int),
                ("life_io", C.c_int), ("life_kernel", C.c_int), ("grid_limit", C.c_int),
                ("reserved", C.c_int * 4)]


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load libom_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: build it with paraiso_gb300.build.build()")
    L = C.CDLL(p)
    vp, i, ip = C.c_void_p, C.c_int, C.POINTER(C.c_int)
    sig = {
        "om_config_default": (None, [C.POINTER(Config)]),
        "om_last_error": (C.c_char_p, []),
        "om_version": (C.c_char_p, []),
        "om_create": (i, [i, i, ip, C.POINTER(Config), C.POINTER(vp)]),
        "om_destroy": (i, [vp]),
        "om_size": (i, [vp, i, ip]),
        "om_memory_size": (i, [vp, i, ip]),
        "om_lower_margin": (i, [vp, i, ip]),
        "om_upper_margin": (i, [vp, i, ip]),
        "om_kernel_id": (i, [vp, C.c_char_p, ip]),
        "om_run": (i, [vp, i]),
        "om_run_n": (i, [vp, i, i]),
        "om_scalar_ptr": (i, [vp, C.c_char_p, C.POINTER(vp), ip]),
        "om_array_host": (i, [vp, C.c_char_p, C.POINTER(vp), C.POINTER(C.c_size_t), ip]),
        "om_array_host_const": (i, [vp, C.c_char_p, C.POINTER(vp), C.POINTER(C.c_size_t), ip]),
        "om_array_device": (i, [vp, C.c_char_p, C.POINTER(vp)]),
        "om_array_read": (i, [vp, C.c_char_p, vp, C.c_size_t]),
        "om_array_write": (i, [vp, C.c_char_p, vp, C.c_size_t]),
        "om_life_fill_random": (i, [vp, C.c_uint64, C.c_double]),
        "om_life_population_history": (i, [vp, vp, i, ip]),
        "om_hydro_init_kh": (i, [vp, C.c_uint64]),
        "om_hydro_totals": (i, [vp, vp]),
        "om_hydro_dt_history": (i, [vp, vp, i, ip]),
        "om_time_run": (i, [vp, i, i, C.POINTER(C.c_float)]),
        "om_last_launch_count": (i, [vp, ip]),
        "om_profile_enable": (i, [vp, i]),
        "om_ensemble_create": (i, [i, ip, C.POINTER(Config), C.POINTER(vp)]),
        "om_ensemble_destroy": (i, [vp]),
        "om_ensemble_info": (i, [vp, ip, C.POINTER(C.c_longlong), ip, ip]),
        "om_ensemble_init_kh": (i, [vp, C.c_uint64]),
        "om_ensemble_step": (i, [vp, i]),
        "om_ensemble_time_step": (i, [vp, i, C.POINTER(C.c_float)]),
        "om_ensemble_read": (i, [vp, i, C.c_char_p, vp, C.c_size_t]),
        "om_ensemble_write": (i, [vp, i, C.c_char_p, vp, C.c_size_t]),
        "om_ensemble_scalar": (i, [vp, i, C.c_char_p, C.POINTER(C.c_double)]),
        "om_ensemble_set_scalar": (i, [vp, i, C.c_char_p, C.c_double]),
        "om_ensemble_totals": (i, [vp, i, vp]),
        "om_ensemble_last_launch_count": (i, [vp, ip]),
        "om_autotune": (i, [i, i, ip, C.POINTER(Config), C.POINTER(Config),
                            C.POINTER(C.c_double)]),
        "om_autotune_ensemble": (i, [i, ip, C.POINTER(Config), C.POINTER(Config),
                                     C.POINTER(C.c_double)]),
        "om_hydro_vjp": (i, [vp, C.POINTER(vp), C.POINTER(vp)]),
        "om_hydro_adjoint_run": (i, [vp, i, vp, i, C.POINTER(C.c_double), C.POINTER(vp)]),
        "om_hydro_time_vjp": (i, [vp, i, C.POINTER(C.c_float)]),
        "om_hydro_time_tape": (i, [vp, i, C.POINTER(C.c_float)]),
        "om_hydro_forward": (i, [vp, i, i, C.POINTER(vp)]),
        "om_hydro_backward": (i, [vp, vp, C.POINTER(vp), C.POINTER(vp)]),
        "om_hydro_tape_free": (i, [vp]),
        "om_create_graph": (i, [C.c_char_p, vp, C.POINTER(vp)]),
        "om_graph_source": (i, [vp, C.POINTER(C.c_char_p)]),
        "om_graph_check": (i, [C.c_char_p, i, i, C.POINTER(C.c_char_p)]),
        "om_save": (i, [vp, C.c_char_p]),
        "om_load": (i, [vp, C.c_char_p]),
        "om_hydro_write_snapshot": (i, [vp, C.c_char_p]),
        "om_selftest_wait_bound": (i, [i]),
        "om_profile_query": (i, [vp, C.c_char_p, C.POINTER(C.c_long), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = L
    return L


def _check(status: int) -> None:
    if status != OM_OK:
        msg = load_library().om_last_error().decode(errors="replace")
        raise OMError(status, msg)


def default_config(**kw) -> Config:
    cfg = Config()
    load_library().om_config_default(C.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


class OrthotopeMachine:
    """One generated OM class instance backed by a device handle."""

    kind = 0
    array_dtypes: dict[str, type] = {}

    def __init__(self, size: tuple[int, int], config: Config | None = None, **kw):
        L = load_library()
        self._L = L
        cfg = config if config is not None else default_config(**kw)
        sizes = (C.c_int * 2)(int(size[0]), int(size[1]))
        h = C.c_void_p()
        _check(L.om_create(self.kind, 2, sizes, C.byref(cfg), C.byref(h)))
        self._h = h
        self.config = cfg
        self._kid: dict[str, int] = {}

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.om_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- sizes (PlanTrans.hs:167-215)
    def _q(self, fn, axis: int) -> int:
        out = C.c_int()
        _check(fn(self._h, axis, C.byref(out)))
        return out.value

    def om_size(self, axis: int = -1) -> int:
        return self._q(self._L.om_size, axis)

    def om_memory_size(self, axis: int = -1) -> int:
        return self._q(self._L.om_memory_size, axis)

    def om_lower_margin(self, axis: int) -> int:
        return self._q(self._L.om_lower_margin, axis)

    def om_upper_margin(self, axis: int) -> int:
        return self._q(self._L.om_upper_margin, axis)

    @property
    def memory_shape(self) -> tuple[int, int]:
        return (self.om_memory_size(1), self.om_memory_size(0))

    # -- kernels (PlanTrans.hs:225-277)
    def kernel_id(self, name: str) -> int:
        if name not in self._kid:
            out = C.c_int()
            _check(self._L.om_kernel_id(self._h, name.encode(), C.byref(out)))
            self._kid[name] = out.value
        return self._kid[name]

    def run(self, name: str, n: int = 1) -> None:
        if n == 1:
            _check(self._L.om_run(self._h, self.kernel_id(name)))
        else:
            _check(self._L.om_run_n(self._h, self.kernel_id(name), int(n)))

    def time_run(self, name: str, n: int) -> float:
        """Device time (ms, CUDA events on the handle's stream) of n steps."""
        ms = C.c_float()
        _check(self._L.om_time_run(self._h, self.kernel_id(name), int(n), C.byref(ms)))
        return ms.value

    def last_launch_count(self) -> int:
        out = C.c_int()
        _check(self._L.om_last_launch_count(self._h, C.byref(out)))
        return out.value

    def profile(self, enable: bool = True) -> None:
        _check(self._L.om_profile_enable(self._h, int(enable)))

    def profile_query(self, kernel: str) -> tuple[int, float, float]:
        """(launches, total device ms, total cell-updates) of one kernel."""
        n = C.c_long()
        ms = C.c_double()
        u = C.c_double()
        _check(self._L.om_profile_query(self._h, kernel.encode(), C.byref(n), C.byref(ms), C.byref(u)))
        return n.value, ms.value, u.value

    # -- statics (PlanTrans.hs:117-157)
    def _scalar(self, name: str):
        p = C.c_void_p()
        t = C.c_int()
        _check(self._L.om_scalar_ptr(self._h, name.encode(), C.byref(p), C.byref(t)))
        ctype = {0: C.c_int32, 1: C.c_double, 2: C.c_float}[t.value]
        return C.cast(p, C.POINTER(ctype))

    def get_scalar(self, name: str):
        return self._scalar(name)[0]

    def set_scalar(self, name: str, value) -> None:
        self._scalar(name)[0] = value

    def array(self, name: str) -> np.ndarray:
        """Writable host mirror (memory-sized, [y, x]); marks the host newer."""
        p = C.c_void_p()
        n = C.c_size_t()
        es = C.c_int()
        _check(self._L.om_array_host(self._h, name.encode(), C.byref(p), C.byref(n), C.byref(es)))
        dt = self.array_dtypes[name]
        buf = (C.c_char * (n.value * es.value)).from_address(p.value)
        return np.frombuffer(buf, dtype=dt).reshape(self.memory_shape)

    def read(self, name: str) -> np.ndarray:
        """Copy of an array (memory-sized, [y, x])."""
        dt = self.array_dtypes[name]
        out = np.empty(self.memory_shape, dtype=dt)
        _check(self._L.om_array_read(self._h, name.encode(), out.ctypes.data, out.nbytes))
        return out

    def write(self, name: str, values: np.ndarray) -> None:
        dt = self.array_dtypes[name]
        a = np.ascontiguousarray(values, dtype=dt)
        if a.shape != self.memory_shape:
            raise ValueError(f"{name}: expected shape {self.memory_shape}, got {a.shape}")
        _check(self._L.om_array_write(self._h, name.encode(), a.ctypes.data, a.nbytes))

    def write_from_pointer(self, name: str, ptr: int, nbytes: int) -> None:
        _check(self._L.om_array_write(self._h, name.encode(), C.c_void_p(ptr), nbytes))

    def read_to_pointer(self, name: str, ptr: int, nbytes: int) -> None:
        _check(self._L.om_array_read(self._h, name.encode(), C.c_void_p(ptr), nbytes))

    def save(self, path) -> None:
        """Binary checkpoint of every static (om_save)."""
        _check(self._L.om_save(self._h, str(path).encode()))

    def load(self, path) -> None:
        """Restore a checkpoint written by save (om_load)."""
        _check(self._L.om_load(self._h, str(path).encode()))

    def device_pointer(self, name: str) -> int:
        p = C.c_void_p()
        _check(self._L.om_array_device(self._h, name.encode(), C.byref(p)))
        return p.value


class Life(OrthotopeMachine):
    """examples/Life: cell (Array Int), population, generation (Scalar Int)."""

    kind = KIND_LIFE
    array_dtypes = {"cell": np.int32}

    def __init__(self, size=(80, 48), config: Config | None = None, **kw):
        super().__init__(size, config, **kw)

    def init(self) -> None:
        self.run("init")

    def proceed(self, n: int = 1) -> None:
        self.run("proceed", n)

    @property
    def population(self) -> int:
        return self.get_scalar("population")

    @property
    def generation(self) -> int:
        return self.get_scalar("generation")

    @generation.setter
    def generation(self, v: int) -> None:
        self.set_scalar("generation", v)

    def fill_random(self, seed: int, p: float = 0.3) -> None:
        _check(self._L.om_life_fill_random(self._h, C.c_uint64(seed), p))

    def population_history(self, n: int) -> np.ndarray:
        out = np.zeros(max(n, 1), np.int32)
        w = C.c_int()
        _check(self._L.om_life_population_history(self._h, out.ctypes.data, n, C.byref(w)))
        return out[: w.value]


class Hydro(OrthotopeMachine):
    """examples/Hydro: density, velocity0, velocity1, pressure (Array Real);
    generation (Int), time, cfl, dR0, dR1, extent0, extent1 (Scalar Real)."""

    kind = KIND_HYDRO

    def __init__(self, size=(1024, 1024), config: Config | None = None, **kw):
        super().__init__(size, config, **kw)
        dt = np.float64 if self.config.precision == 64 else np.float32
        self.array_dtypes = {k: dt for k in ("density", "velocity0", "velocity1", "pressure")}

    def init(self) -> None:
        self.run("init")

    def proceed(self, n: int = 1) -> None:
        self.run("proceed", n)

    def write_snapshot(self, path) -> None:
        """The text snapshot of examples/Hydro/main-kh.cpp (om_hydro_write_snapshot)."""
        _check(self._L.om_hydro_write_snapshot(self._h, str(path).encode()))

    def init_kh(self, seed: int) -> None:
        _check(self._L.om_hydro_init_kh(self._h, C.c_uint64(seed)))

    def totals(self) -> np.ndarray:
        out = np.zeros(4, np.float64)
        _check(self._L.om_hydro_totals(self._h, out.ctypes.data))
        return out

    def dt_history(self, n: int) -> np.ndarray:
        out = np.zeros(max(n, 1), np.float64)
        w = C.c_int()
        _check(self._L.om_hydro_dt_history(self._h, out.ctypes.data, n, C.byref(w)))
        return out[: w.value]

    def state(self) -> tuple[np.ndarray, ...]:
        return tuple(self.read(k) for k in ("density", "velocity0", "velocity1", "pressure"))

    # -- adjoint (om_hydro_vjp / om_hydro_adjoint_run)
    def _dev(self, arrays):
        import torch
        dt = torch.float64 if self.config.precision == 64 else torch.float32
        return [torch.as_tensor(np.ascontiguousarray(a, self.array_dtypes["density"]),
                                dtype=dt).cuda() for a in arrays]

    def vjp(self, cot_next):
        """Cotangent of the current state from the cotangent of the state after
        one proceed (four memory-sized arrays)."""
        import torch
        src = self._dev(cot_next)
        dst = [torch.empty_like(src[0]) for _ in range(4)]
        torch.cuda.synchronize()
        a = (C.c_void_p * 4)(*[t.data_ptr() for t in src])
        b = (C.c_void_p * 4)(*[t.data_ptr() for t in dst])
        _check(self._L.om_hydro_vjp(self._h, a, b))
        return tuple(t.cpu().numpy() for t in dst)

    def adjoint_run(self, steps: int, target, checkpoint_every: int = 0):
        """(loss, gradient) of mean((density_T - target)^2) over `steps` steps
        w.r.t. the current state; the handle ends at step T."""
        dt = self.array_dtypes["density"]
        tgt = np.ascontiguousarray(target, dt)
        grads = [np.empty(self.memory_shape, dt) for _ in range(4)]
        ptrs = (C.c_void_p * 4)(*[g.ctypes.data for g in grads])
        loss = C.c_double()
        _check(self._L.om_hydro_adjoint_run(self._h, int(steps), tgt.ctypes.data,
                                            int(checkpoint_every), C.byref(loss), ptrs))
        return loss.value, tuple(grads)

    def forward(self, steps: int, checkpoint_every: int = 0) -> "HydroTape":
        """Run `steps` steps keeping checkpoints (om_hydro_forward); the tape
        then maps any cotangent of the final state back (HydroTape.backward)."""
        t = C.c_void_p()
        _check(self._L.om_hydro_forward(self._h, int(steps), int(checkpoint_every), C.byref(t)))
        return HydroTape(self, t)

    def backward(self, tape: "HydroTape", cot_final):
        """dL/d(start state) of a tape from dL/d(final state) (four
        memory-sized arrays: density, velocity0, velocity1, pressure)."""
        dt = self.array_dtypes["density"]
        cots = [np.ascontiguousarray(c, dt) for c in cot_final]
        if len(cots) != 4 or any(c.shape != tuple(self.memory_shape) for c in cots):
            raise ValueError("backward: four arrays of the memory shape")
        grads = [np.empty(self.memory_shape, dt) for _ in range(4)]
        a = (C.c_void_p * 4)(*[c.ctypes.data for c in cots])
        b = (C.c_void_p * 4)(*[g.ctypes.data for g in grads])
        _check(self._L.om_hydro_backward(self._h, tape._t, a, b))
        return tuple(grads)

    def time_vjp(self, reps: int = 5) -> float:
        """Device ms of one adjoint step (the reverse sweep from its tape)."""
        ms = C.c_float()
        _check(self._L.om_hydro_time_vjp(self._h, int(reps), C.byref(ms)))
        return ms.value

    def time_tape(self, reps: int = 5) -> float:
        """Device ms of one taped forward step (the backward pass's recompute)."""
        ms = C.c_float()
        _check(self._L.om_hydro_time_tape(self._h, int(reps), C.byref(ms)))
        return ms.value

    def set_state(self, st) -> None:
        for k, v in zip(("density", "velocity0", "velocity1", "pressure"), st):
            self.write(k, v)


def ensemble_sizes(count: int, seed: int, lo: int = 256, hi: int = 2048, step: int = 32):
    """Instance sizes (n0, n1) drawn uniformly from the multiples of `step` in
    [lo, hi] with the library's counter hash: n = step * (lo/step + h % m)."""
    def mix(z):
        z &= (1 << 64) - 1
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & ((1 << 64) - 1)
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & ((1 << 64) - 1)
        return z ^ (z >> 31)
    m = (hi - lo) // step + 1
    out = []
    for k in range(count):
        h0 = mix(mix(seed) + (2 * k) * 0x9E3779B97F4A7C15)
        h1 = mix(mix(seed) + (2 * k + 1) * 0x9E3779B97F4A7C15)
        out.append((lo + step * (h0 % m), lo + step * (h1 % m)))
    return out


class GraphMachine(OrthotopeMachine):
    """A general Orthotope Machine from a graph (paraiso_gb300.omgraph.OM or
    its text), compiled into CUDA kernels for this GPU (om_create_graph).
    Kernels run by name: ``m.run("calculate")``; statics through
    ``read``/``write``/``array`` and ``get_scalar``/``set_scalar``.  A 1-D
    machine has arrays of shape (1, n0 + margins)."""

    kind = KIND_GRAPH
    _NP = {"int": np.int32, "float": np.float32, "double": np.float64, "bool": np.bool_}

    def __init__(self, graph, config: Config | None = None, **kw):
        L = load_library()
        self._L = L
        text = graph.to_text() if hasattr(graph, "to_text") else str(graph)
        cfg = config if config is not None else default_config(**kw)
        h = C.c_void_p()
        _check(L.om_create_graph(text.encode(), C.byref(cfg), C.byref(h)))
        self._h = h
        self.config = cfg
        self._kid = {}
        self.text = text
        self.array_dtypes = {}
        for line in text.splitlines():
            w = line.split()
            if w and w[0] == "static" and w[2] == "array":
                self.array_dtypes[w[1]] = self._NP[w[3]]

    @property
    def source(self) -> str:
        """The CUDA source generated for this machine."""
        p = C.c_char_p()
        _check(self._L.om_graph_source(self._h, C.byref(p)))
        return p.value.decode()


class HydroTape:
    """Checkpoints of one om_hydro_forward run, for om_hydro_backward."""

    def __init__(self, hydro: "Hydro", handle: C.c_void_p):
        self._hydro = hydro
        self._t = handle

    def backward(self, cot_final):
        if not self._t:
            raise OMError(1, "tape is closed")
        return self._hydro.backward(self, cot_final)

    def close(self) -> None:
        if self._t:
            self._hydro._L.om_hydro_tape_free(self._t)
            self._t = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """Batched Hydro: independent periodic grids of uneven sizes, one
    persistent launch per step (om_ensemble_* of include/om_gb300.h)."""

    FIELDS = ("density", "velocity0", "velocity1", "pressure")

    def __init__(self, sizes, config: Config | None = None, **kw):
        L = load_library()
        self._L = L
        cfg = config if config is not None else default_config(**kw)
        self.sizes = [(int(a), int(b)) for a, b in sizes]
        flat = (C.c_int * (2 * len(self.sizes)))(*[v for s in self.sizes for v in s])
        h = C.c_void_p()
        _check(L.om_ensemble_create(len(self.sizes), flat, C.byref(cfg), C.byref(h)))
        self._h = h
        self.config = cfg
        self.dtype = np.float64 if cfg.precision == 64 else np.float32

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.om_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        c, t, g, w = C.c_int(), C.c_longlong(), C.c_int(), C.c_int()
        _check(self._L.om_ensemble_info(self._h, C.byref(c), C.byref(t), C.byref(g), C.byref(w)))
        return {"count": c.value, "cells": t.value, "grid": g.value, "work_items": w.value}

    def init_kh(self, base_seed: int) -> None:
        _check(self._L.om_ensemble_init_kh(self._h, C.c_uint64(base_seed)))

    def step(self, n: int = 1) -> None:
        _check(self._L.om_ensemble_step(self._h, int(n)))

    def time_step(self, n: int) -> float:
        ms = C.c_float()
        _check(self._L.om_ensemble_time_step(self._h, int(n), C.byref(ms)))
        return ms.value

    def read(self, k: int, field: str) -> np.ndarray:
        n0, n1 = self.sizes[k]
        out = np.empty((n1, n0), self.dtype)
        _check(self._L.om_ensemble_read(self._h, k, field.encode(), out.ctypes.data, out.nbytes))
        return out

    def write(self, k: int, field: str, values) -> None:
        n0, n1 = self.sizes[k]
        a = np.ascontiguousarray(values, self.dtype).reshape(n1, n0)
        _check(self._L.om_ensemble_write(self._h, k, field.encode(), a.ctypes.data, a.nbytes))

    def write_from_pointer(self, k: int, field: str, ptr: int, nbytes: int) -> None:
        _check(self._L.om_ensemble_write(self._h, k, field.encode(), C.c_void_p(ptr), nbytes))

    def read_to_pointer(self, k: int, field: str, ptr: int, nbytes: int) -> None:
        _check(self._L.om_ensemble_read(self._h, k, field.encode(), C.c_void_p(ptr), nbytes))

    def state(self, k: int):
        return tuple(self.read(k, f) for f in self.FIELDS)

    def set_state(self, k: int, st) -> None:
        for f, v in zip(self.FIELDS, st):
            self.write(k, f, v)

    def scalar(self, k: int, name: str) -> float:
        v = C.c_double()
        _check(self._L.om_ensemble_scalar(self._h, k, name.encode(), C.byref(v)))
        return v.value

    def set_scalar(self, k: int, name: str, value: float) -> None:
        _check(self._L.om_ensemble_set_scalar(self._h, k, name.encode(), float(value)))

    def totals(self, k: int) -> np.ndarray:
        out = np.zeros(4, np.float64)
        _check(self._L.om_ensemble_totals(self._h, k, out.ctypes.data))
        return out

    def last_launch_count(self) -> int:
        v = C.c_int()
        _check(self._L.om_ensemble_last_launch_count(self._h, C.byref(v)))
        return v.value


def measure_rate(kind: str, size, config: Config, steps: int) -> float:
    """Cell-updates/s of one configuration measured as the tuner measures a
    candidate: a settling run, then the best of two timed runs of `steps`
    steps on the Bernoulli(0.3) / Kelvin-Helmholtz start of seed 1."""
    cls = {"life": Life, "hydro": Hydro}[kind]
    m = cls(size, config=config)
    try:
        if kind == "life":
            m.fill_random(1, 0.3)
        else:
            m.init_kh(1)
        m.time_run("proceed", steps)
        best = min(m.time_run("proceed", steps) for _ in range(2))
    finally:
        m.close()
    return size[0] * size[1] * steps / (best * 1e-3)


def ensemble_rate(sizes, config: Config, steps: int = 4) -> float:
    """Cell-updates/s of an ensemble configuration measured as
    om_autotune_ensemble measures a candidate."""
    e = Ensemble(sizes, config=config)
    try:
        e.init_kh(1)
        e.time_step(steps)
        best = min(e.time_step(steps) for _ in range(2))
    finally:
        e.close()
    return sum(a * b for a, b in sizes) * steps / (best * 1e-3)


def autotune(kind: str, size, **base) -> tuple[Config, float]:
    """Fastest launch configuration for a Life or Hydro mesh of this size
    (om_autotune): returns (config, cell-updates/s)."""
    L = load_library()
    k = {"life": KIND_LIFE, "hydro": KIND_HYDRO}[kind]
    cfg = default_config(**base)
    best = Config()
    rate = C.c_double()
    sizes = (C.c_int * 2)(int(size[0]), int(size[1]))
    _check(L.om_autotune(k, 2, sizes, C.byref(cfg), C.byref(best), C.byref(rate)))
    return best, rate.value


def autotune_ensemble(sizes, **base) -> tuple[Config, float]:
    L = load_library()
    cfg = default_config(**base)
    best = Config()
    rate = C.c_double()
    flat = (C.c_int * (2 * len(sizes)))(*[int(v) for s in sizes for v in s])
    _check(L.om_autotune_ensemble(len(sizes), flat, C.byref(cfg), C.byref(best), C.byref(rate)))
    return best, rate.value
