#!/usr/bin/env python3
"""Throughput benchmark of the GB300 Orthotope Machine kernels.

Default workload: Conway's Life (examples/Life) on a 16384x16384 cyclic grid,
int32 cells Bernoulli(0.3) from seed 1; one step = 100 generations with the
population reduce after every generation.  Metric: Gcell-updates/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload life16k|life128|lifegraph|hydro4k|hydrograph|ensemble|adjoint]

Prints one JSON line (rank 0).  Under torchrun (N > 1) every rank advances
its own independent replica (no data-path collective; weak scaling).
`--impl reference` times the CPU restatement of the reference's algorithm
(oracle/) on all host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


# ---------------------------------------------------------------------------
# process group (replicas only: barrier + max-over-ranks timing)
# ---------------------------------------------------------------------------

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# measurement helpers
# ---------------------------------------------------------------------------

def peaks() -> tuple[float, str]:
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows: list[list[str]] = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        time.sleep(0.25)

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = []
        mx = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_cores() -> int:
    return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

def life_workload(args, dist: Dist) -> dict:
    import paraiso_gb300 as pg
    from paraiso_gb300 import build as pgbuild
    pgbuild.build()
    n = args.size or (128 if args.workload == "life128" else 16384)
    gens = args.generations or (1000 if args.workload == "life128" else 100)
    cells = n * n
    life = pg.Life((n, n), device=dist.local_rank, depth=args.depth, tile_x=args.tile_x,
                   tile_y=args.tile_y, life_io=args.life_io)
    life.fill_random(1 + dist.rank, 0.3)
    kid = life.kernel_id("proceed")
    # warm-up
    for _ in range(args.warmup):
        life.run("proceed", gens)
    # timed region: K steps of `gens` generations, device time (CUDA events on
    # the handle's stream), barrier + synchronize on both sides
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    dist.barrier()
    ms = life.time_run("proceed", gens * args.steps)
    launches = life.last_launch_count()
    dist.barrier()
    clk = clocks.stop()
    ms = dist.max(ms)
    updates = cells * gens * args.steps * dist.world
    value = updates / (ms * 1e-3) / 1e9

    # dominant kernel: per-launch device time with events around each launch
    life.profile(True)
    life.time_run("proceed", gens * min(args.steps, 4))
    best = None
    for kn in ("life_reg_kernel", "life_ws_kernel", "life_tb32_kernel", "life_tb_kernel",
               "life_smallreg_kernel", "life_smallgrid_kernel", "life_general_kernel"):
        q = life.profile_query(kn)
        if q[0] and (best is None or q[1] > best[1][1]):
            best = (kn, q)
    kname, (nl, kms, kunits) = best
    life.profile(False)
    peak, peak_kind = peaks()
    bytes_per_update = 8.0           # int32 read + int32 write per cell-update
    per_launch_units = kunits / max(nl, 1)
    per_launch_ms = kms / max(nl, 1)
    achieved = bytes_per_update * per_launch_units / (per_launch_ms * 1e-3) / 1e9
    traffic = profile_traffic(kname, n)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1),
                "peak": peak, "peak_source": f"{peak_kind} MEASURED_PEAKS.json hbm_gbs"
                if peak_kind == "measured" else "fallback 6.8 TB/s",
                "unit": "GB/s", "frac": round(achieved / peak, 3),
                "traffic": traffic["bytes_per_launch"] if traffic else None,
                "algorithmic_bytes_per_launch": bytes_per_update * per_launch_units,
                "launch_ms": round(per_launch_ms, 4), "launches_profiled": nl,
                "note": "algorithmic 8 B per cell-update; temporal blocking re-uses each "
                        "loaded cell for several generations, so frac may exceed 1"}
    if traffic:
        roofline["dram_gbs"] = round(traffic["bytes_per_launch"] / (per_launch_ms * 1e-3) / 1e9, 1)
        roofline["dram_frac"] = round(roofline["dram_gbs"] / peak, 3)

    # end to end through the public API with host buffers: per step, upload
    # the cells from pinned host memory, run `gens` generations, read the
    # cells and the population back
    import torch
    host_in = torch.empty(cells, dtype=torch.int32).pin_memory()
    host_out = torch.empty(cells, dtype=torch.int32).pin_memory()
    life.read_to_pointer("cell", host_in.data_ptr(), cells * 4)
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    dist.barrier()
    t0 = time.perf_counter()
    pops = []
    for _ in range(e2e_steps):
        life.write_from_pointer("cell", host_in.data_ptr(), cells * 4)
        life.run("proceed", gens)
        life.read_to_pointer("cell", host_out.data_ptr(), cells * 4)
        pops.append(life.population)
    t1 = time.perf_counter()
    dist.barrier()
    e2e_s = dist.max(t1 - t0)
    e2e = {"value": round(cells * gens * e2e_steps * dist.world / e2e_s / 1e9, 3),
           "unit": "Gcell-updates/s", "h2d_bytes_per_step": cells * 4,
           "d2h_bytes_per_step": cells * 4 + 4, "steps": e2e_steps,
           "api": "om_array_write + om_run_n(proceed) + om_array_read + population scalar"}
    life.close()

    out = {
        "metric": "Life cell-updates/s (Gcell-updates/s), bit-exact vs the oracle",
        "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": f"life {n}x{n} cyclic, Bernoulli(0.3) seed 1+rank, "
                               f"{gens} generations per step, population reduce every generation",
                   "n0": n, "n1": n, "generations_per_step": gens,
                   "parallelism": f"replicas x{dist.world}",
                   "l2": f"inputs larger than L2 (2 x {cells * 4 / 2**20:.0f} MiB int32 buffers)"
                   if cells * 4 > 129 * 2**20
                   else "grid fits in L2; no flush (launch-bound case)"},
        "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = life_cpu_baseline(n, args)
    return out


def profile_traffic(kernel: str, n: int):
    """DRAM bytes per launch of `kernel` at grid size n, from the committed ncu
    summary profiles/<kernel>_traffic.txt ("key: value" lines)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_traffic.txt")
    try:
        d = {}
        with open(path) as f:
            for line in f:
                if ":" in line and not line.startswith("#"):
                    k, v = line.split(":", 1)
                    d[k.strip()] = v.strip()
        if int(d["n"]) == n:
            return {"bytes_per_launch": float(d["bytes_per_launch"]), "source": path}
    except Exception:
        pass
    return None


def lifegraph_workload(args, dist: Dist) -> dict:
    """examples/Life as a general OM graph (paraiso_gb300.omgraph), compiled
    at run time: the generic executor on the Life headline workload."""
    import paraiso_gb300 as pg
    from paraiso_gb300 import build as pgbuild
    from paraiso_gb300 import omgraph_examples as ex
    pgbuild.build()
    n = args.size or 16384
    gens = args.generations or 100
    cells = n * n
    m = pg.GraphMachine(ex.life((n, n)), device=dist.local_rank)
    life = pg.Life((n, n), device=dist.local_rank)       # the same Bernoulli(0.3) start
    life.fill_random(1 + dist.rank, 0.3)
    m.write("cell", life.read("cell"))
    life.close()
    m.run("proceed", gens)
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    dist.barrier()
    ms = m.time_run("proceed", gens * args.steps)
    launches = m.last_launch_count()
    dist.barrier()
    clk = clocks.stop()
    ms = dist.max(ms)
    value = cells * gens * args.steps * dist.world / (ms * 1e-3) / 1e9
    peak, _ = peaks()
    per_launch_ms = ms / (gens * args.steps)
    achieved = 8.0 * cells / (per_launch_ms * 1e-3) / 1e9
    traffic = profile_traffic("om_graph_life_stage", n)
    m.close()
    return {
        "metric": "Life cell-updates/s (Gcell-updates/s) through the general OM graph executor",
        "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": {"workload": f"examples/Life graph {n}x{n} cyclic, Bernoulli(0.3), {gens} "
                               "generations per step, one stage kernel per generation",
                   "n0": n, "n1": n, "parallelism": f"replicas x{dist.world}"},
        "roofline": {"bound": "hbm", "kernel": "om_k1_s0 (generated)", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 3),
                     "traffic": traffic["bytes_per_launch"] if traffic else None,
                     "algorithmic_bytes_per_launch": 8.0 * cells},
        "gpu_launches": launches, "clocks": clk,
    }


def hydrograph_workload(args, dist: Dist) -> dict:
    """examples/Hydro (HydroMain.hs with its Manifest annotations) as a
    general OM graph, compiled at run time, on the Hydro 4096^2 periodic
    Kelvin-Helmholtz workload in FP32.  Also checks a few steps against the
    hand-written exact FP32 step (both compute without multiply-add
    contraction in the generator's operation order)."""
    import numpy as np
    import paraiso_gb300 as pg
    from paraiso_gb300 import build as pgbuild
    from paraiso_gb300 import omgraph as og
    from paraiso_gb300 import omgraph_examples as ex
    pgbuild.build()
    n = args.size or 4096
    cells = n * n
    h = pg.Hydro((n, n), precision=32, variant=2, gamma=1.4, device=dist.local_rank)
    h.init_kh(1 + dist.rank)
    h.set_scalar("cfl", 0.4)
    st = h.state()
    m = pg.GraphMachine(ex.hydro((n, n), 1.4, "cyclic", og.Float), device=dist.local_rank)
    f = np.float32
    for name, v in (("cfl", f(0.4)), ("dR0", f(1) / f(n)), ("dR1", f(1) / f(n)),
                    ("extent0", f(1)), ("extent1", f(1)), ("time", f(0))):
        m.set_scalar(name, float(v))
    for name, a in zip(("density", "velocity0", "velocity1", "pressure"), st):
        m.write(name, a)
    check = 5
    m.run("proceed", check)
    h.proceed(check)
    same = all(np.array_equal(m.read(k), a)
               for k, a in zip(("density", "velocity0", "velocity1", "pressure"), h.state()))
    h.close()
    m.run("proceed", max(args.warmup, 1))
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    dist.barrier()
    ms = m.time_run("proceed", args.steps)
    launches = m.last_launch_count()
    dist.barrier()
    clk = clocks.stop()
    ms = dist.max(ms)
    value = cells * args.steps * dist.world / (ms * 1e-3) / 1e9
    peak, _ = peaks()
    achieved = 32.0 * cells / (ms / args.steps * 1e-3) / 1e9
    m.close()
    return {
        "metric": "Hydro cell-updates/s (Gcell-updates/s) through the general OM graph executor",
        "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"examples/Hydro graph (HydroMain.hs, Manifest annotations) {n}x{n} "
                               "periodic Kelvin-Helmholtz, gamma 1.4, CFL 0.4, FP32",
                   "n0": n, "n1": n, "parallelism": f"replicas x{dist.world}"},
        "bit_identical_to_exact_fused_step": {"steps": check, "equal": bool(same)},
        "roofline": {"bound": "hbm", "kernel": "om_k1_s* (generated)", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 3),
                     "traffic": None, "algorithmic_bytes_per_launch": 32.0 * cells,
                     "note": "state in + out per step; the manifest arrays add traffic"},
        "gpu_launches": launches, "clocks": clk,
    }


def hydro_workload(args, dist: Dist) -> dict:
    import paraiso_gb300 as pg
    from paraiso_gb300 import build as pgbuild
    pgbuild.build()
    n = args.size or 4096
    cells = n * n
    h = pg.Hydro((n, n), precision=32, gamma=1.4, device=dist.local_rank,
                 tile_x=args.tile_x, tile_y=args.tile_y)
    h.init_kh(1 + dist.rank)
    h.set_scalar("cfl", 0.4)
    h.proceed(max(args.warmup, 1))
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    dist.barrier()
    ms = h.time_run("proceed", args.steps)
    launches = h.last_launch_count()
    dist.barrier()
    clk = clocks.stop()
    ms = dist.max(ms)
    value = cells * args.steps * dist.world / (ms * 1e-3) / 1e9
    # dominant kernel per launch
    h.profile(True)
    h.time_run("proceed", min(args.steps, 10))
    nl, kms, _ = h.profile_query("hydro_fused_kernel_f32")
    h.profile(False)
    peak, peak_kind = peaks()
    per_launch_ms = kms / max(nl, 1)
    achieved = 32.0 * cells / (per_launch_ms * 1e-3) / 1e9
    traffic = profile_traffic("hydro_fused_kernel_f32", n)
    roofline = {"bound": "hbm", "kernel": "hydro_fused_kernel_f32", "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": traffic["bytes_per_launch"] if traffic else None,
                "algorithmic_bytes_per_launch": 32.0 * cells, "launch_ms": round(per_launch_ms, 4),
                "peak_source": f"{peak_kind} MEASURED_PEAKS.json hbm_gbs",
                "note": "32 B per cell-update (4 FP32 fields in + out); the fused step is "
                        "bound by FP32 CUDA-core issue, not HBM"}
    # end to end: per step upload the four fields from pinned host memory, one
    # step, read the four fields back
    import torch
    hosts = [torch.empty(cells, dtype=torch.float32).pin_memory() for _ in range(4)]
    names = ("density", "velocity0", "velocity1", "pressure")
    for t, nm in zip(hosts, names):
        h.read_to_pointer(nm, t.data_ptr(), cells * 4)
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for t, nm in zip(hosts, names):
            h.write_from_pointer(nm, t.data_ptr(), cells * 4)
        h.proceed(1)
        for t, nm in zip(hosts, names):
            h.read_to_pointer(nm, t.data_ptr(), cells * 4)
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e = {"value": round(cells * e2e_steps * dist.world / e2e_s / 1e9, 3),
           "unit": "Gcell-updates/s", "h2d_bytes_per_step": 4 * cells * 4,
           "d2h_bytes_per_step": 4 * cells * 4, "steps": e2e_steps}
    # the plain FP64 GPU path (the generated structure) and FP64 accuracy reference
    plain = pg.Hydro((n, n), precision=64, variant=1, gamma=1.4, device=dist.local_rank)
    plain.init_kh(1 + dist.rank)
    plain.set_scalar("cfl", 0.4)
    plain.proceed(1)
    pms = plain.time_run("proceed", 2) / 2
    plain.close()
    plain_gcell = cells / (pms * 1e-3) / 1e9
    acc = None
    if args.accuracy_steps > 0:
        import numpy as np
        a = pg.Hydro((n, n), precision=32, gamma=1.4, device=dist.local_rank)
        b = pg.Hydro((n, n), precision=64, gamma=1.4, device=dist.local_rank)
        for x in (a, b):
            x.init_kh(1 + dist.rank)
            x.set_scalar("cfl", 0.4)
        a.proceed(args.accuracy_steps)
        b.proceed(args.accuracy_steps)
        sa = [x.astype(np.float64) for x in a.state()]
        sb = b.state()
        def cons(st):
            r, u, v, p = st
            return {"density": r, "momentum0": r * u, "momentum1": r * v,
                    "energy": 0.5 * r * (u * u + v * v) + p / 0.4}
        ca, cb = cons(sa), cons(sb)
        acc = {"steps": args.accuracy_steps, "reference": "FP64 fused path (bit-exact with the oracle)"}
        for k in ca:
            d = np.abs(ca[k] - cb[k])
            acc[k] = {"l1_rel": float(d.mean() / np.abs(cb[k]).mean()), "linf": float(d.max())}
        ta, tb = a.totals(), b.totals()
        acc["totals_rel_diff"] = [float((x - y) / y) if y else float(x - y) for x, y in zip(ta, tb)]
        a.close()
        b.close()
    h.close()
    out = {
        "metric": "Hydro cell-updates/s (Gcell-updates/s), FP32 bulk, FP64 dt/totals",
        "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"hydro {n}x{n} periodic Kelvin-Helmholtz, gamma 1.4, CFL 0.4, "
                               "noise seed 1+rank, one step per step", "n0": n, "n1": n,
                   "parallelism": f"replicas x{dist.world}",
                   "l2": "inputs larger than L2" if n >= 4096 else "inputs may fit in L2"},
        "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
        "plain_fp64_gpu": {"value": round(plain_gcell, 4), "unit": "Gcell-updates/s",
                           "speedup": round(value / dist.world / plain_gcell, 1)},
        "accuracy": acc,
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        from oracle import pyoracle as O
        O.build()
        m = min(n, 2048)
        st = O.hydro_init_kh(m, m, 1)
        t0 = time.perf_counter()
        O.hydro_run(st, 1, cyclic=True, gamma=1.4, cfl=0.4)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(m * m / dt / 1e9, 5), "unit": "Gcell-updates/s",
                               "cores": O.lib().oracle_num_threads(), "kind": "port",
                               "sample": f"1 FP64 step of {m}x{m} Kelvin-Helmholtz, "
                                         f"oracle/om_oracle.cpp (OpenMP), {dt:.2f} s"}
    return out


def ensemble_workload(args, dist: Dist) -> dict:
    import paraiso_gb300 as pg
    from paraiso_gb300 import build as pgbuild
    pgbuild.build()
    count = args.count
    sizes = pg.ensemble_sizes(count, 1 + dist.rank)
    tile_x, tile_y, tiles_by = args.tile_x, args.tile_y, "command line"
    if tile_x == 0 and tile_y == 0:
        # tile shape picked by the autotuner on these very instance sizes
        best, _ = pg.autotune_ensemble(sizes, precision=32, gamma=1.4, device=dist.local_rank)
        tile_x, tile_y, tiles_by = best.tile_x, best.tile_y, "om_autotune_ensemble"
    e = pg.Ensemble(sizes, precision=32, gamma=1.4, device=dist.local_rank,
                    tile_x=tile_x, tile_y=tile_y)
    e.init_kh(1000 * (1 + dist.rank))
    info = e.info()
    cells = info["cells"]
    e.step(max(args.warmup, 1))
    # timed: K steps replayed from the CUDA graph of K steps (captured in warm-up)
    e.step(args.steps)
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    dist.barrier()
    ms = e.time_step(args.steps)
    dist.barrier()
    clk = clocks.stop()
    ms = dist.max(ms)
    t0 = time.perf_counter()
    e.step(args.steps)              # the public call: graph replay + scalar sync
    graph_s = dist.max(time.perf_counter() - t0)
    value = cells * args.steps * dist.world / (ms * 1e-3) / 1e9
    # the same instances advanced one grid at a time through the single-grid API
    seq_ms = 0.0
    nseq = min(count, args.seq_instances)
    seq_cells = 0
    for k in range(nseq):
        h = pg.Hydro(sizes[k], precision=32, gamma=1.4, device=dist.local_rank)
        h.init_kh(1000 * (1 + dist.rank) + k)
        h.set_scalar("cfl", 0.4)
        h.proceed(1)
        seq_ms += h.time_run("proceed", 10)
        seq_cells += sizes[k][0] * sizes[k][1]
        h.close()
    seq_gcell = seq_cells * 10 / (seq_ms * 1e-3) / 1e9
    peak, _ = peaks()
    achieved = 32.0 * cells / (ms / args.steps * 1e-3) / 1e9
    times = [e.scalar(k, "time") for k in range(count)]
    out = {
        "metric": "Hydro ensemble cell-updates/s (Gcell-updates/s), FP32, per-instance CFL dt",
        "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{count} periodic Kelvin-Helmholtz instances, n0,n1 uniform over "
                               "multiples of 32 in [256,2048] (seed 1+rank), one persistent "
                               "launch per step, CUDA graph", "instances": count,
                   "cells": cells, "work_items": info["work_items"], "grid": info["grid"],
                   "tile": {"tile_x": tile_x, "tile_y": tile_y, "picked_by": tiles_by},
                   "parallelism": f"replicas x{dist.world}"},
        "roofline": {"bound": "hbm", "kernel": "hydro_ensemble_kernel", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": None, "algorithmic_bytes_per_launch": 32.0 * cells,
                     "launch_ms": round(ms / args.steps, 4)},
        "e2e": {"value": round(cells * args.steps * dist.world / graph_s / 1e9, 3),
                "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "om_ensemble_step(K) through the public API, scalars synced once"},
        "gpu_launches": 2 * args.steps, "clocks": clk,
        "single_grid_launches": {"value": round(seq_gcell, 3), "unit": "Gcell-updates/s",
                                 "instances": nseq,
                                 "note": "same instances, one grid at a time (om_run_n per grid)"},
        "instance_time_range": [min(times), max(times)],
    }
    e.close()
    return out


def adjoint_target(n: int, seed: int = 7):
    """Smooth periodic target density: 1.5 + sum of 8 Fourier modes with
    small integer wave numbers, amplitudes scaled to a total of 0.1."""
    import numpy as np
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x)
    amps = rng.uniform(0.2, 1.0, 8)
    amps *= 0.1 / amps.sum()
    t = np.full((n, n), 1.5)
    for a in amps:
        p, q = rng.integers(-4, 5, 2)
        if p == 0 and q == 0:
            p = 1
        t += a * np.sin(2 * np.pi * (p * X + q * Y) + rng.uniform(0, 2 * np.pi))
    return t


def adjoint_workload(args, dist: Dist) -> dict:
    import numpy as np
    import paraiso_gb300 as pg
    from paraiso_gb300 import build as pgbuild
    pgbuild.build()
    n = args.size or 1024
    T = args.adj_steps
    cells = n * n
    target = adjoint_target(n)
    h = pg.Hydro((n, n), precision=args.adj_precision, gamma=1.4, device=dist.local_rank)
    h.init_kh(1)
    h.set_scalar("cfl", 0.4)
    st0 = h.state()
    if args.tie_noise > 0:
        # break the ties of the CFL minimum of the Kelvin-Helmholtz start
        rng0 = np.random.default_rng(99)
        st0 = tuple(a * (1 + args.tie_noise * rng0.standard_normal(a.shape)).astype(a.dtype)
                    for a in st0)
        h.set_state(st0)
    # forward step and adjoint step, device time on the handle's stream
    h.proceed(max(args.warmup, 1))
    fwd_ms = h.time_run("proceed", 50) / 50
    vjp_ms = h.time_vjp(50)      # reverse sweep of one step from its tape
    tape_ms = h.time_tape(50)    # the taped forward step of the recompute
    # the full gradient: forward with sqrt(T) checkpoints, recompute, backward
    h.set_state(st0)
    h.set_scalar("time", 0.0)
    t0 = time.perf_counter()
    loss, grad = h.adjoint_run(T, target.astype(st0[0].dtype))
    grad_s = time.perf_counter() - t0
    grad64 = [g.astype(np.float64) for g in grad]
    h.close()
    # finite differences with the FP64 forward along seeded directions
    f64 = pg.Hydro((n, n), precision=64, gamma=1.4, device=dist.local_rank)
    st64 = tuple(a.astype(np.float64) for a in st0)

    def L(s):
        f64.set_state(s)
        f64.set_scalar("time", 0.0)
        f64.set_scalar("cfl", 0.4)
        f64.set_scalar("dR0", 1.0 / n)
        f64.set_scalar("dR1", 1.0 / n)
        f64.proceed(T)
        return float(((f64.read("density") - target) ** 2).mean())

    rng = np.random.default_rng(2024)
    fd_rows = []
    for k in range(args.fd_dirs):
        d = [rng.standard_normal((n, n)) * s for s in (0.1, 0.05, 0.05, 0.0)]
        ad = sum(float((g * b).sum()) for g, b in zip(grad64, d))
        row = {"ad": ad}
        for eps in args.fd_eps:
            lp = L(tuple(a + eps * b for a, b in zip(st64, d)))
            lm = L(tuple(a - eps * b for a, b in zip(st64, d)))
            fd = (lp - lm) / (2 * eps)
            row[f"fd_{eps:g}"] = fd
            row[f"rel_{eps:g}"] = abs(ad - fd) / max(abs(fd), 1e-300)
        fd_rows.append(row)
    f64.close()
    summary = {}
    for eps in args.fd_eps:
        rels = sorted(r[f"rel_{eps:g}"] for r in fd_rows)
        if not rels:
            continue
        summary[f"{eps:g}"] = {"median_rel": rels[len(rels) // 2], "max_rel": rels[-1],
                               "within_1e-4": sum(x <= 1e-4 for x in rels)}
    out = {
        "metric": "Hydro adjoint: adjoint step / forward step time, gradient vs FD",
        "adjoint_precision": args.adj_precision, "tie_noise": args.tie_noise,
        "value": round(vjp_ms / fwd_ms, 3), "unit": "adjoint_step/forward_step",
        "higher_is_better": False, "n_gpus": dist.world, "steps": T, "warmup": args.warmup,
        "dtype": "f32", "data": "synthetic", "vs_baseline": None, "scaling": "weak",
        "config": {"workload": f"hydro adjoint {n}x{n} Kelvin-Helmholtz (seed 1), {T} FP32 steps, "
                               "loss mean((rho_T - target)^2), target 1.5 + 8 Fourier modes "
                               "(amplitude 0.1), gradient w.r.t. initial rho, vx, vy, p",
                   "n0": n, "n1": n},
        "forward_step_ms": round(fwd_ms, 4), "adjoint_step_ms": round(vjp_ms, 4),
        "taped_step_ms": round(tape_ms, 4),
        "adjoint_step_note": "reverse sweep of one step from the tape its forward step wrote "
                             "when the backward pass recomputed the segment; per gradient step "
                             "the work is forward + taped recompute + reverse",
        "per_step_cost_over_forward": {
            "reverse": round(vjp_ms / fwd_ms, 3),
            "taped_recompute": round(tape_ms / fwd_ms, 3),
            "gradient_wall": round(grad_s * 1e3 / T / fwd_ms, 3)},
        "gradient_run_s": round(grad_s, 3), "loss": loss,
        "forward_gcell_s": round(cells / (fwd_ms * 1e-3) / 1e9, 3),
        "fd": {"directions": args.fd_dirs, "forward": "FP64 fused (bit-exact with the oracle)",
               "summary": summary, "rows": fd_rows[: min(4, len(fd_rows))]},
    }
    return out


def life_cpu_baseline(n: int, args) -> dict:
    from oracle import pyoracle as O
    O.build()
    gens = 3 if n >= 8192 else 200
    a = O.life_bernoulli(n, n, 1, 0.3)
    t0 = time.perf_counter()
    O.life_run(a, gens, cyclic=True)
    dt = time.perf_counter() - t0
    return {"value": round(n * n * gens / dt / 1e9, 4), "unit": "Gcell-updates/s",
            "cores": O.lib().oracle_num_threads(), "kind": "port",
            "sample": f"{n}x{n} cyclic Bernoulli(0.3), {gens} generations, oracle/om_oracle.cpp "
                      f"(OpenMP), {dt:.2f} s"}


def reference_arm(args, dist: Dist) -> dict | None:
    if dist.rank != 0:
        return None
    if args.workload == "adjoint":
        return {"impl": "reference",
                "unavailable": "the reference has no adjoint of the Hydro step to time"}
    if args.workload in ("hydro4k", "hydrograph", "ensemble"):
        return reference_hydro(args, dist)
    from oracle import pyoracle as O
    O.build()
    n = args.size or (128 if args.workload == "life128" else 16384)
    gens_full = args.generations or (1000 if args.workload == "life128" else 100)
    sample_gens = 2 if n >= 8192 else gens_full
    a = O.life_bernoulli(n, n, 1, 0.3)
    for _ in range(min(args.warmup, 1)):
        a, _ = O.life_run(a, 1, cyclic=True)
    times = []
    for _ in range(args.steps if n < 8192 else min(args.steps, 5)):
        t0 = time.perf_counter()
        a, _ = O.life_run(a, sample_gens, cyclic=True)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = n * n * sample_gens * len(times) / tot / 1e9
    cores = O.lib().oracle_num_threads()
    return {
        "impl": "reference",
        "metric": ("Life cell-updates/s (Gcell-updates/s) through the general OM graph executor"
                   if args.workload == "lifegraph"
                   else "Life cell-updates/s (Gcell-updates/s), bit-exact vs the oracle"),
        "value": round(value, 4), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": len(times), "warmup": args.warmup,
        "ms_per_step": round(tot / len(times) * 1e3 * gens_full / sample_gens, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": {"workload": f"life {n}x{n} cyclic, Bernoulli(0.3) seed 1, {gens_full} "
                               f"generations per step", "n0": n, "n1": n},
        "cpu_baseline": {"value": round(value, 4), "unit": "Gcell-updates/s", "cores": cores,
                         "kind": "port",
                         "sample": f"{sample_gens} of {gens_full} generations per step on {n}x{n}; "
                                   "CPU restatement (oracle/om_oracle.cpp, OpenMP) of the "
                                   "generated Life loop, pinned bit-exact to the reference's "
                                   "pre-generated Life.cpp"},
        "e2e": {"value": round(value, 4), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def reference_hydro(args, dist: Dist) -> dict:
    """The oracle's FP32 Hydro step (the reference's generated Hydro is
    float) on the host cores: one step of the 4096^2 grid, or one step of
    every ensemble instance, per timed step."""
    import paraiso_gb300 as pg
    from oracle import pyoracle as O
    O.build()
    if args.workload in ("hydro4k", "hydrograph"):
        n = args.size or 4096
        grids = [(n, n, 1)]
        metric = ("Hydro cell-updates/s (Gcell-updates/s) through the general OM graph executor"
                  if args.workload == "hydrograph"
                  else "Hydro cell-updates/s (Gcell-updates/s), FP32 bulk, FP64 dt/totals")
        workload = f"hydro {n}x{n} periodic Kelvin-Helmholtz, gamma 1.4, CFL 0.4"
    else:
        sizes = pg.ensemble_sizes(args.count, 1)
        grids = [(a, b, 1000 + k) for k, (a, b) in enumerate(sizes)]
        metric = "Hydro ensemble cell-updates/s (Gcell-updates/s), FP32, per-instance CFL dt"
        workload = (f"{args.count} periodic Kelvin-Helmholtz instances, n0,n1 uniform over "
                    "multiples of 32 in [256,2048] (seed 1)")
    states = [tuple(a.astype(np.float32) for a in O.hydro_init_kh(a, b, seed))
              for a, b, seed in grids]
    cells = sum(a * b for a, b, _ in grids)
    steps = max(1, min(args.steps, 3))
    for k, st in enumerate(states):       # warm-up: one step
        states[k], _, _ = O.hydro_run(st, 1, cyclic=True, gamma=1.4, cfl=0.4, dtype=np.float32)
    t0 = time.perf_counter()
    for _ in range(steps):
        for k, st in enumerate(states):
            states[k], _, _ = O.hydro_run(st, 1, cyclic=True, gamma=1.4, cfl=0.4,
                                          dtype=np.float32)
    tot = time.perf_counter() - t0
    value = cells * steps / tot / 1e9
    cores = O.lib().oracle_num_threads()
    return {
        "impl": "reference", "metric": metric, "value": round(value, 5),
        "unit": "Gcell-updates/s", "n_gpus": dist.world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": round(tot / steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload, "cells": cells},
        "cpu_baseline": {"value": round(value, 5), "unit": "Gcell-updates/s", "cores": cores,
                         "kind": "port",
                         "sample": f"{steps} FP32 steps of {len(grids)} grid(s), {cells} cells; "
                                   "CPU restatement (oracle/om_oracle.cpp, OpenMP) of the "
                                   "generated Hydro step, pinned bit-exact to the reference's "
                                   "pre-generated Hydro.cpp"},
        "e2e": {"value": round(value, 5), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 1000 for hydro4k, else 200)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="life16k",
                    choices=["life16k", "life128", "lifegraph", "hydro4k", "hydrograph",
                             "ensemble", "adjoint"])
    ap.add_argument("--adj-steps", type=int, default=200)
    ap.add_argument("--adj-precision", type=int, default=32)
    ap.add_argument("--tie-noise", type=float, default=0.0)
    ap.add_argument("--fd-dirs", type=int, default=32)
    ap.add_argument("--fd-eps", type=float, nargs="+", default=[1e-3, 1e-5, 1e-7])
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--seq-instances", type=int, default=16)
    ap.add_argument("--accuracy-steps", type=int, default=1000)
    ap.add_argument("--size", type=int, default=0)
    ap.add_argument("--generations", type=int, default=0)
    ap.add_argument("--depth", type=int, default=0)
    ap.add_argument("--tile-x", type=int, default=0)
    ap.add_argument("--tile-y", type=int, default=0)
    ap.add_argument("--life-io", type=int, default=0, help="0: 128-bit cell I/O, 1: 32-bit")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"hydro4k": 1000, "lifegraph": 10}.get(args.workload, 200)
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    dist = Dist()
    try:
        if args.impl == "reference":
            out = reference_arm(args, dist)
        elif args.workload == "hydro4k":
            out = hydro_workload(args, dist)
        elif args.workload == "ensemble":
            out = ensemble_workload(args, dist)
        elif args.workload == "adjoint":
            out = adjoint_workload(args, dist)
        elif args.workload == "lifegraph":
            out = lifegraph_workload(args, dist)
        elif args.workload == "hydrograph":
            out = hydrograph_workload(args, dist)
        else:
            out = life_workload(args, dist)
        if out is not None and dist.rank == 0:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
