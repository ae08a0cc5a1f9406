#!/usr/bin/env python3
"""Throughput benchmark of the GB300 Orthotope Machine kernels.

Default workload (the headline line): Conway's Life (examples/Life) on a
16384x16384 cyclic grid, int32 cells Bernoulli(0.3) from seed 1; one step =
100 generations with the population reduce after every generation.  Metric:
Gcell-updates/s.  The line checks its own claim outside the timed region
(the timed path against the one-cell-per-thread integer kernel over a whole
step, and against the oracle's generations of the CPU-baseline sample) and,
at N=1, carries under "configs" the other measured configurations: Life
128^2 x 1000, Hydro 4096^2 x 1000 FP32, the 64-instance Hydro ensemble and
the 1024^2 x 200 Hydro adjoint, each with its roofline, CPU baseline,
end-to-end figure and accuracy against FP64.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload life16k|life128|lifegraph|hydro4k|hydrograph|ensemble|adjoint]
                  [--headline-only]

Prints one JSON line (rank 0).  Under torchrun (N > 1) every rank advances
its own independent replica (no data-path collective; weak scaling).
`--impl reference` times the CPU restatement of the reference's algorithm
(oracle/) on all host cores, K steps of a bounded sample of the same
workload, plus one full step.
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

# Floating-point operations of one Hydro step per cell-update, counted on the
# CPU restatement of examples/Hydro/HydroMain.hs:134-276 (each wall's flux
# evaluated once, only the HLLC branch taken; the periodic Kelvin-Helmholtz
# start, the same for every size).  tests/test_oracle.py recounts them.
HYDRO_OPS_PER_CELL = {"add": 242, "mul": 197, "div": 93, "sqrt": 17}
HYDRO_FLOPS_PER_CELL = sum(HYDRO_OPS_PER_CELL.values())
# FP32 lanes per SM (four sub-partitions of 32) and flops per lane per clock
# (one fused multiply-add): the CUDA-core FP32 peak is SMs x 128 x 2 x clock.
FP32_LANES_PER_SM = 128


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


def peak_source(kind: str) -> str:
    return ("measured MEASURED_PEAKS.json hbm_gbs" if kind == "measured"
            else "fallback 6.8 TB/s (MEASURED_PEAKS.json absent)")


class NearGpu:
    """Within the block, this process runs on the host CPUs local to GPU `dev`
    (its PCI function's sysfs local_cpulist, intersected with the allowed
    CPUs), so that pinned host buffers allocated there sit in the memory the
    GPU reaches directly; the affinity is restored on exit.  `info` says what
    was done (None when the topology could not be read)."""

    def __init__(self, dev: int):
        self.dev = dev
        self.saved = None
        self.info = None

    def __enter__(self):
        try:
            import torch
            p = torch.cuda.get_device_properties(self.dev)
            addr = f"{p.pci_domain_id:04x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0"
            with open(f"/sys/bus/pci/devices/{addr}/local_cpulist") as f:
                text = f.read().strip()
            cpus = set()
            for part in text.split(","):
                if "-" in part:
                    a, b = part.split("-")
                    cpus.update(range(int(a), int(b) + 1))
                elif part:
                    cpus.add(int(part))
            allowed = os.sched_getaffinity(0)
            use = cpus & allowed
            self.info = {"pci": addr, "local_cpus": len(use), "allowed_cpus": len(allowed)}
            if use and use != allowed:
                self.saved = allowed
                os.sched_setaffinity(0, use)
        except Exception:
            self.info = None
        return self

    def __exit__(self, *exc):
        if self.saved:
            os.sched_setaffinity(0, self.saved)
        return False


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
                   tile_y=args.tile_y, life_io=args.life_io, life_kernel=args.life_kernel)
    life.fill_random(1 + dist.rank, 0.3)
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
    for kn in ("life_reg_kernel", "life_ws_kernel", "life_ws_tma_kernel", "life_tb32_kernel",
               "life_tb_kernel",
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
                "peak": peak, "peak_source": peak_source(peak_kind),
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
    with NearGpu(dist.local_rank) as near:
        host_in = torch.empty(cells, dtype=torch.int32).pin_memory()
        host_out = torch.empty(cells, dtype=torch.int32).pin_memory()
        life.read_to_pointer("cell", host_in.data_ptr(), cells * 4)
        e2e_steps = max(1, min(args.steps, args.e2e_steps))
        # one untimed round trip first (its first use of this path's graph)
        life.write_from_pointer("cell", host_in.data_ptr(), cells * 4)
        life.run("proceed", gens)
        life.read_to_pointer("cell", host_out.data_ptr(), cells * 4)
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
        del host_in, host_out
    e2e_s = dist.max(t1 - t0)
    e2e = {"value": round(cells * gens * e2e_steps * dist.world / e2e_s / 1e9, 3),
           "unit": "Gcell-updates/s", "h2d_bytes_per_step": cells * 4,
           "d2h_bytes_per_step": cells * 4 + 4, "steps": e2e_steps,
           "api": "om_array_write + om_run_n(proceed) + om_array_read + population scalar",
           "host_cpus": near.info}
    life.close()

    out = {
        "metric": LIFE_METRIC,
        "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": life_config(n, gens, dist.world),
        "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
    }
    oracle_sample = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"], oracle_sample = life_cpu_baseline(n, args)
    if not args.no_self_check:
        out["self_check"] = life_self_check(pg, n, gens, dist, args, oracle_sample)
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
    for kname in ("hydro_pair_kernel", "hydro_pair2_kernel", "hydro_persist_kernel",
                  "hydro_fused_kernel_f32"):
        nl, kms, _ = h.profile_query(kname)
        if nl > 0:
            break
    h.profile(False)
    peak, peak_kind = peaks()
    per_launch_ms = kms / max(nl, 1)
    achieved = 32.0 * cells / (per_launch_ms * 1e-3) / 1e9
    traffic = profile_traffic(kname, n)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": traffic["bytes_per_launch"] if traffic else None,
                "algorithmic_bytes_per_launch": 32.0 * cells, "launch_ms": round(per_launch_ms, 4),
                "peak_source": peak_source(peak_kind),
                "note": "32 B per cell-update (4 FP32 fields in + out); the fused step is "
                        "bound by FP32 CUDA-core issue, not HBM (see compute_roofline)"}
    kernel_gcell = cells / (per_launch_ms * 1e-3) / 1e9
    compute = fp32_compute_roofline(kernel_gcell, dist.local_rank, clk)
    compute["kernel"] = kname
    # end to end: per step upload the four fields from pinned host memory, one
    # step, read the four fields back
    import torch
    names = ("density", "velocity0", "velocity1", "pressure")
    with NearGpu(dist.local_rank) as near:
        hosts = [torch.empty(cells, dtype=torch.float32).pin_memory() for _ in range(4)]
        for t, nm in zip(hosts, names):
            h.read_to_pointer(nm, t.data_ptr(), cells * 4)
        e2e_steps = max(1, min(args.steps, args.e2e_steps))
        # one untimed round trip first
        for t, nm in zip(hosts, names):
            h.write_from_pointer(nm, t.data_ptr(), cells * 4)
        h.proceed(1)
        for t, nm in zip(hosts, names):
            h.read_to_pointer(nm, t.data_ptr(), cells * 4)
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            for t, nm in zip(hosts, names):
                h.write_from_pointer(nm, t.data_ptr(), cells * 4)
            h.proceed(1)
            for t, nm in zip(hosts, names):
                h.read_to_pointer(nm, t.data_ptr(), cells * 4)
        e2e_s = dist.max(time.perf_counter() - t0)
        del hosts
    e2e = {"value": round(cells * e2e_steps * dist.world / e2e_s / 1e9, 3),
           "unit": "Gcell-updates/s", "h2d_bytes_per_step": 4 * cells * 4,
           "d2h_bytes_per_step": 4 * cells * 4, "steps": e2e_steps,
           "api": "om_array_write x4 + om_run(proceed) + om_array_read x4",
           "host_cpus": near.info}
    h.close()
    # FP64 comparators: the fused FP64 kernel (the same tile code in double)
    # and the plain FP64 GPU path (the generated structure)
    f64 = pg.Hydro((n, n), precision=64, gamma=1.4, device=dist.local_rank)
    f64.init_kh(1 + dist.rank)
    f64.set_scalar("cfl", 0.4)
    f64.proceed(max(args.warmup, 1))
    f64_ms = f64.time_run("proceed", 50) / 50
    f64.close()
    fused64_gcell = cells / (f64_ms * 1e-3) / 1e9
    plain = pg.Hydro((n, n), precision=64, variant=1, gamma=1.4, device=dist.local_rank)
    plain.init_kh(1 + dist.rank)
    plain.set_scalar("cfl", 0.4)
    plain.proceed(1)
    pms = plain.time_run("proceed", 2) / 2
    plain.close()
    plain_gcell = cells / (pms * 1e-3) / 1e9
    acc = None
    if args.accuracy_steps > 0:
        a = pg.Hydro((n, n), precision=32, gamma=1.4, device=dist.local_rank)
        b = pg.Hydro((n, n), precision=64, gamma=1.4, device=dist.local_rank)
        for x in (a, b):
            x.init_kh(1 + dist.rank)
            x.set_scalar("cfl", 0.4)
        a.proceed(args.accuracy_steps)
        b.proceed(args.accuracy_steps)
        acc = {"steps": args.accuracy_steps,
               "reference": "FP64 fused path (bit-exact with the oracle)"}
        acc.update(hydro_conserved_errors(a.state(), b.state()))
        ta, tb = a.totals(), b.totals()
        acc["totals_rel_diff"] = [float((x - y) / y) if y else float(x - y) for x, y in zip(ta, tb)]
        acc["density_l1_target"] = 1e-5
        acc["meets_target"] = acc["density"]["l1_rel"] <= 1e-5
        a.close()
        b.close()
    out = {
        "metric": HYDRO_METRIC,
        "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": hydro_config(n, dist.world),
        "roofline": roofline, "compute_roofline": compute, "e2e": e2e, "gpu_launches": launches,
        "clocks": clk,
        "fused_fp64_gpu": {"value": round(fused64_gcell, 3), "unit": "Gcell-updates/s",
                           "fp32_speedup": round(value / dist.world / fused64_gcell, 2),
                           "note": "the same fused tile kernel in FP64"},
        "plain_fp64_gpu": {"value": round(plain_gcell, 4), "unit": "Gcell-updates/s",
                           "speedup": round(value / dist.world / plain_gcell, 1),
                           "note": "the generated structure in FP64: unfused sub-kernels, "
                                   "every Delayed value recomputed, host round trip for dt"},
        "accuracy": acc,
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = hydro_cpu_baseline([(n, n, 1)])
    return out


def ensemble_workload(args, dist: Dist) -> dict:
    import numpy as np
    import paraiso_gb300 as pg
    from paraiso_gb300 import build as pgbuild
    pgbuild.build()
    count = args.count
    sizes = pg.ensemble_sizes(count, 1 + dist.rank)
    tile_x, tile_y, grid_limit, tiles_by = args.tile_x, args.tile_y, 0, "command line"
    if tile_x == 0 and tile_y == 0 and args.tune:
        # tile shape and persistent grid size picked by the autotuner on these
        # very instance sizes
        best, _ = pg.autotune_ensemble(sizes, precision=32, gamma=1.4, device=dist.local_rank)
        tile_x, tile_y, grid_limit = best.tile_x, best.tile_y, best.grid_limit
        tiles_by = "om_autotune_ensemble"
    e = pg.Ensemble(sizes, precision=32, gamma=1.4, device=dist.local_rank,
                    tile_x=tile_x, tile_y=tile_y, grid_limit=grid_limit)
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
    value = cells * args.steps * dist.world / (ms * 1e-3) / 1e9
    # end to end through the public API with host buffers: per step, every
    # instance's four fields up from pinned host memory, one step, the four
    # fields and the instance time back
    import torch
    with NearGpu(dist.local_rank) as near:
        hosts = []
        for k, (a, b) in enumerate(sizes):
            row = []
            for f in pg.Ensemble.FIELDS:
                t = torch.empty(a * b, dtype=torch.float32).pin_memory()
                e.read_to_pointer(k, f, t.data_ptr(), a * b * 4)
                row.append(t)
            hosts.append(row)
        e2e_steps = max(1, min(args.steps, args.e2e_steps))
        # one untimed round trip first
        for k, (a, b) in enumerate(sizes):
            for f, t in zip(pg.Ensemble.FIELDS, hosts[k]):
                e.write_from_pointer(k, f, t.data_ptr(), a * b * 4)
        e.step(1)
        for k, (a, b) in enumerate(sizes):
            for f, t in zip(pg.Ensemble.FIELDS, hosts[k]):
                e.read_to_pointer(k, f, t.data_ptr(), a * b * 4)
        dist.barrier()
        t0 = time.perf_counter()
        times = []
        for _ in range(e2e_steps):
            for k, (a, b) in enumerate(sizes):
                for f, t in zip(pg.Ensemble.FIELDS, hosts[k]):
                    e.write_from_pointer(k, f, t.data_ptr(), a * b * 4)
            e.step(1)
            for k, (a, b) in enumerate(sizes):
                for f, t in zip(pg.Ensemble.FIELDS, hosts[k]):
                    e.read_to_pointer(k, f, t.data_ptr(), a * b * 4)
            times.append(e.scalar(0, "time"))
        e2e_s = dist.max(time.perf_counter() - t0)
        del hosts
    e2e = {"value": round(cells * e2e_steps * dist.world / e2e_s / 1e9, 3),
           "unit": "Gcell-updates/s", "h2d_bytes_per_step": 16 * cells,
           "d2h_bytes_per_step": 16 * cells + 8, "steps": e2e_steps,
           "api": "om_ensemble_write x4 per instance + om_ensemble_step(1) + "
                  "om_ensemble_read x4 per instance + om_ensemble_scalar(time)",
           "host_cpus": near.info}
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
    # one 4096^2 instance through the ensemble kernel against the single-grid
    # fused step on the same grid (the same tile shape)
    one = None
    if args.one_instance:
        n1 = 4096
        e1 = pg.Ensemble([(n1, n1)], precision=32, gamma=1.4, device=dist.local_rank,
                         tile_x=tile_x, tile_y=tile_y)
        e1.init_kh(7)
        e1.step(3)
        e1_ms = min(e1.time_step(20) for _ in range(2))
        e1.close()
        h1 = pg.Hydro((n1, n1), precision=32, gamma=1.4, device=dist.local_rank,
                      tile_x=tile_x, tile_y=tile_y)
        h1.init_kh(7)
        h1.set_scalar("cfl", 0.4)
        h1.proceed(3)
        h1_ms = min(h1.time_run("proceed", 20) for _ in range(2))
        h1.close()
        ens1 = n1 * n1 * 20 / (e1_ms * 1e-3) / 1e9
        fus1 = n1 * n1 * 20 / (h1_ms * 1e-3) / 1e9
        one = {"instance": [n1, n1], "ensemble": round(ens1, 3), "single_grid": round(fus1, 3),
               "ensemble_over_single": round(ens1 / fus1, 3), "unit": "Gcell-updates/s",
               "note": "one instance through om_ensemble_step against om_run_n(proceed) on the "
                       "same grid, 20 steps each, best of two"}
    peak, peak_kind = peaks()
    launch_ms = ms / args.steps
    achieved = 32.0 * cells / (launch_ms * 1e-3) / 1e9
    # the persistent 32 x 32 kernel (tile_y 0: tile_x 0 two groups per CTA,
    # which the library runs on work lists of at least 16 items per group,
    # as here; 16 or 32 one group) or the tile kernel
    persistent = tile_y == 0 and tile_x in (0, 16, 32)
    ens_kernel = ("hydro_pair2_ensemble_kernel" if persistent and tile_x == 0
                  else "hydro_persist_ensemble_kernel" if persistent else "hydro_ensemble_kernel")
    traffic = profile_traffic_cells(ens_kernel, cells)
    out_times = [e.scalar(k, "time") for k in range(count)]
    e.close()
    acc = None
    if args.accuracy_steps > 0:
        # every instance in production FP32 against the FP64 ensemble (bit-exact
        # per instance with the oracle) over the configuration's steps
        steps = min(args.accuracy_steps, 200)
        a = pg.Ensemble(sizes, precision=32, gamma=1.4, device=dist.local_rank,
                        tile_x=tile_x, tile_y=tile_y)
        b = pg.Ensemble(sizes, precision=64, gamma=1.4, device=dist.local_rank)
        a.init_kh(1000 * (1 + dist.rank))
        b.init_kh(1000 * (1 + dist.rank))
        a.step(steps)
        b.step(steps)
        worst = {}
        per_density = []
        for k in range(count):
            errs = hydro_conserved_errors(a.state(k), b.state(k))
            per_density.append(errs["density"]["l1_rel"])
            for f, d in errs.items():
                w = worst.setdefault(f, {"l1_rel": 0.0, "linf": 0.0})
                w["l1_rel"] = max(w["l1_rel"], d["l1_rel"])
                w["linf"] = max(w["linf"], d["linf"])
        acc = {"steps": steps, "reference": "FP64 ensemble (bit-exact per instance with the oracle)",
               "worst_instance": worst,
               "density_l1_rel_median": float(np.median(per_density)),
               "density_l1_target": 1e-5,
               "meets_target": max(per_density) <= 1e-5}
        a.close()
        b.close()
    out = {
        "metric": ENSEMBLE_METRIC,
        "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(launch_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": ensemble_config(count, cells, dist.world),
        "launch": {"work_items": info["work_items"], "grid": info["grid"],
                   "tile": {"tile_x": tile_x, "tile_y": tile_y, "grid_limit": grid_limit,
                            "picked_by": tiles_by}},
        "roofline": {"bound": "hbm", "kernel": ens_kernel, "achieved": round(achieved, 1),
                     "peak": peak, "peak_source": peak_source(peak_kind),
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic["bytes_per_launch"] if traffic else None,
                     "traffic_source": traffic["source"] if traffic else None,
                     "algorithmic_bytes_per_launch": 32.0 * cells,
                     "launch_ms": round(launch_ms, 4),
                     "note": "one launch per step; 32 B per cell-update summed over instances; "
                             "compute-bound like the single-grid step (see compute_roofline)"},
        "compute_roofline": fp32_compute_roofline(value / dist.world, dist.local_rank, clk),
        "e2e": e2e, "gpu_launches": 2 * args.steps, "clocks": clk,
        "single_grid_launches": {"value": round(seq_gcell, 3), "unit": "Gcell-updates/s",
                                 "instances": nseq,
                                 "persistent_over_single": round(value / dist.world / seq_gcell, 3),
                                 "note": "the first instances, one grid at a time (om_run_n per grid)"},
        "instance_time_range": [min(out_times), max(out_times)],
        "one_instance": one,
        "accuracy": acc,
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = hydro_cpu_baseline(
            [(a, b, 1000 + k) for k, (a, b) in enumerate(sizes)])
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


ADJOINT_METRIC = "Hydro adjoint: adjoint step / forward step time, gradient vs FD"


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
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    fwd_ms = h.time_run("proceed", 50) / 50
    vjp_ms = h.time_vjp(50)      # reverse sweep of one step from its tape
    tape_ms = h.time_tape(50)    # the taped forward step of the recompute
    clk = clocks.stop()
    # the full gradient through the public call from host buffers: forward
    # with sqrt(T) checkpoints, recompute, backward, loss and gradient back
    h.set_state(st0)
    h.set_scalar("time", 0.0)
    t0 = time.perf_counter()
    loss, grad = h.adjoint_run(T, target.astype(st0[0].dtype))
    grad_s = time.perf_counter() - t0
    grad64 = [g.astype(np.float64) for g in grad]
    # the forward alone through the same public calls
    h.set_state(st0)
    h.set_scalar("time", 0.0)
    t0 = time.perf_counter()
    h.proceed(T)
    fin32 = h.state()
    fwd_s = time.perf_counter() - t0
    h.close()
    es = 4 if args.adj_precision == 32 else 8
    # finite differences with the FP64 forward along seeded directions
    f64 = pg.Hydro((n, n), precision=64, gamma=1.4, device=dist.local_rank)
    st64 = tuple(a.astype(np.float64) for a in st0)

    def run64(s):
        f64.set_state(s)
        f64.set_scalar("time", 0.0)
        f64.set_scalar("cfl", 0.4)
        f64.set_scalar("dR0", 1.0 / n)
        f64.set_scalar("dR1", 1.0 / n)
        f64.proceed(T)

    def L(s):
        run64(s)
        return float(((f64.read("density") - target) ** 2).mean())

    # accuracy of the FP32 forward of this workload against FP64
    run64(st64)
    fwd_acc = hydro_conserved_errors(fin32, f64.state())
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
        "metric": ADJOINT_METRIC,
        "adjoint_precision": args.adj_precision,
        "cotangent_accumulation": f"fp{args.adj_precision}",
        "tie_noise": args.tie_noise,
        "value": round(vjp_ms / fwd_ms, 3), "unit": "adjoint_step/forward_step",
        "higher_is_better": False, "n_gpus": dist.world, "steps": T, "warmup": args.warmup,
        "ms_per_step": round(vjp_ms, 4),
        "dtype": f"f{args.adj_precision}", "data": "synthetic", "vs_baseline": None,
        "scaling": "weak",
        "config": {"workload": f"hydro adjoint {n}x{n} Kelvin-Helmholtz (seed 1), {T} FP"
                               f"{args.adj_precision} steps, loss mean((rho_T - target)^2), "
                               "target 1.5 + 8 Fourier modes (amplitude 0.1), gradient w.r.t. "
                               "initial rho, vx, vy, p", "n0": n, "n1": n,
                   "parallelism": f"replicas x{dist.world}",
                   "l2": (f"no flush: a {n}x{n} state ({4 * n * n * args.adj_precision // 8 >> 20} "
                          "MiB) fits in L2 and the forward and reverse steps are compute- and "
                          "latency-bound; a reverse step reads 24 taped arrays of the same "
                          "size")},
        "forward_step_ms": round(fwd_ms, 4), "adjoint_step_ms": round(vjp_ms, 4),
        "taped_step_ms": round(tape_ms, 4),
        "per_step_cost_over_forward": {
            "reverse": round(vjp_ms / fwd_ms, 3),
            "reverse_plus_taped_recompute": round((vjp_ms + tape_ms) / fwd_ms, 3),
            "taped_recompute": round(tape_ms / fwd_ms, 3),
            "gradient_wall": round(grad_s * 1e3 / T / fwd_ms, 3),
            "note": "reverse: the reverse sweep of one step from its tape (the headline "
                    "value); a gradient step also recomputes its forward step with the tape "
                    "written (taped_recompute); gradient_wall is the whole sqrt(T) "
                    "checkpointed gradient through the public call, host copies included, "
                    "per step over the device-timed forward step"},
        "gpu_launches": 2 * 50,
        "clocks": clk,
        "e2e": {"value": round(grad_s / fwd_s, 3), "unit": "gradient_run/forward_run",
                "h2d_bytes_per_step": round((4 + 1) * cells * es / T),
                "d2h_bytes_per_step": round(4 * cells * es / T),
                "note": "om_hydro_adjoint_run (state and target up, loss and the four "
                        "gradient arrays back) over om_run_n(proceed, T) with the state read "
                        "back, both from host buffers; bytes are per step of the T-step run"},
        "gradient_run_s": round(grad_s, 3), "forward_run_s": round(fwd_s, 3), "loss": loss,
        "forward_gcell_s": round(cells / (fwd_ms * 1e-3) / 1e9, 3),
        "forward_accuracy": {"steps": T, "reference": "FP64 fused path",
                             **fwd_acc},
        "fd": {"directions": args.fd_dirs, "forward": "FP64 fused (bit-exact with the oracle)",
               "summary": summary, "rows": fd_rows[: min(4, len(fd_rows))]},
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        from oracle import pyoracle as O
        O.build()
        st = O.hydro_init_kh(n, n, 1)
        dd = tuple(np.full_like(a, 1e-3) for a in st)
        t0 = time.perf_counter()
        O.hydro_tl_run(st, dd, 1, gamma=1.4, cfl=0.4)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(cells / dt / 1e9, 5), "unit": "Gcell-updates/s",
                               "cores": O.lib().oracle_num_threads(), "kind": "port",
                               "sample": f"1 FP64 tangent-linear step of {n}x{n} (the oracle's "
                                         f"derivative of the step, oracle/om_oracle.cpp, "
                                         f"OpenMP), {dt:.2f} s"}
    return out


def life_cpu_baseline(n: int, args):
    """The oracle on all host cores over a bounded sample of the workload.
    Returns (cpu_baseline, (generations, cells, populations)): the sample's
    result also serves the line's self-check."""
    from oracle import pyoracle as O
    O.build()
    gens = 3 if n >= 8192 else 200
    a = O.life_bernoulli(n, n, 1, 0.3)
    t0 = time.perf_counter()
    cells, pops = O.life_run(a, gens, cyclic=True)
    dt = time.perf_counter() - t0
    return ({"value": round(n * n * gens / dt / 1e9, 4), "unit": "Gcell-updates/s",
             "cores": O.lib().oracle_num_threads(), "kind": "port",
             "sample": f"{n}x{n} cyclic Bernoulli(0.3), {gens} generations, "
                       f"oracle/om_oracle.cpp (OpenMP), {dt:.2f} s"},
            (gens, cells, pops))


def reference_arm(args, dist: Dist) -> dict | None:
    """The reference's algorithm on the host cores: the CPU restatement
    (oracle/om_oracle.cpp, OpenMP, pinned bit-exact to the reference's
    pre-generated Life.cpp / Hydro.cpp) on the same configuration as our arm.
    Each of the K timed steps runs a bounded sample of one step's work, so
    that the whole run ends within minutes; ms_per_step is that sample's
    measured time.  One full step is timed once besides."""
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
    for _ in range(args.warmup if sample_gens == gens_full else 1):
        a, _ = O.life_run(a, sample_gens, cyclic=True)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        a, _ = O.life_run(a, sample_gens, cyclic=True)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = n * n * sample_gens * len(times) / tot / 1e9
    full = None
    if sample_gens != gens_full:
        t0 = time.perf_counter()
        O.life_run(a, gens_full, cyclic=True)
        fs = time.perf_counter() - t0
        full = {"generations": gens_full, "ms": round(fs * 1e3, 1),
                "value": round(n * n * gens_full / fs / 1e9, 4), "unit": "Gcell-updates/s"}
    cores = O.lib().oracle_num_threads()
    metric = ("Life cell-updates/s (Gcell-updates/s) through the general OM graph executor"
              if args.workload == "lifegraph" else LIFE_METRIC)
    return {
        "impl": "reference", "metric": metric,
        "value": round(value, 4), "unit": "Gcell-updates/s", "n_gpus": dist.world,
        "steps": len(times), "warmup": args.warmup,
        "ms_per_step": round(tot / len(times) * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": life_config(n, gens_full, dist.world),
        "sample_generations_per_step": sample_gens,
        "full_step": full,
        "cpu_baseline": {"value": round(value, 4), "unit": "Gcell-updates/s", "cores": cores,
                         "kind": "port",
                         "sample": f"{sample_gens} of the {gens_full} generations of a step per "
                                   f"timed step on {n}x{n} (ms_per_step is the sample's), plus "
                                   "one full step timed once (full_step); CPU restatement "
                                   "(oracle/om_oracle.cpp, OpenMP) of the generated Life loop, "
                                   "pinned bit-exact to the reference's pre-generated Life.cpp"},
        "e2e": {"value": round(value, 4), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def reference_hydro(args, dist: Dist) -> dict:
    """The oracle's FP32 Hydro step (the reference's generated Hydro is
    float) on the host cores: per timed step one step of the 4096^2 grid, or
    one step of a bounded sample of the ensemble's instances."""
    import paraiso_gb300 as pg
    from oracle import pyoracle as O
    O.build()
    if args.workload in ("hydro4k", "hydrograph"):
        n = args.size or 4096
        grids = [(n, n, 1)]
        metric = ("Hydro cell-updates/s (Gcell-updates/s) through the general OM graph executor"
                  if args.workload == "hydrograph" else HYDRO_METRIC)
        config = hydro_config(n, dist.world)
        sample = "one FP32 step of the grid per timed step"
    else:
        sizes = pg.ensemble_sizes(args.count, 1)
        cells_all = sum(a * b for a, b in sizes)
        grids = [(a, b, 1000 + k) for k, (a, b) in enumerate(sizes)][:8]
        metric = ENSEMBLE_METRIC
        config = ensemble_config(args.count, cells_all, dist.world)
        sample = f"one FP32 step of the first {len(grids)} of {args.count} instances per timed step"
    states = [tuple(a.astype(np.float32) for a in O.hydro_init_kh(a, b, seed))
              for a, b, seed in grids]
    cells = sum(a * b for a, b, _ in grids)
    for k, st in enumerate(states):       # warm-up: one step
        states[k], _, _ = O.hydro_run(st, 1, cyclic=True, gamma=1.4, cfl=0.4, dtype=np.float32)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for k, st in enumerate(states):
            states[k], _, _ = O.hydro_run(st, 1, cyclic=True, gamma=1.4, cfl=0.4,
                                          dtype=np.float32)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = cells * len(times) / tot / 1e9
    cores = O.lib().oracle_num_threads()
    return {
        "impl": "reference", "metric": metric, "value": round(value, 5),
        "unit": "Gcell-updates/s", "n_gpus": dist.world, "steps": len(times),
        "warmup": args.warmup, "ms_per_step": round(tot / len(times) * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config,
        "cpu_baseline": {"value": round(value, 5), "unit": "Gcell-updates/s", "cores": cores,
                         "kind": "port",
                         "sample": f"{sample} ({cells} cells; ms_per_step is the sample's); CPU "
                                   "restatement (oracle/om_oracle.cpp, OpenMP) of the generated "
                                   "Hydro step, pinned bit-exact to the reference's "
                                   "pre-generated Hydro.cpp"},
        "e2e": {"value": round(value, 5), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def life_config(n: int, gens: int, world: int) -> dict:
    cells = n * n
    return {"workload": f"life {n}x{n} cyclic, Bernoulli(0.3) seed 1+rank, "
                        f"{gens} generations per step, population reduce every generation",
            "n0": n, "n1": n, "generations_per_step": gens,
            "parallelism": f"replicas x{world}",
            "l2": f"inputs larger than L2 (2 x {cells * 4 / 2**20:.0f} MiB int32 buffers)"
            if cells * 4 > 129 * 2**20
            else "grid fits in L2; no flush (launch-bound case)"}


LIFE_METRIC = "Life cell-updates/s (Gcell-updates/s), bit-exact vs the oracle"


def life_self_check(pg, n: int, gens: int, dist: Dist, args, oracle_sample) -> dict:
    """Outside the timed region: one step of the timed path from the same
    start against (a) the one-cell-per-thread integer kernel over all `gens`
    generations (final cells and every generation's population) and (b) the
    oracle's generations of the CPU-baseline sample (same seed)."""
    import numpy as np
    t0 = time.perf_counter()
    life = pg.Life((n, n), device=dist.local_rank, depth=args.depth, tile_x=args.tile_x,
                   tile_y=args.tile_y, life_io=args.life_io, life_kernel=args.life_kernel)
    life.fill_random(1 + dist.rank, 0.3)
    init = life.read("cell")
    use_oracle = oracle_sample is not None and oracle_sample[0] <= gens
    k = oracle_sample[0] if use_oracle else min(3, gens)
    life.run("proceed", k)
    cells_k = life.read("cell")
    pops_k = life.population_history(k)
    if gens > k:
        life.run("proceed", gens - k)
        pops = np.concatenate([pops_k, life.population_history(gens - k)])
    else:
        pops = pops_k
    cells = life.read("cell")
    life.close()
    gen = pg.Life((n, n), variant=1, device=dist.local_rank)
    gen.write("cell", init)
    gen.run("proceed", gens)
    general_ok = bool(np.array_equal(gen.read("cell"), cells)
                      and np.array_equal(gen.population_history(gens), pops))
    gen.close()
    check = {"timed_path_vs_general_kernel": {"generations": gens, "equal": general_ok}}
    ok = general_ok
    if use_oracle and dist.rank == 0:
        ok_k = bool(np.array_equal(oracle_sample[1], cells_k)
                    and np.array_equal(oracle_sample[2], pops_k))
        check["timed_path_vs_oracle"] = {"generations": k, "equal": ok_k}
        ok = ok and ok_k
    check["ok"] = ok
    check["seconds"] = round(time.perf_counter() - t0, 2)
    return check


def sm_count(device: int) -> int:
    try:
        import torch
        return int(torch.cuda.get_device_properties(device).multi_processor_count)
    except Exception:
        return 152


def fp32_compute_roofline(gcell_s: float, device: int, clk: dict) -> dict:
    """The fused step's FP32 work against the CUDA-core FP32 peak: flops per
    cell-update counted on the restatement x cell-updates/s, over SMs x 128
    lanes x 2 flops (one fused multiply-add) x the SM clock (the maximum
    clock nvidia-smi reports during the timed region, else 2070 MHz)."""
    sms = sm_count(device)
    mhz = (clk or {}).get("sm_max_mhz") or 2070.0
    peak = sms * FP32_LANES_PER_SM * 2 * mhz * 1e6 / 1e12
    achieved = HYDRO_FLOPS_PER_CELL * gcell_s * 1e9 / 1e12
    return {"bound": "fp32", "flops_per_cell_update": HYDRO_FLOPS_PER_CELL,
            "ops_per_cell_update": HYDRO_OPS_PER_CELL, "achieved": round(achieved, 2),
            "peak": round(peak, 1), "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
            "peak_derivation": f"{sms} SMs x {FP32_LANES_PER_SM} FP32 lanes x 2 flops (FMA) "
                               f"x {mhz:.0f} MHz",
            "note": "algorithmic flops (each wall's flux once, only the HLLC branch taken); "
                    "division and square root count one flop each though they issue several "
                    "instructions, and the kernel also evaluates the halo's walls"}


def hydro_conserved_errors(got, ref, gamma: float = 1.4) -> dict:
    """L1 (relative to the mean magnitude of the reference) and Linf of the
    conserved fields of `got` against `ref` (primitive states)."""
    import numpy as np

    def cons(st):
        r, u, v, p = (x.astype(np.float64) for x in st)
        return {"density": r, "momentum0": r * u, "momentum1": r * v,
                "energy": 0.5 * r * (u * u + v * v) + p / (gamma - 1.0)}
    ca, cb = cons(got), cons(ref)
    out = {}
    for k in ca:
        d = np.abs(ca[k] - cb[k])
        out[k] = {"l1_rel": float(d.mean() / np.abs(cb[k]).mean()), "linf": float(d.max())}
    return out


HYDRO_METRIC = "Hydro cell-updates/s (Gcell-updates/s), FP32 bulk, FP64 dt/totals"


def hydro_config(n: int, world: int) -> dict:
    return {"workload": f"hydro {n}x{n} periodic Kelvin-Helmholtz, gamma 1.4, CFL 0.4, "
                        "noise seed 1+rank, one step per step", "n0": n, "n1": n,
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2" if n >= 4096 else "inputs may fit in L2"}


def hydro_cpu_baseline(grids) -> dict:
    """The oracle's FP32 Hydro step (the reference's generated Hydro is
    float) on all host cores: one step of every grid (n0, n1, seed)."""
    from oracle import pyoracle as O
    O.build()
    states = [tuple(a.astype(np.float32) for a in O.hydro_init_kh(a, b, seed))
              for a, b, seed in grids]
    cells = sum(a * b for a, b, _ in grids)
    t0 = time.perf_counter()
    for st in states:
        O.hydro_run(st, 1, cyclic=True, gamma=1.4, cfl=0.4, dtype=np.float32)
    dt = time.perf_counter() - t0
    return {"value": round(cells / dt / 1e9, 5), "unit": "Gcell-updates/s",
            "cores": O.lib().oracle_num_threads(), "kind": "port",
            "sample": f"1 FP32 step of {len(grids)} grid(s), {cells} cells, "
                      f"oracle/om_oracle.cpp (OpenMP), {dt:.2f} s"}


ENSEMBLE_METRIC = "Hydro ensemble cell-updates/s (Gcell-updates/s), FP32, per-instance CFL dt"


def ensemble_config(count: int, cells: int, world: int) -> dict:
    return {"workload": f"{count} periodic Kelvin-Helmholtz instances, n0,n1 uniform over "
                        "multiples of 32 in [256,2048] (seed 1+rank), one persistent "
                        "launch per step, CUDA graph", "instances": count, "cells": cells,
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2" if cells * 16 > 129 * 2**20 else "inputs may fit in L2"}


def profile_traffic_cells(kernel: str, cells: int):
    """DRAM bytes per launch of `kernel` over `cells` cell-updates, scaled by
    cells from the committed capture profiles/<kernel>_traffic.txt
    ("bytes_per_cell" line)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_traffic.txt")
    try:
        d = {}
        with open(path) as f:
            for line in f:
                if ":" in line and not line.startswith("#"):
                    k, v = line.split(":", 1)
                    d[k.strip()] = v.strip()
        return {"bytes_per_launch": round(float(d["bytes_per_cell"]) * cells),
                "source": os.path.relpath(path, ROOT) + " (scaled by cells)"}
    except Exception:
        return None


def run_configs(args, dist: Dist) -> dict:
    """The other measured configurations, each as its own complete line
    (N=1 only): Life 128^2 x 1000, Hydro 4096^2 x 1000 FP32, the 64-instance
    ensemble over 200 steps and the 1024^2 x 200 adjoint.  A failure in one
    is reported in its place and does not stop the others."""
    runs = {
        "life128": (life_workload, dict(workload="life128", size=0, generations=0,
                                        depth=0, tile_x=0, tile_y=0, life_kernel=0)),
        "hydro4k": (hydro_workload, dict(workload="hydro4k", size=0, steps=1000,
                                         accuracy_steps=1000, tile_x=0, tile_y=0)),
        "ensemble": (ensemble_workload, dict(workload="ensemble", size=0, steps=200,
                                             accuracy_steps=200, count=64, tile_x=0,
                                             tile_y=0)),
        "adjoint": (adjoint_workload, dict(workload="adjoint", size=0, adj_steps=200,
                                           adj_precision=32, tie_noise=1e-4, fd_dirs=32,
                                           fd_eps=[1e-7])),
    }
    out = {}
    for name, (fn, over) in runs.items():
        sub = argparse.Namespace(**vars(args))
        for k, v in over.items():
            setattr(sub, k, v)
        t0 = time.perf_counter()
        try:
            r = fn(sub, dist)
        except Exception as e:  # reported, not hidden
            r = {"error": f"{type(e).__name__}: {e}"}
        r["wall_s"] = round(time.perf_counter() - t0, 1)
        out[name] = r
    return out

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
    ap.add_argument("--no-tune", dest="tune", action="store_false",
                    help="ensemble line: run the command line's tile shape without tuning")
    ap.add_argument("--no-one-instance", dest="one_instance", action="store_false",
                    help="ensemble line: skip the one-4096^2-instance comparison")
    ap.add_argument("--accuracy-steps", type=int, default=1000)
    ap.add_argument("--size", type=int, default=0)
    ap.add_argument("--generations", type=int, default=0)
    ap.add_argument("--depth", type=int, default=0)
    ap.add_argument("--tile-x", type=int, default=0)
    ap.add_argument("--tile-y", type=int, default=0)
    ap.add_argument("--life-io", type=int, default=0, help="0: 128-bit cell I/O, 1: 32-bit")
    ap.add_argument("--life-kernel", type=int, default=0,
                    help="Life packed kernel (om_config.life_kernel; 0 = automatic)")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-self-check", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="the default line without the other configurations")
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
            if (args.workload == "life16k" and not args.headline_only and dist.world == 1
                    and not args.size and not args.generations):
                out["configs"] = run_configs(args, dist)
        if out is not None and dist.rank == 0:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
