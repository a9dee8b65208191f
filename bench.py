"""Benchmark: zone-updates/s of one Mara2 time step on the 2-D Kelvin-Helmholtz
workload (1024^2 zones, periodic, PLM + HLLC, RK2), mixed precision against
the plain FP64 path, on synthetic seeded initial data.

One zone-update = one interior zone advanced one full time step (all RK
stages), Mara's kzps x 1e3 (src/Mara.cpp:68).  A "step" is one
MethodOfLinesTVD::advance of the whole grid, with dt = CFL x Courant step
computed on the device.

  value      mixed path, state resident in HBM, L2 flushed between steps
  e2e        mixed path through the drop-in C-ABI call with host buffers:
             every step copies MeshData::P (FP64 AoS with guards) host ->
             device, advances, and copies it back
  plain_fp64 the plain FP64 path (bit-identical to the reference's CPU
             build) on the same workload, same timing rules
  roofline   the fused stage kernel: algorithmic bytes / mean launch time
             from CUDA events on the handle's stream, against measured HBM
  cpu_baseline  the CPU oracle (restatement of the reference's algorithm,
             OpenMP over zones) on the host cores, bounded sample

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "zone-updates/s per RK step, mixed vs plain FP64 GPU at stated L1 err; p50/p99 latency"
UNIT = "zone-updates/s"
N_SIDE = 1024
L2_FLUSH_BYTES = 512 << 20
SOAK_S = 1.5


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_per_zone_stage():
    """DRAM bytes per zone and stage of the fused kernel from the committed ncu
    summary (profiles/hydro_tile_kh.txt, line 'dram_bytes_per_zone_stage=...')."""
    p = os.path.join(ROOT, "profiles", "hydro_tile_kh.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_zone_stage="):
            return float(line.split("=", 1)[1].split()[0])
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, 0
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    dist.init_process_group("nccl" if os.environ.get("MARA_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return dist, rank, ws, local


def aggregate(dist, local_ms: float, local_units: float):
    """Whole-job throughput: units of all ranks / max time over ranks
    (replicas: every rank advances its own grid)."""
    if dist is None:
        return local_ms, local_units
    import torch
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([local_ms], dtype=torch.float64, device=dev)
    u = torch.tensor([local_units], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


# ----------------------------------------------------------------------------
def time_resident(solver, steps: int, warmup: int, device: int):
    """Mean device ms per step over `steps` steps, each bracketed by CUDA events
    on the handle's stream, with an L2 flush (a 512 MiB write) between steps
    outside the events."""
    import torch
    stream = torch.cuda.ExternalStream(solver.stream, device=torch.device("cuda", device))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=torch.device("cuda", device))
    solver.run(1)  # computes the first Courant step
    solver.run_async(warmup)
    solver.synchronize()
    launches0 = solver.stats().kernel_launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for a, b in ev:
            flush.fill_(1.0)
            a.record(stream)
            solver.run_async(1)
            b.record(stream)
    torch.cuda.synchronize(device)
    solver.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    launches = solver.stats().kernel_launches - launches0
    return float(np.mean(ms)), ms, int(launches)


def soak(solver, seconds: float) -> int:
    """Advance untimed for `seconds` of wall time; returns the steps taken."""
    solver.run(1)
    n, chunk, t0 = 1, 256, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        solver.run_async(chunk)
        solver.synchronize()
        n += chunk
    return n


def kernel_roofline(solver, steps: int, zones: int, nq: int, rk: int, peak: float, peak_kind: str):
    """Per-launch timing of the fused stage kernel with events around each
    launch (eager, no graph), then achieved = algorithmic bytes / time."""
    solver.set_kernel_timing(True)
    solver.run(steps)
    ms, n = solver.kernel_times()
    solver.set_kernel_timing(False)
    # algorithmic bytes per zone and stage: the stage input (8 B/field, an
    # FP32 pair) and the output; stages after the first also read U0
    per_zone_step = (2 + 3 * (rk - 1)) * nq * 8
    bytes_total = per_zone_step * zones * (n[0] / rk)
    achieved = bytes_total / (ms[0] * 1e-3) / 1e9 if ms[0] > 0 else None
    tr = _traffic_per_zone_stage()
    return {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak if achieved else None,
        "traffic": tr * zones if tr else None,
        "kernel": "hydro_tile_kernel<2D,PLM,HLLC>", "launches_timed": n[0],
        "mean_launch_ms": ms[0] / n[0] if n[0] else None,
        "algorithmic_bytes_per_launch": per_zone_step * zones / rk,
        "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
    }


def l1_vs_fp64(s, P0, steps: int, device: int):
    """Relative L1 density error of the mixed path against the plain FP64 path
    (bit-identical to the reference's CPU build) after `steps` steps of the
    same dt sequence."""
    from mara2_gb300.solver import Solver
    with Solver(s, "fp64", device) as a, Solver(s, "mixed", device) as b:
        a.upload(P0.copy())
        b.upload(P0.copy())
        for _ in range(steps):
            a.run(1)
            dt = a.stats().last_dt
            b.advance(dt)
        pa = a.download()[s.interior()]
        pb = b.download()[s.interior()]
    rho = np.sum(np.abs(pb[..., 0] - pa[..., 0])) / np.sum(np.abs(pa[..., 0]))
    linf = np.max(np.abs(pb[..., 0] - pa[..., 0])) / np.max(np.abs(pa[..., 0]))
    return float(rho), float(linf)


def e2e(solver, P0, steps: int, warmup: int):
    """The drop-in call with host buffers: pinned host P, H2D + advance + D2H
    per step, timed on the host around the synchronous call."""
    import torch
    host = torch.from_numpy(P0.copy()).pin_memory()
    ptr = host.data_ptr()
    solver.upload(P0.copy())
    dt = solver.courant() * solver.scheme.cfl
    for _ in range(warmup):
        solver.advance_host_ptr(ptr, dt)
    launches0 = solver.stats().kernel_launches
    t0 = time.perf_counter()
    for _ in range(steps):
        rc = solver.advance_host_ptr(ptr, dt)
        if rc:
            raise RuntimeError(f"advance_host failed: {rc}")
    t1 = time.perf_counter()
    nbytes = P0.nbytes
    return (t1 - t0) * 1e3 / steps, nbytes, solver.stats().kernel_launches - launches0


def cpu_baseline(s, P0, budget_s: float = 20.0):
    """The oracle (C restatement of the reference's advance, OpenMP over zones)
    on the host cores: whole KH steps until the time budget is spent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(False)
    port = O.Oracle("port")
    c = O.make_config(law=s.law, recon=s.recon, riemann=s.riemann, bc=s.bc, rk_order=s.rk_order,
                      shape=s.shape, lower=s.lower, upper=s.upper, gamma=s.gamma, plm_theta=s.plm_theta)
    threads = port.lib.mo_max_threads()
    P = P0.copy()
    _, dtc = port.courant(c, P)
    dt = s.cfl * dtc
    port.advance(c, P, dt)  # warm the allocator / threads
    n, t0 = 0, time.perf_counter()
    while True:
        st, _ = port.advance(c, P, dt)
        n += 1
        if st or time.perf_counter() - t0 > budget_s or n >= 50:
            break
    el = time.perf_counter() - t0
    return {"value": s.zones * n / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} whole steps of the {s.shape[0]}x{s.shape[1]} KH workload in {el:.1f} s "
                      f"(oracle C restatement, OpenMP, {threads} threads)"}


def _l1_rho(a, b, s):
    pa, pb = a[s.interior()], b[s.interior()]
    return float(np.sum(np.abs(pb[..., 0] - pa[..., 0])) / np.sum(np.abs(pa[..., 0])))


def _rate(g, s, steps, t_final=None):
    """Zone-updates/s of `steps` device-resident steps (host wall clock around
    a synchronising run; the first Courant step is computed beforehand)."""
    import torch
    g.run(1, s.cfl, t_final)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n = g.run(steps, s.cfl, t_final)
    el = time.perf_counter() - t0
    return s.zones * n / el, n, el


def workload_suite(device: int, serving_requests: int = 512):
    """The other benchmark workloads, each on both precisions."""
    from mara2_gb300 import workloads as W
    from mara2_gb300.batch import autotune, serve
    from mara2_gb300.solver import Solver
    out = {}

    # 1. Sod shock tube, 1024 zones, to t = 0.2 (whole run)
    s, P0 = W.sod(1024)
    res = {}
    for prec in ("mixed", "fp64"):
        with Solver(s, prec, device) as g:
            g.upload(P0.copy())
            t0 = time.perf_counter()
            n = g.run(100_000, s.cfl, s.t_final)
            el = time.perf_counter() - t0
            res[prec] = (g.download(), n, el)
    out["sod_1024_t0.2"] = {
        "mixed_zone_updates_per_s": s.zones * res["mixed"][1] / res["mixed"][2],
        "plain_fp64_zone_updates_per_s": s.zones * res["fp64"][1] / res["fp64"][2],
        "steps_mixed": res["mixed"][1], "steps_fp64": res["fp64"][1],
        "l1_density_vs_fp64_at_t_final": _l1_rho(res["fp64"][0], res["mixed"][0], s),
        "note": "mixed: the whole run on one thread-block cluster (grid in shared memory, 1024 steps per launch); "
                "plain FP64: three kernels per step"}

    # 3. 3-D MHD turbulence with CT, 256^3, RK3
    s, P0 = W.mhd_turbulence(256)
    dx = 1.0 / 256
    bmax = float(np.abs(P0[..., 5:8]).max())
    entry = {}
    with Solver(s, "mixed", device) as g:
        g.upload(P0.copy())
        entry["mixed_zone_updates_per_s"], n, _ = _rate(g, s, 6)
        entry["mixed_max_div_b_dx_over_bmax"] = g.monopole_max(dx) * dx / bmax
    with Solver(s, "fp64", device) as g:
        g.upload(P0.copy())
        entry["plain_fp64_zone_updates_per_s"], n, _ = _rate(g, s, 2)
        entry["plain_max_div_b_dx_over_bmax"] = g.monopole_max(dx) * dx / bmax
    with Solver(s, "fp64", device) as a, Solver(s, "mixed", device) as b:
        a.upload(P0.copy())
        b.upload(P0.copy())
        for _ in range(3):
            a.run(1)
            b.advance(a.stats().last_dt)
        entry["l1_density_vs_fp64_3_steps"] = _l1_rho(a.download(), b.download(), s)
    out["mhd_ct_256cube_rk3"] = entry
    del P0

    # 4. relativistic MHD blast, 512^2, WENO5 + HLLE, RK3
    s, P0 = W.rmhd_blast(512)
    entry = {}
    with Solver(s, "mixed", device) as g:
        g.upload(P0.copy())
        entry["mixed_zone_updates_per_s"], n, _ = _rate(g, s, 20)
        entry["mixed_failures"] = g.stats().failures
    with Solver(s, "fp64", device) as g:
        g.upload(P0.copy())
        entry["plain_fp64_zone_updates_per_s"], n, _ = _rate(g, s, 3)
    with Solver(s, "fp64", device) as a, Solver(s, "mixed", device) as b:
        a.upload(P0.copy())
        b.upload(P0.copy())
        for _ in range(10):
            a.run(1)
            b.advance(a.stats().last_dt)
        entry["l1_density_vs_fp64_10_steps"] = _l1_rho(a.download(), b.download(), s)
        entry["plain_failures"] = a.stats().failures
    out["rmhd_blast_512_weno5_rk3"] = entry

    # 5. serving: a bounded Poisson stream of Riemann problems
    tiles = autotune(device)
    reqs = W.riemann_stream(serving_requests, rate=2000.0)
    r = serve(reqs, budget_bytes=32 << 30, tile_1d=tiles["tile_1d"], tile_2d=tiles["tile_2d"], device=device)
    out["serving_riemann_stream"] = {**r.summary(), "requests_in_sample": serving_requests,
                                     "stream": "1-D N log-uniform [256, 8192] / 2-D side log-uniform [128, 512], "
                                               "Poisson 2000/s, t = 0.2, PLM + HLLC, RK2",
                                     "tiles": {"tile_1d": tiles["tile_1d"], "tile_2d": tiles["tile_2d"]}}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mara2_gb300")
    ap.add_argument("--n", type=int, default=N_SIDE)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-workloads", action="store_true", help="skip the per-workload section")
    ap.add_argument("--serving-requests", type=int, default=512)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    from mara2_gb300 import workloads as W
    s, P0 = W.kelvin_helmholtz(args.n)
    config = {"workload": f"kelvin-helmholtz {args.n}x{args.n} periodic, gamma 5/3, PLM(theta 1.5)+HLLC, RK2, CFL 0.4",
              "zones": s.zones, "seed": W.KH_SEED, "l2": "flushed between timed steps (512 MiB write)",
              "parallelism": f"replicas x{args.gpus}"}

    dist, rank, ws, local = _dist()

    if args.impl == "reference":
        # the reference's algorithm on the host cores (the oracle restatement:
        # the reference's own build needs its source tree, absent on the GPU
        # host); rank 0 only
        if rank != 0:
            return
        cb = cpu_baseline(s, P0, args.cpu_budget)
        line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": s.zones / cb["value"] * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "impl": "reference", "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    from mara2_gb300 import build
    from mara2_gb300.solver import Solver
    build.build()
    torch.cuda.set_device(local)
    peak, peak_kind = _peaks()

    with Solver(s, "mixed", local) as g:
        with ClockSampler(local) as clk:
            # the timed region lasts a few ms, shorter than the sampler's
            # period: the same step runs untimed for SOAK_S seconds first, so
            # the samples show the clocks the timed steps ran at
            g.upload(P0.copy())
            soak_steps = soak(g, SOAK_S)
            g.upload(P0.copy())
            if dist:
                dist.barrier()
            torch.cuda.synchronize()
            ms_mixed, ms_all, launches = time_resident(g, args.steps, args.warmup, local)
            torch.cuda.synchronize()
            if dist:
                dist.barrier()
        clocks = clk.summary()
        clocks["window"] = f"{soak_steps} untimed steps ({SOAK_S} s) of the same workload, then the timed region"
        ms_job, units = aggregate(dist, ms_mixed, float(s.zones))
        value = units / (ms_job * 1e-3)
        roof = kernel_roofline(g, min(args.steps, 20), s.zones, s.nq, s.rk_order, peak, peak_kind)
        e2e_ms, pbytes, e2e_launches = e2e(g, P0, max(3, args.steps // 3), 2)

    with Solver(s, "fp64", local) as gp:
        gp.upload(P0.copy())
        ms_plain, _, _ = time_resident(gp, max(3, args.steps // 5), 3, local)
    l1_rho, linf_rho = l1_vs_fp64(s, P0, 20, local)
    suite = None if args.no_workloads or rank != 0 else workload_suite(local, args.serving_requests)

    if rank != 0:
        return
    cb = cpu_baseline(s, P0, args.cpu_budget)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_job, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 flux arithmetic, f32-pair accumulator", "data": "synthetic", "config": config,
        "precision": "mixed",
        "l1_density_vs_fp64": l1_rho, "linf_density_vs_fp64": linf_rho, "l1_steps": 20,
        "plain_fp64": {"value": s.zones / (ms_plain * 1e-3), "unit": UNIT, "ms_per_step": ms_plain,
                       "dtype": "f64", "parity": "bit-identical to the reference's CPU build"},
        "mixed_over_plain": (s.zones / (ms_mixed * 1e-3)) / (s.zones / (ms_plain * 1e-3)),
        "e2e": {"value": s.zones / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": pbytes, "d2h_bytes_per_step": pbytes,
                "call": "mara_gpu_advance_host (MeshData::P host FP64 AoS in and out)"},
        "gpu_launches": launches,
        "roofline": roof,
        "cpu_baseline": cb,
        "clocks": clocks,
        "step_ms_min": min(ms_all), "step_ms_max": max(ms_all),
        "workloads": suite,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
