"""Benchmark: zone-updates/s of one Mara2 time step on the 2-D Kelvin-Helmholtz
workload (1024^2 zones, periodic, PLM + HLLC, RK2), mixed precision against
the plain FP64 path, on synthetic seeded initial data; then every workload
configuration at its stated length.

One zone-update = one interior zone advanced one full time step (all RK
stages), Mara's kzps x 1e3 (src/Mara.cpp:68).  A "step" is one
MethodOfLinesTVD::advance of the whole grid, with dt = CFL x Courant step
computed on the device.

  value      mixed path (FP32 flux arithmetic, FP32-pair accumulator), state
             resident in HBM, L2 flushed between steps
  fp64_accumulator  the same with an FP64 accumulator (the benchmark spec's
             recipe), same rules
  e2e        mixed path through the drop-in C-ABI call with host buffers:
             every step copies MeshData::P (FP64 AoS with guards) host ->
             device, advances, and copies it back
  plain_fp64 the plain FP64 path (bit-identical to the reference's CPU
             build) on the same workload, same timing rules, with its HBM
             and FP64-pipe rooflines
  roofline   the fused stage kernel: algorithmic bytes / mean launch time
             from CUDA events on the handle's stream, against measured HBM
  cpu_baseline  the CPU oracle (restatement of the reference's algorithm,
             OpenMP over zones) on the host cores, bounded sample
  workloads  Sod 1024 to t = 0.2, KH 1024^2 to t = 1, MHD + CT 256^3 for 100
             steps, RMHD blast 512^2 to t = 4: plain FP64 and both mixed
             recipes, each recipe's relative L1 / L-inf error in every
             conserved field against the plain path on its dt sequence,
             failure counts, div B; the 4096-request serving stream, a stream
             below saturation and the requests solved alone on the plain path

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


def _profile_value(name, key):
    """A figure recorded in a committed ncu summary (profiles/<name>, a line
    'key=value ...')."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + "="):
            return float(line.split("=", 1)[1].split()[0])
    return None


def plain_roofline(ms_step, zones, nq, rk, peak_hbm, device):
    """The plain FP64 path against both of its ceilings: HBM (the compulsory
    state bytes per zone-update) and the FP64 pipe (its FP64 operations per
    zone-update from the committed ncu instruction counts, against the DFMA
    throughput measured here)."""
    import ctypes as C
    from mara2_gb300 import _native as N
    rate = zones / (ms_step * 1e-3)
    per_zone = (2 + 3 * (rk - 1)) * nq * 8
    hbm = rate * per_zone / 1e9
    tf = C.c_double(0.0)
    rc = N.load().mara_gpu_fp64_peak(device, C.byref(tf))
    flops = _profile_value("plain_fp64_kh.txt", "fp64_flops_per_zone_update")
    insts = _profile_value("plain_fp64_kh.txt", "fp64_pipe_inst_per_zone_update")
    out = {"hbm": {"achieved": hbm, "peak": peak_hbm, "unit": "GB/s", "frac": hbm / peak_hbm,
                   "algorithmic_bytes_per_zone_update": per_zone},
           "fp64_pipe": {"peak_tflops_measured": tf.value if rc == 0 else None,
                         "flops_per_zone_update": flops, "pipe_inst_per_zone_update": insts,
                         "achieved_tflops": rate * flops / 1e12 if flops else None,
                         "source": "per-zone FP64 counts from profiles/plain_fp64_kh.txt (ncu), "
                                   "peak from independent DFMA chains timed here"}}
    if rc == 0 and flops:
        out["fp64_pipe"]["frac_flops"] = out["fp64_pipe"]["achieved_tflops"] / tf.value
    if rc == 0 and insts:
        # one FMA instruction = two flops: the pipe's instruction rate is half the flop rate
        out["fp64_pipe"]["frac_pipe_issue"] = rate * insts / (tf.value * 1e12 / 2)
    return out


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


def l1_vs_fp64(s, P0, steps: int, device: int, precision: str = "mixed"):
    """Relative L1 density error of a mixed recipe against the plain FP64 path
    (bit-identical to the reference's CPU build) after `steps` steps of the
    same dt sequence."""
    from mara2_gb300.solver import Solver
    with Solver(s, "fp64", device) as a, Solver(s, precision, device) as b:
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


def _ref_worker(args):
    """One host process: the reference's own advance (its hot-path sources
    compiled in place, serial as the reference is) on its own copy of the
    workload, whole steps until the time budget is spent."""
    n_side, budget_s = args
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from mara2_gb300 import workloads as W
    s, P = W.kelvin_helmholtz(n_side)
    ref = O.Oracle("ref")
    c = O.make_config(law=s.law, recon=s.recon, riemann=s.riemann, bc=s.bc, rk_order=s.rk_order,
                      shape=s.shape, lower=s.lower, upper=s.upper, gamma=s.gamma, plm_theta=s.plm_theta)
    _, dtc = ref.courant(c, P)
    dt = s.cfl * dtc
    n, t0 = 0, time.perf_counter()
    while True:
        st, _ = ref.advance(c, P, dt)
        n += 1
        if st or time.perf_counter() - t0 > budget_s:
            break
    return n, time.perf_counter() - t0


def cpu_baseline(s, P0, budget_s: float = 20.0):
    """The reference's algorithm on the host cores.  Where its own hot-path
    sources built on this host (oracle/_ref, from the staged source tree), one
    serial process per host core, each advancing its own copy of the
    workload (the reference parallelises only by MPI ranks, absent here);
    else the oracle restatement with OpenMP over zones."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(False)
    if O.ref_available():
        import multiprocessing as mp
        procs = os.cpu_count() or 1
        with mp.get_context("spawn").Pool(procs) as pool:
            res = pool.map(_ref_worker, [(s.shape[0], budget_s)] * procs)
        steps = sum(n for n, _ in res)
        wall = max(t for _, t in res)
        return {"value": s.zones * steps / wall, "unit": UNIT, "cores": procs, "kind": "reference",
                "sample": f"{steps} whole steps of the {s.shape[0]}x{s.shape[1]} KH workload over {wall:.1f} s: "
                          f"the reference's own sources (compiled in place, g++ -O2 -ffp-contract=off), one "
                          f"serial process per host core, each on its own copy of the grid"}
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


def field_errors(s, out, ref):
    """Relative L1 and L-inf difference of every conserved field (out against
    ref, interior zones): L1 against the field's own L1 norm, and against the
    largest field's (fields that start at exactly zero have no norm of their
    own); L-inf against the field's largest magnitude."""
    from mara2_gb300 import workloads as W
    Ua = W.conserved(s, out[s.interior()])
    Ub = W.conserved(s, ref[s.interior()])
    big = max(float(np.sum(np.abs(Ub[..., q]))) for q in range(Ub.shape[-1]))
    res = {}
    for q, name in enumerate(W.CONSERVED_NAMES[s.law]):
        d = np.abs(Ua[..., q] - Ub[..., q])
        n1 = float(np.sum(np.abs(Ub[..., q])))
        ninf = float(np.max(np.abs(Ub[..., q])))
        res[name] = {"l1": float(np.sum(d)) / n1 if n1 > 0 else None,
                     "l1_vs_largest": float(np.sum(d)) / big,
                     "linf": float(np.max(d)) / ninf if ninf > 0 else None}
    return res


def run_plain_recorded(s, P0, device, t_final=None, steps=None):
    """The plain FP64 path (bit-identical to the reference's CPU build) one
    driver-loop step at a time, dt = CFL x Courant computed on the device
    (src/Problems.cpp:181-186): the dt sequence, the final state, the device
    time (CUDA events around each step on the handle's stream) and the
    failure count."""
    import torch
    from mara2_gb300.solver import Solver
    dts, ms = [], 0.0
    limit = steps if steps is not None else 10_000_000
    with Solver(s, "fp64", device) as g:
        g.upload(P0.copy())
        stream = torch.cuda.ExternalStream(g.stream, device=torch.device("cuda", device))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        while len(dts) < limit:
            a.record(stream)
            n = g.run(1, s.cfl, t_final)
            b.record(stream)
            if n == 0:
                break
            b.synchronize()
            ms += a.elapsed_time(b)
            dts.append(g.stats().last_dt)
        out = g.download()
        failures = g.stats().failures
    return out, dts, ms, failures


def run_replayed(s, P0, precision, dts, device):
    """A mixed recipe advanced with a given dt sequence (the plain path's):
    the final state and the failure count."""
    from mara2_gb300.solver import Solver
    with Solver(s, precision, device) as g:
        g.upload(P0.copy())
        for dt in dts:
            g.advance(dt)
        g.synchronize()
        return g.download(), g.stats().failures


def run_timed(s, P0, precision, device, t_final=None, steps=None):
    """Zone-updates/s of a device-driven run (dt on the device; with an end
    time the host looks at the device's done flag every 64 steps): CUDA
    events on the handle's stream around the run, after one untimed step
    that computes the first Courant step (a run of a stated step count takes
    that many steps in all)."""
    import torch
    from mara2_gb300.solver import Solver
    with Solver(s, precision, device) as g:
        g.upload(P0.copy())
        stream = torch.cuda.ExternalStream(g.stream, device=torch.device("cuda", device))
        g.run(1, s.cfl, t_final)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        n = g.run(steps - 1 if steps is not None else 10_000_000, s.cfl, t_final)
        b.record(stream)
        b.synchronize()
        ms = a.elapsed_time(b)
        return s.zones * n / (ms * 1e-3), n + 1, ms


RECIPES = {"mixed": "FP32 flux arithmetic, FP32-pair (~48-bit) accumulator, RMHD Newton residuals in pairs "
                    "with the FP64 iteration as fallback",
           "mixed_fp64": "FP32 flux arithmetic, FP64 accumulator, FP64 RMHD Newton iteration"}


def config_run(name, s, P0, device, t_final=None, steps=None, extra=None, control=False):
    """One workload at its stated length: the plain FP64 path (the reference's
    arithmetic) and both mixed recipes, the recipes' per-field error against
    the plain path on the plain path's dt sequence, failure counts.  With
    control, also the plain path itself from the initial state moved by one
    unit in the last place in every zone's density (same dt sequence): how
    far round-off alone carries the solution apart over the run."""
    out = {"zones": s.zones, "length": f"t = {t_final}" if t_final is not None else f"{steps} steps"}
    t0 = time.perf_counter()
    ref, dts, ms, fail = run_plain_recorded(s, P0, device, t_final, steps)
    out["steps"] = len(dts)
    out["plain_fp64"] = {"zone_updates_per_s": s.zones * len(dts) / (ms * 1e-3), "ms": ms, "failures": fail,
                         "timing": "CUDA events around each driver step (host reads dt between steps)"}
    if extra:
        out["plain_fp64"].update(extra(ref))
    for prec in RECIPES:
        rate, n, rms = run_timed(s, P0, prec, device, t_final, steps)
        res, rfail = run_replayed(s, P0, prec, dts, device)
        entry = {"zone_updates_per_s": rate, "steps": n, "ms": rms, "failures": rfail,
                 "over_plain": rate / out["plain_fp64"]["zone_updates_per_s"],
                 "error_vs_plain_fp64": field_errors(s, res, ref)}
        if extra:
            entry.update(extra(res))
        out[prec] = entry
        del res
    if control:
        P1 = P0.copy()
        P1[..., 0] = np.nextafter(P1[..., 0], np.inf)
        res, _ = run_replayed(s, P1, "fp64", dts, device)
        out["fp64_one_ulp_control"] = {
            "perturbation": "initial density + 1 ulp in every zone (guards alike), plain FP64, same dt sequence",
            "error_vs_plain_fp64": field_errors(s, res, ref)}
        del res, P1
    out["wall_s"] = time.perf_counter() - t0
    del ref
    return out


def serving_suite(device, requests=4096, rate=2000.0, sample=8, budget_gb=96.0):
    """configs[4]: the Poisson stream of Riemann problems served with
    continuous batching, then a stream below saturation, and the baseline
    of a seeded sample of the same requests each solved alone on the plain
    FP64 path (with the served results' error against it)."""
    from mara2_gb300 import workloads as W
    from mara2_gb300.batch import autotune, run_alone, serve
    from mara2_gb300.solver import Solver
    tiles = autotune(device)
    reqs = W.riemann_stream(requests, rate=rate)
    rng = np.random.default_rng(20261204)
    pick = sorted(int(i) for i in rng.choice(len(reqs), size=sample, replace=False))
    form = {"tile_1d": tiles["tile_1d"], "tile_2d": tiles["tile_2d"], "persistent": tiles["persistent"],
            "ctas_per_sm": tiles["ctas_per_sm"]}
    res = serve(reqs, budget_bytes=int(budget_gb * (1 << 30)), device=device, keep_results=set(pick), **form)
    out = {"stream": f"{requests} Riemann problems (1-D N log-uniform [256, 8192], 2-D side log-uniform "
                     f"[128, 512]), Poisson {rate}/s, t = 0.2, PLM + HLLC, RK2, seed {W.RIEMANN_SEED}",
           "saturated": res.summary(), "launch_form": form, "autotune": tiles,
           "budget_bytes": int(budget_gb * (1 << 30))}
    # below saturation: the same distribution at half the measured capacity
    zu_mean = res.zone_updates / max(1, res.completed)
    cap = res.summary()["zone_updates_per_s"] / zu_mean
    sub_rate = 0.5 * cap
    sub = W.riemann_stream(512, rate=sub_rate, seed=W.RIEMANN_SEED + 7)
    r2 = serve(sub, budget_bytes=int(budget_gb * (1 << 30)), device=device, **form)
    out["below_saturation"] = {**r2.summary(), "rate_per_s": sub_rate,
                               "offered_load": "half the saturated stream's capacity (requests/s)"}
    # each sampled request alone: plain FP64 (the configs' baseline) and mixed
    zu = secs = zm = msecs = 0.0
    errs, lat = [], []
    for i in pick:
        r = reqs[i]
        s, P = W.riemann_initial(r)
        t0 = time.perf_counter()
        with Solver(s, "fp64", device) as g:
            g.upload(P.copy())
            n = g.run(10_000_000, s.cfl, s.t_final)
            ref = g.download()
        el = time.perf_counter() - t0
        zu += s.zones * n
        secs += el
        lat.append(el)
        t0 = time.perf_counter()
        _, _, nm = run_alone(s, P, s.t_final)
        msecs += time.perf_counter() - t0
        zm += s.zones * nm
        e = field_errors(s, res.results[i][0], ref)
        errs.append({"request": i, "dims": s.dims, "n": r.n, "density_l1": e["density"]["l1"],
                     "density_linf": e["density"]["linf"],
                     "max_field_l1_vs_largest": max(v["l1_vs_largest"] for v in e.values())})
    out["alone_plain_fp64"] = {"zone_updates_per_s": zu / secs, "latency_mean_s": float(np.mean(lat)),
                               "requests": len(pick), "sample": "seeded random sample of the stream"}
    out["alone_mixed"] = {"zone_updates_per_s": zm / msecs}
    out["served_vs_alone_plain_fp64"] = errs
    out["served_over_alone_plain"] = out["saturated"]["zone_updates_per_s"] / out["alone_plain_fp64"]["zone_updates_per_s"]
    return out


def workload_suite(device: int, serving_requests: int = 4096):
    """Every configuration at its stated length: plain FP64 (the reference's
    arithmetic on the GPU) beside both mixed recipes."""
    from mara2_gb300 import workloads as W
    out = {"recipes": RECIPES}

    # configs[0]: Sod 1024 to t = 0.2
    s, P0 = W.sod(1024)
    out["sod_1024_t0.2"] = config_run("sod", s, P0, device, t_final=s.t_final)

    # configs[1]: Kelvin-Helmholtz 1024^2 to t = 1.0
    s, P0 = W.kelvin_helmholtz(1024)
    out["kh_1024_t1.0"] = config_run("kh", s, P0, device, t_final=1.0, control=True)

    # configs[2]: MHD turbulence with CT, 256^3, RK3, 100 steps
    s, P0 = W.mhd_turbulence(256)
    dx = 1.0 / 256
    bmax = float(np.abs(P0[..., 5:8]).max())

    def div_b(P):
        from mara2_gb300.solver import ct_monopole
        B = np.ascontiguousarray(P[s.interior()][..., 5:8])
        M = ct_monopole(B, "periodic", "vert", device)
        return {"max_abs_div_b_dx_over_bmax": float(np.abs(M).max()) / bmax}

    out["mhd_ct_256cube_100steps"] = config_run("mhd", s, P0, device, steps=100, extra=div_b)
    out["mhd_ct_256cube_100steps"]["div_b_measure"] = (
        "UniformCartesianCT vertex monopole (sum of face-averaged field differences, i.e. div B x dx) of the "
        "final cell field, over max |B| of the initial state")
    del P0

    # configs[3]: relativistic MHD blast 512^2 to t = 4.0
    s, P0 = W.rmhd_blast(512)
    out["rmhd_blast_512_t4.0"] = config_run("rmhd", s, P0, device, t_final=4.0, control=True)

    # configs[4]: the serving stream
    out["serving_riemann_4096"] = serving_suite(device, requests=serving_requests)
    return out


def _events_ms(solver, device, fn, reps: int) -> float:
    """Mean device ms of fn() (work enqueued on the handle's stream), CUDA
    events on that stream around each call, one untimed call first."""
    import torch
    stream = torch.cuda.ExternalStream(solver.stream, device=torch.device("cuda", device))
    fn()
    ms = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
    return float(np.mean(ms))


def next_rows_suite(device: int, peak_hbm: float):
    """The rows beside the time step (device diagnostics, device initial
    data, source terms) measured on the resident state: device ms per call
    (CUDA events on the handle's stream; each call also returns its result to
    the host), the algorithmic bytes each call must move in HBM and the
    achieved fraction of the measured HBM rate."""
    from mara2_gb300 import workloads as W
    from mara2_gb300.solver import Solver
    out = {}

    def hbm(ms, nbytes):
        gbs = nbytes / (ms * 1e-3) / 1e9
        return {"ms": ms, "algorithmic_bytes": nbytes, "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / peak_hbm}

    # FieldOperator::volumeIntegratedDiagnostics and the largest
    # CellCenteredFieldCT::monopole on MHD 256^3: each reads the resident
    # state once (8 fields; the field's 3 for the monopole) at 8 B a value
    s, P0 = W.mhd_turbulence(256)
    for prec in ("fp64", "mixed"):
        with Solver(s, prec, device) as g:
            g.upload(P0)
            ms = _events_ms(g, device, g.volume_diagnostics, 10)
            out[f"volume_diagnostics_mhd256_{prec}"] = hbm(ms, s.zones * 8 * 8)
            ms = _events_ms(g, device, lambda: g.monopole_max(1.0 / 256), 10)
            out[f"monopole_max_mhd256_{prec}"] = hbm(ms, s.zones * 3 * 8)
    # the checkpoint's cell fields (monopole, current) to the host: 4 doubles a
    # cell with guards over the host link, into page-locked and into pageable
    # host memory
    import torch
    with Solver(s, "fp64", device) as g:
        g.upload(P0)
        cells = int(np.prod(s.full_shape[:3]))
        pinned = torch.empty(tuple(s.full_shape[:3]) + (4,), dtype=torch.float64).pin_memory().numpy()
        for name, buf in (("page_locked", pinned), ("pageable", None)):
            ms = _events_ms(g, device, lambda: g.field_diagnostics(1.0 / 256, buf), 3)
            out[f"field_diagnostics_mhd256_to_host_{name}"] = {"ms": ms, "bytes_to_host": cells * 32,
                                                               "achieved_gbs": cells * 32 / (ms * 1e-3) / 1e9}
        del pinned
    del P0

    # MeshOperator::generate on the device: the KH shear layer with its
    # seeded perturbation written into the resident state (FP64 primitives
    # with guards; FP32 pairs of conserved densities)
    s, spec = W.device_initial_data("kh", 1024)
    for prec in ("fp64", "mixed"):
        with Solver(s, prec, device) as g:
            ms = _events_ms(g, device, lambda: g.generate(spec), 10)
            nbytes = int(np.prod(s.full_shape[:3])) * 5 * 8 if prec == "fp64" else s.zones * 5 * 8
            out[f"generate_kh1024_{prec}"] = hbm(ms, nbytes)

    # source terms (SolutionSchemes.cpp:219-228): the plain step of KH 1024^2
    # with the library's uniform gravity against the same step without
    s, P0 = W.kelvin_helmholtz(1024)
    with Solver(s, "fp64", device) as g:
        g.upload(P0)
        dt = 0.2 * g.courant()
        base = _events_ms(g, device, lambda: g.advance(dt), 5)
        g.set_source_terms(gravity=(0.0, -0.1, 0.0))
        with_src = _events_ms(g, device, lambda: g.advance(dt), 5)
        g.set_source_terms()
        out["source_terms_gravity_kh1024_fp64"] = {"step_ms": base, "step_ms_with_source": with_src,
                                                   "overhead": with_src / base - 1.0}
    # NewtonianMHD cooling (an auxiliary field, ConservationLaws.cpp:489-501)
    # on the plain MHD 128^3 step against the same step without
    s, P0 = W.mhd_turbulence(128)
    sc, P1 = W.with_cooling(s, P0.copy(), 0.4, aux=0.02)
    steps = {}
    for name, ss, PP in (("base", s, P0), ("cooling", sc, P1)):
        with Solver(ss, "fp64", device) as g:
            g.upload(PP)
            dt = 0.2 * g.courant()
            steps[name] = _events_ms(g, device, lambda: g.advance(dt), 3)
    out["source_terms_cooling_mhd128_fp64"] = {"step_ms": steps["base"], "step_ms_with_cooling": steps["cooling"],
                                               "overhead": steps["cooling"] / steps["base"] - 1.0}
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
    ap.add_argument("--serving-requests", type=int, default=4096)
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
        # the reference's own CPU implementation on the host cores (rank 0
        # only; no GPU work in this process, so the spawned workers start clean)
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

    # the benchmark spec's recipe (FP64 accumulator), same workload and timing rules
    with Solver(s, "mixed_fp64", local) as g64:
        g64.upload(P0.copy())
        ms_fp64acc, _, _ = time_resident(g64, args.steps, args.warmup, local)
        roof64 = kernel_roofline(g64, min(args.steps, 20), s.zones, s.nq, s.rk_order, peak, peak_kind)
    with Solver(s, "fp64", local) as gp:
        gp.upload(P0.copy())
        ms_plain, _, _ = time_resident(gp, max(3, args.steps // 5), 3, local)
    l1_rho, linf_rho = l1_vs_fp64(s, P0, 20, local)
    l1_64, linf_64 = l1_vs_fp64(s, P0, 20, local, "mixed_fp64")
    suite = None if args.no_workloads or rank != 0 else workload_suite(local, args.serving_requests)
    next_rows = None if args.no_workloads or rank != 0 else next_rows_suite(local, peak)

    if rank != 0:
        return
    cb = cpu_baseline(s, P0, args.cpu_budget)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_job, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 flux arithmetic, f32-pair accumulator", "data": "synthetic", "config": config,
        "precision": "mixed",
        "recipe": RECIPES["mixed"],
        "fp64_accumulator": {"value": s.zones / (ms_fp64acc * 1e-3), "unit": UNIT, "ms_per_step": ms_fp64acc,
                             "recipe": RECIPES["mixed_fp64"], "l1_density_vs_fp64": l1_64,
                             "linf_density_vs_fp64": linf_64, "l1_steps": 20,
                             "roofline": {k: roof64[k] for k in ("achieved", "frac", "mean_launch_ms")}},
        "l1_density_vs_fp64": l1_rho, "linf_density_vs_fp64": linf_rho, "l1_steps": 20,
        "plain_fp64": {"value": s.zones / (ms_plain * 1e-3), "unit": UNIT, "ms_per_step": ms_plain,
                       "dtype": "f64", "parity": "bit-identical to the reference's CPU build",
                       "roofline": plain_roofline(ms_plain, s.zones, s.nq, s.rk_order, peak, local)},
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
        "next_rows": next_rows,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
