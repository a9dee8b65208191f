"""Batched grids and the serving loop over include/mara_batch.h.

``Batch``  -- many resident hydro grids advanced together: a launch per
             tile list and RK stage (the step replayed from a CUDA graph),
             or the whole step in one cooperative launch (``persistent``).
``serve``  -- continuous batching of a stream of requests: each request is
             admitted as soon as it has arrived and the HBM budget / grid
             table has room, advanced together with whatever else is
             resident, and retired (result copied to the host) as soon as it
             reaches its end time; reports throughput and p50/p99 latency.
``autotune`` -- picks the 1-D and 2-D tile shapes and the launch form (and
             its CTAs per SM) by timing each candidate on a representative
             mix, and caches the choice.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .scheme import Scheme

MARA_ERR_NO_ROOM = 36
TILE_2D = {1: "32x8", 2: "32x16", 3: "64x8", 4: "32x16-oneface"}
CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")


class MaraBatchConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget_bytes", C.c_int64), ("max_grids", C.c_int),
                ("max_zones_per_grid", C.c_int), ("recon", C.c_int), ("riemann", C.c_int),
                ("rk_order", C.c_int), ("tile_1d", C.c_int), ("tile_2d", C.c_int), ("lockstep_1d", C.c_int),
                ("persistent", C.c_int), ("ctas_per_sm", C.c_int)]


class MaraBatchStats(C.Structure):
    _fields_ = [("active", C.c_int), ("finished", C.c_int), ("zones", C.c_int64), ("bytes_in_use", C.c_int64),
                ("zone_updates", C.c_int64), ("steps", C.c_int64), ("kernel_launches", C.c_int64)]


_H = C.c_void_p
SIGNATURES = {
    "mara_batch_create": (C.c_int, [C.POINTER(MaraBatchConfig), C.POINTER(C.c_void_p)]),
    "mara_batch_destroy": (C.c_int, [_H]),
    "mara_batch_admit": (C.c_int, [_H, C.POINTER(N.MaraGpuConfig), C.c_void_p, C.c_double, C.c_double,
                                   C.POINTER(C.c_int)]),
    "mara_batch_step": (C.c_int, [_H, C.c_int]),
    "mara_batch_poll": (C.c_int, [_H, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int)]),
    "mara_batch_retire": (C.c_int, [_H, C.c_int, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "mara_batch_stats": (C.c_int, [_H, C.POINTER(MaraBatchStats)]),
    "mara_batch_tiles": (C.c_int, [_H, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mara_batch_launch_form": (C.c_int, [_H, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
}


def load():
    lib = N.load()
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


class Batch:
    def __init__(self, budget_bytes: int, max_grids: int = 4096, max_zones_per_grid: int = 600 * 600,
                 recon: str = "plm", riemann: str = "hllc", rk_order: int = 2, tile_1d: int = 0,
                 tile_2d: int = 0, device: int = 0, lockstep_1d: bool = False, persistent: bool = False,
                 ctas_per_sm: int = 0):
        self.lib = load()
        c = MaraBatchConfig()
        c.device, c.hbm_budget_bytes, c.max_grids = device, int(budget_bytes), max_grids
        c.max_zones_per_grid, c.recon, c.riemann = max_zones_per_grid, N.RECON[recon], N.RIEMANN[riemann]
        c.rk_order, c.tile_1d, c.tile_2d = rk_order, tile_1d, tile_2d
        c.lockstep_1d = int(lockstep_1d)
        c.persistent, c.ctas_per_sm = int(persistent), ctas_per_sm
        self.cfg = c
        h = C.c_void_p()
        N.check(self.lib.mara_batch_create(C.byref(c), C.byref(h)), "mara_batch_create")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.mara_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def admit(self, s: Scheme, P: np.ndarray, t_final: float, cfl: float | None = None) -> int | None:
        """Admit one grid; None when the budget or the grid table is full."""
        cfg = N.config_from_scheme(s, "mixed", self.device)
        P = np.ascontiguousarray(P, dtype=np.float64)
        slot = C.c_int(-1)
        rc = self.lib.mara_batch_admit(self.h, C.byref(cfg), P.ctypes.data, t_final,
                                       s.cfl if cfl is None else cfl, C.byref(slot))
        if rc == MARA_ERR_NO_ROOM:
            return None
        N.check(rc, "mara_batch_admit")
        return slot.value

    def step(self, n: int = 1) -> None:
        N.check(self.lib.mara_batch_step(self.h, n), "mara_batch_step")

    def poll(self, cap: int = 4096) -> list:
        buf = (C.c_int * cap)()
        n = C.c_int(0)
        N.check(self.lib.mara_batch_poll(self.h, buf, cap, C.byref(n)), "mara_batch_poll")
        return [buf[k] for k in range(min(n.value, cap))]

    def retire(self, slot: int, shape) -> tuple:
        out = np.empty(shape, dtype=np.float64)
        t = C.c_double()
        st = C.c_int64()
        N.check(self.lib.mara_batch_retire(self.h, slot, out.ctypes.data, C.byref(t), C.byref(st)),
                "mara_batch_retire")
        return out, t.value, st.value

    def stats(self) -> MaraBatchStats:
        s = MaraBatchStats()
        self.lib.mara_batch_stats(self.h, C.byref(s))
        return s

    def tiles(self):
        a, b = C.c_int(), C.c_int()
        self.lib.mara_batch_tiles(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def launch_form(self):
        """(persistent, CTAs): one cooperative launch per step call, or the
        per-stage launches."""
        a, b = C.c_int(), C.c_int()
        self.lib.mara_batch_launch_form(self.h, C.byref(a), C.byref(b))
        return bool(a.value), b.value


def run_alone(s: Scheme, P: np.ndarray, t_final: float, **kw):
    """One request by itself in a batch (the reference form of the invariance
    test): returns (P, t, steps)."""
    with Batch(budget_bytes=max(1 << 26, 200 * s.zones), max_grids=4, max_zones_per_grid=int(np.prod(s.full_shape[:3])),
               **kw) as b:
        slot = b.admit(s, P, t_final)
        while True:
            b.step(16)
            if slot in b.poll():
                return b.retire(slot, s.full_shape)


# ----------------------------------------------------------------------------
@dataclass
class ServeResult:
    completed: int = 0
    wall_s: float = 0.0
    zone_updates: int = 0
    latencies: list = field(default_factory=list)
    queue_waits: list = field(default_factory=list)
    peak_active: int = 0
    peak_bytes: int = 0
    results: dict = field(default_factory=dict)
    # per request, in completion order: (index, latency s, queue wait s, steps)
    records: list = field(default_factory=list)

    def summary(self) -> dict:
        lat = np.array(self.latencies) if self.latencies else np.array([np.nan])
        return {"requests": self.completed, "wall_s": self.wall_s,
                "zone_updates": self.zone_updates,
                "zone_updates_per_s": self.zone_updates / self.wall_s if self.wall_s else None,
                "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
                "latency_max_s": float(np.max(lat)),
                "queue_wait_p50_s": float(np.percentile(self.queue_waits, 50)) if self.queue_waits else None,
                "peak_active_grids": self.peak_active, "peak_bytes": self.peak_bytes}


def serve(requests, budget_bytes: int, steps_per_poll: int = 8, keep_results=False,
          max_grids: int = 4096, tile_1d: int = 0, tile_2d: int = 0, device: int = 0, make=None,
          lockstep_1d: bool = False, persistent: bool = False, ctas_per_sm: int = 0) -> ServeResult:
    """Continuous batching of `requests` (objects with .arrival seconds and a
    way to build (Scheme, P) through `make(req)`), arrivals replayed against
    the wall clock.  keep_results: True keeps every result, a set of request
    indices keeps those."""
    from . import workloads as W
    make = make or W.riemann_initial
    pending = deque(sorted(requests, key=lambda r: r.arrival))
    queue = deque()
    inflight = {}
    res = ServeResult()
    max_cells = max(int(np.prod(make(r)[0].full_shape[:3])) for r in [max(requests, key=lambda r: r.zones())])
    with Batch(budget_bytes, max_grids=max_grids, max_zones_per_grid=max_cells, tile_1d=tile_1d,
               tile_2d=tile_2d, device=device, lockstep_1d=lockstep_1d, persistent=persistent,
               ctas_per_sm=ctas_per_sm) as b:
        t0 = time.perf_counter()
        while pending or queue or inflight:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                s, P = make(r)
                queue.append((r, s, P))
            # admit in arrival order while there is room
            while queue:
                r, s, P = queue[0]
                slot = b.admit(s, P, s.t_final)
                if slot is None:
                    break
                queue.popleft()
                inflight[slot] = (r, s, time.perf_counter() - t0)
            if inflight:
                # while requests wait to arrive or to be admitted, poll often;
                # afterwards only retirement waits on a poll
                b.step(steps_per_poll if (queue or pending) else 4 * steps_per_poll)
                for slot in b.poll():
                    r, s, t_admit = inflight.pop(slot)
                    out, t, nsteps = b.retire(slot, s.full_shape)
                    done_t = time.perf_counter() - t0
                    res.latencies.append(done_t - r.arrival)
                    res.queue_waits.append(t_admit - r.arrival)
                    res.zone_updates += s.zones * nsteps
                    res.completed += 1
                    res.records.append((r.index, done_t - r.arrival, t_admit - r.arrival, nsteps))
                    if keep_results is True or (keep_results and r.index in keep_results):
                        res.results[r.index] = (out, t, nsteps)
                st = b.stats()
                res.peak_active = max(res.peak_active, st.active)
                res.peak_bytes = max(res.peak_bytes, st.bytes_in_use)
            elif pending:
                time.sleep(max(0.0, min(0.001, pending[0].arrival - (time.perf_counter() - t0))))
        res.wall_s = time.perf_counter() - t0
    return res


# ----------------------------------------------------------------------------
def autotune(device: int = 0, sample: int = 48, steps: int = 40, force: bool = False) -> dict:
    """Time the launch configurations on a representative mix of the
    Riemann workload (grids of the stream's size distribution) and cache the
    fastest: the 1-D tile (128 / 256 / 512 zones, 1-D grids in the tile
    lists), then for the 2-D grids the launch form - per-stage launches with
    each 2-D tile shape (32x8, 32x16, 64x8; PLM faces in runs along their
    normal) and 32x16 with one face per thread, or the persistent cooperative
    launch with each tile shape it supports (32x8, 32x16) and 2, 3 or 4 CTAs
    per SM."""
    if not force and os.path.exists(CACHE):
        with open(CACHE) as f:
            best = json.load(f)
        if "persistent" in best:
            return best
    import torch
    from . import workloads as W
    reqs = W.riemann_stream(sample, seed=W.RIEMANN_SEED + 1)
    grids = [W.riemann_initial(r) for r in reqs]

    def time_batch(sel, **kw):
        zones = sum(s.zones for s, _ in sel)
        with Batch(budget_bytes=200 * zones + (1 << 26), max_grids=len(sel) + 1,
                   max_zones_per_grid=max(int(np.prod(s.full_shape[:3])) for s, _ in sel), device=device,
                   **kw) as b:
            for s, P in sel:
                b.admit(s, P, 1e9)
            b.step(3)
            b.poll()
            torch.cuda.synchronize(device)
            t0 = time.perf_counter()
            b.step(steps)
            b.poll()
            return (time.perf_counter() - t0) / steps

    best = {}
    sel1 = [(s, P) for s, P in grids if s.dims == 1]
    timing1 = {c: time_batch(sel1, tile_1d=c, lockstep_1d=True) for c in (128, 256, 512)}
    best["tile_1d"] = min(timing1, key=timing1.get)
    best["timing_1d_ms"] = {str(k): v * 1e3 for k, v in timing1.items()}
    sel2 = [(s, P) for s, P in grids if s.dims == 2]
    cands = [("stage", t2, 0) for t2 in (1, 2, 3, 4)] + [("persistent", t2, c) for t2 in (1, 2) for c in (2, 3, 4)]
    timing = {}
    for form, t2, ctas in cands:
        timing[(form, t2, ctas)] = time_batch(sel2, tile_2d=t2, persistent=form == "persistent", ctas_per_sm=ctas)
    form, t2, ctas = min(timing, key=timing.get)
    best["tile_2d"] = t2
    best["persistent"] = form == "persistent"
    best["ctas_per_sm"] = ctas
    best["timing_2d_ms"] = {f"{f}/{TILE_2D[t]}/{c}": v * 1e3 for (f, t, c), v in timing.items()}
    if best["persistent"] and best["tile_1d"] not in (256, 512):
        best["tile_1d"] = 256 if timing1[256] <= timing1[512] else 512
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    with open(CACHE, "w") as f:
        json.dump(best, f, indent=1)
    return best
