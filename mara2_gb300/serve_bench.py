"""Serving benchmark of the batched path: a seeded Poisson stream of Riemann
problems (1-D N log-uniform in [256, 8192], 2-D side log-uniform in
[128, 512], PLM + HLLC, RK2, t = 0.2), continuously batched on one GPU.

  python -m mara2_gb300.serve_bench --requests 4096 --rate 2000 --budget-gb 64

Prints one JSON object: throughput (zone-updates/s over the whole stream),
p50 / p99 latency (arrival -> result on the host), the tile shapes the
autotuner chose, and the baselines: a sample of the same requests each solved
alone with the plain FP64 path and alone in the mixed path.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import build, workloads as W
from .batch import autotune, run_alone, serve


def alone_rates(reqs, sample: int, precision: str):
    """Zone-updates/s of requests each solved by itself (plain FP64 through
    the single-grid handle, or mixed through a batch of one)."""
    from .solver import Solver
    zu, secs = 0, 0.0
    for r in reqs[:sample]:
        s, P = W.riemann_initial(r)
        t0 = time.perf_counter()
        if precision == "fp64":
            with Solver(s, "fp64") as g:
                g.upload(P)
                n = g.run(1_000_000, s.cfl, s.t_final)
        else:
            _, _, n = run_alone(s, P, s.t_final)
        secs += time.perf_counter() - t0
        zu += s.zones * n
    return zu / secs, zu, secs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=4096)
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--budget-gb", type=float, default=64.0)
    ap.add_argument("--steps-per-poll", type=int, default=8)
    ap.add_argument("--alone-sample", type=int, default=6)
    ap.add_argument("--retune", action="store_true")
    args = ap.parse_args()
    build.build()
    tiles = autotune(force=args.retune)
    reqs = W.riemann_stream(args.requests, rate=args.rate)
    res = serve(reqs, budget_bytes=int(args.budget_gb * (1 << 30)), steps_per_poll=args.steps_per_poll,
                tile_1d=tiles["tile_1d"], tile_2d=tiles["tile_2d"])
    out = {"workload": f"{args.requests} Riemann problems, Poisson rate {args.rate}/s, seed {W.RIEMANN_SEED}",
           **res.summary(), "tiles": tiles, "budget_bytes": int(args.budget_gb * (1 << 30))}
    # baselines on the smallest-work requests of the stream (bounded time)
    small = sorted(reqs, key=lambda r: r.zones())[: max(args.alone_sample * 4, 1)]
    pick = small[:: max(1, len(small) // args.alone_sample)][: args.alone_sample]
    out["alone_plain_fp64_zone_updates_per_s"], zu, secs = alone_rates(pick, len(pick), "fp64")
    out["alone_mixed_zone_updates_per_s"], _, _ = alone_rates(pick, len(pick), "mixed")
    out["alone_sample"] = f"{len(pick)} of the stream's smallest requests, each solved by itself"
    print(json.dumps(out))


if __name__ == "__main__":
    main()
