"""Run one workload for a few steps (the target of the ncu captures whose
summaries live in profiles/).

  python -m mara2_gb300.profile_case --workload kh --n 2048 --precision mixed --steps 4
"""
from __future__ import annotations

import argparse

from . import build, workloads as W
from .solver import Solver


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="kh", choices=["kh", "sod", "mhd", "rmhd"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--steps", type=int, default=4)
    args = ap.parse_args()
    build.build()
    make = {"kh": W.kelvin_helmholtz, "sod": W.sod, "mhd": W.mhd_turbulence, "rmhd": W.rmhd_blast}[args.workload]
    s, P = make(args.n)
    with Solver(s, args.precision) as g:
        g.upload(P)
        n = g.run(args.steps)
        g.synchronize()
    print(f"{args.workload} n={args.n} {args.precision}: {n} steps ok")


if __name__ == "__main__":
    main()
