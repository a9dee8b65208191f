"""Generate the golden fixtures in this directory from the reference itself.

Run where the reference tree is available (the reference's hot-path sources
are compiled in place by ``make -C oracle ref``):

    python tests/golden/make_golden.py

Each fixture holds a seeded initial state, the dt sequence the reference's
driver loop chose (Courant step x CFL), the reference's final state after
those steps, and for one magnetised case the CT-corrected Godunov fluxes of
the initial state.  The files are small and are committed so that machines
without the reference tree (the GPU machine) can check against them.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from mara2_gb300 import workloads as W  # noqa: E402

sys.path.insert(0, os.path.join(ROOT, "tests"))
from helpers import oracle_config  # noqa: E402

CASES = {
    "sod64_plm_hlle_rk2": (lambda: W.sod(64), 25),
    "kh24_plm_hllc_rk2": (lambda: W.kelvin_helmholtz(24), 6),
    "kh24_pcm_hlle_rk1_reflecting": (lambda: _with(W.kelvin_helmholtz(24), recon="pcm", riemann="hlle",
                                                    rk_order=1, bc="reflecting", guard=2), 6),
    "mhd8cube_plm_hlle_rk3_ct": (lambda: W.mhd_turbulence(8), 3),
    "rmhd16_weno5_hlle_rk3": (lambda: W.rmhd_blast(16), 3),
}


def _with(sp, **kw):
    s, P = sp
    return s.with_(**kw), P


def main():
    O.build(ref=True)
    ref = O.Oracle("ref")
    for name, (make, steps) in CASES.items():
        s, P0 = make()
        c = oracle_config(s)
        P = P0.copy()
        status, t, dts = ref.run(c, P, steps, s.cfl, s.t_final)
        assert status == 0, (name, status)
        extra = {}
        if s.law != "hydro":
            st, F = ref.godunov(c, P0.copy())
            assert st == 0
            extra["godunov_fluxes"] = F
        np.savez_compressed(os.path.join(HERE, name + ".npz"), P0=P0, P=P, dts=np.array(dts),
                            scheme=repr(s), **extra)
        print(name, steps, "steps", os.path.getsize(os.path.join(HERE, name + ".npz")), "bytes")


if __name__ == "__main__":
    main()
