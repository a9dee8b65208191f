"""Shared test helpers: oracle configs from a Scheme, error metrics."""
from __future__ import annotations

import numpy as np

import oracle as O


def oracle_config(s):
    return O.make_config(law=s.law, recon=s.recon, riemann=s.riemann, bc=s.bc, rk_order=s.rk_order,
                         shape=s.shape, lower=s.lower, upper=s.upper, gamma=s.gamma,
                         plm_theta=s.plm_theta, weno_is=s.weno_is, shenzha_A=s.shenzha_A,
                         pressure_floor=s.pressure_floor, disable_ct=s.disable_ct,
                         ng=max(s.ng))


def rel_l1(a, b, axis_q=None):
    """Relative L1 difference per conserved field (last axis)."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    nq = a.shape[-1]
    out = []
    for q in range(nq):
        den = np.sum(np.abs(b[..., q]))
        num = np.sum(np.abs(a[..., q] - b[..., q]))
        out.append(num / den if den > 0 else num)
    return np.array(out)


def interior(s, P):
    return P[s.interior()]
