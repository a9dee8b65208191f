"""Shared test helpers: oracle configs from a Scheme, error metrics."""
from __future__ import annotations

import numpy as np

import oracle as O


def oracle_config(s):
    return O.make_config(law=s.law, recon=s.recon, riemann=s.riemann, bc=s.bc, rk_order=s.rk_order,
                         shape=s.shape, lower=s.lower, upper=s.upper, gamma=s.gamma,
                         plm_theta=s.plm_theta, weno_is=s.weno_is, shenzha_A=s.shenzha_A,
                         pressure_floor=s.pressure_floor, disable_ct=s.disable_ct,
                         ng=max(s.ng), cooling_rate=s.cooling_rate)


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


def parity_error(s, a, b):
    """The parity metric of the plain path: relative L1 difference per
    conserved field, for every law."""
    return rel_l1(a, b)


def rel_linf(a, b):
    """L-infinity difference per conserved field relative to the field's
    largest magnitude."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    out = []
    for q in range(a.shape[-1]):
        den = np.max(np.abs(b[..., q]))
        num = np.max(np.abs(a[..., q] - b[..., q]))
        out.append(num / den if den > 0 else num)
    return np.array(out)


def rel_l1_max(a, b):
    """L1 difference per conserved field relative to the largest field's L1
    norm: the mixed path's measure for fields that start at exactly zero
    (a transverse field or momentum), which have no norm of their own."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    big = max(np.sum(np.abs(b[..., q])) for q in range(a.shape[-1]))
    return np.array([np.sum(np.abs(a[..., q] - b[..., q])) / big for q in range(a.shape[-1])])
