"""Constrained transport on the GPU: the device monopole diagnostic
(CellCenteredFieldCT::monopole) against the oracle's, and div B kept at
roundoff by the flux-CT update on the 3-D MHD workload."""
import numpy as np
import pytest

from helpers import oracle_config
from mara2_gb300 import workloads as W
from mara2_gb300.solver import Solver


@pytest.mark.gpu
def test_monopole_matches_oracle(gpu_lib, port):
    s, P = W.mhd_turbulence(12)
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        g.run(3)
        m_gpu = g.monopole_max(1.0)
        out = g.download()
    B = np.ascontiguousarray(out[..., 5:8])
    M = port.monopole_cell(B, 1.0)[s.interior()]
    m_ref = float(np.abs(M).max())
    assert abs(m_gpu - m_ref) <= 1e-12 * max(m_ref, 1e-300) + 1e-300


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-5)])
def test_ct_keeps_div_b_at_roundoff(gpu_lib, precision, tol):
    s, P = W.mhd_turbulence(24)
    dx = 1.0 / 24
    bmax = float(np.abs(P[..., 5:8]).max())
    with Solver(s, precision) as g:
        g.upload(P.copy())
        m0 = g.monopole_max(dx)
        g.run(20)
        m1 = g.monopole_max(dx)
    # |div B| relative to |B| / dx, the scale of one cell's flux imbalance;
    # the mixed path holds B in FP32, so its initial field already carries
    # FP32 rounding in the divergence
    assert m0 * dx / bmax < tol
    assert m1 * dx / bmax < tol, (precision, m1 * dx / bmax)
