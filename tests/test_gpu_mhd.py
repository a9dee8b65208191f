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


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [{}, dict(disable_ct=True, rk_order=3)])
def test_cooling_matches_oracle_bitwise(gpu_lib, port, kw):
    """NewtonianMHD with a cooling rate on the plain path: the auxiliary
    field, the cooling source terms and the CT of the three field components
    (not of the auxiliary), through eager advances and the captured driver
    loop; the volume diagnostics gain auxiliary1."""
    s, P = W.mhd_turbulence(10)
    s, P = W.with_cooling(s.with_(**kw), P, 0.4, aux=0.02)
    c = oracle_config(s)
    A = P.copy()
    dts = []
    for _ in range(4):
        _, dt = port.courant(c, A)
        dts.append(s.cfl * dt)
        assert port.advance(c, A, s.cfl * dt)[0] == 0
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        for dt in dts[:2]:
            g.advance(dt)
        mid = g.download()
        g.upload(mid)
        g.run(2)
        out = g.download()
        d = g.volume_diagnostics()
    assert np.array_equal(out.view(np.uint64), A.view(np.uint64))
    st, D, Dabs = port.volume_diagnostics(c, A)
    assert st == 0 and list(d)[-1] == "auxiliary1" and len(d) == 18
    got = np.array(list(d.values()))
    assert np.all(np.abs(got - D) <= 1e-13 * Dabs + 1e-300)


@pytest.mark.gpu
def test_cooling_needs_plain_path(gpu_lib):
    from mara2_gb300 import _native as N
    s, P = W.mhd_turbulence(8)
    s, P = W.with_cooling(s, P, 0.4)
    with pytest.raises(N.MaraError) as e:
        Solver(s, "mixed")
    assert e.value.code == N.MARA_ERR_CONFIG
