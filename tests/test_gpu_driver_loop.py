"""The device-resident driver loop (mara_gpu_run: dt = min(CFL x Courant,
t_final - t) on the device, the step replayed from a captured CUDA graph per
ping-pong parity) against the same steps taken one mara_gpu_advance(dt) at a
time with the loop's own dt sequence, and against the oracle's driver loop
(src/Problems.cpp:181-188), for every law, both precisions' plain form and
RK1-3: the same step count, dt sequence and bits."""
import numpy as np
import pytest

from helpers import oracle_config, parity_error
from mara2_gb300 import workloads as W
from mara2_gb300.solver import Solver


def _cases():
    out = []
    s, P = W.kelvin_helmholtz(32)
    out.append(("kh32-rk2", s.with_(t_final=0.05), P))
    out.append(("kh32-rk3-outflow", s.with_(rk_order=3, bc="outflow", t_final=0.05), W.apply_bc_numpy(
        s.with_(bc="outflow"), P.copy())))
    out.append(("kh32-rk1", s.with_(rk_order=1, t_final=0.03), P))
    s, P = W.mhd_turbulence(8)
    out.append(("mhd8cube-rk3", s.with_(t_final=0.02), P))
    s, P = W.rmhd_blast(24)
    out.append(("rmhd24-weno5-rk3", s.with_(t_final=0.4), P))
    out.append(("rmhd24-weno5-rk2", s.with_(rk_order=2, t_final=0.4), P))
    return out


CASES = _cases()


@pytest.mark.gpu
@pytest.mark.parametrize("name,s,P", CASES, ids=[c[0] for c in CASES])
def test_driver_loop_equals_replayed_advances_and_oracle(gpu_lib, port, name, s, P):
    # the device loop, one step per call, recording the dt of each step
    dts = []
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        while g.run(1, s.cfl, s.t_final) == 1:
            dts.append(g.stats().last_dt)
        a = g.download()
        t_a = g.t
    # the same loop in one call
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        n = g.run(100_000, s.cfl, s.t_final)
        b = g.download()
        assert g.t == t_a and n == len(dts), name
    # the dt sequence replayed through advance
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        for dt in dts:
            g.advance(dt)
        g.synchronize()
        c = g.download()
    i = s.interior()
    bits = lambda x: x[i].view(np.uint64)
    assert np.array_equal(bits(a), bits(b)), name
    assert np.array_equal(bits(a), bits(c)), name
    # the oracle's loop
    ref = P.copy()
    st, t_ref, dts_ref = port.run(oracle_config(s), ref, 100_000, s.cfl, s.t_final)
    assert st == 0 and len(dts_ref) == len(dts), (name, len(dts_ref), len(dts))
    if s.law != "rmhd":
        assert dts == list(dts_ref) and t_a == t_ref, name
        assert np.array_equal(bits(a), bits(ref)), name
    else:
        assert np.max(np.abs(np.array(dts) / np.array(dts_ref) - 1)) <= 1e-12, name
        assert np.all(parity_error(s, a[i], ref[i]) <= 1e-12), name


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "mixed_fp64"])
@pytest.mark.parametrize("rk", [1, 2, 3])
def test_mixed_driver_loop_equals_replayed_advances(gpu_lib, precision, rk):
    """The mixed paths' loop (fused tiles: with RK1 the state alternates
    between two buffers) stepped one call at a time up to t_final, in one
    call, and replayed through advance: the same bits and clock."""
    s, P = W.kelvin_helmholtz(48)
    s = s.with_(rk_order=rk, t_final=0.03)
    dts = []
    with Solver(s, precision) as g:
        g.upload(P.copy())
        while g.run(1, s.cfl, s.t_final) == 1:
            dts.append(g.stats().last_dt)
        a = g.download()
        t_a = g.t
    with Solver(s, precision) as g:
        g.upload(P.copy())
        n = g.run(100_000, s.cfl, s.t_final)
        b = g.download()
        assert g.t == t_a and n == len(dts)
    with Solver(s, precision) as g:
        g.upload(P.copy())
        for dt in dts:
            g.advance(dt)
        c = g.download()
    i = s.interior()
    assert np.array_equal(a[i].view(np.uint64), b[i].view(np.uint64))
    assert np.array_equal(a[i].view(np.uint64), c[i].view(np.uint64))
