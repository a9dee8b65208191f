"""Mixed-precision path against the FP64 oracle.

FP32 reconstruction / Riemann / flux arithmetic with an FP32-pair (or FP64)
conserved accumulator must stay within the stated tolerance of the FP64 reference on
the same inputs and the same dt sequence: relative L1 density error <= 1e-5
(the precision contract), checked here over short runs where it is met with
a wide margin, for every law and both kernel families."""
import numpy as np
import pytest

from helpers import oracle_config, rel_l1, rel_l1_max, rel_linf
from mara2_gb300 import workloads as W
from mara2_gb300.solver import Solver

TOL_RHO = 1e-5  # relative L1 of the density against the FP64 oracle


def _cases():
    out = []
    s, P = W.sod(512)
    out.append(("sod512-fused", s, P, 60))
    s, P = W.kelvin_helmholtz(96)
    out.append(("kh96-fused-hllc", s, P, 20))
    out.append(("kh96-fused-hlle-rk3", s.with_(riemann="hlle", rk_order=3), P, 10))
    # guards must agree with the boundary condition, as the reference's drivers
    # ensure by calling applyBoundaryCondition after generating initial data
    sr = s.with_(recon="pcm", rk_order=1, bc="reflecting", guard=2)
    out.append(("kh96-fused-pcm-rk1-reflect", sr, W.apply_bc_numpy(sr, P.copy()), 10))
    so = s.with_(bc="outflow")
    out.append(("kh96-fused-plm-outflow", so, W.apply_bc_numpy(so, P.copy()), 10))
    # hydro on the general form: WENO5 (the fused tiles take PCM / PLM only)
    # with HLLC, and a 3-D blast (the fused tiles are 1-D / 2-D), so the
    # face fluxes run on every compile-time axis
    sw = s.with_(recon="weno5")
    Pw = W.empty_state(sw)
    g, gw, n = s.ng[0], sw.ng[0], s.shape[0]
    Pw[gw:gw + n, gw:gw + n] = P[g:g + n, g:g + n]
    out.append(("kh96-general-weno5-hllc", sw, W.apply_bc_numpy(sw, Pw), 8))
    sb = W.Scheme(law="hydro", recon="plm", riemann="hllc", bc="periodic", rk_order=2, shape=(24, 24, 24),
                  gamma=1.4, plm_theta=1.5, cfl=0.4, t_final=None, steps=8)
    Pb = W.empty_state(sb)
    X, Y, Z = W.cell_centres(sb)
    r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2)
    Pb[..., 0] = 1.0
    Pb[..., 4] = np.where(r < 0.2, 10.0, 0.1)
    out.append(("blast24cube-general-plm-hllc", sb, W.apply_bc_numpy(sb, Pb), 8))
    s, P = W.mhd_turbulence(16, rk_order=3)
    out.append(("mhd16cube-general-ct", s, P, 6))
    s, P = W.rmhd_blast(48)
    out.append(("rmhd48-general-weno5", s, P, 6))
    # a dense quadrant (rho 1e9, p 1e7) beside the blast: its conserved
    # density lies above the FP32-pair recovery's range, so those zones take
    # the FP64 Newton solve, the rest the pair iteration
    x, y, _ = W.cell_centres(s)
    dense = (x < -0.5) & (y < -0.5)
    Q = P.copy()
    Q[..., 0] = np.where(dense, 1e9, Q[..., 0])
    Q[..., 4] = np.where(dense, 1e7, Q[..., 4])
    out.append(("rmhd48-dense-fp64-recovery", s, W.apply_bc_numpy(s, Q), 6))
    return out


CASES = _cases()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "mixed_fp64"])
@pytest.mark.parametrize("name,s,P,steps", CASES, ids=[c[0] for c in CASES])
def test_mixed_close_to_fp64_oracle(gpu_lib, port, name, s, P, steps, precision):
    """Both mixed recipes: the FP32-pair accumulator, and the FP64
    accumulator with the FP64 RMHD Newton solve."""
    c = oracle_config(s)
    ref = P.copy()
    status, _, dts = port.run(c, ref, steps, s.cfl, s.t_final)
    assert status == 0
    with Solver(s, precision) as g:
        g.upload(P.copy())
        for dt in dts:
            g.advance(dt)
        g.synchronize()
        out = g.download()
    a, b = out[s.interior()], ref[s.interior()]
    err = rel_l1(a, b)
    print(name, "L1 per field:", err.tolist(), "Linf per field:", rel_linf(a, b).tolist())
    assert err[0] <= TOL_RHO, (name, err)
    # every field, against the largest field's norm (fields that start at
    # zero have no norm of their own to measure against)
    assert np.all(rel_l1_max(a, b) <= TOL_RHO), (name, rel_l1_max(a, b))
    assert np.all(np.isfinite(out))


@pytest.mark.gpu
def test_mixed_driver_loop_runs_to_end_time(gpu_lib, port):
    s, P = W.sod(256)
    s = s.with_(t_final=0.05)
    c = oracle_config(s)
    ref = P.copy()
    _, t_ref, dts = port.run(c, ref, 100_000, s.cfl, s.t_final)
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        n = g.run(len(dts) + 50, s.cfl, s.t_final)
        out = g.download()
    assert abs(g.t - s.t_final) < 1e-12
    assert abs(n - len(dts)) <= 2          # FP32 Courant steps may differ slightly
    err = rel_l1(out[s.interior()], ref[s.interior()])
    assert err[0] <= TOL_RHO, err


@pytest.mark.gpu
def test_mixed_courant_close(gpu_lib, port):
    s, P = W.kelvin_helmholtz(64)
    _, dt_ref = port.courant(oracle_config(s), P.copy())
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        dt = g.courant()
    assert abs(dt - dt_ref) / dt_ref < 1e-6


@pytest.mark.gpu
def test_kernel_timing_counts_stage_launches(gpu_lib):
    """Per-launch kernel timing (the benchmark's roofline source) sees every
    stage launch of the fused path, through run() and advance()."""
    s, P = W.kelvin_helmholtz(64)
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        g.set_kernel_timing(True)
        g.run(3)
        dt = g.courant() * s.cfl
        g.advance(dt)
        ms, n = g.kernel_times()
        g.set_kernel_timing(False)
    assert n[0] == 4 * s.rk_order, n
    assert ms[0] > 0.0


def _riemann_1d(n, bc, recon, riemann, rk):
    r = W.riemann_stream(1, seed=W.RIEMANN_SEED + 3)[0]
    r.n, r.dims = n, 1
    s, P = W.riemann_initial(r)
    s = s.with_(bc=bc, recon=recon, riemann=riemann, rk_order=rk, guard=2)
    return s, W.apply_bc_numpy(s, P)


CLUSTER_CASES = [(256, "outflow", "plm", "hlle", 2), (1000, "periodic", "plm", "hllc", 3),
                 (777, "reflecting", "pcm", "hllc", 1), (8192, "outflow", "plm", "hllc", 2),
                 (131, "periodic", "pcm", "hlle", 2)]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "mixed_fp64"])
@pytest.mark.parametrize("n,bc,recon,riemann,rk", CLUSTER_CASES)
def test_cluster_run_matches_tile_steps(gpu_lib, n, bc, recon, riemann, rk, precision):
    """A 1-D grid's driver loop on one thread-block cluster (the grid held in
    shared memory across many steps) against the same steps taken one launch
    per stage by the tile kernels: the same clock, step count and bits (the
    fused kernels share explicitly rounded arithmetic), with either
    accumulator."""
    s, P = _riemann_1d(n, bc, recon, riemann, rk)
    steps = 40
    with Solver(s, precision) as g:
        g.upload(P.copy())
        taken = g.run(steps, s.cfl)
        a = g.download()
        t_cluster = g.t
    with Solver(s, precision) as g:
        g.upload(P.copy())
        t = 0.0
        for _ in range(steps):
            dt = g.courant() * s.cfl
            g.advance(dt)
            t += dt
        b = g.download()
    assert taken == steps
    assert t_cluster == t
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.gpu
def test_cluster_run_stops_at_t_final_and_continues(gpu_lib, port):
    """Runs that end at t_final inside a launch, and a second run that picks
    up the clock and the Courant step the first one left."""
    s, P = W.sod(1024)
    c = oracle_config(s)
    ref = P.copy()
    _, t_ref, dts = port.run(c, ref, 100_000, s.cfl, s.t_final)
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        n1 = g.run(100, s.cfl, s.t_final)
        n2 = g.run(100_000, s.cfl, s.t_final)
        out = g.download()
        assert abs(g.t - s.t_final) < 1e-12
    assert n1 == 100 and abs((n1 + n2) - len(dts)) <= 2
    err = rel_l1(out[s.interior()], ref[s.interior()])
    assert err[0] <= TOL_RHO, err


@pytest.mark.gpu
@pytest.mark.parametrize("make", [lambda: W.mhd_turbulence(16), lambda: W.rmhd_blast(32)], ids=["mhd", "rmhd"])
def test_general_run_split_at_t_final_continues_identically(gpu_lib, make):
    """The general form reduces the Courant step in the last stage's update;
    a driver loop that stops at t_final, or an advance that is not taken,
    keeps the step the last stage left: runs split anywhere give the same
    clock and bits as one run."""
    s, P = make()
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        dt = g.courant()
    t_final = 7.5 * dt * s.cfl
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        n = g.run(100, s.cfl, t_final)
        a = g.download()
        t_a = g.t
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        n1 = g.run(3, s.cfl, t_final)
        n2 = g.run(100, s.cfl, t_final)
        n3 = g.run(100, s.cfl, t_final)
        b = g.download()
        t_b = g.t
    assert n1 == 3 and n1 + n2 == n and n3 == 0
    assert t_a == t_b
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
