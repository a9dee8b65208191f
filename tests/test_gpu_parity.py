"""Plain FP64 GPU path against the oracle (which is pinned bit-for-bit to the
reference's own build): the same seeded inputs, the same dt sequence, then the
relative L1 difference of every conserved field, each relative to its own
norm, must be <= 1e-12, and for laws without transcendental eigenvalues the
primitive arrays match bit for bit.  (RMHD's quartic calls pow, acos, cos
and sin: the device evaluates them correctly rounded, the host's libm on
all but ~0.1 % of arguments.)  Calls go through the C ABI
(mara2_gb300/_native.py)."""
import numpy as np
import pytest

from helpers import oracle_config, parity_error, rel_l1
from mara2_gb300 import workloads as W
from mara2_gb300.scheme import Scheme
from mara2_gb300.solver import Solver

TOL = 1e-12  # relative L1 per conserved field, stated by the plain-path contract


def _repad(s_old, P, s_new):
    """The interior of P in a state array with s_new's guard width, guards
    filled by the boundary condition."""
    Q = W.empty_state(s_new)
    Q[s_new.interior()] = P[s_old.interior()]
    return W.apply_bc_numpy(s_new, Q)


def _rmhd_oblique(n, recon, rk):
    """A smooth relativistic MHD state with every velocity and field
    component non-zero everywhere (an oblique field and an oblique flow), so
    that no conserved field starts at zero and the per-field relative L1
    difference is meaningful for each of them."""
    s = Scheme(law="rmhd", recon=recon, riemann="hlle", bc="periodic", rk_order=rk, shape=(n, n, 1),
               gamma=4.0 / 3, cfl=0.3)
    x, y, _ = W.cell_centres(s)
    X, Y = x[..., 0], y[..., 0]
    two_pi = 2 * np.pi
    P = W.empty_state(s)
    P[..., 0, 0] = 1.0 + 0.2 * np.sin(two_pi * X) * np.cos(two_pi * Y)
    P[..., 0, 1] = 0.3 + 0.05 * np.sin(two_pi * Y)
    P[..., 0, 2] = -0.2 + 0.05 * np.cos(two_pi * X)
    P[..., 0, 3] = 0.1 + 0.02 * np.sin(two_pi * (X + Y))
    P[..., 0, 4] = 1.0 + 0.1 * np.cos(two_pi * (X - Y))
    P[..., 0, 5] = 0.5 + 0.1 * np.sin(two_pi * Y)
    P[..., 0, 6] = 0.3 + 0.1 * np.sin(two_pi * X)
    P[..., 0, 7] = -0.4 + 0.05 * np.cos(two_pi * (X + Y))
    return s, W.apply_bc_numpy(s, P)


def _cases():
    out = []
    s, P = W.sod(256)
    out.append(("sod256-plm-hlle-rk2", s, P, 30))
    s, P = W.kelvin_helmholtz(48)
    out.append(("kh48-plm-hllc-rk2", s, P, 8))
    out.append(("kh48-pcm-hlle-rk1-reflect", s.with_(recon="pcm", riemann="hlle", rk_order=1, bc="reflecting", guard=2), P, 8))
    out.append(("kh48-plm-hlle-rk3-outflow", s.with_(riemann="hlle", rk_order=3, bc="outflow"), P, 6))
    # WENO5 with each of the reference's three smoothness indicators
    # (Reconstruction.cpp:68-132) on a law without transcendental functions
    for wis in ("js96", "borges08", "shenzha10"):
        sw = s.with_(recon="weno5", riemann="hlle", rk_order=3, weno_is=wis)
        out.append((f"kh48-weno5-{wis}-hlle-rk3", sw, _repad(s, P, sw), 5))
    s, P = W.mhd_turbulence(12, rk_order=3)
    out.append(("mhd12cube-plm-hlle-rk3-ct", s, P, 4))
    out.append(("mhd12cube-noct", s.with_(disable_ct=True, rk_order=2), P, 3))
    s, P = W.rmhd_blast(24)
    out.append(("rmhd24-weno5-hlle-rk3", s, P, 4))
    for wis in ("js96", "borges08"):
        out.append((f"rmhd24-weno5-{wis}-hlle-rk3", s.with_(weno_is=wis), P, 3))
    s, P = _rmhd_oblique(24, "plm", 2)
    out.append(("rmhd24-oblique-plm-hlle-rk2", s, P, 6))
    s, P = _rmhd_oblique(24, "weno5", 3)
    out.append(("rmhd24-oblique-weno5-hlle-rk3", s, P, 4))
    return out


CASES = _cases()


def _oracle_dts(port, s, P, steps):
    c = oracle_config(s)
    Q = P.copy()
    status, t, dts = port.run(c, Q, steps, s.cfl, s.t_final)
    assert status == 0
    return Q, dts


def _conserved(port, s, P):
    st, U = port.generate_conserved(oracle_config(s), np.ascontiguousarray(P))
    assert st == 0
    return U[s.interior()]


@pytest.mark.gpu
@pytest.mark.parametrize("name,s,P,steps", CASES, ids=[c[0] for c in CASES])
def test_advance_matches_oracle(gpu_lib, port, name, s, P, steps):
    ref, dts = _oracle_dts(port, s, P, steps)
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        for dt in dts:
            g.advance(dt)
        g.synchronize()
        out = g.download()
    err = parity_error(s, _conserved(port, s, out), _conserved(port, s, ref))
    same = np.array_equal(out[s.interior()].view(np.uint64), ref[s.interior()].view(np.uint64))
    print(name, "bit-identical:", same, "relative L1 per conserved field:", err.tolist())
    assert np.all(err <= TOL), (name, err.tolist())
    if s.law != "rmhd":
        assert same, name


@pytest.mark.gpu
@pytest.mark.parametrize("name,s,P,steps", CASES[:3], ids=[c[0] for c in CASES[:3]])
def test_courant_matches_oracle(gpu_lib, port, name, s, P, steps):
    st, dt_ref = port.courant(oracle_config(s), np.ascontiguousarray(P))
    assert st == 0
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        assert g.courant() == dt_ref


@pytest.mark.gpu
def test_device_driver_loop_matches_oracle(gpu_lib, port):
    """mara_gpu_run (dt = min(cfl*courant, t_final - t) on the device) against
    the oracle's driver loop, through the end time."""
    s, P = W.sod(128)
    s = s.with_(t_final=0.02)
    ref, dts = _oracle_dts(port, s, P, 10_000)
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        n = g.run(len(dts) + 5, s.cfl, s.t_final)
        out = g.download()
    assert n == len(dts)
    assert abs(g.t - sum(dts)) <= 1e-15
    assert np.array_equal(out.view(np.uint64)[s.interior()], ref.view(np.uint64)[s.interior()])


@pytest.mark.gpu
def test_advance_host_dropin(gpu_lib, port):
    """The drop-in form: host MeshData::P in, advanced P out."""
    s, P = W.kelvin_helmholtz(32)
    ref, dts = _oracle_dts(port, s, P, 3)
    Q = P.copy()
    with Solver(s, "fp64") as g:
        for dt in dts:
            g.advance_host(Q, dt)
    assert np.array_equal(Q[s.interior()].view(np.uint64), ref[s.interior()].view(np.uint64))


@pytest.mark.gpu
def test_uniform_state_is_bit_identical(gpu_lib):
    """TestSuite.cpp:1476-1488: a uniform state is unchanged by advance(dt=1)."""
    s = Scheme(law="hydro", recon="plm", bc="periodic", rk_order=2, shape=(16, 16, 1))
    P = np.zeros(s.full_shape)
    P[..., 0] = 1.0
    P[..., 4] = 1.0
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        g.advance(1.0)
        out = g.download()
    assert np.array_equal(out, P)


@pytest.mark.gpu
def test_guard_too_small_is_rejected(gpu_lib):
    """TestSuite.cpp:1491-1511: guards thinner than the stencil throw."""
    from mara2_gb300 import _native as N
    s = Scheme(law="hydro", recon="plm", shape=(32, 1, 1), guard=1)
    with pytest.raises(N.MaraError) as e:
        Solver(s, "fp64")
    assert e.value.code == N.MARA_ERR_GUARD_TOO_SMALL


@pytest.mark.gpu
@pytest.mark.parametrize("recon", ["plm", "weno5"])
def test_signed_zeros_and_flat_regions_bitwise(gpu_lib, port, recon):
    """Reconstruction on exactly flat data and on signed zeros: minmod's sign
    tests and MIN3 (done on bit patterns on the device) must give the
    reference's result including the sign of zero; checked bit for bit over
    the whole array with guards."""
    s = Scheme(law="hydro", recon=recon, riemann="hllc", bc="periodic", rk_order=2, shape=(40, 24, 1))
    rng = np.random.default_rng(11)
    P = np.zeros(s.full_shape)
    P[..., 0] = 1.0
    P[..., 4] = 1.0
    P[10:20, ..., 0] = 2.0                       # a step: flat on both sides
    P[..., 1] = -0.0                             # negative zeros
    P[::3, ..., 2] = -0.0
    P[5:9, 4:9, :, 3] = rng.choice([0.0, -0.0, 1e-300, -1e-300, 5e-324], size=(4, 5, 1))
    P = W.apply_bc_numpy(s, P)
    ref, dts = _oracle_dts(port, s, P, 3)
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        for dt in dts:
            g.advance(dt)
        out = g.download()
    assert np.array_equal(out.view(np.uint64), ref.view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("make", [lambda: W.kelvin_helmholtz(96), lambda: W.mhd_turbulence(10)])
def test_page_locked_buffers_match_pageable(gpu_lib, precision, make):
    """A page-locked host array is read and written in place by the
    conversion kernels; a pageable one is staged in chunks: same bits."""
    import torch
    s, P = make()
    P = W.apply_bc_numpy(s, P)
    with Solver(s, precision) as g:
        g.upload(P.copy())
        dt = g.courant() * s.cfl
        g.advance(dt)
        a = g.download()
        pin = torch.from_numpy(P.copy()).pin_memory()
        g.upload_ptr(pin.data_ptr())
        g.advance(dt)
        out = torch.empty(pin.shape, dtype=torch.float64).pin_memory()
        g.download_ptr(out.data_ptr())
        b = out.numpy()
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
        # the drop-in call with the page-locked array, in place
        assert g.advance_host_ptr(pin.data_ptr(), dt) == 0
        assert np.array_equal(pin.numpy().view(np.uint64), a.view(np.uint64))


def _rect_state(ni, nj, bc, seed, **scheme):
    """A smooth positive state on a rectangular 2-D grid (density and pressure
    waves, a shear flow), guards by the boundary condition."""
    s0, _ = W.kelvin_helmholtz(8)
    s = s0.with_(shape=(ni, nj, 1), bc=bc, **scheme)
    x, y, _ = W.cell_centres(s)
    X, Y = x[..., 0], y[..., 0]
    rng = np.random.default_rng(seed)
    k = rng.integers(1, 4, size=4)
    P = W.empty_state(s)
    P[..., 0, 0] = 1.0 + 0.3 * np.sin(2 * np.pi * (k[0] * X + k[1] * Y))
    P[..., 0, 1] = 0.5 * np.cos(2 * np.pi * k[2] * Y)
    P[..., 0, 2] = 0.2 * np.sin(2 * np.pi * k[3] * X)
    P[..., 0, 4] = 1.0 + 0.2 * np.cos(2 * np.pi * (k[1] * X - k[0] * Y))
    return s, W.apply_bc_numpy(s, P)


# grids of at least 2^19 zones (the pipelined form's threshold): square and
# rectangular, partial last tile columns and rows (1058 = 33 x 32 + 2, 498 =
# 31 x 16 + 2, 830, 3000), few tile rows (176 = 11 x 16), 2048^2
PIPELINED = [(736, 736, "periodic", "plm", "hllc", 2), (740, 740, "outflow", "plm", "hlle", 3),
             (726, 726, "reflecting", "pcm", "hllc", 1), (1058, 498, "periodic", "pcm", "hlle", 1),
             (2048, 256, "periodic", "plm", "hllc", 2), (640, 830, "outflow", "plm", "hllc", 2),
             (3000, 176, "reflecting", "plm", "hlle", 2), (2048, 2048, "periodic", "plm", "hllc", 2)]


@pytest.mark.gpu
@pytest.mark.parametrize("ni,nj,bc,recon,riemann,rk", PIPELINED)
def test_pipelined_host_step_matches_unpipelined(gpu_lib, ni, nj, bc, recon, riemann, rk):
    """The drop-in call on a page-locked 2-D array runs as one launch that
    pipelines the transfers in, the stages and the transfers out by bands of
    host rows; a pageable array takes the unpipelined path (whole-grid
    transfers, then the stages).  Several calls in a row (the rotation
    parity of RK1 alternates), then a resident step: the same bits in the
    host array and on the device, and the same Courant step."""
    import torch
    s, P = _rect_state(ni, nj, bc, seed=ni + nj, recon=recon, riemann=riemann, rk_order=rk, guard=2)
    with Solver(s, "mixed") as a, Solver(s, "mixed") as b:
        a.upload(P.copy())
        dt = a.courant() * s.cfl
        ref = P.copy()
        pin = torch.from_numpy(P.copy()).pin_memory()
        for _ in range(3):
            a.advance_host(ref, dt)
            launches = b.stats().kernel_launches
            assert b.advance_host_ptr(pin.data_ptr(), dt) == 0
            # the pipelined form: status reset, step start, the one launch
            assert b.stats().kernel_launches - launches == 3
            assert np.array_equal(pin.numpy().view(np.uint64), ref.view(np.uint64))
        assert a.courant() == b.courant()
        assert a.stats().steps == b.stats().steps
        # the device state after the pipelined call continues like the other
        a.advance(dt)
        b.advance(dt)
        assert np.array_equal(a.download().view(np.uint64), b.download().view(np.uint64))


@pytest.mark.gpu
def test_host_register_makes_an_array_page_locked(gpu_lib):
    """mara_gpu_host_register page-locks a caller's array (the C++ drop-in's
    pinHostState): advance_host then reads and writes it in place, with the
    bits of the pageable path."""
    from mara2_gb300 import _native as N
    s, P = W.kelvin_helmholtz(768)
    lib = N.load()
    with Solver(s, "mixed") as a, Solver(s, "mixed") as b:
        a.upload(P.copy())
        dt = a.courant() * s.cfl
        ref = P.copy()
        a.advance_host(ref, dt)
        arr = np.ascontiguousarray(P.copy())
        assert lib.mara_gpu_host_register(arr.ctypes.data, arr.nbytes) == 0
        try:
            assert b.advance_host_ptr(arr.ctypes.data, dt) == 0
        finally:
            assert lib.mara_gpu_host_unregister(arr.ctypes.data) == 0
        assert np.array_equal(arr.view(np.uint64), ref.view(np.uint64))
