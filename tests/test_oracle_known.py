"""Known answers of the reference's own unit tests (src/TestSuite.cpp),
re-asserted on the oracle restatement, plus the MethodOfLinesTVD contract."""
import math

import numpy as np
import pytest

import oracle as O


def approx(a, b, eps=np.finfo(np.float32).eps * 100, scale=1.0):
    """Catch's Approx: |a - b| < eps (scale + max(|a|, |b|))."""
    return abs(a - b) < eps * (scale + max(abs(a), abs(b)))


# TestSuite.cpp:431-478
@pytest.mark.parametrize("coeffs,roots,eps", [
    ((1, 0, -5, 0, 4), (-2, -1, 1, 2), 1e-14),
    ((1., 0., -1., 0., 1e-10), (-1, -1e-5, 1e-5, 1), 1e-10),
    ((-1, 0, 0, 0, 1), (-1, 1), 1e-14),
])
def test_quartic_known_roots(port, coeffs, roots, eps):
    nr, r = port.quartic(*coeffs)
    assert nr == len(roots)
    for a, b in zip(r, roots):
        assert approx(a, b, eps)


# TestSuite.cpp:636-731
def test_rmhd_eigenvalues_match_newtonian_when_slow(port):
    nr = O.make_config(law="mhd")
    sr = O.make_config(law="rmhd")
    for P in ([1., 0., 0., 0., 1e-6, 0, 0, 0], [1., 1e-6, 1e-6, 1e-6, 1e-6, 1e-6, 1e-6, 1e-6]):
        for d in range(3):
            n = [0.0, 0.0, 0.0]
            n[d] = 1.0
            s1, _, _, A1 = port.from_primitive(nr, P, n)
            s2, _, _, A2 = port.from_primitive(sr, P, n)
            assert s1 == s2 == 0
            for i in range(8):
                assert approx(A1[i], A2[i]), (P, d, i, A1[i], A2[i])


@pytest.mark.parametrize("P,eps", [
    ([1., 0., 0., 0., 1e-6, 0, 0, 0], np.finfo(np.float32).eps * 100),
    ([1., 1e-6, 1e-6, 1e-6, 1e-6, 1e-6, 1e-6, 1e-6], 1e-12),
    ([1., 0.5, 0.4, 0.3, 1, 1, 1, 1], 1e-12),
])
def test_rmhd_prim_cons_round_trip(port, P, eps):
    c = O.make_config(law="rmhd")
    s, U, _, _ = port.from_primitive(c, P)
    assert s == 0
    s, Q, _ = port.from_conserved(c, U[:8])
    assert s == 0
    for i in range(8):
        assert approx(P[i], Q[i], eps)


# TestSuite.cpp:1147-1239
def test_field_operator_round_trip_and_courant(port):
    c = O.make_config(law="hydro", shape=(128, 1, 1), ng=0, recon="pcm")
    c.ng[0] = 0  # the unit test works on guard-free arrays
    x = (np.arange(128) + 0.5) / 128
    P = np.zeros((128, 1, 1, 5))
    P[:, 0, 0, 0] = 1 + 0.5 * np.cos(math.pi * x)
    P[..., 1], P[..., 2], P[..., 3], P[..., 4] = 1., 2., 3., 1.
    st, U = port.generate_conserved(c, P)
    assert st == 0
    for i in range(128):
        _, Ui, _, _ = port.from_primitive(c, P[i, 0, 0])
        assert np.array_equal(U[i, 0, 0], Ui[:5])
        s, Q, _ = port.from_conserved(c, U[i, 0, 0])
        assert all(approx(a, b) for a, b in zip(P[i, 0, 0], Q[:5]))
    # rho = 1, v = 1, p = 0: the Courant step equals the cell length
    P2 = np.zeros((128, 1, 1, 5))
    P2[..., 0], P2[..., 1] = 1.0, 1.0
    st, dt = port.courant(c, P2)
    assert st == 0 and dt == 1.0 / 128


# TestSuite.cpp:1213-1233: the volume-integrated mass of rho = 1 on the unit
# interval is the mesh volume, and the first diagnostic is "mass"
def test_volume_diagnostics_mass_is_mesh_volume(port):
    from mara2_gb300.solver import diagnostic_names
    c = O.make_config(law="hydro", shape=(128, 1, 1), ng=0, recon="pcm")
    c.ng[0] = 0
    P = np.zeros((128, 1, 1, 5))
    P[..., 0], P[..., 1] = 1.0, 1.0
    st, D, _ = port.volume_diagnostics(c, P)
    assert st == 0 and D[0] == 1.0
    assert diagnostic_names("hydro")[0] == "mass" and len(diagnostic_names("mhd")) == 17


def _divergence(F, dx):
    dA = [dx[1] * dx[2], dx[2] * dx[0], dx[0] * dx[1]]
    dV = dx[0] * dx[1] * dx[2]
    n0, n1, n2 = F.shape[0] - 1, F.shape[1] - 1, F.shape[2] - 1
    return (1.0 / dV) * (F[1:, :n1, :n2, :, 0] * dA[0] - F[:n0, :n1, :n2, :, 0] * dA[0]
                         + F[:n0, 1:, :n2, :, 1] * dA[1] - F[:n0, :n1, :n2, :, 1] * dA[1]
                         + F[:n0, :n1, 1:, :, 2] * dA[2] - F[:n0, :n1, :n2, :, 2] * dA[2])


# TestSuite.cpp:1340-1436: CT-corrected fluxes give a zero cell monopole
def test_ct_monopole_2d(port):
    rng = np.random.default_rng(2017)
    F = np.zeros((17, 17, 2, 3, 3))
    F[:, :, 0] = rng.integers(0, 2**31, (17, 17, 3, 3)).astype(float)
    F[:, :, 1] = F[:, :, 0]
    G = port.ct_correct(F, 0)
    dx = (1 / 16, 1 / 16, 1.0)
    Mf = port.monopole_cell(_divergence(F, dx))
    Mg = port.monopole_cell(_divergence(G, dx))
    assert Mf.shape == (16, 16, 1)
    assert not approx(Mf[8, 8, 0], 0.0)
    assert approx(Mg[8, 8, 0], 0.0)


def test_ct_monopole_3d(port):
    rng = np.random.default_rng(2018)
    F = rng.integers(0, 2**31, (17, 17, 17, 3, 3)).astype(float)
    G = port.ct_correct(F, 0)
    dx = (1 / 16, 1 / 16, 1 / 16)
    Mf = port.monopole_cell(_divergence(F, dx))[2:-2, 2:-2, 2:-2]
    Mg = port.monopole_cell(_divergence(G, dx))[2:-2, 2:-2, 2:-2]
    assert np.all([not approx(v, 0.0) for v in Mf.ravel()])
    assert np.all([approx(v, 0.0) for v in Mg.ravel()])


# TestSuite.cpp:1476-1511
def test_uniform_state_unchanged_and_guard_check(port):
    c = O.make_config(law="hydro", recon="plm", bc="periodic", shape=(16, 16, 1))
    P = np.zeros((20, 20, 1, 5))
    P[..., 0] = 1.0
    P[..., 4] = 1.0
    Q = P.copy()
    s, _ = port.advance(c, Q, 1.0)
    assert s == 0 and np.array_equal(P, Q)
    c.ng[0] = c.ng[1] = 1
    s, _ = port.advance(c, np.zeros((18, 18, 1, 5)), 1.0)
    assert s == O.ERR_GUARD_TOO_SMALL
