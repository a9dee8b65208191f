"""Constrained transport beyond the flux CT of the step, on the device.

* The divergence-free initial field of the reference's MHD drivers
  (src/Problems.cpp:660-667: vector potential -> Godunov fluxes -> flux CT ->
  divergence, then applyBoundaryCondition) built on the device from an
  uploaded face-centred A, against the oracle (pinned bit for bit to the
  reference build): the same bits on the plain path, the FP32-pair
  round-off on the mixed path, and a plain step taken from it equal to the
  oracle's step (bit for bit, or within 1e-12 per field for RMHD).
* The ConstrainedTransport interface (src/Mara.hpp:341-349) as
  UniformCartesianCT implements it: monopole at vertices and cells, and the
  adaptor's current, bit for bit against the oracle.
"""
import numpy as np
import pytest

from helpers import oracle_config, rel_l1
from mara2_gb300 import workloads as W
from mara2_gb300.solver import Solver, ct_current, ct_monopole


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def _cases():
    out = []
    s, P, A, scale, _ = W.mhd_turbulence_parts(10)
    out.append(("mhd10cube-periodic", s, P, A, scale))
    s, P = W.rmhd_blast(16)
    A = W.face_vector_potential(s, lambda x, y, z: W._fourier_vector(9, x, y, z))
    out.append(("rmhd16-outflow", s, P, A, 0.05))
    sr = s.with_(law="mhd", recon="plm", bc="reflecting", gamma=5.0 / 3)
    Pr = W.empty_state(sr)
    Pr[..., 0] = 1.0
    Pr[..., 4] = 1.0
    Pr[..., 1] = 0.1
    Pr = W.apply_bc_numpy(sr, Pr)
    Ar = W.face_vector_potential(sr, lambda x, y, z: W._fourier_vector(11, x, y, z))
    out.append(("mhd2d-reflecting", sr, Pr, Ar, 1.0))
    return out


CASES = _cases()


def _expected(port, s, P, A, scale):
    c = oracle_config(s)
    st, B = port.vector_potential_to_cell_b(c, A, scale)
    assert st == 0
    Q = np.ascontiguousarray(P.copy())
    Q[..., 5:8] = B
    assert port.apply_bc(c, Q) == 0
    return Q


@pytest.mark.gpu
@pytest.mark.parametrize("name,s,P,A,scale", CASES, ids=[c[0] for c in CASES])
def test_assign_vector_potential_plain_matches_oracle(gpu_lib, port, name, s, P, A, scale):
    want = _expected(port, s, P, A, scale)
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        g.assign_vector_potential(A, scale)
        out = g.download()
        # and a step from it
        dt = 0.2 * g.courant()
        g.advance(dt)
        stepped = g.download()
    assert np.array_equal(_bits(out), _bits(want)), name
    ref = want.copy()
    st, _ = port.advance(oracle_config(s), ref, dt)
    assert st == 0
    i = s.interior()
    if s.law == "rmhd":
        # the quartic's pow / acos / cos / sin: correctly rounded on the
        # device, the host's libm on all but ~0.1 % of arguments
        err = rel_l1(stepped[i], ref[i])
        assert np.all(err <= 1e-12), (name, err.tolist())
    else:
        assert np.array_equal(_bits(stepped[i]), _bits(ref[i])), name


@pytest.mark.gpu
@pytest.mark.parametrize("name,s,P,A,scale", CASES[:2], ids=[c[0] for c in CASES[:2]])
def test_assign_vector_potential_mixed_close_to_oracle(gpu_lib, port, name, s, P, A, scale):
    want = _expected(port, s, P, A, scale)
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        g.assign_vector_potential(A, scale)
        out = g.download()
    i = s.interior()
    big = np.abs(want[i][..., 5:8]).max()
    assert np.abs(out[i][..., 5:8] - want[i][..., 5:8]).max() <= 1e-12 * big


@pytest.mark.gpu
def test_mhd_workload_field_built_on_device(gpu_lib, port):
    """The MHD turbulence workload's field from its vector potential on the
    device: the oracle's bits, divergence-free at round-off, and within
    round-off of the host-built workload state."""
    s, P, A, scale, _ = W.mhd_turbulence_parts(16)
    want = _expected(port, s, P, A, scale)
    _, host = W.mhd_turbulence(16)
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        g.assign_vector_potential(A, scale)
        out = g.download()
        m = g.monopole_max(1.0 / 16)
    assert np.array_equal(_bits(out), _bits(want))
    assert np.allclose(out, host, rtol=0, atol=1e-13)
    assert m * (1.0 / 16) / np.abs(out[..., 5:8]).max() < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(6, 5, 4), (12, 9, 1), (17, 1, 1)])
@pytest.mark.parametrize("bc", ["periodic", "outflow"])
def test_constrained_transport_interface_matches_oracle(gpu_lib, port, shape, bc):
    rng = np.random.default_rng(3 * sum(shape) + len(bc))
    B = rng.standard_normal(shape + (3,))
    for loc in ("vert", "cell"):
        st, want = port.uct_monopole(B, bc, loc)
        assert st == 0
        assert np.array_equal(_bits(ct_monopole(B, bc, loc)), _bits(want)), loc
    st, want = port.uct_current(B, bc, 0.5)
    assert st == 0
    assert np.array_equal(_bits(ct_current(B, bc, 0.5)), _bits(want))


@pytest.mark.gpu
def test_constrained_transport_monopole_of_a_ct_field_vanishes(gpu_lib, port):
    """A field built by flux CT has a vanishing monopole at vertices away from
    the guards' influence (TestSuite.cpp:1340-1436 asks the same of
    CellCenteredFieldCT)."""
    s, P, A, scale, _ = W.mhd_turbulence_parts(12)
    want = _expected(port, s, P, A, scale)
    B = np.ascontiguousarray(want[s.interior()][..., 5:8])
    Mv = ct_monopole(B, "periodic", "vert")
    assert np.abs(Mv).max() < 1e-12 * np.abs(B).max()
