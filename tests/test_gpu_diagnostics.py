"""Device diagnostics against the oracle: FieldOperator::
volumeIntegratedDiagnostics (totals to rounding: the device sums in a
different order than the reference's sequential loop) and the checkpoint's
cell fields CellCenteredFieldCT::monopole / ::current (bit for bit on the
plain path)."""
import numpy as np
import pytest

from helpers import oracle_config
from mara2_gb300 import workloads as W
from mara2_gb300.solver import Solver, diagnostic_names

# |device - oracle| <= SUM_TOL x (sum over zones of |term|): the two sums
# differ only in association order
SUM_TOL = 1e-13


def _stepped(make, port, steps=2):
    s, P = make()
    c = oracle_config(s)
    for _ in range(steps):
        _, dt = port.courant(c, P)
        assert port.advance(c, P, s.cfl * dt)[0] == 0
    return s, P


CASES = [("kh", lambda: W.kelvin_helmholtz(64)), ("sod", lambda: W.sod(256)),
         ("mhd", lambda: W.mhd_turbulence(16)), ("rmhd", lambda: W.rmhd_blast(32))]


@pytest.mark.gpu
@pytest.mark.parametrize("name,make", CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_volume_diagnostics_match_oracle(gpu_lib, port, name, make, precision):
    s, P = _stepped(make, port)
    with Solver(s, precision) as g:
        g.upload(P.copy())
        d = g.volume_diagnostics()
        Q = g.download()  # the state the diagnostics describe
    st, D, Dabs = port.volume_diagnostics(oracle_config(s), Q)
    assert st == 0
    assert list(d) == diagnostic_names(s.law)
    got = np.array(list(d.values()))
    finite = np.isfinite(D)
    assert np.array_equal(np.isfinite(got), finite)
    assert np.all(np.abs(got - D)[finite] <= SUM_TOL * Dabs[finite] + 1e-300), (got - D, Dabs)


@pytest.mark.gpu
def test_volume_diagnostics_uniform_mass(gpu_lib):
    """The reference's known answer (TestSuite.cpp:1213-1233) on the device:
    rho = 1 integrates to the mesh volume."""
    s, P = W.sod(128)
    P[..., 0], P[..., 1], P[..., 4] = 1.0, 1.0, 1.0
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        assert g.volume_diagnostics()["mass"] == 1.0


@pytest.mark.gpu
def test_volume_diagnostics_superluminal_reports_status(gpu_lib, port):
    s, P = W.rmhd_blast(16)
    P[s.interior()][3, 3, 0, 1] = 1.5  # |v| > 1 in one interior zone
    st, _, _ = port.volume_diagnostics(oracle_config(s), P)
    assert st != 0
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        with pytest.raises(RuntimeError) as e:
            g.volume_diagnostics()
        assert e.value.code == st
        g.upload(W.rmhd_blast(16)[1])  # the handle stays usable
        assert g.volume_diagnostics()["mass"] > 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("make", [lambda: W.mhd_turbulence(12), lambda: W.rmhd_blast(24)])
def test_field_diagnostics_plain_bitwise(gpu_lib, port, make):
    s, P = _stepped(make, port)
    h = 1.0 / s.shape[0]
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        out = g.field_diagnostics(h)
    B = P[..., 5:8]
    assert np.array_equal(out[..., 0].view(np.uint64), port.monopole_cell(B, h).view(np.uint64))
    assert np.array_equal(out[..., 1:].view(np.uint64), port.current_cell(B, h).view(np.uint64))


@pytest.mark.gpu
def test_field_diagnostics_mixed_close(gpu_lib, port):
    s, P = _stepped(lambda: W.mhd_turbulence(12), port)
    h = 1.0 / s.shape[0]
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        out = g.field_diagnostics(h)
    J = port.current_cell(P[..., 5:8], h)
    assert np.max(np.abs(out[..., 1:] - J)) <= 1e-5 * np.max(np.abs(J))
    # the monopole of a CT-initialised field stays at FP32 round-off
    assert np.max(np.abs(out[..., 0])) * h <= 1e-5 * np.max(np.abs(P[..., 5:8]))
