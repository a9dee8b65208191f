"""Failure detection on the GPU, made on the host side by uploading states the
reference cannot invert (no GPU fault is involved): the status codes, the
failure count and the first failed zone must agree with the oracle, which
agrees with the reference's FieldOperator::InversionFailure and runtime
errors (tests/test_oracle_vs_ref.py)."""
import numpy as np
import pytest

from helpers import oracle_config
from mara2_gb300 import _native as N
from mara2_gb300 import workloads as W
from mara2_gb300.solver import Solver


def _planted_mhd():
    s, P = W.mhd_turbulence(6)
    Q = P.copy()
    Q[4, 5, 3, 4] = 1e-9     # near-vacuum pressure next to a strong velocity jump
    Q[4, 5, 3, 1] = 3.0
    return s, Q


@pytest.mark.gpu
def test_inversion_failure_matches_oracle(gpu_lib, port):
    s, Q = _planted_mhd()
    st, fail = port.advance(oracle_config(s), Q.copy(), 0.05)
    assert st == N.MARA_ERR_INVERSION_FAILURE and fail.count == 1
    with Solver(s, "fp64") as g:
        g.upload(Q.copy())
        g.advance(0.05)
        assert g.status() == N.MARA_ERR_INVERSION_FAILURE
        stats = g.stats()
    assert stats.failures == fail.count
    assert tuple(stats.first_zone) == tuple(fail.first)


@pytest.mark.gpu
def test_mixed_path_reports_inversion_failure(gpu_lib):
    s, Q = _planted_mhd()
    with Solver(s, "mixed") as g:
        g.upload(Q.copy())
        g.advance(0.05)
        assert g.status() == N.MARA_ERR_INVERSION_FAILURE
        assert g.stats().failures >= 1


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_superluminal_state_is_an_error(gpu_lib, port, precision):
    s, P = W.rmhd_blast(16)
    Q = P.copy()
    Q[8, 8, 0, 1] = 1.2
    st, _ = port.advance(oracle_config(s), Q.copy(), 0.01)
    assert st == N.MARA_ERR_SUPERLUMINAL
    with Solver(s, precision) as g:
        g.upload(Q.copy())
        g.advance(0.01)
        assert g.status() == N.MARA_ERR_SUPERLUMINAL


@pytest.mark.gpu
def test_handle_recovers_after_failure(gpu_lib):
    """The context stays usable: a fresh upload on a new handle steps normally."""
    s, Q = _planted_mhd()
    with Solver(s, "fp64") as g:
        g.upload(Q.copy())
        g.advance(0.05)
        assert g.status() != 0
    s2, P2 = W.mhd_turbulence(6)
    with Solver(s2, "fp64") as g:
        g.upload(P2.copy())
        assert g.run(2) == 2
