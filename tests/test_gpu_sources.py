"""Source terms on the GPU (MethodOfLinesTVD::setSourceTermsFunction,
SolutionSchemes.cpp:219-228) against the oracle with the same function:
bit-identical on the plain path, through eager advances and captured
driver-loop graphs; caller-supplied functions and their errors."""
import ctypes as C

import numpy as np
import pytest

from helpers import oracle_config
from mara2_gb300 import _native as N
from mara2_gb300 import workloads as W
from mara2_gb300.solver import Solver


def _gravity(g):
    def S(x, y, z, aux, P):
        rho = P[0]
        return [0.0, rho * g[0], rho * g[1], rho * g[2], rho * (P[1] * g[0] + P[2] * g[1] + P[3] * g[2])] + [0.0] * 5
    return S


def _oracle_steps(port, s, P, g, n):
    c = oracle_config(s)
    A = P.copy()
    port.set_source_terms(_gravity(g))
    try:
        for _ in range(n):
            _, dt = port.courant(c, A)
            assert port.advance(c, A, s.cfl * dt)[0] == 0
    finally:
        port.set_source_terms(None)
    return A


CASES = [("kh", lambda: W.kelvin_helmholtz(48), (0.0, -1.0, 0.0)),
         ("sod", lambda: W.sod(128), (-0.5, 0.0, 0.0)),
         ("mhd", lambda: W.mhd_turbulence(8), (0.3, -0.2, 0.1))]


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,g", CASES)
def test_gravity_source_bitwise(gpu_lib, port, name, make, g):
    s, P = make()
    ref = _oracle_steps(port, s, P, g, 4)
    with Solver(s, "fp64") as h:
        h.set_source_terms(gravity=g)
        h.upload(P.copy())
        h.run(2)                                   # captured graph
        out = h.download()
        h.upload(out)
        for _ in range(2):                         # eager advances
            h.advance(h.courant() * s.cfl)
        out = h.download()
    assert np.array_equal(out[s.interior()].view(np.uint64), ref[s.interior()].view(np.uint64))


@pytest.mark.gpu
def test_python_source_function_and_removal(gpu_lib, port):
    """A caller's function (here a Python callable that enqueues the
    library's gravity kernel with its own g) is called once per stage."""
    s, P = W.kelvin_helmholtz(32)
    g = (C.c_double * 3)(0.0, -2.0, 0.0)
    calls = []
    lib = N.load()

    def fn(user, args):
        calls.append(args.contents.nq)
        return lib.mara_source_uniform_gravity(C.cast(g, C.c_void_p), args)

    ref = _oracle_steps(port, s, P, (0.0, -2.0, 0.0), 1)
    with Solver(s, "fp64") as h:
        h.set_source_terms(fn)
        h.upload(P.copy())
        h.advance(h.courant() * s.cfl)
        out = h.download()
        assert calls == [5] * s.rk_order
        assert np.array_equal(out[s.interior()].view(np.uint64), ref[s.interior()].view(np.uint64))
        h.set_source_terms(None)                   # back to no source terms
        h.upload(P.copy())
        h.advance(h.courant() * s.cfl)
        plain = h.download()
    c = oracle_config(s)
    A = P.copy()
    _, dt = port.courant(c, A)
    port.advance(c, A, s.cfl * dt)
    assert np.array_equal(plain[s.interior()].view(np.uint64), A[s.interior()].view(np.uint64))


@pytest.mark.gpu
def test_source_function_error_and_mixed_rejection(gpu_lib):
    s, P = W.kelvin_helmholtz(32)
    with Solver(s, "fp64") as h:
        h.set_source_terms(lambda user, args: 7)
        h.upload(P.copy())
        with pytest.raises(N.MaraError) as e:
            h.advance(1e-4)
        assert e.value.code == 7
        with pytest.raises(N.MaraError):
            h.run(2)
        h.set_source_terms(None)
        h.upload(P.copy())
        h.run(2)                                   # usable again
    with Solver(s, "mixed") as h:
        with pytest.raises(N.MaraError) as e:
            h.set_source_terms(gravity=(0.0, -1.0, 0.0))
        assert e.value.code == N.MARA_ERR_CONFIG
