"""Initial data generated on the device (MeshOperator::generate of the
built-in functions, guards by the boundary condition) against the host
generators of the same workloads: the arrays a download returns must be the
same bits as uploading the host arrays."""
import numpy as np
import pytest

from mara2_gb300 import workloads as W
from mara2_gb300.solver import Solver


def _host(name, n=None, req=None):
    if name == "sod":
        return W.sod(n)
    if name == "kh":
        return W.kelvin_helmholtz(n)
    if name == "rmhd_blast":
        return W.rmhd_blast(n)
    return W.riemann_initial(req)


REQS = W.riemann_stream(40, seed=W.RIEMANN_SEED + 7, n1=(64, 256), n2=(32, 96))
CASES = [("sod", 200, None), ("kh", 72, None), ("rmhd_blast", 40, None),
         ("riemann", None, next(r for r in REQS if r.dims == 1)),
         ("riemann", None, next(r for r in REQS if r.dims == 2))]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name,n,req", CASES)
def test_device_generation_matches_host(gpu_lib, precision, name, n, req):
    s, spec = W.device_initial_data(name, n, req)
    hs, P = _host(name, n, req)
    assert hs == s
    with Solver(s, precision) as g:
        g.generate(spec)
        a = g.download()
        g.upload(P.copy())
        b = g.download()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    if precision == "fp64":
        assert np.array_equal(a.view(np.uint64), P.view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("bc", ["reflecting", "outflow"])
def test_device_generation_guard_images(gpu_lib, bc):
    """Guards of other boundary conditions (reflecting negates the normal
    velocity) on the perturbed shear layer."""
    s, spec = W.device_initial_data("kh", 40)
    s = s.with_(bc=bc)
    _, P = W.kelvin_helmholtz(40)
    P = W.apply_bc_numpy(s, P)
    with Solver(s, "fp64") as g:
        g.generate(spec)
        a = g.download()
    assert np.array_equal(a.view(np.uint64), P.view(np.uint64))


@pytest.mark.gpu
def test_generated_state_runs_like_uploaded(gpu_lib):
    s, spec = W.device_initial_data("kh", 64)
    _, P = W.kelvin_helmholtz(64)
    with Solver(s, "fp64") as g:
        g.generate(spec)
        g.run(3)
        a = g.download()
        g.upload(P.copy())
        g.run(3)
        b = g.download()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
