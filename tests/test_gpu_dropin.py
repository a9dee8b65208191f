"""The C++ drop-in run on the GPU: a driver compiled against the reference's
own interface headers and hot-path objects (tests/dropin_driver.cpp) swaps
MethodOfLinesTVD for GpuMethodOfLinesTVD and calls advance the way the
reference's drivers do (src/Problems.cpp:188), and uses GpuConstrainedTransport
through the ConstrainedTransport interface (src/Mara.hpp:341-349).

* Sod 64 through SolutionScheme::advance reproduces the golden fixture made
  by the reference's build, bit for bit, and getCourantTimestep the oracle's.
* A state the reference cannot invert throws FieldOperator::InversionFailure
  naming the zone the oracle names.
* The ConstrainedTransport adaptor's monopole and current equal the oracle's.

Needs the reference's sources (MARA_REF_SRC, else baseline/_ref/src) and
their objects (oracle/_ref, built by __graft_entry__.build()); skipped where
they are absent."""
import glob
import os
import subprocess

import numpy as np
import pytest

from helpers import oracle_config
from mara2_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.environ.get("MARA_REF_SRC", os.path.join(ROOT, "baseline", "_ref", "src"))
OBJS = sorted(glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o")))


@pytest.fixture(scope="module")
def driver(tmp_path_factory, gpu_lib):
    if not os.path.isfile(os.path.join(REF_SRC, "SolutionSchemes.hpp")) or not OBJS:
        pytest.skip("reference sources or objects not available")
    from mara2_gb300 import build
    lib = build.build()
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_driver")
    cmd = ["g++", "-std=c++14", "-O1", "-ffp-contract=off", "-I" + os.path.join(ROOT, "oracle", "cowshim"),
           "-I" + REF_SRC, "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "mara2_gb300", "csrc"),
           os.path.join(ROOT, "tests", "dropin_driver.cpp"), *OBJS, "-L" + os.path.dirname(lib), "-lmara_gpu",
           "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _run(exe, mode, tmp_path, data):
    fin, fout = str(tmp_path / f"{mode}.in"), str(tmp_path / f"{mode}.out")
    np.ascontiguousarray(data, dtype=np.float64).tofile(fin)
    r = subprocess.run([exe, mode, fin, fout], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return np.fromfile(fout, dtype=np.float64), r.stdout


@pytest.mark.gpu
def test_dropin_advance_reproduces_golden(driver, port, tmp_path):
    z = np.load(os.path.join(ROOT, "tests", "golden", "sod64_plm_hlle_rk2.npz"))
    s = eval(str(z["scheme"]), {"Scheme": __import__("mara2_gb300.scheme", fromlist=["Scheme"]).Scheme})
    out, _ = _run(driver, "sod", tmp_path, np.concatenate([z["P0"].ravel(), z["dts"]]))
    P = out[:-1].reshape(z["P"].shape)
    assert np.array_equal(P.view(np.uint64), z["P"].view(np.uint64))
    st, dt = port.courant(oracle_config(s), z["P0"].copy())
    assert st == 0 and out[-1] == dt


@pytest.mark.gpu
def test_dropin_throws_inversion_failure(driver, port, tmp_path):
    s, P = W.mhd_turbulence(6)
    Q = P.copy()
    Q[4, 5, 3, 4] = 1e-9
    Q[4, 5, 3, 1] = 3.0
    st, fail = port.advance(oracle_config(s), Q.copy(), 0.05)
    assert st == 16 and fail.count == 1
    zone, msg = _run(driver, "fail", tmp_path, Q)
    assert zone[3] == 1, msg
    assert tuple(int(v) for v in zone[:3]) == tuple(fail.first), msg


@pytest.mark.gpu
def test_dropin_constrained_transport_interface(driver, port, tmp_path):
    n = (7, 6, 5)
    B = np.random.default_rng(5).standard_normal(n + (3,))
    out, _ = _run(driver, "ct", tmp_path, np.concatenate([np.array(n, dtype=float), B.ravel()]))
    nv = (n[0] + 1) * (n[1] + 1) * (n[2] + 1)
    nc = n[0] * n[1] * n[2]
    _, Mv = port.uct_monopole(B, "periodic", "vert")
    _, Mc = port.uct_monopole(B, "periodic", "cell")
    _, J = port.uct_current(B, "periodic", 1.0)
    assert np.array_equal(out[:nv].view(np.uint64), Mv.ravel().view(np.uint64))
    assert np.array_equal(out[nv:nv + nc].view(np.uint64), Mc.ravel().view(np.uint64))
    assert np.array_equal(out[nv + nc:nv + nc + 3 * nc].view(np.uint64), J.ravel().view(np.uint64))
    assert out[-1] == 1.0   # computeCurrent at vertices throws std::logic_error
