"""Golden fixtures produced by the reference's own build (make_golden.py):
the oracle must reproduce them bit for bit on any machine, and the plain GPU
path must match them (bit for bit where no transcendental function enters,
relative L1 <= 1e-12 per conserved field otherwise)."""
import glob
import os

import numpy as np
import pytest

from helpers import oracle_config, parity_error, rel_l1
from mara2_gb300.scheme import Scheme  # noqa: F401  (eval of the stored repr)

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = sorted(glob.glob(os.path.join(HERE, "*.npz")))


def _load(path):
    z = np.load(path, allow_pickle=False)
    s = eval(str(z["scheme"]))  # a Scheme(...) repr written by make_golden.py
    return s, z


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_oracle_reproduces_golden(port, path):
    s, z = _load(path)
    c = oracle_config(s)
    P = z["P0"].copy()
    for dt in z["dts"]:
        st, _ = port.advance(c, P, float(dt))
        assert st == 0
    assert np.array_equal(P.view(np.uint64), z["P"].view(np.uint64))
    if "godunov_fluxes" in z:
        st, F = port.godunov(c, z["P0"].copy())
        assert np.array_equal(F.view(np.uint64), z["godunov_fluxes"].view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_gpu_plain_reproduces_golden(gpu_lib, port, path):
    from mara2_gb300.solver import Solver
    s, z = _load(path)
    with Solver(s, "fp64") as g:
        g.upload(z["P0"].copy())
        for dt in z["dts"]:
            g.advance(float(dt))
        out = g.download()
    ref = z["P"]
    c = oracle_config(s)
    _, Uo = port.generate_conserved(c, np.ascontiguousarray(out))
    _, Ur = port.generate_conserved(c, np.ascontiguousarray(ref))
    err = parity_error(s, Uo[s.interior()], Ur[s.interior()])
    assert np.all(err <= 1e-12), err.tolist()
    if s.law != "rmhd":
        assert np.array_equal(out[s.interior()].view(np.uint64), ref[s.interior()].view(np.uint64))
