"""QuarticPolynomial::solve (src/QuarticPolynomial.cpp:19-144) on the device,
through mara_gpu_quartic_solve: the known answers of the reference's unit
test (src/TestSuite.cpp:431-478) and, on seeded random quartics, the
oracle's roots (the oracle is pinned bit for bit to the reference build).
The device's pow(x, 1/3), acos, cos and sin are correctly rounded, the
host's libm is on all but ~0.1 % of arguments, so nearly every root set is
bit-identical; the rest differ by a rounding that the printed table
bounds."""
import ctypes as C

import numpy as np
import pytest

from test_oracle_known import approx


def _device_roots(lib, coeffs):
    coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
    n = coeffs.shape[0]
    roots = np.zeros((n, 4))
    nr = np.zeros(n, dtype=np.int32)
    rc = lib.mara_gpu_quartic_solve(coeffs.ctypes.data, n, roots.ctypes.data, nr.ctypes.data, 0)
    assert rc == 0
    return nr, roots


@pytest.mark.gpu
@pytest.mark.parametrize("coeffs,roots,eps", [
    ((1, 0, -5, 0, 4), (-2, -1, 1, 2), 1e-14),
    ((1., 0., -1., 0., 1e-10), (-1, -1e-5, 1e-5, 1), 1e-10),
    ((-1, 0, 0, 0, 1), (-1, 1), 1e-14),
])
def test_device_quartic_known_roots(gpu_lib, coeffs, roots, eps):
    nr, r = _device_roots(gpu_lib, [coeffs])
    assert nr[0] == len(roots)
    for a, b in zip(r[0], roots):
        assert approx(a, b, eps)


def _random_quartics(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.uniform(-3, 3, (n, 5))
    # also the quartics of RMHD wave speeds: real roots of both counts, wide
    # coefficient ranges
    e = rng.uniform(-3, 3, (n, 5)) * 10.0 ** rng.uniform(-4, 4, (n, 5))
    return np.concatenate([d, e])


@pytest.mark.gpu
def test_device_quartic_matches_oracle(gpu_lib, port):
    Q = _random_quartics(2000, 7)
    nr, r = _device_roots(gpu_lib, Q)
    same = 0
    worst = 0.0
    for i, d in enumerate(Q):
        na, ra = port.quartic(*d)
        assert na == nr[i], (i, d)
        ra = np.asarray(ra)[:na]
        rb = r[i, :na]
        if np.array_equal(ra.view(np.uint64), rb.view(np.uint64)):
            same += 1
        elif na:
            worst = max(worst, float(np.max(np.abs(ra - rb)) / (1.0 + np.max(np.abs(ra)))))
    print(f"\n{same} of {len(Q)} root sets bit-identical to the oracle; largest difference "
          f"of the others {worst:.3g} relative to 1 + max |root|")
    assert same >= 0.98 * len(Q)
    assert worst <= 1e-7
