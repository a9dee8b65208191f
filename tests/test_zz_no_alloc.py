"""mara_gpu_advance_noalloc: the advance for callers that cannot allocate
device memory when they step a grid (an application whose memory pool
already reserves the GPU, a latency-critical loop that must not block in an
allocation, code that must avoid cudaFree's device-wide synchronisation).

The entry point runs the same plain FP64 kernels as the handle-based entry
points (mara_gpu_create / upload / advance / download), so it is checked
against them bit for bit, through the C ABI, two calls in a row on the same
device buffers: a 2-D hydro Kelvin-Helmholtz grid (RK2, HLLC) and a 3-D MHD
grid with constrained transport (RK3, HLLE, three face-flux arrays carved
from the scratch array).  A planted state that cannot be inverted must come
back as the same status code the handle path reports, and the caller's
current device must be unchanged afterwards.  This file is collected last,
so that a run stopping at the first failure has already run every other
test; it passes alone in a fresh process too.
"""
import ctypes as C

import numpy as np
import pytest


def _noalloc(lib, cfg, d_in, d_out, dt, stream):
    return lib.mara_gpu_advance_noalloc(C.byref(cfg), C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                        dt, C.c_void_p(stream))


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def _two_steps_both_ways(lib, s, P0):
    import torch
    from mara2_gb300 import _native as N
    from mara2_gb300.solver import Solver

    cfg = N.config_from_scheme(s, "fp64", 0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)

    # the existing entry points
    with Solver(s, "fp64") as g:
        g.upload(P0.copy())
        dt1 = g.courant() * s.cfl
        g.advance(dt1)
        ref1 = g.download()
        dt2 = 0.9 * dt1
        g.advance(dt2)
        ref2 = g.download()

    # the allocation-free entry point on caller-owned device buffers
    d_in = torch.from_numpy(P0.copy()).to(dev)
    d_out = torch.empty_like(d_in)
    torch.cuda.synchronize(dev)
    assert _noalloc(lib, cfg, d_in, d_out, dt1, stream.cuda_stream) == N.MARA_OK
    out1 = d_out.cpu().numpy()
    assert _noalloc(lib, cfg, d_out, d_out, dt2, stream.cuda_stream) == N.MARA_OK  # in place
    out2 = d_out.cpu().numpy()
    assert torch.cuda.current_device() == 0
    return (ref1, ref2), (out1, out2)


@pytest.mark.gpu
def test_noalloc_matches_handle_path_two_calls_hydro(gpu_lib):
    from mara2_gb300 import workloads as W

    s, P0 = W.kelvin_helmholtz(64)
    (ref1, ref2), (out1, out2) = _two_steps_both_ways(gpu_lib, s, P0)
    i = s.interior()
    assert np.array_equal(_bits(out1[i]), _bits(ref1[i]))
    assert np.array_equal(_bits(out2[i]), _bits(ref2[i]))
    assert np.all(np.isfinite(out2))


@pytest.mark.gpu
def test_noalloc_matches_handle_path_two_calls_mhd3d_rk3(gpu_lib):
    from mara2_gb300 import workloads as W

    s, P0 = W.mhd_turbulence(12)
    assert s.rk_order == 3 and s.law == "mhd" and s.dims == 3
    (ref1, ref2), (out1, out2) = _two_steps_both_ways(gpu_lib, s, P0)
    i = s.interior()
    assert np.array_equal(_bits(out1[i]), _bits(ref1[i]))
    assert np.array_equal(_bits(out2[i]), _bits(ref2[i]))


@pytest.mark.gpu
def test_noalloc_reports_inversion_failure_like_the_handle_path(gpu_lib):
    import torch
    from mara2_gb300 import _native as N
    from mara2_gb300 import workloads as W
    from mara2_gb300.solver import Solver

    s, P = W.mhd_turbulence(6)
    Q = P.copy()
    Q[4, 5, 3, 4] = 1e-9     # near-vacuum pressure next to a strong velocity jump
    Q[4, 5, 3, 1] = 3.0
    with Solver(s, "fp64") as g:
        g.upload(Q.copy())
        g.advance(0.05)
        want = g.status()
    assert want == N.MARA_ERR_INVERSION_FAILURE
    cfg = N.config_from_scheme(s, "fp64", 0)
    d = torch.from_numpy(Q.copy()).to("cuda:0")
    out = torch.empty_like(d)
    torch.cuda.synchronize()
    assert _noalloc(gpu_lib, cfg, d, out, 0.05, torch.cuda.current_stream().cuda_stream) == want
    # the next call starts from cleared status words
    s2, P2 = W.mhd_turbulence(6)
    d2 = torch.from_numpy(P2.copy()).to("cuda:0")
    assert _noalloc(gpu_lib, cfg, d2, out, 1e-3, torch.cuda.current_stream().cuda_stream) == N.MARA_OK


@pytest.mark.gpu
def test_noalloc_rejects_grids_beyond_the_scratch_limit(gpu_lib):
    from mara2_gb300 import _native as N
    from mara2_gb300.scheme import Scheme

    import torch
    s = Scheme(law="mhd", recon="plm", shape=(256, 256, 256), bc="periodic")
    cfg = N.config_from_scheme(s, "fp64", 0)
    small = torch.zeros(8, dtype=torch.float64, device="cuda:0")  # never touched: rejected before any GPU work
    rc = gpu_lib.mara_gpu_advance_noalloc(C.byref(cfg), C.c_void_p(small.data_ptr()), C.c_void_p(small.data_ptr()),
                                          1e-3, None)
    assert rc == N.MARA_ERR_TOO_LARGE
