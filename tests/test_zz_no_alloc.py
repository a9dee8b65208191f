"""mara_gpu_advance_noalloc: the advance for callers that cannot allocate
device memory when they step a grid (an application whose memory pool
already reserves the GPU, a latency-critical loop that must not block in an
allocation, code that must avoid cudaFree's device-wide synchronisation).

Checked through the C ABI against the handle-based entry points
(mara_gpu_create / upload / advance / download), two calls in a row on the
same device buffers, within the tolerance of the plain-path parity tests.
This file is collected last so that a run stopping at the first failure has
already run every other test; it passes alone in a fresh process too.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_l1

TOL = 1e-12  # relative L1 per conserved field, as in the plain-path parity tests


def _noalloc(lib, cfg, d_in, d_out, dt, stream):
    return lib.mara_gpu_advance_noalloc(C.byref(cfg), C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                        dt, C.c_void_p(stream))


@pytest.mark.gpu
def test_noalloc_matches_handle_path_two_calls(gpu_lib):
    import torch
    from mara2_gb300 import _native as N
    from mara2_gb300 import workloads as W
    from mara2_gb300.solver import Solver

    s, P0 = W.kelvin_helmholtz(64)
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
    assert _noalloc(gpu_lib, cfg, d_in, d_out, dt1, stream.cuda_stream) == N.MARA_OK
    out1 = d_out.cpu().numpy()
    assert _noalloc(gpu_lib, cfg, d_out, d_out, dt2, stream.cuda_stream) == N.MARA_OK  # in place
    out2 = d_out.cpu().numpy()

    i = s.interior()
    assert np.all(rel_l1(out1[i], ref1[i]) <= TOL)
    assert np.all(rel_l1(out2[i], ref2[i]) <= TOL)
    assert np.all(np.isfinite(out2))


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
