"""The FP32 <-> FP64 conversions and the exact halving that the
FP64-accumulator form runs on the integer pipes
(mara2_gb300/csrc/hydro_tile.cuh: f2d_exact, d2f_rn_ftz, half_exact): bit for
bit the conversion instructions (and the FP64 multiply by 0.5) as the fused
kernels compile them (-ftz=true), on seeded arguments of every kind -
random magnitudes, rounding ties and their neighbours, values at the ends of
the FP32 range, signed zeros, and random bit patterns (subnormals,
infinities, NaNs)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROBE = os.path.join(ROOT, "tests", "conv_probe.cu")


def _arguments(n, seed=2027):
    rng = np.random.default_rng(seed)
    kind = np.arange(n) % 6
    mag = (rng.random(n) - 0.5) * 10.0 ** ((rng.random(n) - 0.5) * 90)
    f = ((rng.random(n) - 0.5) * 100).astype(np.float32).astype(np.float64)
    ties = (f.view(np.uint64) + np.uint64(1 << 28) + rng.integers(-2, 3, n).astype(np.int64).view(np.uint64)).view(
        np.float64)
    ends = rng.random(n) * np.where(rng.random(n) < 0.5, 3.4e38 * 1.02, 1.2e-38 * 1.5) * np.where(
        rng.random(n) < 0.5, -1.0, 1.0)
    sign = np.where(rng.random(n) < 0.5, np.uint64(1 << 63), np.uint64(0))
    bits = (rng.integers(0, 2**63, n, dtype=np.int64).view(np.uint64) | sign).view(np.float64)
    zeros = np.where(rng.random(n) < 0.5, 0.0, -0.0)
    d = np.select([kind == 0, kind == 1, kind == 2, kind == 3, kind == 4], [mag, ties, ends, bits, zeros], mag)
    fb = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    fv = ((rng.random(n) - 0.5) * 10.0 ** ((rng.random(n) - 0.5) * 70)).astype(np.float32)
    f32 = np.where(np.arange(n) % 3 == 0, fb, fv).astype(np.float32)
    return np.ascontiguousarray(d), np.ascontiguousarray(f32)


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    nan = np.isnan(a) & np.isnan(b)
    return np.all((a.view(np.uint32 if a.dtype == np.float32 else np.uint64) ==
                   b.view(np.uint32 if b.dtype == np.float32 else np.uint64)) | nan)


@pytest.mark.gpu
def test_integer_pipe_conversions_match_the_instructions(tmp_path):
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    so = os.path.join(str(tmp_path), "libconvprobe.so")
    subprocess.run([nvcc, "-O3", "-std=c++17", "--fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true",
                    "-gencode", "arch=compute_103a,code=sm_103a", "-I" + os.path.join(ROOT, "include"),
                    "-Xcompiler", "-fPIC", "-shared", PROBE, "-o", so], check=True)
    lib = C.CDLL(so)
    n = 1 << 21
    d, f = _arguments(n)
    outs = [np.empty(n, np.float32), np.empty(n, np.float32), np.empty(n), np.empty(n), np.empty(n), np.empty(n)]
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    assert lib.conv_eval(ptr(d), ptr(f), C.c_int(n), *[ptr(o) for o in outs]) == 0
    assert _same(outs[0], outs[1]), "double -> float"
    assert _same(outs[2], outs[3]), "float -> double"
    assert _same(outs[4], outs[5]), "x / 2"
