"""ctypes front end to the oracle libraries (TEST INFRASTRUCTURE ONLY).

Two libraries expose the same entry points:

* ``libmara_oracle.so`` -- the CPU restatement in ``mara_oracle.c`` (prefix
  ``mo_``), built by ``make`` in this directory on any machine;
* ``_ref/libmara_ref.so`` -- the reference's own hot-path sources compiled in
  place (prefix ``mr_``), built by ``make ref`` only where the reference tree
  exists.

Only tests, the smoke check and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

LAW = {"hydro": 0, "mhd": 1, "rmhd": 2}
RECON = {"pcm": 0, "plm": 1, "weno5": 2}
RIEMANN = {"hlle": 0, "hllc": 1}
BC = {"periodic": 0, "outflow": 1, "reflecting": 2}
WENO_IS = {"js96": 0, "borges08": 1, "shenzha10": 2}
NFIELDS = {"hydro": 5, "mhd": 8, "rmhd": 8}
STENCIL = {"pcm": 1, "plm": 2, "weno5": 3}

OK = 0
ERR_INVERSION_FAILURE = 16
ERR_SUPERLUMINAL = 17
ERR_BAD_EIGENVALUES = 18
ERR_GUARD_TOO_SMALL = 19
ERR_CONFIG = 20


SOURCE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double),
                        C.POINTER(C.c_double), C.POINTER(C.c_double))


class Config(C.Structure):
    """Mirror of ``mo_config`` in mara_oracle.h."""

    _fields_ = [
        ("law", C.c_int), ("recon", C.c_int), ("riemann", C.c_int), ("bc", C.c_int),
        ("rk_order", C.c_int), ("disable_ct", C.c_int), ("weno_is", C.c_int),
        ("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("ng", C.c_int * 3),
        ("lower", C.c_double * 3), ("upper", C.c_double * 3),
        ("gamma", C.c_double), ("plm_theta", C.c_double), ("shenzha_A", C.c_double),
        ("pressure_floor", C.c_double), ("cooling_rate", C.c_double),
    ]


class Failure(C.Structure):
    _fields_ = [("count", C.c_int), ("first", C.c_int * 3), ("code", C.c_int)]


def make_config(law="hydro", recon="plm", riemann="hlle", bc="outflow", rk_order=2,
                shape=(64, 1, 1), lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0), gamma=5.0 / 3,
                plm_theta=1.5, weno_is="shenzha10", shenzha_A=50.0, pressure_floor=-1.0,
                disable_ct=False, ng=None, cooling_rate=-1.0) -> Config:
    c = Config()
    c.law, c.recon, c.riemann, c.bc = LAW[law], RECON[recon], RIEMANN[riemann], BC[bc]
    c.rk_order, c.disable_ct, c.weno_is = rk_order, int(disable_ct), WENO_IS[weno_is]
    c.ni, c.nj, c.nk = shape
    g = STENCIL[recon] if ng is None else ng
    for a in range(3):
        c.ng[a] = g if shape[a] > 1 else 0
        c.lower[a], c.upper[a] = lower[a], upper[a]
    c.gamma, c.plm_theta, c.shenzha_A, c.pressure_floor = gamma, plm_theta, shenzha_A, pressure_floor
    c.cooling_rate = cooling_rate
    return c


def config_nq(c: Config) -> int:
    return (5, 9 if c.cooling_rate > 0.0 else 8, 8)[c.law]


def full_shape(c: Config) -> tuple:
    return (c.ni + 2 * c.ng[0], c.nj + 2 * c.ng[1], c.nk + 2 * c.ng[2], config_nq(c))


def interior(c: Config):
    return (slice(c.ng[0], c.ng[0] + c.ni), slice(c.ng[1], c.ng[1] + c.nj), slice(c.ng[2], c.ng[2] + c.nk))


def build(ref: bool = False) -> None:
    subprocess.run(["make", "-s", "-C", HERE] + (["ref"] if ref else []), check=True)


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libmara_ref.so"))


_D = C.POINTER(C.c_double)


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


class Oracle:
    """One library (restatement or reference build) behind a numpy API."""

    def __init__(self, which: str = "port"):
        self.which = which
        if which == "port":
            path, self.p = os.path.join(HERE, "libmara_oracle.so"), "mo_"
            if not os.path.exists(path):
                build(False)
        elif which == "ref":
            path, self.p = os.path.join(HERE, "_ref", "libmara_ref.so"), "mr_"
            if not os.path.exists(path):
                raise FileNotFoundError("the reference build is absent (make -C oracle ref)")
        else:
            raise ValueError(which)
        self.lib = L = C.CDLL(path)
        cp = C.POINTER(Config)
        f = self._f
        f("advance").argtypes = [cp, _D, C.c_double, C.c_double, C.POINTER(Failure)]
        f("courant").argtypes = [cp, _D, _D]
        f("apply_bc").argtypes = [cp, _D]
        f("godunov").argtypes = [cp, _D, _D]
        f("generate_conserved").argtypes = [cp, _D, _D]
        f("from_primitive").argtypes = [cp, _D, _D, _D, _D, _D]
        f("from_conserved").argtypes = [cp, _D, _D, C.POINTER(C.c_int)]
        f("quartic").argtypes = [C.c_double] * 5 + [_D]
        f("ct_correct").argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        f("ct_correct").restype = None
        f("monopole_cell").argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_double, _D]
        f("monopole_cell").restype = None
        f("set_source_terms").argtypes = [C.c_void_p, C.c_void_p]
        f("set_source_terms").restype = None
        self._src = None
        f("volume_diagnostics").argtypes = [cp, _D, _D, _D]
        f("current_cell").argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_double, _D]
        f("current_cell").restype = None
        f("uct_monopole").argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _D]
        f("uct_current").argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _D]
        f("vector_potential_to_cell_b_scaled").argtypes = [cp, _D, C.c_double, _D]
        if which == "port":
            L.mo_max_threads.restype = C.c_int
            L.mo_set_threads.argtypes = [C.c_int]
            L.mo_set_threads.restype = None
        else:
            L.mr_vector_potential_to_cell_b.argtypes = [cp, _D, _D]

    def _f(self, name):
        return getattr(self.lib, self.p + name)

    # -- whole-array operations ------------------------------------------------
    def advance(self, c: Config, P: np.ndarray, dt: float, t0: float = 0.0):
        fail = Failure()
        status = self._f("advance")(C.byref(c), _ptr(P), t0, dt, C.byref(fail))
        return status, fail

    def uct_monopole(self, B: np.ndarray, bc: str, location: str):
        """UniformCartesianCT::computeMonopole of cell data B (n0, n1, n2, 3)."""
        B = np.ascontiguousarray(B, dtype=float)
        n = B.shape[:3]
        M = np.zeros(tuple(m + 1 for m in n) if location == "vert" else n)
        st = self._f("uct_monopole")(_ptr(B), *n, BC[bc], 0 if location == "vert" else 1, _ptr(M))
        return st, M

    def uct_current(self, B: np.ndarray, bc: str, h: float = 1.0):
        B = np.ascontiguousarray(B, dtype=float)
        J = np.zeros_like(B)
        st = self._f("uct_current")(_ptr(B), *B.shape[:3], BC[bc], h, _ptr(J))
        return st, J

    def vector_potential_to_cell_b(self, c: Config, A: np.ndarray, scale: float = 1.0):
        """B = scale x div(CT(fluxes of A)) at every cell with guards."""
        A = np.ascontiguousarray(A, dtype=float)
        B = np.zeros((A.shape[0] - 1, A.shape[1] - 1, A.shape[2] - 1, 3))
        st = self._f("vector_potential_to_cell_b_scaled")(C.byref(c), _ptr(A), scale, _ptr(B))
        return st, B

    def courant(self, c: Config, P: np.ndarray):
        dt = np.zeros(1)
        status = self._f("courant")(C.byref(c), _ptr(P), _ptr(dt))
        return status, float(dt[0])

    def apply_bc(self, c: Config, P: np.ndarray) -> int:
        return self._f("apply_bc")(C.byref(c), _ptr(P))

    def godunov(self, c: Config, P: np.ndarray):
        N = full_shape(c)
        F = np.zeros((N[0] + 1, N[1] + 1, N[2] + 1, N[3], 3))
        status = self._f("godunov")(C.byref(c), _ptr(P), _ptr(F))
        return status, F

    def generate_conserved(self, c: Config, P: np.ndarray):
        U = np.zeros_like(P)
        status = self._f("generate_conserved")(C.byref(c), _ptr(P), _ptr(U))
        return status, U

    # -- point operations -------------------------------------------------------
    def from_primitive(self, c: Config, P, n=(1.0, 0.0, 0.0)):
        P = np.ascontiguousarray(np.pad(np.asarray(P, float), (0, 10 - len(P))))
        n = np.ascontiguousarray(np.asarray(n, float))
        U, F, A = np.zeros(10), np.zeros(10), np.zeros(10)
        status = self._f("from_primitive")(C.byref(c), _ptr(P), _ptr(n), _ptr(U), _ptr(F), _ptr(A))
        return status, U, F, A

    def from_conserved(self, c: Config, U):
        U = np.ascontiguousarray(np.pad(np.asarray(U, float), (0, 10 - len(U))))
        P = np.zeros(10)
        h = C.c_int(0)
        status = self._f("from_conserved")(C.byref(c), _ptr(U), _ptr(P), C.byref(h))
        return status, P, h.value

    def quartic(self, d4, d3, d2, d1, d0):
        r = np.zeros(4)
        nr = self._f("quartic")(d4, d3, d2, d1, d0, _ptr(r))
        return nr, r[:nr].copy()

    def ct_correct(self, F: np.ndarray, ib: int = 5) -> np.ndarray:
        G = np.ascontiguousarray(F.copy())
        n0, n1, n2, nq, _ = G.shape
        self._f("ct_correct")(_ptr(G), n0, n1, n2, nq, ib)
        return G

    def monopole_cell(self, B: np.ndarray, h: float = 1.0) -> np.ndarray:
        B = np.ascontiguousarray(B, dtype=float)
        n0, n1, n2, _ = B.shape
        M = np.zeros((n0, n1, n2))
        self._f("monopole_cell")(_ptr(B), n0, n1, n2, h, _ptr(M))
        return M

    def set_source_terms(self, fn=None):
        """MethodOfLinesTVD::setSourceTermsFunction for later advances:
        fn(x, y, z, aux, P) -> S, with P and S of MARA_NUM_FIELDS (10) slots;
        None removes it."""
        if fn is None:
            self._src = None
            self._f("set_source_terms")(None, None)
            return

        def tramp(user, x, y, z, aux, P, S):
            out = fn(x, y, z, [aux[n] for n in range(8)], [P[n] for n in range(10)])
            for q, v in enumerate(out):
                S[q] = v

        self._src = SOURCE_FN(tramp)
        self._f("set_source_terms")(C.cast(self._src, C.c_void_p), None)

    def current_cell(self, B: np.ndarray, h: float = 1.0) -> np.ndarray:
        B = np.ascontiguousarray(B, dtype=float)
        n0, n1, n2, _ = B.shape
        J = np.zeros((n0, n1, n2, 3))
        self._f("current_cell")(_ptr(B), n0, n1, n2, h, _ptr(J))
        return J

    def volume_diagnostics(self, c: Config, P: np.ndarray):
        """(status, D, Dabs): FieldOperator::volumeIntegratedDiagnostics over
        the interior of P, and the sum of the terms' magnitudes (zeros from the
        reference build, which does not form it)."""
        nd = 5 if c.law == LAW["hydro"] else 18 if (c.law == LAW["mhd"] and c.cooling_rate > 0.0) else 17
        D, Dabs = np.zeros(nd), np.zeros(nd)
        status = self._f("volume_diagnostics")(C.byref(c), _ptr(np.ascontiguousarray(P, dtype=float)), _ptr(D),
                                                _ptr(Dabs))
        return status, D, Dabs

    # -- driver -----------------------------------------------------------------
    def run(self, c: Config, P: np.ndarray, steps: int, cfl: float, t_final: float | None = None,
            dts=None):
        """The regression drivers' main loop (src/Problems.cpp:181-188 with
        src/Mara.cpp:56-76): dt = min(cfl * courant, t_final - t).  Returns
        (status, t, dt list)."""
        t, out = 0.0, []
        for n in range(steps):
            if t_final is not None and not t < t_final:
                break
            if dts is not None:
                dt = dts[n]
            else:
                s, dc = self.courant(c, P)
                if s:
                    return s, t, out
                dt = cfl * dc
                if t_final is not None:
                    dt2 = t_final - t
                    dt = dt if dt < dt2 else dt2
            s, _ = self.advance(c, P, dt)
            out.append(dt)
            if s:
                return s, t, out
            t += dt
        return OK, t, out
