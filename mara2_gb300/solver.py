"""Python host API over the C ABI: one ``Solver`` per resident grid.

``Solver`` holds a ``MaraGpuHandle``: the device state of one MeshData plus
the scheme that advances it.  Host arrays are the reference's MeshData::P
layout (numpy float64, shape ``Scheme.full_shape``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .scheme import Scheme


def diagnostic_names(law: str, aux: int = 0) -> list:
    """ConservationLaw::getDiagnosticNames (src/ConservationLaws.cpp:332-341,
    576-601, 924-945); aux auxiliary fields of NewtonianMHD add
    auxiliary1..."""
    base = ["mass", "momentum1", "momentum2", "momentum3", "total_energy"]
    if law == "hydro":
        return base
    return base + ["magnetic_flux1", "magnetic_flux2", "magnetic_flux3", "kinetic_energy", "internal_energy",
                   "magnetic_energy", "sound_speed", "alfven_speed", "sonic_mach_number", "alfven_mach_number",
                   "specific_entropy", "cross_helicity"] + [f"auxiliary{n + 1}" for n in range(aux)]


class Solver:
    def __init__(self, scheme: Scheme, precision: str = "fp64", device: int = 0):
        self.scheme = scheme
        self.precision = precision
        self.lib = N.load()
        self._cfg = N.config_from_scheme(scheme, precision, device)
        h = C.c_void_p()
        N.check(self.lib.mara_gpu_create(C.byref(self._cfg), C.byref(h)), "mara_gpu_create")
        self.h = h
        self.t = 0.0

    # -- life cycle ---------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.mara_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state ----------------------------------------------------------------------
    def upload(self, P: np.ndarray) -> None:
        P = self._as_state(P)
        N.check(self.lib.mara_gpu_upload(self.h, P.ctypes.data), "mara_gpu_upload")

    def upload_ptr(self, ptr: int) -> None:
        N.check(self.lib.mara_gpu_upload(self.h, C.c_void_p(ptr)), "mara_gpu_upload")

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.scheme.full_shape, dtype=np.float64)
        N.check(self.lib.mara_gpu_download(self.h, out.ctypes.data), "mara_gpu_download")
        return out

    def download_ptr(self, ptr: int) -> None:
        N.check(self.lib.mara_gpu_download(self.h, C.c_void_p(ptr)), "mara_gpu_download")

    def _as_state(self, P):
        if P.shape != self.scheme.full_shape or P.dtype != np.float64 or not P.flags["C_CONTIGUOUS"]:
            raise ValueError(f"state must be C-contiguous float64 {self.scheme.full_shape}")
        return P

    # -- stepping -------------------------------------------------------------------
    def advance(self, dt: float, t0: float = 0.0) -> None:
        N.check(self.lib.mara_gpu_advance(self.h, t0, dt), "mara_gpu_advance")

    def advance_host(self, P: np.ndarray, dt: float, t0: float = 0.0) -> None:
        """SolutionScheme::advance on a host MeshData::P array, in place."""
        P = self._as_state(P)
        N.check(self.lib.mara_gpu_advance_host(self.h, P.ctypes.data, t0, dt), "mara_gpu_advance_host")

    def advance_host_ptr(self, ptr: int, dt: float, t0: float = 0.0) -> int:
        return self.lib.mara_gpu_advance_host(self.h, C.c_void_p(ptr), t0, dt)

    def courant(self) -> float:
        dt = C.c_double()
        N.check(self.lib.mara_gpu_courant(self.h, C.byref(dt)), "mara_gpu_courant")
        return dt.value

    def run(self, steps: int, cfl: float | None = None, t_final: float | None = None) -> int:
        """Device-resident driver loop; returns steps taken and updates self.t."""
        s = self.scheme
        cfl = s.cfl if cfl is None else cfl
        tf = -1.0 if t_final is None else t_final
        t = C.c_double(self.t)
        n = C.c_int(0)
        N.check(self.lib.mara_gpu_run(self.h, steps, cfl, tf, C.byref(t), C.byref(n)), "mara_gpu_run")
        self.t = t.value
        return n.value

    def run_async(self, steps: int, cfl: float | None = None, t_final: float | None = None) -> None:
        """Enqueue steps of the driver loop on the handle's stream and return
        at once (continues from the device-side time of the last run)."""
        cfl = self.scheme.cfl if cfl is None else cfl
        tf = -1.0 if t_final is None else t_final
        N.check(self.lib.mara_gpu_run_async(self.h, steps, cfl, tf), "mara_gpu_run_async")

    def synchronize(self) -> None:
        N.check(self.lib.mara_gpu_synchronize(self.h), "mara_gpu_synchronize")

    def stats(self) -> N.MaraGpuStats:
        st = N.MaraGpuStats()
        self.lib.mara_gpu_stats(self.h, C.byref(st))
        return st

    def status(self) -> int:
        return self.lib.mara_gpu_synchronize(self.h)

    @property
    def stream(self) -> int:
        return self.lib.mara_gpu_stream(self.h)

    def monopole_max(self, mesh_spacing: float = 1.0) -> float:
        """Largest |div B| (CellCenteredFieldCT::monopole at cells) over the
        interior of the resident state."""
        m = C.c_double()
        N.check(self.lib.mara_gpu_monopole(self.h, mesh_spacing, C.byref(m)), "mara_gpu_monopole")
        return m.value

    def device_bytes(self) -> int:
        return self.lib.mara_gpu_device_bytes(self.h)

    def set_kernel_timing(self, on: bool) -> None:
        self.lib.mara_gpu_set_kernel_timing(self.h, int(on))

    def generate(self, spec: dict) -> None:
        """MeshOperator::generate of a built-in initial-data function on the
        device (mara_gpu_generate); spec as workloads.device_initial_data
        builds it."""
        d = N.MaraInitialData()
        d.kind = spec["kind"]
        for name in ("left", "right"):
            for q, v in enumerate(spec.get(name, ())):
                getattr(d, name)[q] = v
        for name in ("x0", "normal"):
            for a, v in enumerate(spec.get(name, (0.0, 0.0, 0.0))):
                getattr(d, name)[a] = v
        d.radius = spec.get("radius", 0.0)
        d.noise = spec.get("noise", 0.0)
        d.seed = spec.get("seed", 0)
        N.check(self.lib.mara_gpu_generate(self.h, C.byref(d)), "mara_gpu_generate")

    def set_source_terms(self, fn=None, gravity=None) -> None:
        """MethodOfLinesTVD::setSourceTermsFunction on the plain path:
        gravity=(g1, g2, g3) installs the library's uniform-gravity source; fn
        is a MaraSourceTermsFn (a ctypes function pointer or a Python callable
        (user, args) -> status that enqueues device work on args.stream);
        neither removes the source terms."""
        self._src_keep = None
        if gravity is not None:
            g = (C.c_double * 3)(*[float(v) for v in gravity])
            fptr = C.cast(self.lib.mara_source_uniform_gravity, C.c_void_p)
            self._src_keep = (g,)
            N.check(self.lib.mara_gpu_set_source_terms(self.h, fptr, C.cast(g, C.c_void_p)),
                    "mara_gpu_set_source_terms")
        elif fn is not None:
            cb = fn if isinstance(fn, N.SOURCE_FN) else N.SOURCE_FN(fn)
            self._src_keep = (cb,)
            N.check(self.lib.mara_gpu_set_source_terms(self.h, C.cast(cb, C.c_void_p), None),
                    "mara_gpu_set_source_terms")
        else:
            N.check(self.lib.mara_gpu_set_source_terms(self.h, None, None), "mara_gpu_set_source_terms")

    def volume_diagnostics(self) -> dict:
        """FieldOperator::volumeIntegratedDiagnostics of the resident state,
        by the names ConservationLaw::getDiagnosticNames gives them."""
        n = self.lib.mara_gpu_num_diagnostics(self.h)
        D = np.zeros(n)
        cnt = C.c_int(0)
        N.check(self.lib.mara_gpu_volume_diagnostics(self.h, D.ctypes.data, C.byref(cnt)),
                "mara_gpu_volume_diagnostics")
        return dict(zip(diagnostic_names(self.scheme.law, self.scheme.aux), D.tolist()))

    def field_diagnostics(self, mesh_spacing: float = 1.0, out: np.ndarray | None = None) -> np.ndarray:
        """[monopole, current1, current2, current3] at every cell of the array
        with guards, shape full_shape[:3] + (4,) (MHD and RMHD); out, if
        given, receives them (C-contiguous float64 of that shape; page-locked
        memory takes the full rate of the host link)."""
        shape = tuple(self.scheme.full_shape[:3]) + (4,)
        if out is None:
            out = np.zeros(shape)
        elif out.shape != shape or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError(f"field diagnostics buffer must be C-contiguous float64 of shape {shape}")
        N.check(self.lib.mara_gpu_field_diagnostics(self.h, mesh_spacing, out.ctypes.data),
                "mara_gpu_field_diagnostics")
        return out

    def assign_vector_potential(self, A: np.ndarray, scale: float = 1.0) -> None:
        """The divergence-free field of src/Problems.cpp:660-667 from the
        face-centred vector potential A (shape (N0+1, N1+1, N2+1, 3, 3)),
        times scale, on the resident state (mara_gpu_assign_vector_potential)."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        want = tuple(n + 1 for n in self.scheme.full_shape[:3]) + (3, 3)
        if A.shape != want:
            raise ValueError(f"vector potential shape {A.shape}, expected {want}")
        N.check(self.lib.mara_gpu_assign_vector_potential(self.h, A.ctypes.data, scale),
                "mara_gpu_assign_vector_potential")

    def kernel_times(self):
        ms = (C.c_double * 3)()
        n = (C.c_int64 * 3)()
        self.lib.mara_gpu_kernel_times(self.h, ms, n)
        return list(ms), list(n)


_BC = {"periodic": 0, "outflow": 1, "reflecting": 2}


def ct_monopole(B: np.ndarray, bc: str, location: str = "cell", device: int = 0) -> np.ndarray:
    """UniformCartesianCT::computeMonopole (the ConstrainedTransport interface,
    src/Mara.hpp:341-349) of a cell-centred field B (n0, n1, n2, 3) on the
    device: at vertices ((n+1)^3) or cells (n^3)."""
    B = np.ascontiguousarray(B, dtype=np.float64)
    n = np.array(B.shape[:3], dtype=np.int32)
    M = np.zeros(tuple(int(m) + 1 for m in n) if location == "vert" else tuple(int(m) for m in n))
    N.check(N.load().mara_gpu_ct_monopole(B.ctypes.data, n.ctypes.data, _BC[bc], 0 if location == "vert" else 1,
                                          M.ctypes.data, device), "mara_gpu_ct_monopole")
    return M


def ct_current(B: np.ndarray, bc: str, mesh_spacing: float = 1.0, device: int = 0) -> np.ndarray:
    """computeCurrent of the same adaptor (CellCenteredFieldCT::current of the
    guarded field) at the interior cells: J (n0, n1, n2, 3)."""
    B = np.ascontiguousarray(B, dtype=np.float64)
    n = np.array(B.shape[:3], dtype=np.int32)
    J = np.zeros_like(B)
    N.check(N.load().mara_gpu_ct_current(B.ctypes.data, n.ctypes.data, _BC[bc], mesh_spacing, J.ctypes.data,
                                         device), "mara_gpu_ct_current")
    return J
