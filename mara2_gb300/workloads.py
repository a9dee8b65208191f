"""Seeded synthetic initial data for the five benchmark workloads.

The reference's regression drivers build initial data by evaluating an
``InitialDataFunction`` at cell centres (``MeshOperator::generate``,
src/MeshOperator.cpp:168-189) and, for magnetised problems, by turning a
face-centred vector potential into a divergence-free cell field
(src/Problems.cpp:660-667).  These generators do the same in numpy, in the
reference's AoS layout ``(ni+2g, nj+2g, nk+2g, nq)`` with guards filled by
the boundary condition, so one array feeds the GPU solver and the CPU oracle
identically.

Randomness comes from SplitMix64 (Steele, Lea & Flood 2014) so that every
machine produces the same bits.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .scheme import Scheme

MASK64 = (1 << 64) - 1


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n successive SplitMix64 outputs as uint64."""
    out = np.empty(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed & MASK64) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        out[:] = z ^ (z >> np.uint64(31))
    return out


def uniform(seed: int, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    """n doubles uniform in [lo, hi) from the top 53 bits of SplitMix64."""
    u = (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


def cell_centres(s: Scheme):
    """Cell-centre coordinates of every cell including guards
    (CartesianMeshGeometry::coordinateAtIndex, lower + dx * (i + 0.5))."""
    out = []
    for a in range(3):
        n, g = s.shape[a], s.ng[a]
        dx = (s.upper[a] - s.lower[a]) / n
        idx = np.arange(-g, n + g, dtype=np.float64)
        out.append(s.lower[a] + dx * (idx + 0.5))
    return np.meshgrid(*out, indexing="ij")


def apply_bc_numpy(s: Scheme, P: np.ndarray) -> np.ndarray:
    """Guard fill of BoundaryCondition::applySimple (src/BoundaryConditions.cpp:
    8-176): axis by axis, left then right, over the full transverse extent."""
    for a in range(3):
        g = s.ng[a]
        if g == 0:
            continue
        N = P.shape[a]
        P = np.moveaxis(P, a, 0)
        for n in range(g):
            if s.bc == "periodic":
                P[n] = P[N - 2 * g + n]
            elif s.bc == "outflow":
                P[n] = P[g]
            else:
                P[n] = P[2 * g - n - 1]
                P[n, ..., 1 + a] *= -1
        for n in range(g):
            if s.bc == "periodic":
                P[N - g + n] = P[g + n]
            elif s.bc == "outflow":
                P[N - n - 1] = P[N - g - 1]
            else:
                P[N - n - 1] = P[N - 2 * g + n]
                P[N - n - 1, ..., 1 + a] *= -1
        P = np.moveaxis(P, 0, a)
    return P


def empty_state(s: Scheme) -> np.ndarray:
    return np.zeros(s.full_shape, dtype=np.float64)


# ----------------------------------------------------------------------------
# workload 1: Sod shock tube (src/Problems.cpp:37-42 states)
# ----------------------------------------------------------------------------
def _sod_scheme(n: int, gamma: float = 1.4) -> Scheme:
    return Scheme(law="hydro", recon="plm", riemann="hlle", bc="outflow", rk_order=2,
                  shape=(n, 1, 1), gamma=gamma, plm_theta=1.5, cfl=0.4, t_final=0.2)


def sod(n: int = 1024, gamma: float = 1.4):
    s = _sod_scheme(n, gamma)
    P = empty_state(s)
    x, _, _ = cell_centres(s)
    left = x < 0.5
    P[..., 0] = np.where(left, 1.0, 0.125)
    P[..., 4] = np.where(left, 1.0, 0.1)
    return s, apply_bc_numpy(s, P)


# ----------------------------------------------------------------------------
# workload 2: Kelvin-Helmholtz, periodic [0,1]^2
# ----------------------------------------------------------------------------
KH_SEED = 20261203


def _kh_scheme(n: int, riemann: str = "hllc") -> Scheme:
    return Scheme(law="hydro", recon="plm", riemann=riemann, bc="periodic", rk_order=2,
                  shape=(n, n, 1), gamma=5.0 / 3, plm_theta=1.5, cfl=0.4, t_final=1.0)


def kelvin_helmholtz(n: int = 1024, seed: int = KH_SEED, riemann: str = "hllc"):
    s = _kh_scheme(n, riemann)
    P = empty_state(s)
    g = s.ng[0]
    _, y, _ = cell_centres(s)
    band = np.abs(y - 0.5) < 0.25
    P[..., 0] = np.where(band, 2.0, 1.0)
    P[..., 1] = np.where(band, 0.5, -0.5)
    P[..., 4] = 2.5
    vy = uniform(seed, n * n, -1.0, 1.0).reshape(n, n) * 0.01
    P[g:g + n, g:g + n, 0, 2] = vy
    return s, apply_bc_numpy(s, P)


# ----------------------------------------------------------------------------
# workload 3: 3-D Newtonian MHD turbulence with a vector-potential B field
# ----------------------------------------------------------------------------
MHD_SEED = 314159


def _fourier_modes(seed: int, kmax: int = 4):
    ks = [(a, b, c) for a in range(-kmax, kmax + 1) for b in range(-kmax, kmax + 1)
          for c in range(-kmax, kmax + 1) if 0 < a * a + b * b + c * c <= kmax * kmax]
    r = uniform(seed, 4 * len(ks)).reshape(len(ks), 4)
    return np.array(ks, dtype=np.float64), r


def _fourier_vector(seed, X, Y, Z, kmax=4):
    """Sum over modes 0 < |k| <= kmax of a random-amplitude, random-phase
    vector wave, amp_k cos(2 pi (k.x + phi_k)), on the tensor-product grid
    X, Y, Z (meshgrid, 'ij'); returns (3, *X.shape).  Evaluated as a
    separable inverse DFT: cos(2 pi (k.x + phi)) = Re e^{2 pi i phi}
    e^{2 pi i kx x} e^{2 pi i ky y} e^{2 pi i kz z}, contracted one axis at a
    time over the 2 kmax + 1 wavenumbers per axis."""
    ks, r = _fourier_modes(seed, kmax)
    K = 2 * kmax + 1
    C = np.zeros((3, K, K, K), dtype=np.complex128)
    for m, k in enumerate(ks):
        amp = (r[m, :3] - 0.5) / max(1.0, float(np.dot(k, k)))
        a, b, c = (int(v) + kmax for v in k)
        C[:, a, b, c] += amp * np.exp(2j * math.pi * r[m, 3])
    wav = np.arange(-kmax, kmax + 1, dtype=np.float64)
    x, y, z = X[:, 0, 0], Y[0, :, 0], Z[0, 0, :]
    ex = np.exp(2j * math.pi * np.outer(wav, x))
    ey = np.exp(2j * math.pi * np.outer(wav, y))
    ez = np.exp(2j * math.pi * np.outer(wav, z))
    T = np.einsum("cabd,dk->cabk", C, ez)
    T = np.einsum("cabk,bj->cajk", T, ey)
    out = np.empty((3,) + X.shape)
    for comp in range(3):
        out[comp] = np.tensordot(ex, T[comp], axes=([0], [0])).real
    return out


def vector_potential_to_cell_b(s: Scheme, A: np.ndarray) -> np.ndarray:
    """B = divergence(CT(fluxes of A)) on every cell including guards, as in
    src/Problems.cpp:660-667 with CellCenteredFieldCT::vectorPotentialToFluxes
    (src/CellCenteredFieldCT.cpp:136-150), the flux CT stencil (:14-134) and
    MeshOperator::divergence with factor 1 (src/MeshOperator.cpp:323-381).
    A has shape (N0+1, N1+1, N2+1, 3, 3): component, face axis."""
    F = np.zeros_like(A)
    F[..., 1, 0] = -A[..., 2, 0]
    F[..., 2, 0] = +A[..., 1, 0]
    F[..., 2, 1] = -A[..., 0, 1]
    F[..., 0, 1] = +A[..., 2, 1]
    F[..., 0, 2] = -A[..., 1, 2]
    F[..., 1, 2] = +A[..., 0, 2]
    G = ct_correct_numpy(F, 0)
    dx = [(s.upper[a] - s.lower[a]) / s.shape[a] for a in range(3)]
    dA = [dx[1] * dx[2], dx[2] * dx[0], dx[0] * dx[1]]
    dV = dx[0] * dx[1] * dx[2]
    n0, n1, n2 = A.shape[0] - 1, A.shape[1] - 1, A.shape[2] - 1
    B = (1.0 / dV) * (
        + G[1:, :n1, :n2, :, 0] * dA[0] - G[:n0, :n1, :n2, :, 0] * dA[0]
        + G[:n0, 1:, :n2, :, 1] * dA[1] - G[:n0, :n1, :n2, :, 1] * dA[1]
        + G[:n0, :n1, 1:, :, 2] * dA[2] - G[:n0, :n1, :n2, :, 2] * dA[2])
    return B


def ct_correct_numpy(F: np.ndarray, ib: int) -> np.ndarray:
    """CellCenteredFieldCT::correctGodunovFluxes (src/CellCenteredFieldCT.cpp:
    14-134), Toth (2000) eq. 25, vectorised."""
    G = F.copy()
    n0, n1, n2 = F.shape[:3]
    B0, B1, B2 = ib, ib + 1, ib + 2
    G[..., B0, 0] = 0.0
    G[..., B1, 1] = 0.0
    G[..., B2, 2] = 0.0
    f = F
    if n0 >= 3:
        if n1 >= 3:
            G[1:, 1:-1, :, B1, 0] = 0.125 * (
                + 2 * f[1:, 1:-1, :, B1, 0] + f[1:, 2:, :, B1, 0] + f[1:, :-2, :, B1, 0]
                - f[1:, 2:, :, B0, 1] - f[:-1, 2:, :, B0, 1] - f[1:, 1:-1, :, B0, 1] - f[:-1, 1:-1, :, B0, 1])
        if n2 >= 3:
            G[1:, :, 1:-1, B2, 0] = 0.125 * (
                + 2 * f[1:, :, 1:-1, B2, 0] + f[1:, :, 2:, B2, 0] + f[1:, :, :-2, B2, 0]
                - f[1:, :, 2:, B0, 2] - f[:-1, :, 2:, B0, 2] - f[1:, :, 1:-1, B0, 2] - f[:-1, :, 1:-1, B0, 2])
    if n1 >= 3:
        if n2 >= 3:
            G[:, 1:, 1:-1, B2, 1] = 0.125 * (
                + 2 * f[:, 1:, 1:-1, B2, 1] + f[:, 1:, 2:, B2, 1] + f[:, 1:, :-2, B2, 1]
                - f[:, 1:, 2:, B1, 2] - f[:, :-1, 2:, B1, 2] - f[:, 1:, 1:-1, B1, 2] - f[:, :-1, 1:-1, B1, 2])
        if n0 >= 3:
            G[1:-1, 1:, :, B0, 1] = 0.125 * (
                + 2 * f[1:-1, 1:, :, B0, 1] + f[2:, 1:, :, B0, 1] + f[:-2, 1:, :, B0, 1]
                - f[2:, 1:, :, B1, 0] - f[2:, :-1, :, B1, 0] - f[1:-1, 1:, :, B1, 0] - f[1:-1, :-1, :, B1, 0])
    if n2 >= 3:
        if n0 >= 3:
            G[1:-1, :, 1:, B0, 2] = 0.125 * (
                + 2 * f[1:-1, :, 1:, B0, 2] + f[2:, :, 1:, B0, 2] + f[:-2, :, 1:, B0, 2]
                - f[2:, :, 1:, B2, 0] - f[2:, :, :-1, B2, 0] - f[1:-1, :, 1:, B2, 0] - f[1:-1, :, :-1, B2, 0])
        if n1 >= 3:
            G[:, 1:-1, 1:, B1, 2] = 0.125 * (
                + 2 * f[:, 1:-1, 1:, B1, 2] + f[:, 2:, 1:, B1, 2] + f[:, :-2, 1:, B1, 2]
                - f[:, 2:, 1:, B2, 1] - f[:, 2:, :-1, B2, 1] - f[:, 1:-1, 1:, B2, 1] - f[:, 1:-1, :-1, B2, 1])
    return G


def face_vector_potential(s: Scheme, fn) -> np.ndarray:
    """MeshOperator::generate(face, scalars, boundaryShape) (src/MeshOperator.
    cpp:119-167): fn(x, y, z) -> (3, ...) evaluated at the three face centres of
    every index of the guard-extended mesh plus one."""
    N = [s.shape[a] + 2 * s.ng[a] for a in range(3)]
    dx = [(s.upper[a] - s.lower[a]) / s.shape[a] for a in range(3)]
    idx = [np.arange(N[a] + 1, dtype=np.float64) - s.ng[a] for a in range(3)]
    A = np.zeros((N[0] + 1, N[1] + 1, N[2] + 1, 3, 3))
    for face in range(3):
        c = []
        for a in range(3):
            off = -0.5 if a == face else 0.0
            c.append(s.lower[a] + dx[a] * (idx[a] + off + 0.5))
        X, Y, Z = np.meshgrid(*c, indexing="ij")
        A[..., :, face] = np.moveaxis(fn(X, Y, Z), 0, -1)
    return A


def mhd_turbulence_parts(n: int = 256, seed: int = MHD_SEED, v_rms: float = 0.1, b_rms: float = 0.5,
                         rk_order: int = 3):
    """The MHD turbulence workload before its magnetic field is built: the
    scheme, the state with B = 0, the face-centred vector potential A and the
    factor that brings the rms of B over the interior to b_rms.  B follows
    as scale x div(CT(fluxes of A)) (src/Problems.cpp:660-667), on the host
    (mhd_turbulence) or on the device (Solver.assign_vector_potential)."""
    s = Scheme(law="mhd", recon="plm", riemann="hlle", bc="periodic", rk_order=rk_order,
               shape=(n, n, n), gamma=5.0 / 3, plm_theta=1.5, cfl=0.3, t_final=None, steps=100)
    P = empty_state(s)
    X, Y, Z = cell_centres(s)
    v = _fourier_vector(seed, X, Y, Z)
    g = s.ng[0]
    inner = v[:, g:-g, g:-g, g:-g]
    v *= v_rms / math.sqrt(float(np.mean(np.sum(inner ** 2, axis=0))))
    P[..., 0] = 1.0
    P[..., 4] = 1.0
    P[..., 1:4] = np.moveaxis(v, 0, -1)
    A = face_vector_potential(s, lambda x, y, z: _fourier_vector(seed + 1, x, y, z))
    B = vector_potential_to_cell_b(s, A)
    inner_b = B[g:-g, g:-g, g:-g]
    scale = b_rms / math.sqrt(float(np.mean(np.sum(inner_b ** 2, axis=-1))))
    return s, apply_bc_numpy(s, P), A, scale, B


def mhd_turbulence(n: int = 256, seed: int = MHD_SEED, v_rms: float = 0.1, b_rms: float = 0.5,
                   rk_order: int = 3):
    s, P, A, scale, B = mhd_turbulence_parts(n, seed, v_rms, b_rms, rk_order)
    P[..., 5:8] = B * scale
    return s, apply_bc_numpy(s, P)


# ----------------------------------------------------------------------------
# workload 4: relativistic MHD cylindrical blast wave on [-6, 6]^2
# ----------------------------------------------------------------------------
def with_cooling(s: Scheme, P: np.ndarray, rate: float, aux: float = 0.0):
    """NewtonianMHD with cooling (setCoolingRate, ConservationLaws.cpp:355-358):
    the scheme with the rate and the state with the auxiliary field (index 8)
    set to aux."""
    if s.law != "mhd" or not rate > 0.0:
        raise ValueError("cooling needs the MHD law and a positive rate")
    s2 = s.with_(cooling_rate=rate)
    P2 = np.concatenate([P[..., :8], np.full(P.shape[:3] + (1,), float(aux))], axis=-1)
    return s2, P2


def _rmhd_blast_scheme(n: int, pressure_floor: float = -1.0) -> Scheme:
    return Scheme(law="rmhd", recon="weno5", riemann="hlle", bc="outflow", rk_order=3,
                  shape=(n, n, 1), lower=(-6.0, -6.0, 0.0), upper=(6.0, 6.0, 1.0), gamma=4.0 / 3,
                  cfl=0.3, t_final=4.0, pressure_floor=pressure_floor)


def rmhd_blast(n: int = 512, pressure_floor: float = -1.0):
    s = _rmhd_blast_scheme(n, pressure_floor)
    P = empty_state(s)
    x, y, _ = cell_centres(s)
    r = np.sqrt(x * x + y * y)
    P[..., 0] = 0.01
    P[..., 4] = np.where(r < 0.8, 1.0, 0.01)
    P[..., 5] = 0.1
    return s, apply_bc_numpy(s, P)


# ----------------------------------------------------------------------------
# workload 5: stream of Riemann problems of uneven sizes
# ----------------------------------------------------------------------------
RIEMANN_SEED = 27182818


@dataclass
class RiemannRequest:
    index: int
    arrival: float
    dims: int
    n: int
    theta: float
    left: tuple
    right: tuple
    scheme: Scheme = field(repr=False, default=None)

    def zones(self) -> int:
        return self.n ** self.dims


def riemann_stream(count: int = 4096, rate: float = 2000.0, seed: int = RIEMANN_SEED,
                   n1=(256, 8192), n2=(128, 512)):
    """Seeded Poisson arrivals (rate per second) of 1-D / 2-D Riemann problems.
    Half are 1-D with N log-uniform in n1, half 2-D with side log-uniform in n2;
    rho log-uniform in [0.1, 10], p in [0.01, 100], velocities uniform in
    [-1, 1]; the 2-D interface passes through the centre at a random angle."""
    r = uniform(seed, count * 16).reshape(count, 16)
    out, t = [], 0.0
    for m in range(count):
        t += -math.log(1.0 - r[m, 0]) / rate
        dims = 1 if r[m, 1] < 0.5 else 2
        lo, hi = (n1 if dims == 1 else n2)
        nn = int(round(math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * r[m, 2])))
        def logu(u, a, b):
            return math.exp(math.log(a) + (math.log(b) - math.log(a)) * u)
        left = (logu(r[m, 3], 0.1, 10), 2 * r[m, 4] - 1, (2 * r[m, 5] - 1) if dims == 2 else 0.0, 0.0,
                logu(r[m, 6], 0.01, 100))
        right = (logu(r[m, 7], 0.1, 10), 2 * r[m, 8] - 1, (2 * r[m, 9] - 1) if dims == 2 else 0.0, 0.0,
                 logu(r[m, 10], 0.01, 100))
        theta = 2 * math.pi * r[m, 11]
        out.append(RiemannRequest(m, t, dims, nn, theta, left, right))
    return out


def _riemann_scheme(req: RiemannRequest, gamma: float = 5.0 / 3) -> Scheme:
    shape = (req.n, 1, 1) if req.dims == 1 else (req.n, req.n, 1)
    return Scheme(law="hydro", recon="plm", riemann="hllc", bc="outflow", rk_order=2, shape=shape,
                  gamma=gamma, plm_theta=1.5, cfl=0.4, t_final=0.2)


def riemann_initial(req: RiemannRequest, gamma: float = 5.0 / 3):
    s = _riemann_scheme(req, gamma)
    P = empty_state(s)
    x, y, _ = cell_centres(s)
    if req.dims == 1:
        side = (x - 0.5) < 0
    else:
        side = (x - 0.5) * math.cos(req.theta) + (y - 0.5) * math.sin(req.theta) < 0
    for q in range(5):
        P[..., q] = np.where(side, req.left[q], req.right[q])
    return s, apply_bc_numpy(s, P)


# ----------------------------------------------------------------------------
# the same initial data as built-in functions generated on the device
# (mara_gpu_generate): Scheme plus the MaraInitialData fields
# ----------------------------------------------------------------------------
def device_initial_data(name: str, n: int = None, req: RiemannRequest = None):
    """(Scheme, spec) whose device generation equals the host generator's
    array bit for bit: "sod", "kh", "rmhd_blast" or "riemann" (req)."""
    from ._native import MARA_INIT_CYLINDER, MARA_INIT_PLANAR_RIEMANN, MARA_INIT_SHEAR_LAYER
    if name == "sod":
        s = _sod_scheme(n)
        return s, {"kind": MARA_INIT_PLANAR_RIEMANN, "left": (1.0, 0.0, 0.0, 0.0, 1.0),
                   "right": (0.125, 0.0, 0.0, 0.0, 0.1), "x0": (0.5, 0.5, 0.5), "normal": (1.0, 0.0, 0.0)}
    if name == "kh":
        s = _kh_scheme(n)
        return s, {"kind": MARA_INIT_SHEAR_LAYER, "left": (2.0, 0.5, 0.0, 0.0, 2.5), "right": (1.0, -0.5, 0.0, 0.0, 2.5),
                   "x0": (0.5, 0.5, 0.5), "radius": 0.25, "noise": 0.01, "seed": KH_SEED}
    if name == "rmhd_blast":
        s = _rmhd_blast_scheme(n)
        return s, {"kind": MARA_INIT_CYLINDER, "left": (0.01, 0.0, 0.0, 0.0, 1.0, 0.1, 0.0, 0.0),
                   "right": (0.01, 0.0, 0.0, 0.0, 0.01, 0.1, 0.0, 0.0), "x0": (0.0, 0.0, 0.0), "radius": 0.8}
    if name == "riemann":
        s = _riemann_scheme(req)
        nrm = (1.0, 0.0, 0.0) if req.dims == 1 else (math.cos(req.theta), math.sin(req.theta), 0.0)
        return s, {"kind": MARA_INIT_PLANAR_RIEMANN, "left": req.left, "right": req.right, "x0": (0.5, 0.5, 0.5),
                   "normal": nrm}
    raise ValueError(name)


# ----------------------------------------------------------------------------
# conserved densities of a primitive array (for error reports)
# ----------------------------------------------------------------------------
CONSERVED_NAMES = {
    "hydro": ["density", "momentum1", "momentum2", "momentum3", "energy"],
    "mhd": ["density", "momentum1", "momentum2", "momentum3", "energy", "magnetic1", "magnetic2", "magnetic3"],
    "rmhd": ["density", "momentum1", "momentum2", "momentum3", "energy", "magnetic1", "magnetic2", "magnetic3"],
}


def conserved(s: Scheme, P: np.ndarray) -> np.ndarray:
    """U of every zone of P (..., nq) by the law's fromPrimitive
    (NewtonianHydro ConservationLaws.cpp:253-290, NewtonianMHD :416-447,
    RelativisticMHD :659-720), in numpy FP64."""
    P = np.asarray(P, dtype=np.float64)
    U = np.empty_like(P)
    rho, v, p = P[..., 0], P[..., 1:4], P[..., 4]
    gm1 = s.gamma - 1.0
    vv = np.sum(v * v, axis=-1)
    if s.law == "hydro":
        U[..., 0] = rho
        U[..., 1:4] = rho[..., None] * v
        U[..., 4] = rho * 0.5 * vv + p / gm1
    elif s.law == "mhd":
        B = P[..., 5:8]
        U[..., 0] = rho
        U[..., 1:4] = rho[..., None] * v
        U[..., 4] = rho * 0.5 * vv + 0.5 * np.sum(B * B, axis=-1) + p / gm1
        U[..., 5:] = P[..., 5:]
    else:
        B = P[..., 5:8]
        BB = np.sum(B * B, axis=-1)
        Bv = np.sum(B * v, axis=-1)
        W2 = 1.0 / (1.0 - vv)
        W0 = np.sqrt(W2)
        b0 = W0 * Bv
        bb = (BB + b0 * b0) / W2
        b = (B + (b0 * W0)[..., None] * v) / W0[..., None]
        e0 = (p / rho) / gm1
        es = e0 + 0.5 * bb / rho
        ps = p + 0.5 * bb
        hs = 1.0 + es + ps / rho
        U[..., 0] = rho * W0
        U[..., 4] = rho * hs * W2 - ps - b0 * b0 - U[..., 0]
        U[..., 1:4] = (rho * hs * W2)[..., None] * v - b0[..., None] * b
        U[..., 5:8] = B
    return U
