"""Checkpoint and restart of a resident state (CheckpointWriter,
src/Checkpoint.cpp:96-277), and the time series the drivers append to
(TimeSeriesManager, src/TimeSeriesManager.cpp:43-91).

The reference writes HDF5 groups status, scheduler, time_series, user,
primitive, diagnostic, mesh and particles.  HDF5 is not available here, so a
checkpoint is one file with the same groups and dataset names:

    8 bytes   b"MARACHK1"
    8 bytes   header length H (little-endian unsigned)
    H bytes   JSON header (UTF-8)
    padding   to a multiple of 64 bytes
    data      every dataset as little-endian float64, C order, at the
              offset (from the start of the data section) its header entry
              gives: {"dtype": "<f8", "shape": [...], "offset": N}

Header groups:
  run_name     "Mara"
  status       SimulationStatus::pack: simulationIter, simulationTime
  user         the run's user parameters (JSON values)
  mesh         type "cartesian", points {x, y, z}: the cell-face coordinates
               CartesianMeshGeometry::getPointCoordinates gives
  primitive    one dataset per ConservationLaw::getPrimitiveName, interior
               zones only (MeshData::getPrimitive(q))
  diagnostic   one dataset per diagnostic field (e.g. monopole, current1-3),
               interior zones only
  time_series  one dataset per double column, one JSON list per int column
  scheduler    the task scheduler's state (JSON values)
  particles    {data: dataset}
  scheme       the solution scheme's configuration, so that a restart can
               rebuild it (not in the reference's file)
"""
from __future__ import annotations

import json
import struct
from dataclasses import dataclass, field

import numpy as np

from .scheme import Scheme
from .workloads import apply_bc_numpy

MAGIC = b"MARACHK1"
ALIGN = 64


def primitive_names(law: str, aux: int = 0) -> list:
    """ConservationLaw::getPrimitiveName (src/ConservationLaws.cpp:310-318,
    522-533, 861-872); NewtonianMHD's auxiliary fields are auxiliary1..."""
    base = ["density", "velocity1", "velocity2", "velocity3", "pressure"]
    if law == "hydro":
        return base
    return base + ["magnetic1", "magnetic2", "magnetic3"] + [f"auxiliary{n + 1}" for n in range(aux)]


def point_coordinates(s: Scheme, axis: int) -> np.ndarray:
    """CartesianMeshGeometry::getPointCoordinates (src/CartesianMeshGeometry.
    cpp:121-131): lower + dx (n - 0.5 + 0.5) for n = 0..shape."""
    n = s.shape[axis]
    dx = (s.upper[axis] - s.lower[axis]) / n
    return np.array([s.lower[axis] + dx * ((k - 0.5) + 0.5) for k in range(n + 1)])


class TimeSeries:
    """TimeSeriesManager: columns of doubles and ints, each appended once per
    entry; append(status, columns) adds the iteration and time first."""

    def __init__(self):
        self.doubles: dict = {}
        self.ints: dict = {}

    def append_value(self, name: str, value) -> None:
        if isinstance(value, (bool, np.bool_)):
            raise TypeError("[TimeSeriesManager] only accepts entries of type int and double")
        if isinstance(value, (int, np.integer)):
            self.ints.setdefault(name, []).append(int(value))
        elif isinstance(value, (float, np.floating)):
            self.doubles.setdefault(name, []).append(float(value))
        else:
            raise TypeError("[TimeSeriesManager] only accepts entries of type int and double")

    def append(self, status: dict, columns: dict) -> None:
        self.append_value("iteration", int(status["simulationIter"]))
        self.append_value("time", float(status["simulationTime"]))
        for k, v in columns.items():
            self.append_value(k, v)

    def series_double(self, name: str) -> list:
        return self.doubles[name]

    def series_int(self, name: str) -> list:
        return self.ints[name]

    def clear(self) -> None:
        self.doubles.clear()
        self.ints.clear()


@dataclass
class Checkpoint:
    scheme: Scheme
    P: np.ndarray                       # primitives with guards filled by the boundary condition
    status: dict
    user: dict = field(default_factory=dict)
    time_series: TimeSeries = field(default_factory=TimeSeries)
    scheduler: dict = field(default_factory=dict)
    diagnostic: dict = field(default_factory=dict)   # name -> interior array
    particles: np.ndarray = field(default_factory=lambda: np.zeros(0))


def _scheme_dict(s: Scheme) -> dict:
    keys = ("law", "recon", "riemann", "bc", "rk_order", "disable_ct", "weno_is", "shape", "lower", "upper",
            "gamma", "plm_theta", "shenzha_A", "pressure_floor", "cooling_rate", "guard", "cfl", "t_final", "steps")
    out = {}
    for k in keys:
        v = getattr(s, k)
        out[k] = list(v) if isinstance(v, tuple) else v
    return out


def _scheme_from(d: dict) -> Scheme:
    kw = dict(d)
    for k in ("shape", "lower", "upper"):
        if k in kw and kw[k] is not None:
            kw[k] = tuple(kw[k])
    return Scheme(**kw)


def write_checkpoint(filename: str, s: Scheme, P: np.ndarray, status: dict, user: dict | None = None,
                     time_series: TimeSeries | None = None, scheduler: dict | None = None,
                     diagnostic: dict | None = None, particles: np.ndarray | None = None) -> None:
    """CheckpointWriter::writeCheckpoint for one process (format single).
    P is MeshData::P with guards (a Solver's download()); diagnostic maps a
    field name to an interior or with-guards array of one component."""
    blobs: list = []
    offset = [0]

    def ds(a) -> dict:
        a = np.ascontiguousarray(a, dtype="<f8")
        entry = {"dtype": "<f8", "shape": list(a.shape), "offset": offset[0]}
        blobs.append(a.tobytes())
        offset[0] += a.nbytes
        return entry

    interior = s.interior()
    full = tuple(s.full_shape[:3])
    names = primitive_names(s.law, s.aux)
    if P.shape[-1] != len(names):
        raise ValueError("primitive array does not match the conservation law")
    header = {
        "format": "mara2-gb300-checkpoint", "version": 1,
        "run_name": "Mara",
        "status": {"simulationIter": int(status["simulationIter"]),
                   "simulationTime": float(status["simulationTime"])},
        "user": dict(user or {}),
        "mesh": {"type": "cartesian",
                 "points": {ax: ds(point_coordinates(s, a)) for a, ax in enumerate("xyz")}},
        "primitive": {n: ds(P[interior][..., q]) for q, n in enumerate(names)},
        "diagnostic": {},
        "time_series": {},
        "scheduler": dict(scheduler or {}),
        "particles": {"data": ds(np.zeros(0) if particles is None else particles)},
        "scheme": _scheme_dict(s),
    }
    for name, a in (diagnostic or {}).items():
        a = np.asarray(a, dtype=float)
        if a.shape[:3] == full:
            a = a[interior[:3]]
        header["diagnostic"][name] = ds(a)
    ts = time_series or TimeSeries()
    for name, col in ts.doubles.items():
        header["time_series"][name] = ds(np.array(col, dtype=float))
    for name, col in ts.ints.items():
        header["time_series"][name] = {"int": list(col)}

    h = json.dumps(header, sort_keys=True).encode("utf-8")
    pre = len(MAGIC) + 8 + len(h)
    pad = (-pre) % ALIGN
    with open(filename, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<Q", len(h)))
        f.write(h)
        f.write(b"\0" * pad)
        for b in blobs:
            f.write(b)


def read_header(filename: str) -> tuple:
    with open(filename, "rb") as f:
        if f.read(len(MAGIC)) != MAGIC:
            raise ValueError(f"{filename}: not a checkpoint")
        (hl,) = struct.unpack("<Q", f.read(8))
        header = json.loads(f.read(hl).decode("utf-8"))
    pre = len(MAGIC) + 8 + hl
    return header, pre + (-pre) % ALIGN


def read_checkpoint(filename: str, s: Scheme | None = None) -> Checkpoint:
    """CheckpointWriter::readCheckpoint: the primitives go into the interior
    (MeshData::assignPrimitive) and the guards are filled by the boundary
    condition, as the drivers do before the first step."""
    header, base = read_header(filename)
    data = np.memmap(filename, dtype=np.uint8, mode="r")

    def load(entry) -> np.ndarray:
        n = int(np.prod(entry["shape"])) if entry["shape"] else 0
        start = base + entry["offset"]
        return np.frombuffer(data[start:start + 8 * n].tobytes(), dtype="<f8").reshape(entry["shape"]).copy()

    s = s or _scheme_from(header["scheme"])
    names = primitive_names(s.law, s.aux)
    P = np.zeros(s.full_shape)
    interior = s.interior()
    for q, n in enumerate(names):
        a = load(header["primitive"][n])
        if tuple(a.shape) != tuple(s.shape):
            raise ValueError(f"{filename}: {n} has shape {a.shape}, the scheme has {s.shape}")
        P[interior + (q,)] = a
    P = apply_bc_numpy(s, P)
    ts = TimeSeries()
    for name, e in header["time_series"].items():
        if "int" in e:
            ts.ints[name] = list(e["int"])
        else:
            ts.doubles[name] = load(e).tolist()
    return Checkpoint(scheme=s, P=P, status=dict(header["status"]), user=dict(header["user"]), time_series=ts,
                      scheduler=dict(header["scheduler"]),
                      diagnostic={k: load(v) for k, v in header["diagnostic"].items()},
                      particles=load(header["particles"]["data"]))


def checkpoint_solver(filename: str, solver, status: dict, user: dict | None = None,
                      time_series: TimeSeries | None = None, scheduler: dict | None = None,
                      mesh_spacing: float | None = None) -> None:
    """The drivers' checkpoint task (e.g. src/Problems/MagneticBraiding.cpp:
    176-189) for a resident state: the primitives and, for magnetised laws,
    the cell monopole and current computed on the device."""
    s = solver.scheme
    P = solver.download()
    diag = {}
    if s.law != "hydro":
        h = mesh_spacing if mesh_spacing is not None else (s.upper[0] - s.lower[0]) / s.shape[0]
        F = solver.field_diagnostics(h)
        for c, n in enumerate(("monopole", "current1", "current2", "current3")):
            diag[n] = F[..., c]
    write_checkpoint(filename, s, P, status, user, time_series, scheduler, diag)
