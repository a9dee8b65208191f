"""Checkpoint / restart (CheckpointWriter, src/Checkpoint.cpp:96-277) and the
time series (TimeSeriesManager): the file keeps the reference's groups and
dataset names, a restart reproduces the state bit for bit, and a run
continued from a checkpoint equals the uninterrupted run."""
import numpy as np
import pytest

from helpers import oracle_config
from mara2_gb300 import workloads as W
from mara2_gb300.checkpoint import (TimeSeries, checkpoint_solver, point_coordinates, primitive_names,
                                    read_checkpoint, read_header, write_checkpoint)

MAKERS = [("sod", lambda: W.sod(64)), ("kh", lambda: W.kelvin_helmholtz(24)),
          ("mhd", lambda: W.mhd_turbulence(8)), ("rmhd", lambda: W.rmhd_blast(16))]


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


@pytest.mark.parametrize("name,make", MAKERS)
def test_round_trip_bitwise(tmp_path, name, make):
    s, P = make()
    P = W.apply_bc_numpy(s, P)
    ts = TimeSeries()
    ts.append({"simulationIter": 3, "simulationTime": 0.125}, {"mass": 1.5, "zones": s.zones})
    f = str(tmp_path / "chkpt.0003.mara")
    write_checkpoint(f, s, P, {"simulationIter": 3, "simulationTime": 0.125}, user={"N": 64, "cfl": 0.4},
                     time_series=ts, scheduler={"checkpoint": {"last": 0.1}},
                     diagnostic={"monopole": np.arange(s.zones, dtype=float).reshape(s.shape)})
    c = read_checkpoint(f)
    assert c.scheme == s
    assert np.array_equal(_bits(c.P), _bits(P))
    assert c.status == {"simulationIter": 3, "simulationTime": 0.125}
    assert c.user == {"N": 64, "cfl": 0.4} and c.scheduler == {"checkpoint": {"last": 0.1}}
    assert c.time_series.series_int("iteration") == [3] and c.time_series.series_double("time") == [0.125]
    assert c.time_series.series_double("mass") == [1.5] and c.time_series.series_int("zones") == [s.zones]
    assert np.array_equal(c.diagnostic["monopole"], np.arange(s.zones, dtype=float).reshape(s.shape))


def test_header_groups_and_mesh_points(tmp_path):
    s, P = W.mhd_turbulence(8)
    f = str(tmp_path / "c.mara")
    write_checkpoint(f, s, P, {"simulationIter": 0, "simulationTime": 0.0})
    h, base = read_header(f)
    assert base % 64 == 0
    for g in ("status", "scheduler", "time_series", "user", "primitive", "diagnostic", "mesh", "particles"):
        assert g in h
    assert h["run_name"] == "Mara" and h["mesh"]["type"] == "cartesian"
    assert sorted(h["primitive"]) == sorted(primitive_names("mhd"))
    x = point_coordinates(s, 0)
    assert len(x) == s.shape[0] + 1 and x[0] == s.lower[0] and abs(x[-1] - s.upper[0]) < 1e-15
    c = read_checkpoint(f)
    assert c.particles.size == 0


def test_time_series_rejects_other_types():
    ts = TimeSeries()
    with pytest.raises(TypeError):
        ts.append_value("flag", True)
    with pytest.raises(TypeError):
        ts.append_value("name", "x")


def test_restart_continues_identically_oracle(tmp_path, port):
    """Three steps, checkpoint, restart, three more == six steps (the oracle
    restatement of the reference's advance)."""
    s, P = W.kelvin_helmholtz(24)
    P = W.apply_bc_numpy(s, P)
    c = oracle_config(s)
    A = P.copy()
    _, t, _ = port.run(c, A, 6, s.cfl)
    B = P.copy()
    _, t1, dts = port.run(c, B, 3, s.cfl)
    f = str(tmp_path / "r.mara")
    write_checkpoint(f, s, B, {"simulationIter": 3, "simulationTime": t1})
    r = read_checkpoint(f)
    _, t2, _ = port.run(c, r.P, 3, s.cfl)
    assert np.array_equal(_bits(r.P), _bits(A))
    assert r.status["simulationTime"] + t2 == pytest.approx(t, rel=1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("name,make", [("kh", lambda: W.kelvin_helmholtz(64)), ("mhd", lambda: W.mhd_turbulence(12))])
def test_restart_resident_state_plain(tmp_path, gpu_lib, name, make):
    """A resident plain-FP64 run checkpointed from the device and restarted
    into a fresh handle continues bit for bit."""
    from mara2_gb300.solver import Solver
    s, P = make()
    P = W.apply_bc_numpy(s, P)
    f = str(tmp_path / "g.mara")
    with Solver(s, "fp64") as g:
        g.upload(P.copy())
        g.run(3)
        checkpoint_solver(f, g, {"simulationIter": 3, "simulationTime": g.t})
        g.run(3)
        A = g.download()
    r = read_checkpoint(f)
    if s.law != "hydro":
        assert set(r.diagnostic) == {"monopole", "current1", "current2", "current3"}
        assert r.diagnostic["monopole"].shape == s.shape
    with Solver(r.scheme, "fp64") as g:
        g.upload(r.P)
        g.run(3)
        B = g.download()
    assert np.array_equal(_bits(A), _bits(B))
