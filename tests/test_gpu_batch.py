"""Batched grids and continuous batching (include/mara_batch.h).

Each grid's arithmetic must not depend on the other grids in the batch or on
where its tiles land: a request solved alone and the same request solved in a
mix give bit-identical results and step counts; a grid solved in the batch
matches the single-grid mixed path bit for bit."""
import dataclasses

import numpy as np
import pytest

from mara2_gb300 import workloads as W


def _small_requests(n=8, seed=99):
    reqs = W.riemann_stream(n, rate=1e6, seed=seed, n1=(64, 512), n2=(32, 96))
    return reqs


def _make(r):
    s, P = W.riemann_initial(r)
    s = s.with_(t_final=0.02)
    return s, P


@pytest.mark.gpu
def test_alone_equals_mix(gpu_lib):
    from mara2_gb300.batch import Batch, run_alone
    reqs = _small_requests()
    built = [_make(r) for r in reqs]
    alone = [run_alone(s, P, s.t_final) for s, P in built]
    cells = max(int(np.prod(s.full_shape[:3])) for s, _ in built)
    with Batch(budget_bytes=1 << 28, max_grids=32, max_zones_per_grid=cells) as b:
        slots = {b.admit(s, P, s.t_final): k for k, (s, P) in enumerate(built)}
        out = {}
        while len(out) < len(built):
            b.step(7)
            for sl in b.poll():
                k = slots[sl]
                out[k] = b.retire(sl, built[k][0].full_shape)
    for k, (s, _) in enumerate(built):
        Pa, ta, na = alone[k]
        Pm, tm, nm = out[k]
        assert na == nm and ta == tm, (k, na, nm)
        assert np.array_equal(Pa[s.interior()].view(np.uint64), Pm[s.interior()].view(np.uint64)), k


def _run_batch(built, **kw):
    from mara2_gb300.batch import Batch
    cells = max(int(np.prod(s.full_shape[:3])) for s, _ in built)
    out = {}
    with Batch(budget_bytes=1 << 29, max_grids=64, max_zones_per_grid=cells, **kw) as b:
        slots = {b.admit(s, P, s.t_final): k for k, (s, P) in enumerate(built)}
        while len(out) < len(built):
            b.step(5)
            for sl in b.poll():
                k = slots[sl]
                out[k] = b.retire(sl, built[k][0].full_shape)
    return out


@pytest.mark.gpu
def test_cluster_slots_match_lockstep(gpu_lib):
    """1-D grids of every cluster class (1 to 8 CTAs, up to 1024 zones per
    CTA) run on their own clusters beside 2-D grids in the tile lists, against
    all grids stepping in lockstep: the same clock, step count and bits."""
    reqs = W.riemann_stream(40, rate=1e6, seed=5, n1=(64, 512), n2=(32, 64))
    one = [r for r in reqs if r.dims == 1][:6]
    two = [r for r in reqs if r.dims == 2][:4]
    sizes = [100, 300, 700, 1500, 3000, 8192]
    built = []
    for r, n in zip(one, sizes):
        s, P = W.riemann_initial(dataclasses.replace(r, n=n))
        built.append((s.with_(t_final=0.004), P))
    built += [_make(r) for r in two]
    a = _run_batch(built)
    b = _run_batch(built, lockstep_1d=True)
    for k, (s, _) in enumerate(built):
        Pa, ta, na = a[k]
        Pb, tb, nb = b[k]
        assert na == nb and ta == tb, (k, na, nb, ta, tb)
        assert np.array_equal(Pa[s.interior()].view(np.uint64), Pb[s.interior()].view(np.uint64)), k


@pytest.mark.gpu
@pytest.mark.parametrize("rk,recon,riemann", [(1, "pcm", "hlle"), (3, "plm", "hlle")])
def test_cluster_slots_match_lockstep_other_schemes(gpu_lib, rk, recon, riemann):
    """The same comparison for RK1 (the lockstep path swaps the state buffer
    every step, the clusters update in place) and RK3, PCM and HLLE."""
    reqs = W.riemann_stream(40, rate=1e6, seed=11, n1=(64, 512), n2=(32, 64))
    one = [r for r in reqs if r.dims == 1][:3]
    two = [r for r in reqs if r.dims == 2][:2]
    built = []
    for r, n in zip(one, [100, 700, 3000]):
        s, P = W.riemann_initial(dataclasses.replace(r, n=n))
        built.append((s.with_(t_final=0.004, rk_order=rk, recon=recon, riemann=riemann, guard=2), P))
    for r in two:
        s, P = _make(r)
        built.append((s.with_(rk_order=rk, recon=recon, riemann=riemann, guard=2), P))
    kw = dict(recon=recon, riemann=riemann, rk_order=rk)
    a = _run_batch(built, **kw)
    b = _run_batch(built, lockstep_1d=True, **kw)
    for k, (s, _) in enumerate(built):
        Pa, ta, na = a[k]
        Pb, tb, nb = b[k]
        assert na == nb and ta == tb, (k, na, nb, ta, tb)
        assert np.array_equal(Pa[s.interior()].view(np.uint64), Pb[s.interior()].view(np.uint64)), k


@pytest.mark.gpu
@pytest.mark.parametrize("n", [300, 5000])
def test_cluster_slot_matches_single_grid_run(gpu_lib, n):
    """A 1-D grid in the batch and the same grid run by a single-grid handle
    (both on a thread-block cluster): the same bits and step count."""
    from mara2_gb300.batch import run_alone
    from mara2_gb300.solver import Solver
    r = next(r for r in W.riemann_stream(8, rate=1e6, seed=3) if r.dims == 1)
    s, P = W.riemann_initial(dataclasses.replace(r, n=n))
    s = s.with_(t_final=0.003)
    Pb, tb, nb = run_alone(s, P, s.t_final)
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        ns = g.run(100_000, s.cfl, s.t_final)
        Ps = g.download()
        ts = g.t
    assert ns == nb and ts == tb
    assert np.array_equal(Pb[s.interior()].view(np.uint64), Ps[s.interior()].view(np.uint64))


@pytest.mark.gpu
def test_batch_matches_single_grid_mixed(gpu_lib):
    from mara2_gb300.batch import run_alone
    from mara2_gb300.solver import Solver
    s, P = W.kelvin_helmholtz(96, riemann="hllc")
    s = s.with_(t_final=0.01)
    Pb, tb, nb = run_alone(s, P, s.t_final)
    with Solver(s, "mixed") as g:
        g.upload(P.copy())
        n = g.run(10_000, s.cfl, s.t_final)
        Ps = g.download()
    assert n == nb
    assert np.array_equal(Pb[s.interior()].view(np.uint64), Ps[s.interior()].view(np.uint64))


@pytest.mark.gpu
def test_admission_respects_budget(gpu_lib):
    from mara2_gb300.batch import Batch
    s, P = W.kelvin_helmholtz(64)
    per_grid = 2 * 2 * 5 * s.zones * 4
    with Batch(budget_bytes=int(1.5 * per_grid), max_grids=8, max_zones_per_grid=70 * 70) as b:
        assert b.admit(s, P, 0.01) is not None
        assert b.admit(s, P, 0.01) is None          # over budget
        assert b.stats().bytes_in_use == per_grid


@pytest.mark.gpu
def test_serving_loop_completes_and_matches_alone(gpu_lib):
    from mara2_gb300.batch import run_alone, serve
    reqs = W.riemann_stream(24, rate=400.0, seed=7, n1=(64, 512), n2=(32, 96))
    res = serve(reqs, budget_bytes=1 << 26, keep_results=True, make=_make)
    assert res.completed == 24
    summ = res.summary()
    assert summ["latency_p99_s"] >= summ["latency_p50_s"] > 0
    for r in reqs[:4]:
        s, P = _make(r)
        Pa, ta, na = run_alone(s, P, s.t_final)
        Pm, tm, nm = res.results[r.index]
        assert na == nm
        assert np.array_equal(Pa[s.interior()].view(np.uint64), Pm[s.interior()].view(np.uint64))


PERSISTENT = [("plm", "hllc", 2, 512, 2), ("plm", "hlle", 3, 256, 1), ("pcm", "hllc", 1, 256, 2),
              ("pcm", "hlle", 2, 512, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("recon,riemann,rk,tile_1d,tile_2d", PERSISTENT)
def test_persistent_launch_matches_per_stage_launches(gpu_lib, recon, riemann, rk, tile_1d, tile_2d):
    """The persistent form (every stage of every step of a call in one
    cooperative launch, grid-wide barriers between stages, stage inputs read
    through L2) against one launch per stage and tile list: 1-D and 2-D
    grids together in the tile lists, the same clock, step count and bits;
    and CTAs per SM from 2 to the occupancy limit."""
    from mara2_gb300.batch import Batch
    reqs = W.riemann_stream(24, rate=1e6, seed=17, n1=(64, 2048), n2=(32, 160))
    built = []
    for r in reqs[:14]:
        s, P = W.riemann_initial(r)
        s = s.with_(recon=recon, riemann=riemann, rk_order=rk, t_final=0.01, guard=2)
        built.append((s, W.apply_bc_numpy(s, P)))
    kw = dict(recon=recon, riemann=riemann, rk_order=rk, tile_1d=tile_1d, tile_2d=tile_2d, lockstep_1d=True)
    ref = _run_batch(built, **kw)
    for ctas in (2, 0):
        got = _run_batch(built, persistent=True, ctas_per_sm=ctas, **kw)
        for k, (s, _) in enumerate(built):
            Pa, ta, na = ref[k]
            Pb, tb, nb = got[k]
            assert na == nb and ta == tb, (k, na, nb)
            assert np.array_equal(Pa[s.interior()].view(np.uint64), Pb[s.interior()].view(np.uint64)), k
    cells = max(int(np.prod(s.full_shape[:3])) for s, _ in built)
    with Batch(budget_bytes=1 << 26, max_grids=4, max_zones_per_grid=cells, persistent=True, **kw) as b:
        persistent, ctas = b.launch_form()
        assert persistent and ctas > 0


@pytest.mark.gpu
@pytest.mark.parametrize("riemann,rk", [("hllc", 2), ("hlle", 3)])
def test_tile_shapes_and_face_forms_agree(gpu_lib, riemann, rk):
    """Every 2-D tile choice of the per-stage launches (32x8, 32x16 and 64x8
    with the PLM faces in runs along their normal, 32x16 with one face per
    thread) and the persistent launch with runs: the same clock, step count
    and bits."""
    reqs = W.riemann_stream(24, rate=1e6, seed=23, n1=(64, 2048), n2=(40, 200))
    built = []
    for r in reqs[:12]:
        s, P = W.riemann_initial(r)
        s = s.with_(recon="plm", riemann=riemann, rk_order=rk, t_final=0.01, guard=2)
        built.append((s, W.apply_bc_numpy(s, P)))
    assert any(s.dims == 2 for s, _ in built)
    kw = dict(recon="plm", riemann=riemann, rk_order=rk, tile_1d=256, lockstep_1d=True)
    ref = _run_batch(built, tile_2d=4, **kw)
    for form in ({"tile_2d": 1}, {"tile_2d": 2}, {"tile_2d": 3}, {"tile_2d": 2, "persistent": True}):
        got = _run_batch(built, **form, **kw)
        for k, (s, _) in enumerate(built):
            Pa, ta, na = ref[k]
            Pb, tb, nb = got[k]
            assert na == nb and ta == tb, (form, k, na, nb)
            assert np.array_equal(Pa[s.interior()].view(np.uint64), Pb[s.interior()].view(np.uint64)), (form, k)


@pytest.mark.gpu
def test_persistent_serving_alone_equals_mix(gpu_lib):
    """Continuous batching on the persistent form: each request's result is
    the same alone and in the mix (small 1-D grids on their clusters)."""
    from mara2_gb300.batch import run_alone, serve
    reqs = _small_requests(10, seed=41)
    res = serve(reqs, budget_bytes=1 << 28, max_grids=32, keep_results=True, make=_make, persistent=True)
    assert res.completed == len(reqs)
    for r in reqs:
        s, P = _make(r)
        Pa, ta, na = run_alone(s, P, s.t_final)
        Pm, tm, nm = res.results[r.index]
        assert na == nm and ta == tm
        assert np.array_equal(Pa[s.interior()].view(np.uint64), Pm[s.interior()].view(np.uint64))
