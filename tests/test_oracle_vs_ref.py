"""The oracle restatement (oracle/mara_oracle.c) against the reference's own
hot-path sources compiled in place (oracle/_ref): bit-for-bit on whole
advances, fluxes, Courant steps, guard fills and point operations.  Skipped
where the reference tree is absent."""
import numpy as np
import pytest

import oracle as O
from helpers import oracle_config
from mara2_gb300 import workloads as W


@pytest.fixture(scope="module")
def ref():
    if not O.ref_available():
        try:
            O.build(ref=True)
        except Exception:
            pytest.skip("reference tree not available")
    if not O.ref_available():
        pytest.skip("reference tree not available")
    return O.Oracle("ref")


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


CASES = [
    ("sod", lambda: W.sod(96), {}, 30),
    ("sod-pcm-rk1", lambda: W.sod(64), dict(recon="pcm", rk_order=1), 20),
    ("sod-plm-hllc-rk3", lambda: W.sod(64), dict(riemann="hllc", rk_order=3), 20),
    ("sod-theta2", lambda: W.sod(64), dict(plm_theta=2.0), 10),
    ("kh", lambda: W.kelvin_helmholtz(20), {}, 6),
    ("kh-reflect", lambda: W.kelvin_helmholtz(20), dict(bc="reflecting"), 6),
    ("kh-outflow-hlle", lambda: W.kelvin_helmholtz(20), dict(bc="outflow", riemann="hlle"), 6),
    ("mhd3d", lambda: W.mhd_turbulence(8), {}, 3),
    ("mhd3d-noct", lambda: W.mhd_turbulence(8), dict(disable_ct=True), 2),
    ("mhd3d-floor", lambda: W.mhd_turbulence(8), dict(pressure_floor=1e-3), 2),
    ("rmhd-weno-js", lambda: W.rmhd_blast(16), dict(weno_is="js96"), 2),
    ("rmhd-weno-borges", lambda: W.rmhd_blast(16), dict(weno_is="borges08"), 2),
    ("rmhd-weno-shenzha", lambda: W.rmhd_blast(16), {}, 3),
    ("rmhd-plm", lambda: W.rmhd_blast(16), dict(recon="plm"), 3),
]


@pytest.mark.parametrize("name,make,kw,steps", CASES, ids=[c[0] for c in CASES])
def test_advance_bitwise(port, ref, name, make, kw, steps):
    s, P = make()
    s = s.with_(**kw)
    c = oracle_config(s)
    A, B = P.copy(), P.copy()
    sa, _, da = port.run(c, A, steps, s.cfl, s.t_final)
    sb, _, db = ref.run(c, B, steps, s.cfl, s.t_final)
    assert sa == sb == 0
    assert da == db
    assert np.array_equal(_bits(A), _bits(B))


@pytest.mark.parametrize("make", [lambda: W.kelvin_helmholtz(12), lambda: W.mhd_turbulence(6), lambda: W.rmhd_blast(12)])
def test_godunov_fluxes_bitwise(port, ref, make):
    s, P = make()
    c = oracle_config(s)
    sa, Fa = port.godunov(c, P.copy())
    sb, Fb = ref.godunov(c, P.copy())
    assert sa == sb == 0
    assert np.array_equal(_bits(Fa), _bits(Fb))


def test_bc_and_conserved_bitwise(port, ref):
    for bc in ("periodic", "outflow", "reflecting"):
        s, P = W.kelvin_helmholtz(10)
        s = s.with_(bc=bc)
        c = oracle_config(s)
        rng = np.random.default_rng(5)
        P = P + 0.01 * rng.random(P.shape)
        A, B = P.copy(), P.copy()
        assert port.apply_bc(c, A) == ref.apply_bc(c, B) == 0
        assert np.array_equal(_bits(A), _bits(B))
        sa, Ua = port.generate_conserved(c, A)
        sb, Ub = ref.generate_conserved(c, B)
        assert np.array_equal(_bits(Ua), _bits(Ub))


def test_point_operations_bitwise(port, ref):
    rng = np.random.default_rng(7)
    c = O.make_config(law="rmhd", gamma=4.0 / 3)
    for _ in range(200):
        v = rng.uniform(-0.5, 0.5, 3)
        P = [rng.uniform(0.1, 2), *v, rng.uniform(0.01, 3), *rng.uniform(-2, 2, 3)]
        n = [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0)][rng.integers(3)]
        a = port.from_primitive(c, P, n)
        b = ref.from_primitive(c, P, n)
        assert a[0] == b[0]
        for x, y in zip(a[1:], b[1:]):
            assert np.array_equal(_bits(x), _bits(y))
        if a[0] == 0:
            ra = port.from_conserved(c, a[1][:8])
            rb = ref.from_conserved(c, b[1][:8])
            assert ra[0] == rb[0]
            assert np.array_equal(_bits(ra[1]), _bits(rb[1]))
    for _ in range(200):
        d = rng.uniform(-3, 3, 5)
        na, ra = port.quartic(*d)
        nb, rb = ref.quartic(*d)
        assert na == nb and np.array_equal(_bits(ra), _bits(rb))


def test_ct_and_monopole_bitwise(port, ref):
    rng = np.random.default_rng(11)
    for shape in [(9, 9, 2, 8), (7, 6, 5, 8), (8, 2, 2, 8)]:
        F = rng.standard_normal(shape + (3,))
        assert np.array_equal(_bits(port.ct_correct(F)), _bits(ref.ct_correct(F)))
    B = rng.standard_normal((6, 5, 4, 3))
    assert np.array_equal(_bits(port.monopole_cell(B, 0.5)), _bits(ref.monopole_cell(B, 0.5)))


def test_failure_reporting_matches(port, ref):
    """A zone that cannot be inverted: same status, count and first zone."""
    s, P = W.mhd_turbulence(6)
    c = oracle_config(s)
    P = P.copy()
    P[4, 5, 3, 4] = 1e-9       # near-vacuum pressure next to strong gradients
    P[4, 5, 3, 1] = 3.0
    A, B = P.copy(), P.copy()
    sa, fa = port.advance(c, A, 0.05)
    sb, fb = ref.advance(c, B, 0.05)
    assert sa == sb
    assert fa.count == fb.count
    if fa.count:
        assert tuple(fa.first) == tuple(fb.first)


def test_workload_vector_potential_matches_reference(ref):
    """workloads.vector_potential_to_cell_b restates Problems.cpp:660-667."""
    s, _ = W.mhd_turbulence(6)
    A = W.face_vector_potential(s, lambda x, y, z: W._fourier_vector(5, x, y, z))
    B = W.vector_potential_to_cell_b(s, A)
    c = oracle_config(s)
    Bref = np.zeros(B.shape)
    import ctypes as C
    ref.lib.mr_vector_potential_to_cell_b(C.byref(c), np.ascontiguousarray(A).ctypes.data_as(C.POINTER(C.c_double)),
                                          Bref.ctypes.data_as(C.POINTER(C.c_double)))
    np.testing.assert_allclose(B, Bref, rtol=0, atol=1e-12 * np.abs(Bref).max())


@pytest.mark.parametrize("make", [lambda: W.kelvin_helmholtz(24), lambda: W.sod(64),
                                  lambda: W.mhd_turbulence(8), lambda: W.rmhd_blast(16)])
def test_volume_diagnostics_bitwise(port, ref, make):
    """FieldOperator::volumeIntegratedDiagnostics, every law, after a few
    steps so that velocities and fields are non-trivial."""
    s, P = make()
    c = oracle_config(s)
    for _ in range(2):
        _, dt = port.courant(c, P)
        assert port.advance(c, P, s.cfl * dt)[0] == 0
    a = port.volume_diagnostics(c, P)
    b = ref.volume_diagnostics(c, P)
    assert a[0] == b[0] == 0
    assert np.array_equal(_bits(a[1]), _bits(b[1]))


def test_current_bitwise(port, ref):
    """CellCenteredFieldCT::current on 3-D, 2-D and 1-D cell fields."""
    rng = np.random.default_rng(7)
    for shape in ((9, 8, 7, 3), (12, 10, 1, 3), (16, 1, 1, 3)):
        B = rng.normal(size=shape)
        assert np.array_equal(_bits(port.current_cell(B, 0.1)), _bits(ref.current_cell(B, 0.1)))


def _gravity(g):
    def S(x, y, z, aux, P):
        rho = P[0]
        return [0.0, rho * g[0], rho * g[1], rho * g[2], rho * (P[1] * g[0] + P[2] * g[1] + P[3] * g[2])] + [0.0] * 5
    return S


def _position_source(x, y, z, aux, P):
    # depends on the cell centre, so the coordinates are checked too
    return [0.0, x * y, -z + x, 0.0, P[0] * x] + [0.0] * 5


@pytest.mark.parametrize("make,src", [(lambda: W.kelvin_helmholtz(16), _gravity((0.0, -1.0, 0.0))),
                                      (lambda: W.sod(48), _position_source),
                                      (lambda: W.mhd_turbulence(6), _gravity((0.3, -0.2, 0.1)))])
def test_source_terms_bitwise(port, ref, make, src):
    """MethodOfLinesTVD::setSourceTermsFunction: S from the stage's
    primitives and the cell centres, added to L before the RK combine."""
    s, P = make()
    c = oracle_config(s)
    A, B = P.copy(), P.copy()
    try:
        port.set_source_terms(src)
        ref.set_source_terms(src)
        for _ in range(2):
            _, dt = port.courant(c, A)
            assert port.advance(c, A, s.cfl * dt)[0] == 0
            assert ref.advance(c, B, s.cfl * dt)[0] == 0
    finally:
        port.set_source_terms(None)
        ref.set_source_terms(None)
    assert np.array_equal(_bits(A), _bits(B))
    assert not np.array_equal(_bits(A), _bits(P))


@pytest.mark.parametrize("make,kw", [(lambda: W.mhd_turbulence(6), {}),
                                     (lambda: W.mhd_turbulence(6), dict(disable_ct=True, rk_order=3))])
def test_cooling_bitwise(port, ref, make, kw):
    """NewtonianMHD with a cooling rate: the auxiliary field 8 and
    addSourceTerms (ConservationLaws.cpp:355-358, 479-501), advances and the
    18 volume diagnostics."""
    s, P = make()
    s, P = W.with_cooling(s.with_(**kw), P, 0.4, aux=0.02)
    c = oracle_config(s)
    assert O.config_nq(c) == 9
    A, B = P.copy(), P.copy()
    for _ in range(3):
        _, dt = port.courant(c, A)
        assert port.advance(c, A, s.cfl * dt)[0] == 0
        assert ref.advance(c, B, s.cfl * dt)[0] == 0
    assert np.array_equal(_bits(A), _bits(B))
    assert A[..., 8].mean() > 0.02                      # energy moved into the auxiliary field
    a, b = port.volume_diagnostics(c, A), ref.volume_diagnostics(c, A)
    assert len(a[1]) == 18 and np.array_equal(_bits(a[1]), _bits(b[1]))


@pytest.mark.parametrize("shape", [(6, 5, 4), (7, 6, 1), (9, 1, 1)])
@pytest.mark.parametrize("bc", ["periodic", "outflow"])
def test_uniform_cartesian_ct_bitwise(port, ref, shape, bc):
    """UniformCartesianCT (the reference's ConstrainedTransport
    implementation): monopole at vertices and cells of an assigned
    cell-centred field, and the adaptor's current operator
    (CellCenteredFieldCT::current of the guarded field)."""
    rng = np.random.default_rng(sum(shape) + len(bc))
    B = rng.standard_normal(shape + (3,))
    for loc in ("vert", "cell"):
        sa, Ma = port.uct_monopole(B, bc, loc)
        sb, Mb = ref.uct_monopole(B, bc, loc)
        assert sa == sb == 0
        assert np.array_equal(_bits(Ma), _bits(Mb)), loc
    sa, Ja = port.uct_current(B, bc, 0.25)
    sb, Jb = ref.uct_current(B, bc, 0.25)
    assert sa == sb == 0
    assert np.array_equal(_bits(Ja), _bits(Jb))


@pytest.mark.parametrize("make", [lambda: W.mhd_turbulence(6), lambda: W.rmhd_blast(10)])
def test_vector_potential_to_cell_b_bitwise(port, ref, make):
    """Problems.cpp:660-667 (fluxes of A -> flux CT -> divergence), every cell
    with guards, then scaled."""
    s, _ = make()
    A = W.face_vector_potential(s, lambda x, y, z: W._fourier_vector(5, x, y, z))
    c = oracle_config(s)
    for scale in (1.0, 0.37):
        sa, Ba = port.vector_potential_to_cell_b(c, A, scale)
        sb, Bb = ref.vector_potential_to_cell_b(c, A, scale)
        assert sa == sb == 0
        assert np.array_equal(_bits(Ba), _bits(Bb))
