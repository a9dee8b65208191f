// ref_harness.cpp -- drives the reference's own hot-path code (compiled in
// place from the reference tree, see oracle/Makefile) behind the same C entry
// points as the oracle restatement, with an "mr_" prefix.
//
// TEST INFRASTRUCTURE ONLY: used here, where the reference sources exist, to
// pin oracle/mara_oracle.c and to generate the golden fixtures in
// tests/golden/.  It is never built on a machine without the reference tree.
#include <cstdio>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>

#include "BoundaryConditions.hpp"
#include "CartesianMeshGeometry.hpp"
#include "CellCenteredFieldCT.hpp"
#include "ConservationLaws.hpp"
#include "FieldOperator.hpp"
#include "IntercellFluxSchemes.hpp"
#include "MeshData.hpp"
#include "MeshOperator.hpp"
#include "ConstrainedTransport.hpp"
#include "QuarticPolynomial.hpp"
#include "Reconstruction.hpp"
#include "RiemannSolvers.hpp"
#include "SolutionSchemes.hpp"

#include "mara_oracle.h"

// ----------------------------------------------------------------------------
// MeshGeometry's non-virtual members live in the reference's Mara.cpp, which
// also holds main() and the problem drivers; these are the same trivial
// accessors (src/Mara.cpp:92-130).
MeshGeometry::MeshGeometry() { patchIndex = {{0, 0, 0, 0, 0}}; startIndex = {{0, 0, 0, 0, 0}}; }
std::vector<bool> MeshGeometry::fleshedOutAxes() const
{
    auto s = cellsShape();
    return {s[0] > 1, s[1] > 1, s[2] > 1};
}
void MeshGeometry::assignPatchIndex (PatchIndex p) { patchIndex = p; }
MeshGeometry::PatchIndex MeshGeometry::getPatchIndex() const { return patchIndex; }
Coordinate MeshGeometry::coordinateAtIndex (Cow::Index i) const { return coordinateAtIndex (i[0], i[1], i[2]); }
Cow::Index MeshGeometry::getStartIndex() const { return startIndex; }
void MeshGeometry::assignStartIndex (Index i) { startIndex = i; }

// ----------------------------------------------------------------------------
// The WENO5 + HLLE composition of the relativistic blast-wave workload: the
// shape of MethodOfLinesPlm::intercellFlux with the reference's WENO5 C2R /
// C2L reconstructions on a 6-cell stencil (no reference class composes it).
class MethodOfLinesWeno5Prim : public IntercellFluxScheme
{
public:
    MethodOfLinesWeno5Prim (int mode, double A)
    {
        weno.setSmoothnessIndicator (Reconstruction::SmoothnessIndicator (mode));
        weno.setShenZha10A (A);
        riemannSolver = std::make_shared<HlleRiemannSolver>();
    }
    void setRiemannSolver (std::shared_ptr<RiemannSolver> rs) override { riemannSolver = rs; }
    ConservationLaw::State intercellFlux (const FaceData& fd, std::array<double, 8> t) const override
    {
        ConservationLaw::Request request;
        request.areaElement = fd.areaElement;
        request.auxiliaryData = t;
        const int nq = fd.conservationLaw->getNumConserved();
        std::array<double, MARA_NUM_FIELDS> PL, PR;
        for (int q = 0; q < nq; ++q)
        {
            double ps[6];
            for (int n = 0; n < 6; ++n) ps[n] = (&fd.stencilData (n))[q];
            PL[q] = weno.reconstruct (&ps[2], Reconstruction::WENO5_FD_C2R);
            PR[q] = weno.reconstruct (&ps[3], Reconstruction::WENO5_FD_C2L);
        }
        auto L = fd.conservationLaw->fromPrimitive (request, &PL[0]);
        auto R = fd.conservationLaw->fromPrimitive (request, &PR[0]);
        return riemannSolver->solve (L, R, fd.areaElement);
    }
    int getStencilSize() const override { return 3; }

private:
    Reconstruction weno;
    std::shared_ptr<RiemannSolver> riemannSolver;
};

// ----------------------------------------------------------------------------
// The source terms function every later setup installs (mr_set_source_terms)
static mo_source_fn g_src_fn = nullptr;
static void* g_src_user = nullptr;

// ----------------------------------------------------------------------------
struct Setup
{
    std::shared_ptr<CartesianMeshGeometry> mg;
    std::shared_ptr<MeshOperator> mo;
    std::shared_ptr<ConservationLaw> cl;
    std::shared_ptr<FieldOperator> fo;
    std::shared_ptr<IntercellFluxScheme> fs;
    std::shared_ptr<BoundaryCondition> bc;
    std::shared_ptr<MethodOfLinesTVD> ss;
    std::shared_ptr<MeshData> md;
    int nq;
};

static Setup make_setup (const mo_config* c)
{
    Setup s;
    auto cs = Cow::Shape {{c->ni, c->nj, c->nk, 1, 1}};
    auto bs = Cow::Shape {{c->ng[0], c->ng[1], c->ng[2], 0, 0}};

    s.mg = std::make_shared<CartesianMeshGeometry>();
    s.mg->setCellsShape (cs);
    s.mg->setLowerUpper ({{c->lower[0], c->lower[1], c->lower[2]}}, {{c->upper[0], c->upper[1], c->upper[2]}});
    s.mo = std::make_shared<MeshOperator>();
    s.mo->setMeshGeometry (s.mg);

    switch (c->law)
    {
        case MO_LAW_HYDRO: s.cl = std::make_shared<NewtonianHydro>(); break;
        case MO_LAW_MHD: s.cl = std::make_shared<NewtonianMHD>(); break;
        default: s.cl = std::make_shared<RelativisticMHD>(); break;
    }
    s.cl->setGammaLawIndex (c->gamma);
    s.cl->setPressureFloor (c->pressure_floor);
    s.cl->setCoolingRate (c->cooling_rate);
    s.nq = s.cl->getNumConserved();

    s.fo = std::make_shared<FieldOperator>();
    s.fo->setConservationLaw (s.cl);

    std::shared_ptr<RiemannSolver> rs;
    if (c->riemann == MO_RIEMANN_HLLC) rs = std::make_shared<HllcNewtonianHydroRiemannSolver>();
    else rs = std::make_shared<HlleRiemannSolver>();

    switch (c->recon)
    {
        case MO_RECON_PCM: s.fs = std::make_shared<MethodOfLines>(); break;
        case MO_RECON_PLM: s.fs = std::make_shared<MethodOfLinesPlm>(); s.fs->setPlmTheta (c->plm_theta); break;
        default: s.fs = std::make_shared<MethodOfLinesWeno5Prim> (c->weno_is, c->shenzha_A); break;
    }
    s.fs->setRiemannSolver (rs);

    switch (c->bc)
    {
        case MO_BC_PERIODIC: s.bc = std::make_shared<PeriodicBoundaryCondition>(); break;
        case MO_BC_OUTFLOW: s.bc = std::make_shared<OutflowBoundaryCondition>(); break;
        default:
        {
            auto r = std::make_shared<ReflectingBoundaryCondition>();
            r->setConservationLaw (s.cl);
            s.bc = r;
            break;
        }
    }

    s.ss = std::make_shared<MethodOfLinesTVD>();
    s.ss->setRungeKuttaOrder (c->rk_order);
    s.ss->setDisableFieldCT (c->disable_ct != 0);
    s.ss->setFieldOperator (s.fo);
    s.ss->setMeshOperator (s.mo);
    s.ss->setBoundaryCondition (s.bc);
    s.ss->setIntercellFluxScheme (s.fs);
    if (g_src_fn)
    {
        s.ss->setSourceTermsFunction ([] (double x, double y, double z, std::array<double, 8> t, StateArray P)
        {
            auto S = StateArray();
            g_src_fn (g_src_user, x, y, z, t.data(), P.data(), S.data());
            return S;
        });
    }

    s.md = std::make_shared<MeshData> (cs, bs, s.nq);
    return s;
}

static int zone_from_message (const char* what, int first[3])
{
    // StateFailure::what() starts with "at zone index [i j k]"
    return std::sscanf (what, "at zone index [%d %d %d]", &first[0], &first[1], &first[2]) == 3;
}

static int code_of_runtime_error (const std::runtime_error& e)
{
    const std::string w = e.what();
    if (w.find ("superluminal") != std::string::npos) return MO_ERR_SUPERLUMINAL;
    if (w.find ("eigenvalues") != std::string::npos) return MO_ERR_BAD_EIGENVALUES;
    return MO_ERR_CONFIG;
}

#define GUARD_CALL(...)                                                          \
    try { __VA_ARGS__ }                                                            \
    catch (FieldOperator::InversionFailure& e)                                   \
    {                                                                            \
        if (fail)                                                                \
        {                                                                        \
            fail->count = int (e.failedStates.size());                           \
            fail->code = MO_ERR_INVERSION_FAILURE;                               \
            if (!e.failedStates.empty()) zone_from_message (e.failedStates[0].what(), fail->first); \
        }                                                                        \
        status = MO_ERR_INVERSION_FAILURE;                                       \
    }                                                                            \
    catch (std::runtime_error& e) { status = code_of_runtime_error (e); }       \
    catch (std::logic_error& e)                                                  \
    {                                                                            \
        status = std::string (e.what()).find ("smaller than") != std::string::npos \
            ? MO_ERR_GUARD_TOO_SMALL : MO_ERR_CONFIG;                            \
    }

extern "C" {

int mr_advance (const mo_config* c, double* P, double t0, double dt, mo_failure* fail)
{
    int status = MO_OK;
    if (fail) std::memset (fail, 0, sizeof (*fail));
    GUARD_CALL (
        auto s = make_setup (c);
        std::memcpy (s.md->P.data(), P, sizeof (double) * s.md->P.size());
        try { s.ss->advance (*s.md, t0, dt); }
        catch (...) { std::memcpy (P, s.md->P.data(), sizeof (double) * s.md->P.size()); throw; }
        std::memcpy (P, s.md->P.data(), sizeof (double) * s.md->P.size());
    )
    return status;
}

int mr_courant (const mo_config* c, const double* P, double* dt)
{
    int status = MO_OK;
    mo_failure* fail = nullptr;
    GUARD_CALL (
        auto s = make_setup (c);
        std::memcpy (s.md->P.data(), P, sizeof (double) * s.md->P.size());
        auto L = s.mo->linearCellDimension();
        auto Pi = s.md->getPrimitive();
        *dt = s.fo->getCourantTimestep (Pi, L);
    )
    return status;
}

int mr_apply_bc (const mo_config* c, double* P)
{
    int status = MO_OK;
    mo_failure* fail = nullptr;
    GUARD_CALL (
        auto s = make_setup (c);
        std::memcpy (s.md->P.data(), P, sizeof (double) * s.md->P.size());
        s.md->applyBoundaryCondition (*s.bc);
        std::memcpy (P, s.md->P.data(), sizeof (double) * s.md->P.size());
    )
    return status;
}

int mr_godunov (const mo_config* c, const double* P, double* Fout)
{
    int status = MO_OK;
    mo_failure* fail = nullptr;
    GUARD_CALL (
        auto s = make_setup (c);
        std::memcpy (s.md->P.data(), P, sizeof (double) * s.md->P.size());
        auto footprint = Cow::Shape3D();
        auto startIndex = Cow::Index();
        auto interior = Cow::Region();
        SchemeHelpers::makeFootprint (s.fs->getStencilSize(), s.md->P.shape(), s.md->getBoundaryShape(),
                                      footprint, startIndex, interior);
        auto D = IntercellFluxScheme::FaceData();
        D.conservationLaw = s.cl;
        const int nq = s.nq;
        auto fs = s.fs;
        std::array<double, 8> T = {};
        auto Fhat = [&] (GodunovStencil& stencil)
        {
            D.areaElement = stencil.faceNormal.cartesian();
            D.stencilData = stencil.cellData;
            auto S = fs->intercellFlux (D, T);
            for (int q = 0; q < nq; ++q) stencil.godunovFlux[q] = S.F[q];
        };
        const bool ct = s.cl->getIndexFor (ConservationLaw::VariableType::magnetic) != -1 && !c->disable_ct;
        auto fluxCorrection = [&] (const Cow::Array&, Cow::Array& F)
        {
            if (ct) CellCenteredFieldCT().correctGodunovFluxes (F, 5);
        };
        auto F = s.mo->godunov (Fhat, s.md->P, s.md->B, footprint, startIndex, fluxCorrection);
        std::memcpy (Fout, F.data(), sizeof (double) * F.size());
    )
    return status;
}

int mr_generate_conserved (const mo_config* c, const double* P, double* U)
{
    int status = MO_OK;
    mo_failure* fail = nullptr;
    GUARD_CALL (
        auto s = make_setup (c);
        std::memcpy (s.md->P.data(), P, sizeof (double) * s.md->P.size());
        auto Uarr = s.fo->generateConserved (s.md->P);
        std::memcpy (U, Uarr.data(), sizeof (double) * Uarr.size());
    )
    return status;
}

int mr_from_primitive (const mo_config* c, const double* P, const double n[3], double* U, double* F, double* A)
{
    int status = MO_OK;
    mo_failure* fail = nullptr;
    GUARD_CALL (
        auto s = make_setup (c);
        auto request = ConservationLaw::Request();
        request.areaElement = {{n[0], n[1], n[2]}};
        auto S = s.cl->fromPrimitive (request, P);
        for (int q = 0; q < MARA_NUM_FIELDS; ++q)
        {
            if (U) U[q] = S.U[q];
            if (F) F[q] = S.F[q];
            if (A) A[q] = S.A[q];
        }
    )
    return status;
}

int mr_from_conserved (const mo_config* c, const double* U, double* P, int* health)
{
    int status = MO_OK;
    mo_failure* fail = nullptr;
    try
    {
        auto s = make_setup (c);
        auto request = ConservationLaw::Request();
        auto S = s.cl->fromConserved (request, U);
        for (int q = 0; q < s.nq; ++q) P[q] = S.P[q];
        if (health) *health = S.healthFlag;
    }
    catch (ConservationLaw::StateFailure&) { status = MO_ERR_INVERSION_FAILURE; }
    catch (std::runtime_error& e) { status = code_of_runtime_error (e); }
    (void) fail;
    return status;
}

int mr_quartic (double d4, double d3, double d2, double d1, double d0, double roots[4])
{
    return QuarticPolynomial (d4, d3, d2, d1, d0).solve (roots);
}

void mr_ct_correct (double* F, int n0, int n1, int n2, int nq, int ib)
{
    auto A = Cow::Array (n0, n1, n2, nq, 3);
    std::memcpy (A.data(), F, sizeof (double) * A.size());
    CellCenteredFieldCT().correctGodunovFluxes (A, ib);
    std::memcpy (F, A.data(), sizeof (double) * A.size());
}

void mr_monopole_cell (const double* B, int n0, int n1, int n2, double h, double* M)
{
    auto A = Cow::Array (n0, n1, n2, 3, 1);
    std::memcpy (A.data(), B, sizeof (double) * A.size());
    auto ct = CellCenteredFieldCT();
    ct.setMeshSpacing (h);
    auto Mc = ct.monopole (A, MeshLocation::cell);
    std::memcpy (M, Mc.data(), sizeof (double) * Mc.size());
}

int mr_vector_potential_to_cell_b (const mo_config* c, const double* Aface, double* Bcell)
{
    // Problems.cpp:660-667: B = divergence (CT (fluxes of A)), including guards.
    int status = MO_OK;
    mo_failure* fail = nullptr;
    GUARD_CALL (
        auto s = make_setup (c);
        auto bs = Cow::Shape3D (Cow::Shape {{c->ng[0], c->ng[1], c->ng[2], 0, 0}});
        auto tot = Cow::Shape3D (s.mg->cellsShape()).increased (bs * 2);
        auto A = Cow::Array (tot.increased (1).withComponents (3).withRank (3));
        std::memcpy (A.data(), Aface, sizeof (double) * A.size());
        auto ct = CellCenteredFieldCT();
        auto F = ct.vectorPotentialToFluxes (A);
        auto G = ct.generateGodunovFluxes (F, 0);
        auto B = s.mo->divergence (G, 1.0, {});
        std::memcpy (Bcell, B.data(), sizeof (double) * B.size());
    )
    return status;
}

int mr_vector_potential_to_cell_b_scaled (const mo_config* c, const double* Aface, double scale, double* Bcell)
{
    const int status = mr_vector_potential_to_cell_b (c, Aface, Bcell);
    if (status != MO_OK) return status;
    auto s = make_setup (c);
    auto bs = Cow::Shape3D (Cow::Shape {{c->ng[0], c->ng[1], c->ng[2], 0, 0}});
    auto tot = Cow::Shape3D (s.mg->cellsShape()).increased (bs * 2);
    const long n = (long) tot[0] * tot[1] * tot[2] * 3;
    for (long m = 0; m < n; ++m) Bcell[m] = Bcell[m] * scale;
    return MO_OK;
}

int mr_uct_current (const double* Bc, int n0, int n1, int n2, int bc, double h, double* J)
{
    // the guarded field as UniformCartesianCT::setCellBC fills it (one guard
    // zone, axis by axis), then CellCenteredFieldCT::current at the interior
    if (bc != MO_BC_PERIODIC && bc != MO_BC_OUTFLOW) return MO_ERR_CONFIG;
    std::shared_ptr<BoundaryCondition> b;
    if (bc == MO_BC_PERIODIC) b = std::make_shared<PeriodicBoundaryCondition>();
    else b = std::make_shared<OutflowBoundaryCondition>();
    auto Bg = Cow::Array (n0 + 2, n1 + 2, n2 + 2, 3);
    for (int i = 0; i < n0; ++i)
        for (int j = 0; j < n1; ++j)
            for (int k = 0; k < n2; ++k)
                for (int q = 0; q < 3; ++q)
                    Bg (i + 1, j + 1, k + 1, q) = Bc[(((long) i * n1 + j) * n2 + k) * 3 + q];
    for (int axis = 0; axis < 3; ++axis)
    {
        b->apply (Bg, MeshLocation::cell, MeshBoundary::left, axis, 1);
        b->apply (Bg, MeshLocation::cell, MeshBoundary::right, axis, 1);
    }
    auto ct = CellCenteredFieldCT();
    ct.setMeshSpacing (h);
    auto Jg = ct.current (Bg, MeshLocation::cell);
    for (int i = 0; i < n0; ++i)
        for (int j = 0; j < n1; ++j)
            for (int k = 0; k < n2; ++k)
                for (int q = 0; q < 3; ++q)
                    J[(((long) i * n1 + j) * n2 + k) * 3 + q] = Jg (i + 1, j + 1, k + 1, q);
    return MO_OK;
}

int mr_uct_monopole (const double* Bc, int n0, int n1, int n2, int bc, int location, double* M)
{
    // UniformCartesianCT with a mesh geometry and a boundary condition; the
    // field assigned at the interior cells, its monopole at vertices or cells
    if (bc != MO_BC_PERIODIC && bc != MO_BC_OUTFLOW) return MO_ERR_CONFIG;
    auto mg = std::make_shared<CartesianMeshGeometry>();
    mg->setCellsShape (Cow::Shape {{n0, n1, n2, 1, 1}});
    std::shared_ptr<BoundaryCondition> b;
    if (bc == MO_BC_PERIODIC) b = std::make_shared<PeriodicBoundaryCondition>();
    else b = std::make_shared<OutflowBoundaryCondition>();
    auto ct = UniformCartesianCT();
    ct.setMeshGeometry (mg);
    ct.setBoundaryCondition (b);
    auto B = Cow::Array (n0, n1, n2, 3);
    std::memcpy (B.data(), Bc, sizeof (double) * B.size());
    ct.assignCellCenteredB (B);
    auto Mo = ct.computeMonopole (location == 0 ? MeshLocation::vert : MeshLocation::cell);
    std::memcpy (M, Mo.data(), sizeof (double) * Mo.size());
    return MO_OK;
}

void mr_set_source_terms (mo_source_fn fn, void* user)
{
    g_src_fn = fn;
    g_src_user = user;
}

int mr_volume_diagnostics (const mo_config* c, const double* P, double* D, double* Dabs)
{
    // the drivers' time-series task (e.g. src/Problems/MagneticBraiding.cpp:
    // 165-166, 205): interior primitives and MeshOperator::measure (cell)
    int status = MO_OK;
    mo_failure* fail = nullptr;
    GUARD_CALL (
        auto s = make_setup (c);
        std::memcpy (s.md->P.data(), P, sizeof (double) * s.md->P.size());
        auto V = s.mo->measure (MeshLocation::cell);
        auto Pi = s.md->getPrimitive();
        auto d = s.fo->volumeIntegratedDiagnostics (Pi, V);
        for (unsigned n = 0; n < d.size(); ++n)
        {
            D[n] = d[n];
            if (Dabs) Dabs[n] = 0.0;
        }
    )
    return status;
}

void mr_current_cell (const double* B, int n0, int n1, int n2, double h, double* J)
{
    auto A = Cow::Array (n0, n1, n2, 3, 1);
    std::memcpy (A.data(), B, sizeof (double) * A.size());
    auto ct = CellCenteredFieldCT();
    ct.setMeshSpacing (h);
    auto Jc = ct.current (A, MeshLocation::cell);
    std::memcpy (J, Jc.data(), sizeof (double) * Jc.size());
}

} // extern "C"
