// GpuSolutionScheme.hpp -- the drop-in for Mara2: a SolutionScheme whose
// advance() runs on the GPU through the C ABI of include/mara_gpu.h.
//
// Header-only C++14, meant to be compiled inside a Mara2 build (it includes
// the reference's own interface headers).  It keeps the reference's
// dependency-injection surface (Mara.hpp:44-51, SolutionSchemes.hpp:24-72):
// setBoundaryCondition / setFieldOperator / setMeshOperator /
// setIntercellFluxScheme / setRungeKuttaOrder / setDisableFieldCT, and maps
// the injected objects onto the GPU configuration by their dynamic type.
// Parameters the reference classes keep without getters (the gamma-law index,
// the PLM theta, the Riemann solver inside a flux scheme, the pressure floor,
// the mesh bounds) are given once in Options.
//
// Errors come back as the reference's exception types:
//   FieldOperator::InversionFailure for failed primitive recoveries,
//   std::runtime_error for superluminal states / bad eigenvalues,
//   std::logic_error for configuration errors (guards smaller than the
//   stencil, missing operators, unsupported types).
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <typeinfo>
#include <vector>

#include "BoundaryConditions.hpp"
#include "CartesianMeshGeometry.hpp"
#include "ConservationLaws.hpp"
#include "FieldOperator.hpp"
#include "IntercellFluxSchemes.hpp"
#include "Mara.hpp"
#include "MeshData.hpp"
#include "MeshOperator.hpp"
#include "mara_gpu.h"

struct GpuSchemeOptions
{
    double gammaLawIndex = 5. / 3;   // ConservationLaw::setGammaLawIndex
    double plmTheta = 1.5;           // MethodOfLinesPlm default
    double pressureFloor = -1.0;     // ConservationLaw::setPressureFloor
    double coolingRate = -1.0;       // NewtonianMHD::setCoolingRate (> 0: auxiliary field 8)
    int riemannSolver = MARA_RIEMANN_HLLE;
    int wenoSmoothness = MARA_WENO_SHENZHA10;
    double shenZha10A = 50.0;
    Coordinate lower = {{0.0, 0.0, 0.0}};  // CartesianMeshGeometry::setLowerUpper
    Coordinate upper = {{1.0, 1.0, 1.0}};
    int precision = MARA_PRECISION_FP64;
    int device = 0;
    // page-lock MeshData::P on the first advance (and again if the array
    // moves), so advance() reads and writes it in place; for a 2-D mixed
    // hydro grid the transfers then overlap the stages (mara_gpu_advance_host)
    bool pinHostState = false;
};

class GpuMethodOfLinesTVD : public SolutionScheme
{
public:
    using Options = GpuSchemeOptions;

    GpuMethodOfLinesTVD() {}
    explicit GpuMethodOfLinesTVD (Options options) : opts (options) {}
    ~GpuMethodOfLinesTVD()
    {
        if (handle) mara_gpu_destroy (handle);
        if (pinned) mara_gpu_host_unregister (pinned);
    }
    GpuMethodOfLinesTVD (const GpuMethodOfLinesTVD&) = delete;
    GpuMethodOfLinesTVD& operator= (const GpuMethodOfLinesTVD&) = delete;

    void setRungeKuttaOrder (int order)
    {
        if (0 >= order || order > 3) throw std::logic_error ("Runge-Kutta order not 1, 2, or 3");
        rungeKuttaOrder = order;
        reset();
    }
    void setDisableFieldCT (bool disable) { disableFieldCT = disable; reset(); }
    void setBoundaryCondition (std::shared_ptr<BoundaryCondition> bc) override { boundaryCondition = bc; reset(); }
    void setFieldOperator (std::shared_ptr<FieldOperator> fo) override { fieldOperator = fo; reset(); }
    void setMeshOperator (std::shared_ptr<MeshOperator> mo) override { meshOperator = mo; reset(); }
    void setIntercellFluxScheme (std::shared_ptr<IntercellFluxScheme> fs) override { fluxScheme = fs; reset(); }

    int getStencilSize() const override
    {
        if (! fluxScheme) throw std::logic_error ("No IntercellFluxScheme instance");
        return fluxScheme->getStencilSize();
    }

    /** MethodOfLinesTVD::advance on solution.P (host, in place). */
    void advance (MeshData& solution, double t0, double dt) const override
    {
        ensure (solution);
        if (opts.pinHostState && pinned != solution.P.data())
        {
            if (pinned) mara_gpu_host_unregister (pinned);
            pinned = nullptr;
            if (mara_gpu_host_register (solution.P.data(), solution.P.size() * sizeof (double)) == MARA_OK)
                pinned = solution.P.data();
        }
        raise (mara_gpu_advance_host (handle, solution.P.data(), t0, dt));
    }

    /** FieldOperator::getCourantTimestep of solution.P (interior), on the GPU. */
    double getCourantTimestep (MeshData& solution) const
    {
        ensure (solution);
        raise (mara_gpu_upload (handle, solution.P.data()));
        double dt = 0.0;
        raise (mara_gpu_courant (handle, &dt));
        return dt;
    }

    /** FieldOperator::volumeIntegratedDiagnostics of solution.P (interior)
     *  with the cell volumes, on the GPU; the order of
     *  ConservationLaw::getDiagnosticNames. */
    std::vector<double> volumeIntegratedDiagnostics (MeshData& solution) const
    {
        ensure (solution);
        raise (mara_gpu_upload (handle, solution.P.data()));
        auto D = std::vector<double> (mara_gpu_num_diagnostics (handle));
        raise (mara_gpu_volume_diagnostics (handle, D.data(), nullptr));
        return D;
    }

    /** CellCenteredFieldCT::monopole and ::current (MeshLocation::cell) of
     *  the cell magnetic field of solution.P including guards, as the
     *  drivers' checkpoint task stores them: shape (ni+2g, nj+2g, nk+2g, 4),
     *  components [monopole, current1, current2, current3]. */
    Cow::Array fieldDiagnostics (MeshData& solution, double meshSpacing) const
    {
        ensure (solution);
        raise (mara_gpu_upload (handle, solution.P.data()));
        auto D = Cow::Array (solution.P.size (0), solution.P.size (1), solution.P.size (2), 4, 1);
        raise (mara_gpu_field_diagnostics (handle, meshSpacing, D.data()));
        return D;
    }

private:
    void reset() { if (handle) { mara_gpu_destroy (handle); handle = nullptr; } }

    void ensure (MeshData& solution) const
    {
        if (handle) return;
        if (! fieldOperator)     throw std::logic_error ("No FieldOperator instance");
        if (! meshOperator)      throw std::logic_error ("No MeshOperator instance");
        if (! boundaryCondition) throw std::logic_error ("No BoundaryCondition instance");
        if (! fluxScheme)        throw std::logic_error ("No IntercellFluxScheme instance");

        MaraGpuConfig c = {};
        auto law = fieldOperator->getConservationLaw();
        if      (dynamic_cast<NewtonianHydro*>  (law.get())) c.law = MARA_LAW_HYDRO;
        else if (dynamic_cast<NewtonianMHD*>    (law.get())) c.law = MARA_LAW_MHD;
        else if (dynamic_cast<RelativisticMHD*> (law.get())) c.law = MARA_LAW_RMHD;
        else throw std::logic_error ("GpuMethodOfLinesTVD: unsupported ConservationLaw");

        const auto* fs = fluxScheme.get();
        if      (dynamic_cast<const MethodOfLinesPlm*> (fs)) c.recon = MARA_RECON_PLM;
        else if (dynamic_cast<const MethodOfLines*>    (fs)) c.recon = MARA_RECON_PCM;
        else if (fs->getStencilSize() == 3)                 c.recon = MARA_RECON_WENO5;
        else throw std::logic_error ("GpuMethodOfLinesTVD: unsupported IntercellFluxScheme");

        const auto* bc = boundaryCondition.get();
        if      (dynamic_cast<const PeriodicBoundaryCondition*>   (bc)) c.bc = MARA_BC_PERIODIC;
        else if (dynamic_cast<const OutflowBoundaryCondition*>    (bc)) c.bc = MARA_BC_OUTFLOW;
        else if (dynamic_cast<const ReflectingBoundaryCondition*> (bc)) c.bc = MARA_BC_REFLECTING;
        else throw std::logic_error ("GpuMethodOfLinesTVD: unsupported BoundaryCondition");

        const auto& mg = meshOperator->getMeshGeometry();
        if (! dynamic_cast<const CartesianMeshGeometry*> (&mg))
            throw std::logic_error ("GpuMethodOfLinesTVD: only CartesianMeshGeometry is supported");
        const auto cells = mg.cellsShape();
        const auto guards = solution.getBoundaryShape();

        c.riemann = opts.riemannSolver;
        c.rk_order = rungeKuttaOrder;
        c.disable_ct = disableFieldCT ? 1 : 0;
        c.weno_is = opts.wenoSmoothness;
        c.ni = cells[0]; c.nj = cells[1]; c.nk = cells[2];
        for (int a = 0; a < 3; ++a)
        {
            c.ng[a] = guards[a];
            c.lower[a] = opts.lower[a];
            c.upper[a] = opts.upper[a];
        }
        c.gamma = opts.gammaLawIndex;
        c.plm_theta = opts.plmTheta;
        c.shenzha_A = opts.shenZha10A;
        c.pressure_floor = opts.pressureFloor;
        c.cooling_rate = opts.coolingRate;
        c.precision = opts.precision;
        c.device = opts.device;
        raise (mara_gpu_create (&c, &handle));
    }

    void raise (int status) const
    {
        switch (status)
        {
            case MARA_OK: return;
            case MARA_ERR_INVERSION_FAILURE:
            {
                MaraGpuStats st;
                mara_gpu_stats (handle, &st);
                auto failure = FieldOperator::InversionFailure();
                ConservationLaw::State S;
                auto zone = ConservationLaw::StateFailure (S);
                zone.setZoneIndex (Cow::Index {{st.first_zone[0], st.first_zone[1], st.first_zone[2], 0, 0}});
                failure.failedStates.push_back (zone);
                failure.updateWhatMessage();
                throw failure;
            }
            case MARA_ERR_SUPERLUMINAL:
            case MARA_ERR_BAD_EIGENVALUES:
                throw std::runtime_error (mara_gpu_status_string (status));
            default:
                throw std::logic_error (std::string ("GpuMethodOfLinesTVD: ") + mara_gpu_status_string (status));
        }
    }

    Options opts;
    int rungeKuttaOrder = 1;
    bool disableFieldCT = false;
    std::shared_ptr<BoundaryCondition> boundaryCondition;
    std::shared_ptr<FieldOperator> fieldOperator;
    std::shared_ptr<MeshOperator> meshOperator;
    std::shared_ptr<IntercellFluxScheme> fluxScheme;
    mutable MaraGpuHandle* handle = nullptr;
    mutable double* pinned = nullptr;   // the page-locked MeshData::P, if any
};

/** The ConstrainedTransport interface (src/Mara.hpp:341-349) on the GPU, as
 *  its reference implementation UniformCartesianCT (src/ConstrainedTransport
 *  .cpp) behaves for a cell-centred field: assignCellCenteredB stores the
 *  interior field, the guards (one zone per axis) come from the boundary
 *  condition (periodic or outflow), computeMonopole runs the vertex / cell
 *  monopole on the device (mara_gpu_ct_monopole), computeCurrent the
 *  centred-difference curl of CellCenteredFieldCT::current with unit mesh
 *  spacing (mara_gpu_ct_current).  Errors are std::logic_error, as the
 *  reference throws for a bad mesh location. */
class GpuConstrainedTransport : public ConstrainedTransport
{
public:
    explicit GpuConstrainedTransport (int device = 0) : device (device) {}

    void setMeshGeometry (std::shared_ptr<MeshGeometry> geometry) override { meshGeometry = geometry; }
    void setBoundaryCondition (std::shared_ptr<BoundaryCondition> bc) override
    {
        if      (dynamic_cast<const PeriodicBoundaryCondition*> (bc.get())) bcKind = MARA_BC_PERIODIC;
        else if (dynamic_cast<const OutflowBoundaryCondition*>  (bc.get())) bcKind = MARA_BC_OUTFLOW;
        else throw std::logic_error ("GpuConstrainedTransport: periodic or outflow boundaries only");
    }

    void assignCellCenteredB (Cow::Array newB) override
    {
        if (! meshGeometry) throw std::logic_error ("GpuConstrainedTransport: no mesh geometry");
        const auto cells = meshGeometry->cellsShape();
        if (newB.size (0) != cells[0] || newB.size (1) != cells[1] || newB.size (2) != cells[2] || newB.size (3) != 3)
            throw std::logic_error ("GpuConstrainedTransport: field shape does not match the mesh");
        B = std::move (newB);
    }

    Cow::Array computeMonopole (MeshLocation location) const override
    {
        int n[3];
        shape (n);
        if (location != MeshLocation::vert && location != MeshLocation::cell)
            throw std::logic_error ("Mesh location for monopole calculation not cell or vert");
        const int v = location == MeshLocation::vert ? 1 : 0;
        auto M = Cow::Array (n[0] + v, n[1] + v, n[2] + v);
        check (mara_gpu_ct_monopole (B.data(), n, bcKind, v ? 0 : 1, M.data(), device));
        return M;
    }

    Cow::Array computeCurrent (MeshLocation location) const override
    {
        if (location != MeshLocation::cell)
            throw std::logic_error ("Mesh location for current calculation not cell");
        int n[3];
        shape (n);
        auto J = Cow::Array (n[0], n[1], n[2], 3);
        check (mara_gpu_ct_current (B.data(), n, bcKind, 1.0, J.data(), device));
        return J;
    }

private:
    void shape (int n[3]) const
    {
        if (B.size() == 0) throw std::logic_error ("GpuConstrainedTransport: no field assigned");
        for (int a = 0; a < 3; ++a) n[a] = B.size (a);
    }
    static void check (int status)
    {
        if (status != MARA_OK)
            throw std::logic_error (std::string ("GpuConstrainedTransport: ") + mara_gpu_status_string (status));
    }
    int device = 0;
    int bcKind = MARA_BC_PERIODIC;
    std::shared_ptr<MeshGeometry> meshGeometry;
    Cow::Array B;
};
