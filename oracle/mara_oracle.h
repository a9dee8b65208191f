/*
 * mara_oracle.h -- CPU restatement of Mara2's finite-volume time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * implementation in mara2_gb300/: only tests, the smoke check and the
 * CPU-baseline leg of bench.py may load it.  The product path never calls
 * it and has no CPU fallback.
 *
 * Parity is pinned two ways (see oracle/README.md):
 *   1. oracle/ref_harness.cpp compiles the reference's own hot-path
 *      translation units in place (against the clean-room container shim in
 *      oracle/cowshim/) and exposes the same entry points with an "mr_"
 *      prefix; tests/test_oracle_vs_ref.py checks the two bit-for-bit and
 *      tests/golden/ holds fixtures produced by the reference build.
 *   2. the known answers of the reference's own unit tests
 *      (src/TestSuite.cpp) are re-asserted in tests/test_oracle_known.py.
 *
 * Data layout is the reference's MeshData::P: an AoS array of shape
 * (ni+2g0, nj+2g1, nk+2g2, nq) in C order (i slowest, q fastest), FP64,
 * with guard zones only on axes whose interior size is > 1.
 */
#ifndef MARA_ORACLE_H
#define MARA_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { MO_LAW_HYDRO = 0, MO_LAW_MHD = 1, MO_LAW_RMHD = 2 };
enum { MO_RECON_PCM = 0, MO_RECON_PLM = 1, MO_RECON_WENO5 = 2 };
enum { MO_RIEMANN_HLLE = 0, MO_RIEMANN_HLLC = 1 };
enum { MO_BC_PERIODIC = 0, MO_BC_OUTFLOW = 1, MO_BC_REFLECTING = 2 };
enum { MO_WENO_JS96 = 0, MO_WENO_BORGES08 = 1, MO_WENO_SHENZHA10 = 2 };

/* Status codes.  1..8 mirror ConsToPrimRMHD's error enum
 * (src/ConsToPrimRMHD.hpp:9-20); the rest name the reference's exceptions. */
enum {
    MO_OK = 0,
    MO_C2P_CONS_CONTAINS_NAN = 1,
    MO_C2P_CONS_NEGATIVE_DENSITY = 2,
    MO_C2P_CONS_NEGATIVE_ENERGY = 3,
    MO_C2P_PRIM_CONTAINS_NAN = 4,
    MO_C2P_PRIM_NEGATIVE_PRESSURE = 5,
    MO_C2P_PRIM_NEGATIVE_RESTMASS = 6,
    MO_C2P_PRIM_SUPERLUMINAL = 7,
    MO_C2P_MAXITER = 8,
    MO_ERR_INVERSION_FAILURE = 16, /* FieldOperator::InversionFailure        */
    MO_ERR_SUPERLUMINAL = 17,      /* runtime_error "got superluminal velocity" */
    MO_ERR_BAD_EIGENVALUES = 18,   /* runtime_error "got bad eigenvalues"   */
    MO_ERR_GUARD_TOO_SMALL = 19,   /* logic_error from makeFootprint        */
    MO_ERR_CONFIG = 20
};

typedef struct mo_config {
    int law;            /* MO_LAW_*                                     */
    int recon;          /* MO_RECON_*                                   */
    int riemann;        /* MO_RIEMANN_*                                 */
    int bc;             /* MO_BC_*                                      */
    int rk_order;       /* 1, 2 or 3                                    */
    int disable_ct;     /* MethodOfLinesTVD::setDisableFieldCT          */
    int weno_is;        /* MO_WENO_* smoothness indicator               */
    int ni, nj, nk;     /* interior cells per axis                      */
    int ng[3];          /* guard width per axis (0 on flat axes)        */
    double lower[3];
    double upper[3];
    double gamma;       /* gamma-law index                              */
    double plm_theta;
    double shenzha_A;
    double pressure_floor;
    double cooling_rate; /* NewtonianMHD::setCoolingRate: > 0 adds the     */
                         /* auxiliary field 8 and the cooling source terms  */
} mo_config;

typedef struct mo_failure {
    int count;          /* zones whose inversion failed in the last stage */
    int first[3];       /* interior-relative index of the first failure   */
    int code;           /* status of the first failure                    */
} mo_failure;

int mo_num_fields(const mo_config* c);
int mo_stencil_size(const mo_config* c);

/* Source terms function (MethodOfLinesTVD::setSourceTermsFunction): cell
 * centre, auxiliary data, primitives (MARA_NUM_FIELDS slots) -> source terms
 * added to L.  NULL removes it.  Applies to every later mo_advance. */
typedef void (*mo_source_fn)(void* user, double x, double y, double z, const double aux[8], const double* P,
                             double* S);
void mo_set_source_terms(mo_source_fn fn, void* user);

/* MethodOfLinesTVD::advance (src/SolutionSchemes.cpp:108-275) on the AoS
 * array P (with guards), in place. */
int mo_advance(const mo_config* c, double* P, double t0, double dt, mo_failure* fail);

/* FieldOperator::getCourantTimestep (src/FieldOperator.cpp:125-169) over the
 * interior of P with L = MeshOperator::linearCellDimension. */
int mo_courant(const mo_config* c, const double* P, double* dt);

/* MeshData::applyBoundaryCondition -> BoundaryCondition::applySimple. */
int mo_apply_bc(const mo_config* c, double* P);

/* MeshOperator::godunov (+ CellCenteredFieldCT::correctGodunovFluxes when the
 * law has a magnetic field and CT is enabled).  F has shape
 * (NI+1, NJ+1, NK+1, nq, 3). */
int mo_godunov(const mo_config* c, const double* P, double* F);

/* FieldOperator::generateConserved over every cell of P. */
int mo_generate_conserved(const mo_config* c, const double* P, double* U);

/* ConservationLaw::fromPrimitive for one state along normal n. */
int mo_from_primitive(const mo_config* c, const double* P, const double n[3],
                      double* U, double* F, double* A);

/* ConservationLaw::fromConserved for one state (recovered primitive only). */
int mo_from_conserved(const mo_config* c, const double* U, double* P, int* health);

/* QuarticPolynomial::solve (src/QuarticPolynomial.cpp:19-103). */
int mo_quartic(double d4, double d3, double d2, double d1, double d0, double roots[4]);

/* CellCenteredFieldCT::correctGodunovFluxes on a flux array of shape
 * (n0, n1, n2, nq, 3). */
void mo_ct_correct(double* F, int n0, int n1, int n2, int nq, int ib);

/* CellCenteredFieldCT::monopole with MeshLocation::cell on cell data B of
 * shape (n0, n1, n2, 3); M has shape (n0, n1, n2). */
void mo_monopole_cell(const double* B, int n0, int n1, int n2, double mesh_spacing, double* M);

/* Number of diagnostics ConservationLaw::getDiagnosticNames lists. */
int mo_num_diagnostics(const mo_config* c);

/* FieldOperator::volumeIntegratedDiagnostics (src/FieldOperator.cpp:171-205)
 * over the interior of P; D (and Dabs, the sum of the terms' magnitudes, if
 * not NULL) hold mo_num_diagnostics values. */
int mo_volume_diagnostics(const mo_config* c, const double* P, double* D, double* Dabs);

/* CellCenteredFieldCT::current (src/CellCenteredFieldCT.cpp:231-257) of cell
 * data B (n0, n1, n2, 3); J has the same shape. */
void mo_current_cell(const double* B, int n0, int n1, int n2, double mesh_spacing, double* J);

/* UniformCartesianCT (src/ConstrainedTransport.cpp) on a cell-centred field
 * Bc (n0, n1, n2, 3) given at the interior cells (assignCellCenteredB) with
 * periodic or outflow guards: computeMonopole at vertices (location 0; M
 * (n0+1, n1+1, n2+1)) or cells (location 1; M (n0, n1, n2)). */
int mo_uct_monopole(const double* Bc, int n0, int n1, int n2, int bc, int location, double* M);

/* The current operator of that adaptor: CellCenteredFieldCT::current
 * (src/CellCenteredFieldCT.cpp:231-257) with mesh spacing h of the guarded
 * field, at the interior cells; J (n0, n1, n2, 3). */
int mo_uct_current(const double* Bc, int n0, int n1, int n2, int bc, double h, double* J);

/* B = scale x divergence(CT(vectorPotentialToFluxes(A))) at every cell with
 * guards (src/Problems.cpp:660-667); A (N0+1, N1+1, N2+1, 3, 3), B (N0, N1,
 * N2, 3). */
int mo_vector_potential_to_cell_b_scaled(const mo_config* c, const double* A, double scale, double* B);

/* Face-normal unit vectors as CartesianMeshGeometry::faceNormal returns them
 * (UnitVector::xhat/yhat/zhat, src/UnitVector.cpp:9-11,32-39). */
void mo_face_normals(double n[3][3]);

/* Total threads the oracle's OpenMP loops may use (1 without OpenMP). */
int mo_max_threads(void);
void mo_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
