/*
 * mara_gpu.h -- C ABI of the GB300-native Mara2 finite-volume time step.
 *
 * The drop-in boundary is Mara2's SolutionScheme interface
 * (src/Mara.hpp:87-97): a GPU MethodOfLinesTVD whose advance() mutates
 * MeshData::P in place, plus the separate FieldOperator::getCourantTimestep
 * call that drivers make for dt (src/FieldOperator.hpp:80).  Every entry
 * point takes plain pointers and sizes, returns an int status (0 = success)
 * and never throws; the C++ wrapper in mara2_gb300/csrc/GpuSolutionScheme.hpp
 * turns statuses back into the reference's exception types.
 *
 * Array layout at the boundary is the reference's MeshData::P: FP64 AoS
 * (ni+2g0, nj+2g1, nk+2g2, nq) in C order, q fastest, guard zones only on
 * axes with more than one interior cell (src/MeshData.cpp:8-28).  On the
 * device the state is kept structure-of-arrays with x fastest.
 *
 * A handle owns one CUDA stream and its device memory; it is not
 * thread-safe.  Calls on one handle are ordered on its stream.
 */
#ifndef MARA_GPU_H
#define MARA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ConservationLaw subclasses: NewtonianHydro, NewtonianMHD, RelativisticMHD
 * (src/ConservationLaws.hpp:25-100) */
enum { MARA_LAW_HYDRO = 0, MARA_LAW_MHD = 1, MARA_LAW_RMHD = 2 };
/* IntercellFluxScheme: MethodOfLines (PCM), MethodOfLinesPlm, and the WENO5
 * primitive-reconstruction composition (src/IntercellFluxSchemes.hpp) */
enum { MARA_RECON_PCM = 0, MARA_RECON_PLM = 1, MARA_RECON_WENO5 = 2 };
/* RiemannSolver: HlleRiemannSolver, HllcNewtonianHydroRiemannSolver
 * (src/RiemannSolvers.hpp:27-50) */
enum { MARA_RIEMANN_HLLE = 0, MARA_RIEMANN_HLLC = 1 };
/* BoundaryCondition: Periodic, Outflow, Reflecting (src/BoundaryConditions.hpp) */
enum { MARA_BC_PERIODIC = 0, MARA_BC_OUTFLOW = 1, MARA_BC_REFLECTING = 2 };
/* Reconstruction::SmoothnessIndicator (src/Reconstruction.hpp) */
enum { MARA_WENO_JS96 = 0, MARA_WENO_BORGES08 = 1, MARA_WENO_SHENZHA10 = 2 };
/* arithmetic of the step */
enum {
    MARA_PRECISION_FP64 = 0,  /* plain: matches the reference's FP64 CPU path  */
    MARA_PRECISION_MIXED = 1, /* FP32 reconstruction/Riemann/flux arithmetic,
                                 compensated FP32 pair (hi+lo, ~48 bits)
                                 conserved-state accumulator; RMHD recovery
                                 with its Newton residuals in FP32 pairs and
                                 the FP64 iteration as fallback               */
    MARA_PRECISION_MIXED_FP64 = 2 /* FP32 reconstruction/Riemann/flux
                                 arithmetic, FP64 conserved-state accumulator
                                 and FP64 RMHD Newton iteration (the same 8
                                 bytes per field as the pair)                 */
};

/* Status codes.  1..8 mirror ConsToPrimRMHD's enum (src/ConsToPrimRMHD.hpp:
 * 9-20); 16..20 name the exceptions the reference throws on this path. */
enum {
    MARA_OK = 0,
    MARA_C2P_CONS_CONTAINS_NAN = 1,
    MARA_C2P_CONS_NEGATIVE_DENSITY = 2,
    MARA_C2P_CONS_NEGATIVE_ENERGY = 3,
    MARA_C2P_PRIM_CONTAINS_NAN = 4,
    MARA_C2P_PRIM_NEGATIVE_PRESSURE = 5,
    MARA_C2P_PRIM_NEGATIVE_RESTMASS = 6,
    MARA_C2P_PRIM_SUPERLUMINAL = 7,
    MARA_C2P_MAXITER = 8,
    MARA_ERR_INVERSION_FAILURE = 16, /* FieldOperator::InversionFailure       */
    MARA_ERR_SUPERLUMINAL = 17,      /* std::runtime_error, superluminal      */
    MARA_ERR_BAD_EIGENVALUES = 18,   /* std::runtime_error, bad eigenvalues   */
    MARA_ERR_GUARD_TOO_SMALL = 19,   /* std::logic_error from makeFootprint   */
    MARA_ERR_CONFIG = 20,            /* std::logic_error, bad configuration   */
    MARA_ERR_CUDA = 32,              /* a CUDA runtime call failed            */
    MARA_ERR_NO_DEVICE = 33,
    MARA_ERR_ARGUMENT = 34,
    MARA_ERR_TOO_LARGE = 35
};

typedef struct MaraGpuConfig {
    int law, recon, riemann, bc;
    int rk_order;        /* MethodOfLinesTVD::setRungeKuttaOrder: 1, 2, 3     */
    int disable_ct;      /* MethodOfLinesTVD::setDisableFieldCT              */
    int weno_is;         /* MARA_WENO_*                                      */
    int ni, nj, nk;      /* interior cells (CartesianMeshGeometry cellsShape) */
    int ng[3];           /* guard zones per axis (MeshData boundaryShape)     */
    double lower[3], upper[3];   /* CartesianMeshGeometry::setLowerUpper     */
    double gamma;        /* ConservationLaw::setGammaLawIndex                */
    double plm_theta;    /* IntercellFluxScheme::setPlmTheta                 */
    double shenzha_A;    /* Reconstruction::setShenZha10A                    */
    double pressure_floor; /* ConservationLaw::setPressureFloor              */
    int precision;       /* MARA_PRECISION_*                                 */
    int device;          /* CUDA device ordinal                              */
    double cooling_rate; /* NewtonianMHD::setCoolingRate (ConservationLaws.cpp:
                            355-358, 489-501): > 0 adds the auxiliary field 8
                            and the cooling source terms (plain FP64 path;
                            MHD only, ignored by the other laws); <= 0 none  */
} MaraGpuConfig;

typedef struct MaraGpuStats {
    int status;          /* status of the last advance                       */
    int failures;        /* zones whose primitive recovery failed            */
    int first_zone[3];   /* interior-relative index of the lowest failed zone */
    int first_code;      /* status of that zone                              */
    int64_t steps;       /* advances done on this handle                     */
    int64_t kernel_launches; /* kernels this handle has launched             */
    double last_dt;
} MaraGpuStats;

typedef struct MaraGpuHandle MaraGpuHandle;

/* Replaces the construction of MethodOfLinesTVD + its injected operators
 * (SolutionSchemes.hpp:49-72, Mara.hpp:44-51).  Validates the configuration
 * like SchemeHelpers::makeFootprint (SolutionSchemes.cpp:17-49). */
int mara_gpu_create(const MaraGpuConfig* config, MaraGpuHandle** handle);
int mara_gpu_destroy(MaraGpuHandle* handle);

/* Host <-> device copies of MeshData::P (with guards, AoS FP64).  A
 * page-locked array (cudaHostAlloc / cudaHostRegister) is read or written
 * in place by the layout-conversion kernels over the chip-to-chip link; a
 * pageable one goes through a device staging buffer in chunks.  upload may
 * still be reading the array when it returns: the next call that
 * synchronises the handle (download, synchronize, courant, run, stats)
 * marks the end. */
int mara_gpu_upload(MaraGpuHandle* h, const double* P_aos);
int mara_gpu_download(MaraGpuHandle* h, double* P_aos);

/* Page-lock a host array (MeshData::P) of `bytes` bytes, or undo it, so that
 * the host calls above and mara_gpu_advance_host read and write it in place
 * (cudaHostRegister, mapped).  MARA_ERR_CUDA if the driver refuses. */
int mara_gpu_host_register(void* p, size_t bytes);
int mara_gpu_host_unregister(void* p);

/* MethodOfLinesTVD::advance (SolutionSchemes.cpp:108-275) on the resident
 * state: every RK stage, flux CT when the law is magnetic, primitive recovery
 * and the guard fill.  Asynchronous; the status of earlier steps is reported
 * by the next synchronising call. */
int mara_gpu_advance(MaraGpuHandle* h, double t0, double dt);

/* The drop-in form of advance: P_aos (host) in, advanced P_aos out, as
 * SolutionScheme::advance(MeshData&, t0, dt) does on MeshData::P.  Copies in,
 * advances, copies back and synchronises.  On a page-locked array of a 2-D
 * mixed-precision hydro grid (PCM / PLM, at least 128 zones along x and
 * 2^19 zones in all) the transfers in, the RK stages and the transfers out
 * are pipelined in one launch; the array receives the same bits as upload +
 * advance + download. */
int mara_gpu_advance_host(MaraGpuHandle* h, double* P_aos, double t0, double dt);

/* FieldOperator::getCourantTimestep (FieldOperator.cpp:125-169) with
 * L = MeshOperator::linearCellDimension, on the resident state (without the
 * driver's CFL factor).  Synchronises. */
int mara_gpu_courant(MaraGpuHandle* h, double* dt);

/* Device-resident driver loop (the regression drivers' timestep/advance
 * pair, src/Problems.cpp:181-188): up to max_steps steps of
 * dt = min(cfl * courant, t_final - t) while t < t_final (t_final < 0 means
 * no end time).  dt never leaves the device.  *t is read and updated. */
int mara_gpu_run(MaraGpuHandle* h, int max_steps, double cfl, double t_final, double* t, int* steps_done);

/* The same loop without waiting: the steps are enqueued on the handle's
 * stream and the call returns at once (t and the status are read by the next
 * mara_gpu_run, mara_gpu_synchronize or mara_gpu_stats). */
int mara_gpu_run_async(MaraGpuHandle* h, int max_steps, double cfl, double t_final);

/* Wait for the handle's stream; returns the first error seen. */
int mara_gpu_synchronize(MaraGpuHandle* h);
int mara_gpu_stats(MaraGpuHandle* h, MaraGpuStats* stats);

/* The handle's cudaStream_t, for callers that time or order work on it. */
void* mara_gpu_stream(MaraGpuHandle* h);

/* Optional per-kernel timing with CUDA events around each launch of the
 * stage kernels (off by default).  ms_total/launches are per kernel class:
 * [0] flux / stage kernels, [1] update, [2] courant. */
int mara_gpu_set_kernel_timing(MaraGpuHandle* h, int enable);
int mara_gpu_kernel_times(MaraGpuHandle* h, double ms_total[3], int64_t launches[3]);

/* CellCenteredFieldCT::monopole (MeshLocation::cell, CellCenteredFieldCT.cpp:
 * 159-223) of the resident magnetic field, reduced to the largest |div B| over
 * the interior zones; mesh_spacing is CellCenteredFieldCT::setMeshSpacing
 * (the reference's default is 1).  MHD and RMHD only. */
int mara_gpu_monopole(MaraGpuHandle* h, double mesh_spacing, double* max_abs);

/* ---- initial data generated on the device ----------------------------------
 * MeshOperator::generate (MeshOperator.cpp:168-189) of a built-in initial
 * data function at every cell centre, guards filled as
 * BoundaryCondition::applySimple does, then loaded like mara_gpu_upload: the
 * synthetic problems start without a host array or a host-to-device copy.
 * Cell centre: lower + dx (i + 0.5) per axis (CartesianMeshGeometry).
 *   PLANAR_RIEMANN  left where (x - x0) . normal < 0, right elsewhere
 *                   (shock tubes, Problems.cpp:37-87; oblique interfaces)
 *   SHEAR_LAYER     left where |y - x0[1]| < radius, right elsewhere; with
 *                   noise != 0, interior zone (i, j, k) gets velocity2 =
 *                   (-1 + 2 u) noise, u the top 53 bits of the
 *                   ((i nj + j) nk + k + 1)-th SplitMix64 output of seed
 *                   times 2^-53 (Kelvin-Helmholtz)
 *   CYLINDER        left where sqrt((x - x0)^2 + (y - y0)^2) < radius, right
 *                   elsewhere (cylindrical blast waves, Problems.cpp:350-375)
 * States are primitives (nq values). */
enum { MARA_INIT_PLANAR_RIEMANN = 1, MARA_INIT_SHEAR_LAYER = 2, MARA_INIT_CYLINDER = 3 };

typedef struct MaraInitialData {
    int kind;
    double left[8];
    double right[8];
    double x0[3];
    double normal[3];
    double radius;
    double noise;
    unsigned long long seed;
} MaraInitialData;

int mara_gpu_generate(MaraGpuHandle* h, const MaraInitialData* data);

/* ---- source terms ----------------------------------------------------------
 * MethodOfLinesTVD::setSourceTermsFunction (SolutionSchemes.hpp:36; applied
 * at SolutionSchemes.cpp:219-228): once per RK stage the scheme evaluates the
 * source terms S from the stage's primitives and adds them to the flux
 * divergence L before the RK combine, U = U0 (1 - b) + (U + dt (L + S)) b.
 * The reference calls a per-cell host function; here the caller's function
 * is called on the host each time a stage is enqueued (also while a step is
 * captured into a CUDA graph, whose replays then repeat what it enqueued) and
 * must enqueue device work on args->stream that writes S, without
 * synchronising.  A non-zero return ends the call that enqueued the stage
 * with that status.  Plain FP64 path only (MARA_ERR_CONFIG on a mixed
 * handle). */
typedef struct MaraSourceTermsArgs {
    const double* P;   /* device: the stage's primitives with guards, SoA,
                          P[q * sP + (k * N[1] + j) * N[0] + i]              */
    double* S;         /* device: source terms, the same layout; zero until
                          written; the interior cells are added to L          */
    long long sP;      /* field stride                                        */
    int N[3];          /* cells per axis including guards                     */
    int ng[3];         /* guard cells per axis                                */
    int nq;            /* fields                                              */
    double lower[3];   /* the centre of cell (i, j, k) along axis a is
                          lower[a] + dx[a] * ((i - ng[a]) + 0.5), as
                          coordinateAtIndex with the start index of
                          SchemeHelpers::makeFootprint gives it               */
    double dx[3];
    double aux[8];     /* the auxiliary data the reference passes (star
                          particles): zeros                                   */
    void* stream;      /* the handle's cudaStream_t                           */
} MaraSourceTermsArgs;

typedef int (*MaraSourceTermsFn)(void* user, const MaraSourceTermsArgs* args);

/* Installs fn (NULL removes it); user is passed back unchanged.  Captured
 * step graphs are rebuilt on the next run. */
int mara_gpu_set_source_terms(MaraGpuHandle* h, MaraSourceTermsFn fn, void* user);

/* A ready-made source terms function: a uniform gravitational acceleration
 * g = ((const double*) user)[0..2], read when the stage is enqueued:
 * S = (0, rho g1, rho g2, rho g3, rho (v1 g1 + v2 g2 + v3 g3), 0, ...). */
int mara_source_uniform_gravity(void* user, const MaraSourceTermsArgs* args);

/* Number of volume-integrated diagnostics the law lists
 * (ConservationLaw::getDiagnosticNames, ConservationLaws.cpp:332-341,
 * 576-601, 924-945): 5 for hydro (mass, momentum1-3, total_energy), 17 for
 * MHD and RMHD (those, magnetic_flux1-3, kinetic_energy, internal_energy,
 * magnetic_energy, sound_speed, alfven_speed, sonic_mach_number,
 * alfven_mach_number, specific_entropy, cross_helicity). */
int mara_gpu_num_diagnostics(const MaraGpuHandle* h);

/* FieldOperator::volumeIntegratedDiagnostics (FieldOperator.cpp:171-205) of
 * the resident state over the interior zones: per zone makeDiagnostics of
 * fromPrimitive(P), times the cell volume, summed (totals equal the
 * reference's to rounding; the summation order differs).  On the mixed path
 * P is the FP64 state a download returns.  D holds mara_gpu_num_diagnostics
 * values; *count (if not NULL) receives that number.  A zone whose state the
 * law rejects makes the call return its status code. */
int mara_gpu_volume_diagnostics(MaraGpuHandle* h, double* D, int* count);

/* The cell diagnostic fields a checkpoint carries (the reference's checkpoint
 * task, src/Problems/MagneticBraiding.cpp:176-189):
 * CellCenteredFieldCT::monopole and ::current at cell centres
 * (CellCenteredFieldCT.cpp:159-257) of the resident magnetic field at every
 * cell of the array with guards, as FP64 AoS (ni+2g, nj+2g, nk+2g, 4) =
 * [monopole, current1, current2, current3].  MHD and RMHD only. */
int mara_gpu_field_diagnostics(MaraGpuHandle* h, double mesh_spacing, double* out_aos);

/* Device bytes the handle holds. */
int64_t mara_gpu_device_bytes(const MaraGpuHandle* h);

/* One plain-FP64 advance (the same arithmetic as mara_gpu_advance) on
 * device buffers the caller owns, for callers that cannot allocate device
 * memory when they step a grid: an application whose memory pool already
 * reserves the GPU, a latency-critical loop that must not block in or fail
 * inside an allocation, code that must avoid cudaFree's device-wide
 * synchronisation.  P_in and P_out are device pointers to MeshData::P in the
 * layout above (they may be the same buffer); stream may be 0.  All
 * intermediates live in a fixed 64 MiB scratch array inside the library's
 * device image (held on every GPU that loads the library until the process
 * exits); grids whose intermediates exceed it return MARA_ERR_TOO_LARGE.
 * Calls share that array, so calls whose GPU work overlaps race: order them
 * on one stream.  Each call looks the array's address up with
 * config->device current (a host-side query, no allocation) and restores
 * the caller's current device before it returns; the first call on a
 * device may load the library's device image there, so make it before any
 * stream capture.  Synchronises the stream and returns the step's status
 * (MARA_ERR_CUDA only for this call's own launches and copies).  No counterpart in the reference:
 * it exists for callers of this library that cannot allocate. */
int mara_gpu_advance_noalloc(const MaraGpuConfig* config, const double* P_in, double* P_out,
                             double dt, void* stream);

/* ---- the ConstrainedTransport interface (src/Mara.hpp:341-349) -------------
 * Device forms of UniformCartesianCT (src/ConstrainedTransport.cpp), the
 * reference's implementation of the interface: a cell-centred field B (host,
 * AoS (n[0], n[1], n[2], 3)) as assignCellCenteredB receives it, given one
 * guard zone on every axis by the boundary condition (MARA_BC_PERIODIC or
 * MARA_BC_OUTFLOW; MARA_ERR_CONFIG otherwise).
 *   mara_gpu_ct_monopole: computeMonopole (ConstrainedTransport.cpp:81-89,
 *     302-377) at vertices (location 0; M (n+1)^3 values) or cells
 *     (location 1; M n^3 values).
 *   mara_gpu_ct_current: computeCurrent as CellCenteredFieldCT::current
 *     (CellCenteredFieldCT.cpp:231-257) with the given mesh spacing at the
 *     interior cells (J (n[0], n[1], n[2], 3)).  UniformCartesianCT's own
 *     computeCurrent (ConstrainedTransport.cpp:91-117) reads components 1..3
 *     of a 3-component array and offsets -1..+1 of a 0..2 stencil window, so
 *     it has no defined result to follow.
 * Synchronous; the caller's current device is kept. */
int mara_gpu_ct_monopole(const double* B, const int n[3], int bc, int location, double* M, int device);
int mara_gpu_ct_current(const double* B, const int n[3], int bc, double mesh_spacing, double* J, int device);

/* The divergence-free initial field of the reference's MHD drivers
 * (src/Problems.cpp:660-667) on the resident state: the face-centred vector
 * potential A (host, MeshOperator::generate(ivp, face, scalars, guards):
 * (N0+1, N1+1, N2+1, 3, 3) over the cells with guards, component then face
 * axis) becomes Godunov fluxes (CellCenteredFieldCT::vectorPotentialToFluxes,
 * CellCenteredFieldCT.cpp:136-150), flux CT (generateGodunovFluxes, :152-157)
 * and their divergence (MeshOperator::divergence, factor 1), times scale;
 * the result replaces the magnetic field of every interior cell
 * (MeshData::assignMagneticField) and the guards are refilled by the boundary
 * condition (applyBoundaryCondition).  MHD and RMHD handles, either
 * precision; the arithmetic is FP64 and gives the reference's bits. */
int mara_gpu_assign_vector_potential(MaraGpuHandle* h, const double* A, double scale);

/* The FP64 pipe's throughput in TFLOP/s (one FMA counted as two flops),
 * measured with independent FMA chains in every thread of eight CTAs per SM:
 * the ceiling the plain FP64 path's arithmetic runs against.  No counterpart
 * in the reference; the benchmark reports the plain path against it. */
int mara_gpu_fp64_peak(int device, double* tflops);

/* QuarticPolynomial::solve (src/QuarticPolynomial.cpp:19-144) on the device
 * for n quartics d4 x^4 + d3 x^3 + d2 x^2 + d1 x + d0: coeffs (host) holds
 * (d4, d3, d2, d1, d0) per quartic; roots (host) receives 4 values per
 * quartic, the real roots in ascending order first (the rest 0), nroots
 * (host) their number (0, 2 or 4).  The same device function as the RMHD
 * eigenvalues of the plain path (its pow(x, 1/3), acos, cos and sin
 * correctly rounded).  Synchronous; the caller's current device is kept. */
int mara_gpu_quartic_solve(const double* coeffs, int n, double* roots, int* nroots, int device);

const char* mara_gpu_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif
