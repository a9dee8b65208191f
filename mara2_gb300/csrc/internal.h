// internal.h -- declarations shared by the CUDA translation units of the
// library (not part of the public C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mara_gpu.h"

namespace mara {

// Mesh description passed by value to every kernel.  Device arrays are
// structure-of-arrays with x fastest:
//   P (with guards)   P[q * sP + (k * N1 + j) * N0 + i]
//   U (interior only) U[q * sU + (k * n1 + j) * n0 + i]
//   F_a (face fluxes) F[q * sF + (k * (N1+1) + j) * (N0+1) + i], face i is
//                     the left face of cell i along axis a
struct GridDesc {
    int n[3];          // interior cells
    int g[3];          // guard cells (0 on flat axes)
    int N[3];          // n + 2 g
    long long sP, sU, sF;
    double nrm[3][3];  // face normals exactly as the reference builds them
    double dA[3], dV;  // CartesianMeshGeometry face areas and volume
    double lmin;       // MeshOperator::linearCellDimension
    int bc;
    int ct;            // flux CT on the magnetic fluxes
    int nq;
};

// Device-side status of a handle: the first error and the inversion-failure
// bookkeeping of FieldOperator::recoverPrimitive.
struct DevStatus {
    int code;                       // first non-zero status (0 = ok)
    int failures;                   // zones whose recovery failed
    int first_code;                 // status of the lowest failed zone
    int done;                       // driver loop reached t_final
    unsigned long long first_zone;  // lowest failed interior zone, linear
    unsigned long long dt_bits;     // Courant reduction (min of positive doubles)
    double t;                       // driver-loop time
    double dt;                      // dt of the current step
    long long steps;                // driver-loop steps taken
    long long taken;                // steps that ran since the host last read the
                                    // status: a step enqueued after t_final (or an
                                    // error) does no work, so the ping-pong parity
                                    // of the state follows this count, not the
                                    // number of steps the host enqueued
    int halt;                       // a previous stage had inversion failures: the
                                    // step stops there, as the reference's
                                    // InversionFailure ends MethodOfLinesTVD::advance
};

struct PhysParamsH {
    double gamma, plm_theta, shenzha_A, pressure_floor;
    int weno_is;
    double cooling_rate;
};

// ---- plain FP64 path (plain_fp64.cu) -----------------------------------------
void plain_flux(int law, int recon, int riemann, int axis, const GridDesc& G, const PhysParamsH& pp,
                const double* P, double* F, DevStatus* st, cudaStream_t s);
void plain_update(int law, const GridDesc& G, const PhysParamsH& pp, const double* Pin, double* Pout,
                  double* U0, double* U, const double* Fx, const double* Fy, const double* Fz,
                  double b, int stage, const double* dt, DevStatus* st, cudaStream_t s,
                  const double* S = nullptr);
void plain_courant(int law, const GridDesc& G, const PhysParamsH& pp, const double* P, DevStatus* st,
                   cudaStream_t s);

// ---- diagnostics (diagnostics.cu) ----------------------------------------------
void launch_monopole_max(const void* P, bool fp32, const GridDesc& G, double h, unsigned long long* out,
                         cudaStream_t s);
// monopole and current at every cell of the array with guards, FP64 AoS
// (N0, N1, N2, 4)
void launch_field_diag(const void* P, bool fp32, const GridDesc& G, double h, double* out, cudaStream_t s);
// volume-integrated diagnostics of the plain path's primitives: per-block
// partial sums (DIAG_BLOCKS x 17 doubles), the first error code, the totals
void launch_volume_diag_plain(int law, const double* P, const GridDesc& G, const PhysParamsH& pp, double* partial,
                              int* err, double* out, cudaStream_t s);

// ---- shared helpers (mara_gpu.cu) --------------------------------------------
// the law the kernels are instantiated for (LAW_MHD_COOL for NewtonianMHD
// with a positive cooling rate) and the physics parameters of a configuration
int kernel_law(const MaraGpuConfig* c);
void make_phys(const MaraGpuConfig* c, PhysParamsH* pp);
void launch_courant_init(DevStatus* st, cudaStream_t s);
void launch_dt_from_courant(DevStatus* st, double cfl, double t_final, cudaStream_t s);
void launch_set_dt(DevStatus* st, double dt, cudaStream_t s);
void launch_advance_time(DevStatus* st, cudaStream_t s);
void launch_aos_to_soa(const double* aos, double* soa, const GridDesc& G, cudaStream_t s);
void launch_aos_to_soa_range(const double* aos, double* soa, const GridDesc& G, long long c0, long long c1,
                             cudaStream_t s);
void launch_soa_to_aos_range(const double* soa, double* aos, const GridDesc& G, long long c0, long long c1,
                             cudaStream_t s);
void launch_soa_to_aos(const double* soa, double* aos, const GridDesc& G, cudaStream_t s);

} // namespace mara
