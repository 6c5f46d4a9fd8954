// ccs_kernels.h -- launch descriptors shared by the kernels and the C ABI layer.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "ccs_internal.h"

namespace ccs {

// Raises a kernel's dynamic shared-memory limit once per device: the attribute is
// held per device, so a process driving handles on several devices sets it on each
// (`done` is the kernel's own set of device bits; ordinals above 63 set it every
// launch).
inline cudaError_t smem_attr_once(const void *fn, int smem, std::atomic<uint64_t> &done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = dev >= 0 && dev < 64 ? (uint64_t)1 << dev : 0;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

// One tile of work: instance, panel (0..5) and tile coordinates.
struct WorkItem {
  int16_t inst, panel, tx, ty;
};

// Stage kinds.  RK4 (time_scheme_mod.F90:13-44) keeps the running combination
// acc = k1 (+ 2 k2) (+ 2 k3) so that the final (acc + k4) / 6 has the reference's
// association ((k1 + 2k2) + 2k3) + k4.  RK3-TVD follows :46-67, 85-115.
enum StageKind {
  K_RK4_1 = 0,  // acc = k;          Y = Y0 + c1 k
  K_RK4_2 = 1,  // acc = acc + 2 k;  Y = Y0 + c1 k
  K_RK4_4 = 2,  // Y = Y0 + c1 ((acc + k) / 6)
  K_RK3_1 = 3,  // Y = Y0 + c1 k
  K_RK3_2 = 4,  // Y = 0.75 Y0 + 0.25 Yc + c1 k
  K_RK3_3 = 5,  // Y = Y0 / 3 + 2/3 Yc + c1 k
  K_TEND = 6    // write k only
};

// FP64 lane: everything one instance's stage launch needs.
struct F64Stage {
  Layout L;
  MeshF64 m;
  StateF64 in;   // stencil input Y_k
  StateF64 out;  // Y_{k+1} (may alias the Y0 slot: only the own cell of Y0 is read)
  const double *y0phiG, *y0u, *y0v;
  double *accphiG, *accu, *accv;
  double *zonal, *merid;  // sphere winds of Y_{k+1} when non-null
  double *tphiG, *tu, *tv;
  double dx, dy, dx60, dy60, c1;
  double rdx, rdy, rdx60, rdy60;  // RN(1 / dx) etc.: the divisions by them are corrected to IEEE
  int kind, ediss;
  int op;  // CCS_OP_WENO, or the central-difference order 2 / 4 / 6
};

// Mixed lane: one instance's stage launch.
struct MixedStage {
  Layout L;
  MeshMixed m;
  StateMixed in, out;
  const float *y0hp, *y0u, *y0v;
  float *lohp, *lou, *lov;  // compensation terms of the step-to-step state (interior)
  float *acchp, *accu, *accv;
  float *thp, *tu, *tv;
  float rdx, rdy, rdx60, rdy60;  // reciprocals of dx, dy, 60 dx, 60 dy
  float c1;
  float phibar;  // mean geopotential phibar (m^2 s^-2)
  float a2, inv_a2;
  float eps_E;  // WENO eps of E (m^2 s^-2 units: the reference's 1e-2)
  float eps_F;  // eps of the flux / a^2 (1e-2 / a^4)
  float eps_P;  // eps of phitG / a^2 (1e-2 / a^4)
  int kind, ediss;
  int op;             // CCS_OP_WENO, or the central-difference order 2 / 4 / 6
  float rdxc, rdyc;   // 1 / (2 dx), 1 / (12 dx) or 1 / (60 dx) for the central operator
};

// Kernel variants: the tile shape (cells per work item) of each lane's stage kernel.
// A handle runs one variant; the autotuner picks it per resolution by timing.
struct TileShape {
  int tx, ty;
};
constexpr int F64_NVAR = 3;  // 32 x 8, 16 x 16, 64 x 4 (256 threads, one cell each in phase 3)
constexpr TileShape kF64Tiles[F64_NVAR] = {{32, 8}, {16, 16}, {64, 4}};
// Mixed lane: tile shape x halo-staging schedule of phase 1.  kStageLoads: each
// thread loads its cells' raw inputs into registers and stores the derived cell
// quantities; kStageAsync: asynchronous copies (cp.async) put the raw inputs of all
// of a thread's cells into shared memory at once, then the thread derives the
// quantities in place.
constexpr int kStageLoads = 0, kStageAsync = 1;
constexpr int MX_NVAR = 4;  // 32 x 32 (256 threads), 32 x 16 (128 threads); each with both schedules
constexpr TileShape kMxTiles[MX_NVAR] = {{32, 32}, {32, 16}, {32, 32}, {32, 16}};
constexpr int kMxStaging[MX_NVAR] = {kStageLoads, kStageLoads, kStageAsync, kStageAsync};

// kernel launchers (return cudaGetLastError()); `var` indexes the tile tables
cudaError_t launch_f64_stage(int var, const F64Stage *d_stages, const WorkItem *d_work, int nwork, int grid,
                             cudaStream_t s);
int f64_max_grid(int var, int device);

// central: every stage in d_stages uses a central-difference operator (else WENO-Z);
// ediss: every stage reconstructs the E-flux dissipation (CCS_EDISS_RECONSTRUCT)
cudaError_t launch_mixed_stage(int var, bool central, bool ediss, const MixedStage *d_stages,
                               const WorkItem *d_work, int nwork, int grid, cudaStream_t s);
int mixed_max_grid(int var, int device);
cudaError_t launch_mixed_import(const Layout &L, const double *phi, const double *u, const double *v,
                                double phibar, double inv_a2, StateMixed out, float *lohp, float *lou,
                                float *lov, cudaStream_t s);
cudaError_t launch_mixed_export(const Layout &L, StateMixed st, const float *lohp, const float *lou,
                                const float *lov, const MeshF64 &m, double phibar, double a2, double *const out[8],
                                cudaStream_t s);
cudaError_t launch_mixed_tend_export(const Layout &L, const float *thp, const float *tu, const float *tv,
                                     const MeshF64 &m, double a2, double *op, double *ou, double *ov,
                                     cudaStream_t s);
cudaError_t launch_mixed_diag(const Layout &L, StateMixed st, const float *lohp, const float *lou,
                              const float *lov, const MeshF64 &m, double phibar, double a2, double *partials,
                              int nblocks, cudaStream_t s);


// test support: correctly rounded division by a constant, see ccs_fp64.cu
cudaError_t launch_div_const_check(const double *x, int64_t n, double b, double *out, cudaStream_t s);
// test support: division by a shared divisor from its reciprocal, see ccs_fp64.cu
cudaError_t launch_div_pairs_check(const double *a, const double *b, int64_t n, double *out, cudaStream_t s);

// Bounds-checked build (-DCCS_BOUNDS, ccs_bounds.cuh): the first out-of-range index
// the FP64 / mixed kernels met since the last call, (site << 48) | (index & 2^48-1),
// 0 for none; the call clears it.  Always 0 in the normal build.
unsigned long long f64_bounds_take();
unsigned long long mixed_bounds_take();
// one thread checks index i against [0, n) under `site`, accessing nothing (a no-op
// in the normal build)
cudaError_t launch_bounds_selftest(long long i, long long n, int site, cudaStream_t s);

// zero rows after each face wave-speed metric block of the mixed lane (the line
// sweep fetches one face ahead and reads faces past N in partial tiles)
constexpr int kLamPadRows = 32;

// FP64 reductions (mass / energy) over the interior of an FP64 state
cudaError_t launch_f64_diag(const Layout &L, const double *phiG, const double *phi, const double *u,
                            const double *v, const double *uC, const double *vC, const double *sqrtG,
                            const double *phis, double *partials, int nblocks, cudaStream_t s);

}  // namespace ccs
