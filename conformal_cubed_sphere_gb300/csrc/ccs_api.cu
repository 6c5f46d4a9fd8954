// ccs_api.cu -- the C ABI (include/ccs_gpu.h): handles, device buffers, stage
// descriptors, CUDA-graph capture of a step, state transfer and diagnostics.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "ccs_internal.h"
#include "ccs_kernels.h"

using namespace ccs;

namespace {

int round_up(int x, int m) { return (x + m - 1) / m * m; }

// NVTX range over a host call (named in Nsight Systems / ncu timelines; a no-op when
// no tool is attached)
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

// Health check: counts interior cells whose depth is not positive (NaN included) or
// whose covariant wind is not finite.  phi = phi0 + hp[c] (FP64 lane: phi0 = 0 and
// hp = phi).  One atomic per warp.
template <typename R>
__global__ void health_kernel(Layout L, const R *__restrict__ hp, const R *__restrict__ u,
                              const R *__restrict__ v, double phi0, unsigned long long *bad) {
  const int64_t ncell = (int64_t)L.N * L.N * 6;
  for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x; q0 < ncell; q0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = q0 + threadIdx.x;
    bool b = false;
    if (q < ncell) {
      const int i = 1 + (int)(q % L.N), j = 1 + (int)((q / L.N) % L.N), p = (int)(q / ((int64_t)L.N * L.N));
      const int64_t c = L.idx(i, j, p);
      const double ph = phi0 + (double)hp[c];
      b = !(ph > 0.) || !isfinite((double)u[c]) || !isfinite((double)v[c]);
    }
    const unsigned m = __ballot_sync(0xffffffffu, b);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(bad, (unsigned long long)__popc(m));
  }
}

// Largest wave speed of a state over interior and edge-halo cells (the cells of
// ccs_cfl_dt): max(|uC| + sqrt(IG11 phit), |vC| + sqrt(IG22 phit)), phit = phi0 + hp +
// phis, in FP64; a cell with non-positive phit or a non-finite value counts as +inf.
// FP64 lane: hp = phi, uC / vC from the state.  Mixed lane: hp = phi - phi0 and the
// covariant wind / a^2 in FP32, uC / vC formed with the FP64 metric.  The maximum is
// an atomicMax on the bit patterns (non-negative doubles order as integers).
__global__ void courant_kernel(Layout L, const float *__restrict__ hp32, const float *__restrict__ u32,
                               const float *__restrict__ v32, const double *__restrict__ phi64,
                               const double *__restrict__ uC64, const double *__restrict__ vC64, MeshF64 m,
                               double phi0, double a2, unsigned long long *lmax) {
  const int N = L.N, n2 = N + 2;
  const int64_t ncell = (int64_t)n2 * n2 * 6;
  double best = 0.;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ncell;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % n2), j = (int)((q / n2) % n2), p = (int)(q / ((int64_t)n2 * n2));
    if ((i < 1 || i > N) && (j < 1 || j > N)) continue;  // corner blocks
    const int64_t c = L.idx(i, j, p);
    double pt, uC, vC;
    if (phi64) {
      pt = phi64[c] + m.phis[c];
      uC = uC64[c];
      vC = vC64[c];
    } else {
      pt = phi0 + (double)hp32[c] + m.phis[c];
      const double u = (double)u32[c] * a2, v = (double)v32[c] * a2;
      uC = m.ig11[c] * u + m.ig12[c] * v;
      vC = m.ig21[c] * u + m.ig22[c] * v;
    }
    double x = INFINITY;
    if (pt > 0.) {
      const double lx = fabs(uC) + sqrt(m.ig11[c] * pt), ly = fabs(vC) + sqrt(m.ig22[c] * pt);
      const double l = fmax(lx, ly);
      if (l >= 0. && l < INFINITY) x = l;
    }
    best = fmax(best, x);
  }
  for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0) atomicMax(lmax, (unsigned long long)__double_as_longlong(best));
}

#define CCS_TRY(h, call)                                                       \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      if (h) (h)->err = std::string(#call) + ": " + cudaGetErrorString(e_);    \
      return CCS_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

// Device copy of one grid's metric, shared by every member on that grid.
struct DeviceMesh {
  int device = 0;
  Layout L{};
  double *buf64 = nullptr;  // FP64 lane arrays
  int32_t *push = nullptr;
  MeshF64 m64{};
  float *buf32 = nullptr;   // mixed lane arrays
  double *xf = nullptr;     // mixed lane FP64 halo transforms
  MeshMixed mm{};
  double radius = 0.;
  ~DeviceMesh() {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(device);
    if (buf64) cudaFree(buf64);
    if (push) cudaFree(push);
    if (buf32) cudaFree(buf32);
    if (xf) cudaFree(xf);
    cudaSetDevice(cur);
  }
};

}  // namespace

struct MixedLane;

struct ccs_handle {
  ccs_config cfg{};
  std::shared_ptr<DeviceMesh> mesh;
  Layout L{};
  cudaStream_t stream = nullptr;
  std::string err;
  // FP64 lane buffers
  double *sbuf = nullptr;
  StateF64 S[3]{};
  double *zonal = nullptr, *merid = nullptr;
  double *acc[3]{}, *tend[3]{};
  // stage descriptors: RK stages, final stage with sphere winds, tendency-only
  std::vector<F64Stage> h_stages;
  F64Stage *d_stages = nullptr;
  int n_rk = 0;  // number of RK stages (4 or 3)
  WorkItem *d_work = nullptr;
  int nwork = 0;
  int grid = 0;
  int var = 0;  // tile variant of the FP64 stage kernel (kF64Tiles)
  int op = CCS_OP_WENO;  // spatial operator (ccs_set_operator)
  bool sphere_valid = false;
  cudaGraphExec_t g_step = nullptr, g_step_sw = nullptr;
  // timing
  bool timing = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_order = nullptr;  // orders the handle's stream with a batch step
  double kernel_ms = 0.;
  int64_t launches = 0;
  // diagnostics
  double *d_partials = nullptr;
  unsigned long long *d_bad = nullptr;  // health-check counter
  unsigned long long *d_lmax = nullptr;  // largest wave speed (ccs_courant), as bits
  // mixed lane
  struct MixedLane *mixed = nullptr;
};

static const int kDiagBlocks = 512;

static int upload_field(ccs_handle *h, double *dst, const double *src) {
  const Layout &L = h->L;
  CCS_TRY(h, cudaMemcpy2DAsync(dst, (size_t)L.pitch * sizeof(double), src, (size_t)L.nh * sizeof(double),
                               (size_t)L.nh * sizeof(double), (size_t)L.nh * 6, cudaMemcpyHostToDevice,
                               h->stream));
  return CCS_OK;
}

static int download_field(ccs_handle *h, double *dst, const double *src) {
  const Layout &L = h->L;
  CCS_TRY(h, cudaMemcpy2DAsync(dst, (size_t)L.nh * sizeof(double), src, (size_t)L.pitch * sizeof(double),
                               (size_t)L.nh * sizeof(double), (size_t)L.nh * 6, cudaMemcpyDeviceToHost,
                               h->stream));
  return CCS_OK;
}

static int validate_config(const ccs_config *c) {
  if (!c) return CCS_ERR_ARG;
  if (c->N < 1 || c->N > 8192 || c->halo < 3 || c->halo > c->N) return CCS_ERR_ARG;
  if (c->scheme != CCS_RK4 && c->scheme != CCS_RK3_TVD) return CCS_ERR_ARG;
  if (c->precision != CCS_FP64 && c->precision != CCS_MIXED) return CCS_ERR_ARG;
  if (c->e_dissipation != CCS_EDISS_ZERO && c->e_dissipation != CCS_EDISS_RECONSTRUCT) return CCS_ERR_ARG;
  if (!(c->dx > 0.) || !(c->dy > 0.) || !(c->dt > 0.) || !(c->radius > 0.) || !(c->gravity > 0.))
    return CCS_ERR_ARG;
  if (!std::isfinite(c->dx) || !std::isfinite(c->dy) || !std::isfinite(c->dt) || !std::isfinite(c->omega))
    return CCS_ERR_ARG;
  return CCS_OK;
}

// The mixed lane keeps one copy of sqrtG and G^-1 for all six panels: true of a
// cube map (the panels are rotations of one face map, halo cells included), checked
// here to 1e-12 relative (G^-1 entries relative to its diagonal) on every cell
// outside the corner blocks.
static bool panels_share_metric(int N, int h, const ccs_mesh_view *m) {
  const int nh = N + 2 * h;
  const size_t np = (size_t)nh * nh;
  auto close = [](double a, double b) { return std::fabs(a - b) <= 1e-12 * std::fmax(std::fabs(a), std::fabs(b)); };
  for (int j = 1 - h; j <= N + h; j++)
    for (int i = 1 - h; i <= N + h; i++) {
      if ((i < 1 || i > N) && (j < 1 || j > N)) continue;
      const size_t r0 = (size_t)(i + h - 1) + (size_t)nh * (j + h - 1);
      for (int p = 1; p < 6; p++) {
        const size_t r = r0 + np * p;
        if (!close(m->sqrtG[r], m->sqrtG[r0])) return false;
        // entries against the matrix's scale (off-diagonals vanish on the centre lines)
        const double *a = &m->matrixIG[4 * r], *b = &m->matrixIG[4 * r0];
        const double scale = std::fabs(b[0]) + std::fabs(b[3]);
        for (int q = 0; q < 4; q++)
          if (!(std::fabs(a[q] - b[q]) <= 1e-12 * scale)) return false;
      }
    }
  return true;
}

// matmul of two 2x2 column-major matrices as gfortran inlines it (c = 0; c += ...)
static void matmul22(const double *X, const double *Y, double *M) {
  for (int c = 0; c < 2; c++)
    for (int r = 0; r < 2; r++) {
      double s = 0.;
      for (int k = 0; k < 2; k++) s = s + X[r + 2 * k] * Y[k + 2 * c];
      M[r + 2 * c] = s;
    }
}

static int mixed_mesh_setup(ccs_handle *h, DeviceMesh *dm, const ccs_mesh_view *mv);
static int mixed_handle_create(ccs_handle *h);
static void mixed_handle_destroy(ccs_handle *h);
static int mixed_set_state(ccs_handle *h, const ccs_state_view *s, bool sync);
static int mixed_get_state(ccs_handle *h, ccs_state_view *s, bool sync);
static int mixed_sync(ccs_handle *h);
static int mixed_build_stages(ccs_handle *h);
static bool mixed_has_stages(const ccs_handle *h);
static int mixed_step(ccs_handle *h, int nsteps, bool sync);
static int mixed_tend(ccs_handle *h, double *tp, double *tu, double *tv);
static int mixed_diag(ccs_handle *h, double *mass, double *energy);

static int build_mesh(ccs_handle *h, const ccs_mesh_view *mv) {
  auto dm = std::make_shared<DeviceMesh>();
  dm->device = h->cfg.device;
  dm->L = h->L;
  dm->radius = h->cfg.radius;
  const Layout &L = h->L;
  const size_t nref = (size_t)L.nh * L.nh * 6;
  const size_t nf = (size_t)L.field;
  // 15 FP64 arrays: sqrtG phis f ig11 ig12 ig21 ig22 aig11..22 gia11..22
  CCS_TRY(h, cudaMalloc(&dm->buf64, 15 * nf * sizeof(double)));
  CCS_TRY(h, cudaMemsetAsync(dm->buf64, 0, 15 * nf * sizeof(double), h->stream));
  std::vector<double> tmp(15 * nref, 0.);
  double *t[15];
  for (int k = 0; k < 15; k++) t[k] = tmp.data() + k * nref;
  for (size_t c = 0; c < nref; c++) {
    t[0][c] = mv->sqrtG[c];
    t[1][c] = mv->phis[c];
    t[2][c] = mv->f[c];
    const double *IG = &mv->matrixIG[4 * c];
    t[3][c] = IG[0];  // IG(1,1)
    t[4][c] = IG[2];  // IG(1,2)
    t[5][c] = IG[1];  // IG(2,1)
    t[6][c] = IG[3];  // IG(2,2)
    double M[4];
    matmul22(&mv->matrixA[4 * c], IG, M);  // projection_mod.F90:90
    t[7][c] = M[0]; t[8][c] = M[2]; t[9][c] = M[1]; t[10][c] = M[3];
    matmul22(&mv->matrixG[4 * c], &mv->matrixIA[4 * c], M);  // projection_mod.F90:71
    t[11][c] = M[0]; t[12][c] = M[2]; t[13][c] = M[1]; t[14][c] = M[3];
  }
  for (int k = 0; k < 15; k++) {
    int rc = upload_field(h, dm->buf64 + k * nf, t[k]);
    if (rc) return rc;
  }
  double *b = dm->buf64;
  dm->m64.sqrtG = b + 0 * nf; dm->m64.phis = b + 1 * nf; dm->m64.f = b + 2 * nf;
  dm->m64.ig11 = b + 3 * nf; dm->m64.ig12 = b + 4 * nf; dm->m64.ig21 = b + 5 * nf; dm->m64.ig22 = b + 6 * nf;
  dm->m64.aig11 = b + 7 * nf; dm->m64.aig12 = b + 8 * nf; dm->m64.aig21 = b + 9 * nf; dm->m64.aig22 = b + 10 * nf;
  dm->m64.gia11 = b + 11 * nf; dm->m64.gia12 = b + 12 * nf; dm->m64.gia21 = b + 13 * nf; dm->m64.gia22 = b + 14 * nf;
  std::vector<int32_t> push;
  if (!build_push_table(L, push)) {
    h->err = "ghost tables are inconsistent";
    return CCS_ERR_MESH;
  }
  CCS_TRY(h, cudaMalloc(&dm->push, push.size() * sizeof(int32_t)));
  CCS_TRY(h, cudaMemcpyAsync(dm->push, push.data(), push.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                             h->stream));
  dm->m64.push = dm->push;
  if (h->cfg.precision == CCS_MIXED) {
    int rc = mixed_mesh_setup(h, dm.get(), mv);
    if (rc) return rc;
  }
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  h->mesh = dm;
  return CCS_OK;
}

// (Re)builds a work list of all tiles of the six panels for tile shape ts.
static int build_work(ccs_handle *h, TileShape ts, WorkItem **d_work, int *nwork) {
  const int N = h->L.N;
  const int ntx = (N + ts.tx - 1) / ts.tx, nty = (N + ts.ty - 1) / ts.ty;
  std::vector<WorkItem> work;
  for (int p = 0; p < 6; p++)
    for (int ty = 0; ty < nty; ty++)
      for (int tx = 0; tx < ntx; tx++) work.push_back(WorkItem{0, (int16_t)p, (int16_t)tx, (int16_t)ty});
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  if (*d_work) CCS_TRY(h, cudaFree(*d_work));
  *d_work = nullptr;
  CCS_TRY(h, cudaMalloc(d_work, work.size() * sizeof(WorkItem)));
  CCS_TRY(h, cudaMemcpyAsync(*d_work, work.data(), work.size() * sizeof(WorkItem), cudaMemcpyHostToDevice,
                             h->stream));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  *nwork = (int)work.size();
  return CCS_OK;
}

static int build_f64_lane(ccs_handle *h) {
  const Layout &L = h->L;
  const size_t nf = (size_t)L.field;
  // 3 slots x 6 fields + zonal + merid + acc(3) + tend(3) = 26 fields
  CCS_TRY(h, cudaMalloc(&h->sbuf, 26 * nf * sizeof(double)));
  CCS_TRY(h, cudaMemsetAsync(h->sbuf, 0, 26 * nf * sizeof(double), h->stream));
  double *b = h->sbuf;
  for (int s = 0; s < 3; s++) {
    h->S[s].phiG = b; b += nf;
    h->S[s].u = b; b += nf;
    h->S[s].v = b; b += nf;
    h->S[s].phi = b; b += nf;
    h->S[s].uC = b; b += nf;
    h->S[s].vC = b; b += nf;
  }
  h->zonal = b; b += nf;
  h->merid = b; b += nf;
  for (int k = 0; k < 3; k++) { h->acc[k] = b; b += nf; }
  for (int k = 0; k < 3; k++) { h->tend[k] = b; b += nf; }

  const ccs_config &c = h->cfg;
  F64Stage base{};
  base.L = L;
  base.m = h->mesh->m64;
  base.y0phiG = h->S[0].phiG; base.y0u = h->S[0].u; base.y0v = h->S[0].v;
  base.accphiG = h->acc[0]; base.accu = h->acc[1]; base.accv = h->acc[2];
  base.dx = c.dx; base.dy = c.dy;
  base.dx60 = 60. * c.dx; base.dy60 = 60. * c.dy;
  base.rdx = 1. / base.dx; base.rdy = 1. / base.dy;
  base.rdx60 = 1. / base.dx60; base.rdy60 = 1. / base.dy60;
  base.ediss = c.e_dissipation;
  base.op = h->op;
  auto mk = [&](int kind, int in, int out, double c1) {
    F64Stage s = base;
    s.kind = kind;
    s.in = h->S[in];
    s.out = h->S[out];
    s.c1 = c1;
    return s;
  };
  h->h_stages.clear();
  const double dt = c.dt;
  if (c.scheme == CCS_RK4) {
    h->n_rk = 4;
    h->h_stages.push_back(mk(K_RK4_1, 0, 1, 0.5 * dt));
    h->h_stages.push_back(mk(K_RK4_2, 1, 2, 0.5 * dt));
    h->h_stages.push_back(mk(K_RK4_2, 2, 1, dt));
    h->h_stages.push_back(mk(K_RK4_4, 1, 0, dt));
  } else {
    h->n_rk = 3;
    h->h_stages.push_back(mk(K_RK3_1, 0, 1, dt));
    h->h_stages.push_back(mk(K_RK3_2, 1, 2, 0.25 * dt));
    h->h_stages.push_back(mk(K_RK3_3, 2, 0, 2. / 3. * dt));
  }
  F64Stage sw = h->h_stages.back();
  sw.zonal = h->zonal;
  sw.merid = h->merid;
  h->h_stages.push_back(sw);  // final stage with sphere winds
  F64Stage td = mk(K_TEND, 0, 0, 0.);
  td.tphiG = h->tend[0]; td.tu = h->tend[1]; td.tv = h->tend[2];
  h->h_stages.push_back(td);
  CCS_TRY(h, cudaMalloc(&h->d_stages, h->h_stages.size() * sizeof(F64Stage)));
  CCS_TRY(h, cudaMemcpyAsync(h->d_stages, h->h_stages.data(), h->h_stages.size() * sizeof(F64Stage),
                             cudaMemcpyHostToDevice, h->stream));
  int rc = build_work(h, kF64Tiles[h->var], &h->d_work, &h->nwork);
  if (rc) return rc;
  h->grid = f64_max_grid(h->var, c.device);
  CCS_TRY(h, cudaMalloc(&h->d_partials, 2 * kDiagBlocks * sizeof(double)));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

// enqueue one step; with_sw: the final stage also writes the sphere winds
static int f64_enqueue_step(ccs_handle *h, bool with_sw) {
  for (int k = 0; k < h->n_rk; k++) {
    const F64Stage *d = h->d_stages + ((k == h->n_rk - 1 && with_sw) ? h->n_rk : k);
    if (h->timing) CCS_TRY(h, cudaEventRecord(h->ev0, h->stream));
    CCS_TRY(h, launch_f64_stage(h->var, d, h->d_work, h->nwork, h->grid, h->stream));
    if (h->timing) {
      CCS_TRY(h, cudaEventRecord(h->ev1, h->stream));
      CCS_TRY(h, cudaEventSynchronize(h->ev1));
      float ms = 0.f;
      CCS_TRY(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
      h->kernel_ms += ms;
      h->launches++;
    }
  }
  return CCS_OK;
}

static int f64_capture(ccs_handle *h, bool with_sw, cudaGraphExec_t *out) {
  cudaGraph_t g = nullptr;
  CCS_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const bool t = h->timing;
  h->timing = false;
  int rc = f64_enqueue_step(h, with_sw);
  h->timing = t;
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) {
    h->err = std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e);
    return CCS_ERR_CUDA;
  }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    h->err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e);
    return CCS_ERR_CUDA;
  }
  return CCS_OK;
}

static int f64_step(ccs_handle *h, int nsteps, bool sync) {
  if (nsteps <= 0) return CCS_OK;
  if (h->timing) {
    for (int s = 0; s < nsteps; s++) {
      int rc = f64_enqueue_step(h, s == nsteps - 1);
      if (rc) return rc;
    }
  } else {
    if (!h->g_step) {
      int rc = f64_capture(h, false, &h->g_step);
      if (rc) return rc;
      rc = f64_capture(h, true, &h->g_step_sw);
      if (rc) return rc;
    }
    for (int s = 0; s < nsteps - 1; s++) CCS_TRY(h, cudaGraphLaunch(h->g_step, h->stream));
    CCS_TRY(h, cudaGraphLaunch(h->g_step_sw, h->stream));
  }
  h->sphere_valid = true;
  if (sync) CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

// ---------------------------------------------------------------------------
extern "C" {

int ccs_abi_version(void) { return CCS_ABI_VERSION; }

void *ccs_stream(ccs_handle *h) { return h ? (void *)h->stream : nullptr; }

int ccs_selftest_div(const double *x, int64_t n, double b, double *fast, double *ieee) {
  if (!x || n <= 0 || !fast || !ieee) return CCS_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return CCS_ERR_NODEVICE;
  cudaSetDevice(0);
  double *dx = nullptr, *dout = nullptr;
  if (cudaMalloc(&dx, n * sizeof(double)) != cudaSuccess) return CCS_ERR_NOMEM;
  if (cudaMalloc(&dout, 2 * n * sizeof(double)) != cudaSuccess) {
    cudaFree(dx);
    return CCS_ERR_NOMEM;
  }
  int rc = CCS_OK;
  if (cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      launch_div_const_check(dx, n, b, dout, 0) != cudaSuccess ||
      cudaMemcpy(fast, dout, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(ieee, dout + n, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = CCS_ERR_CUDA;
  cudaFree(dx);
  cudaFree(dout);
  return rc;
}

int ccs_selftest_div_pairs(const double *a, const double *b, int64_t n, double *fast, double *ieee) {
  if (!a || !b || n <= 0 || !fast || !ieee) return CCS_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return CCS_ERR_NODEVICE;
  cudaSetDevice(0);
  double *da = nullptr, *dout = nullptr;
  if (cudaMalloc(&da, 2 * n * sizeof(double)) != cudaSuccess) return CCS_ERR_NOMEM;
  if (cudaMalloc(&dout, 2 * n * sizeof(double)) != cudaSuccess) {
    cudaFree(da);
    return CCS_ERR_NOMEM;
  }
  int rc = CCS_OK;
  if (cudaMemcpy(da, a, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(da + n, b, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      launch_div_pairs_check(da, da + n, n, dout, 0) != cudaSuccess ||
      cudaMemcpy(fast, dout, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(ieee, dout + n, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = CCS_ERR_CUDA;
  cudaFree(da);
  cudaFree(dout);
  return rc;
}

const char *ccs_strerror(int status) {
  switch (status) {
    case CCS_OK: return "ok";
    case CCS_ERR_ARG: return "invalid argument";
    case CCS_ERR_CUDA: return "CUDA error";
    case CCS_ERR_NAN: return "non-finite or non-positive state";
    case CCS_ERR_TIMEOUT: return "device wait timed out";
    case CCS_ERR_UNSUPPORTED: return "unsupported option";
    case CCS_ERR_MESH: return "singular or inconsistent mesh";
    case CCS_ERR_NOMEM: return "out of memory";
    case CCS_ERR_NODEVICE: return "no CUDA device";
    case CCS_ERR_TOO_LARGE: return "size exceeds the fixed scratch capacity";
    case CCS_ERR_IO: return "mesh file missing, unreadable or not in the raw mesh format";
    default: return "unknown status";
  }
}

const char *ccs_last_error(const ccs_handle *h) { return h ? h->err.c_str() : ""; }

static int init_common(const ccs_config *cfg, ccs_handle **out, ccs_handle **hp) {
  if (!out) return CCS_ERR_ARG;
  *out = nullptr;
  int rc = validate_config(cfg);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return CCS_ERR_NODEVICE;
  if (cfg->device < 0 || cfg->device >= ndev) return CCS_ERR_ARG;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return CCS_ERR_CUDA;
  ccs_handle *h = new ccs_handle();
  h->cfg = *cfg;
  const int nh = cfg->N + 2 * cfg->halo;
  h->L = make_layout(cfg->N, cfg->halo, round_up(nh, 4));
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return CCS_ERR_CUDA;
  }
  cudaEventCreate(&h->ev0);
  cudaEventCreate(&h->ev1);
  *hp = h;
  return CCS_OK;
}

static int finish_init(ccs_handle *h) {
  if (h->cfg.precision == CCS_FP64) return build_f64_lane(h);
  return mixed_handle_create(h);
}

int ccs_init(const ccs_config *cfg, const ccs_mesh_view *mesh, ccs_handle **out) {
  if (!mesh || !mesh->sqrtG || !mesh->matrixG || !mesh->matrixIG || !mesh->matrixA || !mesh->matrixIA ||
      !mesh->f || !mesh->phis)
    return CCS_ERR_ARG;
  if (out) *out = nullptr;
  if (validate_config(cfg)) return CCS_ERR_ARG;
  if (cfg->precision == CCS_MIXED && !panels_share_metric(cfg->N, cfg->halo, mesh)) return CCS_ERR_UNSUPPORTED;
  ccs_handle *h = nullptr;
  int rc = init_common(cfg, out, &h);
  if (rc) return rc;
  rc = build_mesh(h, mesh);
  if (!rc) rc = finish_init(h);
  if (rc) {
    fprintf(stderr, "ccs_init: %s (%s)\n", ccs_strerror(rc), h->err.c_str());
    ccs_destroy(h);
    return rc;
  }
  *out = h;
  return CCS_OK;
}

int ccs_init_shared(const ccs_config *cfg, ccs_handle *owner, ccs_handle **out) {
  if (!owner || !cfg) return CCS_ERR_ARG;
  const ccs_config &o = owner->cfg;
  if (cfg->N != o.N || cfg->halo != o.halo || cfg->dx != o.dx || cfg->dy != o.dy || cfg->device != o.device ||
      cfg->precision != o.precision || cfg->radius != o.radius)
    return CCS_ERR_ARG;
  ccs_handle *h = nullptr;
  int rc = init_common(cfg, out, &h);
  if (rc) return rc;
  h->mesh = owner->mesh;
  rc = finish_init(h);
  if (rc) {
    ccs_destroy(h);
    return rc;
  }
  *out = h;
  return CCS_OK;
}

void ccs_destroy(ccs_handle *h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->g_step) cudaGraphExecDestroy(h->g_step);
  if (h->g_step_sw) cudaGraphExecDestroy(h->g_step_sw);
  if (h->sbuf) cudaFree(h->sbuf);
  if (h->d_stages) cudaFree(h->d_stages);
  if (h->d_work) cudaFree(h->d_work);
  if (h->d_partials) cudaFree(h->d_partials);
  if (h->d_bad) cudaFree(h->d_bad);
  if (h->d_lmax) cudaFree(h->d_lmax);
  if (h->mixed) mixed_handle_destroy(h);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev_order) cudaEventDestroy(h->ev_order);
  if (h->ev1) cudaEventDestroy(h->ev1);
  h->mesh.reset();
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

static int set_state_impl(ccs_handle *h, const ccs_state_view *s, bool sync) {
  NvtxRange nvtx("ccs_set_state");
  if (!h || !s || !s->phiG || !s->u || !s->v || !s->phi || !s->uC || !s->vC) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  if (h->cfg.precision == CCS_MIXED) return mixed_set_state(h, s, sync);
  const double *src[6] = {s->phiG, s->u, s->v, s->phi, s->uC, s->vC};
  double *dst[6] = {h->S[0].phiG, h->S[0].u, h->S[0].v, h->S[0].phi, h->S[0].uC, h->S[0].vC};
  for (int k = 0; k < 6; k++) {
    int rc = upload_field(h, dst[k], src[k]);
    if (rc) return rc;
  }
  h->sphere_valid = false;
  if (s->zonal_wind && s->meridional_wind) {
    int rc = upload_field(h, h->zonal, s->zonal_wind);
    if (!rc) rc = upload_field(h, h->merid, s->meridional_wind);
    if (rc) return rc;
    h->sphere_valid = true;
  }
  if (sync) CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

int ccs_set_state(ccs_handle *h, const ccs_state_view *s) { return set_state_impl(h, s, true); }
int ccs_set_state_async(ccs_handle *h, const ccs_state_view *s) { return set_state_impl(h, s, false); }

static int get_state_impl(ccs_handle *h, ccs_state_view *s, bool sync) {
  NvtxRange nvtx("ccs_get_state");
  if (!h || !s) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  if (h->cfg.precision == CCS_MIXED) return mixed_get_state(h, s, sync);
  double *dst[6] = {s->phiG, s->u, s->v, s->phi, s->uC, s->vC};
  const double *src[6] = {h->S[0].phiG, h->S[0].u, h->S[0].v, h->S[0].phi, h->S[0].uC, h->S[0].vC};
  for (int k = 0; k < 6; k++)
    if (dst[k]) {
      int rc = download_field(h, dst[k], src[k]);
      if (rc) return rc;
    }
  if (h->sphere_valid) {
    if (s->zonal_wind) {
      int rc = download_field(h, s->zonal_wind, h->zonal);
      if (rc) return rc;
    }
    if (s->meridional_wind) {
      int rc = download_field(h, s->meridional_wind, h->merid);
      if (rc) return rc;
    }
  }
  if (sync) CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

int ccs_get_state(ccs_handle *h, ccs_state_view *s) { return get_state_impl(h, s, true); }
int ccs_get_state_async(ccs_handle *h, ccs_state_view *s) { return get_state_impl(h, s, false); }

int ccs_step(ccs_handle *h, int nsteps) {
  NvtxRange nvtx("ccs_step");
  if (!h || nsteps < 0) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  if (h->cfg.precision == CCS_MIXED) return mixed_step(h, nsteps, true);
  return f64_step(h, nsteps, true);
}

int ccs_step_async(ccs_handle *h, int nsteps) {
  NvtxRange nvtx("ccs_step_async");
  if (!h || nsteps < 0) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  if (h->cfg.precision == CCS_MIXED) return mixed_step(h, nsteps, false);
  return f64_step(h, nsteps, false);
}

int ccs_sync(ccs_handle *h) {
  if (!h) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  if (h->cfg.precision == CCS_MIXED) return mixed_sync(h);
  return CCS_OK;
}

int ccs_set_operator(ccs_handle *h, int op) {
  if (!h) return CCS_ERR_ARG;
  if (op != CCS_OP_WENO && op != CCS_OP_CENTRAL2 && op != CCS_OP_CENTRAL4 && op != CCS_OP_CENTRAL6)
    return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  h->op = op;
  if (h->cfg.precision == CCS_MIXED) {
    // the stage descriptors exist once the state (and with it phibar) is set
    return mixed_has_stages(h) ? mixed_build_stages(h) : CCS_OK;
  }
  for (F64Stage &s : h->h_stages) s.op = op;
  // the captured graphs read the descriptors from device memory: updating them in
  // place (after the stream's pending steps) is all a change needs
  CCS_TRY(h, cudaMemcpyAsync(h->d_stages, h->h_stages.data(), h->h_stages.size() * sizeof(F64Stage),
                             cudaMemcpyHostToDevice, h->stream));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

int ccs_spatial_operator(ccs_handle *h, double *tp, double *tu, double *tv) {
  if (!h) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  if (h->cfg.precision == CCS_MIXED) return mixed_tend(h, tp, tu, tv);
  const F64Stage *d = h->d_stages + h->n_rk + 1;
  CCS_TRY(h, launch_f64_stage(h->var, d, h->d_work, h->nwork, h->grid, h->stream));
  double *dst[3] = {tp, tu, tv};
  for (int k = 0; k < 3; k++)
    if (dst[k]) {
      int rc = download_field(h, dst[k], h->tend[k]);
      if (rc) return rc;
    }
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

int ccs_diag(ccs_handle *h, double *mass, double *energy) {
  NvtxRange nvtx("ccs_diag");
  if (!h) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  if (h->cfg.precision == CCS_MIXED) return mixed_diag(h, mass, energy);
  const MeshF64 &m = h->mesh->m64;
  CCS_TRY(h, launch_f64_diag(h->L, h->S[0].phiG, h->S[0].phi, h->S[0].u, h->S[0].v, h->S[0].uC, h->S[0].vC,
                             m.sqrtG, m.phis, h->d_partials, kDiagBlocks, h->stream));
  std::vector<double> part(2 * kDiagBlocks);
  CCS_TRY(h, cudaMemcpyAsync(part.data(), h->d_partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  double tm = 0., te = 0.;
  for (int b = 0; b < kDiagBlocks; b++) {
    tm += part[2 * b];
    te += part[2 * b + 1];
  }
  if (mass) *mass = tm;
  if (energy) *energy = te;
  return CCS_OK;
}

int ccs_timing(ccs_handle *h, int enable, int reset, double *kernel_ms, int64_t *launches) {
  if (!h) return CCS_ERR_ARG;
  if (kernel_ms) *kernel_ms = h->kernel_ms;
  if (launches) *launches = h->launches;
  if (reset) {
    h->kernel_ms = 0.;
    h->launches = 0;
  }
  if (enable >= 0) h->timing = enable != 0;
  return CCS_OK;
}

}  // extern "C"


// ---------------------------------------------------------------------------
// mixed lane host side
// ---------------------------------------------------------------------------
struct MixedLane {
  float *buf = nullptr;  // S[3] (3 fields each), lo(3), acc(3), tend(3)
  StateMixed S[3]{};
  float *lo[3]{}, *acc[3]{}, *tend[3]{};
  // Reference-layout FP64 staging, double-buffered so that transfers of consecutive
  // states overlap: in slots hold phi, u, v (3 fields), out slots the 8 exported
  // fields.  Host-to-device copies run on `cin`, device-to-host copies on `cout`,
  // the import / export kernels on the handle's stream; events order the slots.
  double *staging = nullptr;
  double *stage_in[2]{}, *stage_out[2]{};
  cudaStream_t cin = nullptr, cout = nullptr;
  cudaEvent_t in_ready[2]{}, in_free[2]{}, out_ready[2]{}, out_free[2]{};
  int in_slot = 0, out_slot = 0;
  std::vector<MixedStage> h_stages;
  MixedStage *d_stages = nullptr;
  int n_rk = 0;
  WorkItem *d_work = nullptr;
  int nwork = 0, grid = 0;
  int var = 0;  // tile variant of the mixed stage kernel (kMxTiles)
  double phibar = 0.;
  bool have_phibar = false;
  cudaGraphExec_t g_step = nullptr;
};

static int mixed_mesh_setup(ccs_handle *h, DeviceMesh *dm, const ccs_mesh_view *mv) {
  const Layout &L = h->L;
  const int N = L.N, hh = L.h, nh = L.nh;
  const double a2 = h->cfg.radius * h->cfg.radius;
  const size_t nf = (size_t)L.field, np = (size_t)L.panel;
  const size_t nref = (size_t)nh * nh * 6;
  // shared: s inv_s lamx lamy (one panel each; the face metrics followed by 32 zero
  // rows that the stage kernel's one-face-ahead prefetch may read in partial tiles)
  // + ig as float4; per panel: phis fs
  const size_t pad = kLamPadRows * (size_t)L.pitch;  // a multiple of 4 floats: ig stays 16-byte aligned
  const size_t o_lamx = 2 * np, o_lamy = 3 * np + pad, o_ig = 4 * np + 2 * pad;
  const size_t nfloat = o_ig + 4 * np + 2 * nf;  // s, inv_s, lamx, lamy, ig (4 per cell), phis, fs
  CCS_TRY(h, cudaMalloc(&dm->buf32, nfloat * sizeof(float)));
  std::vector<float> hb(nfloat, 0.f);
  float *sh_s = hb.data(), *sh_inv = hb.data() + np, *sh_lamx = hb.data() + o_lamx, *sh_lamy = hb.data() + o_lamy;
  float *sh_ig = hb.data() + o_ig;  // interleaved (11, 12, 21, 22), 16-byte aligned (np % 4 == 0)
  float *phs = hb.data() + o_ig + 4 * np, *fs = phs + nf;
  for (int p = 0; p < 6; p++)
    for (int j = 1 - hh; j <= N + hh; j++)
      for (int i = 1 - hh; i <= N + hh; i++) {
        const size_t r = (size_t)(i + hh - 1) + (size_t)nh * ((size_t)(j + hh - 1) + (size_t)nh * p);
        const int64_t d = L.idx(i, j, p);
        const double sg = mv->sqrtG[r];
        if (p == 0) {
          const double *IG = &mv->matrixIG[4 * r];
          sh_s[d] = (float)(sg / a2);
          sh_ig[4 * d + 0] = (float)(IG[0] * a2);
          sh_ig[4 * d + 1] = (float)(IG[2] * a2);
          sh_ig[4 * d + 2] = (float)(IG[1] * a2);
          sh_ig[4 * d + 3] = (float)(IG[3] * a2);
          sh_inv[d] = sg > 0. ? (float)(a2 / sg) : 0.f;
        }
        phs[d] = (float)mv->phis[r];
        fs[d] = (float)(mv->f[r] * sg / a2);
      }
  // face wave-speed metric (spatial_operators_mod.F90:113-114, 138-139), x-faces i in
  // [0, N] of rows j in [1, N] (stored transposed) and y-faces j in [0, N] of columns
  // i in [1, N]
  for (int j = 0; j <= N; j++)
    for (int i = 0; i <= N; i++) {
      const size_t r = (size_t)(i + hh - 1) + (size_t)nh * (size_t)(j + hh - 1);
      const int64_t d = L.idx(i, j, 0);
      if (j >= 1) sh_lamx[L.idx(j, i, 0)] = (float)(0.5 * (mv->matrixIG[4 * (r + 1)] + mv->matrixIG[4 * r]));
      if (i >= 1) sh_lamy[d] = (float)(0.5 * (mv->matrixIG[4 * (r + nh) + 3] + mv->matrixIG[4 * r + 3]));
    }
  CCS_TRY(h, cudaMemcpyAsync(dm->buf32, hb.data(), nfloat * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  // FP64 halo transforms, one per push-table entry: T = (G IA)_halo (A IG)_source
  const size_t ne = (size_t)24 * hh * N;
  std::vector<double> xf(4 * ne, 0.);
  for (int p = 1; p <= 6; p++)
    for (int side = 0; side < 4; side++)
      for (int k = 1; k <= hh; k++)
        for (int m = 1; m <= N; m++) {
          const GhostSrc s = ghost_source(N, p, side, k, m);
          const int ss = ghost_source_side(p, side);
          int di, dj;
          switch (side) {
            case 0: di = 1 - k; dj = m; break;
            case 1: di = N + k; dj = m; break;
            case 2: di = m; dj = 1 - k; break;
            default: di = m; dj = N + k; break;
          }
          int ks, ms;
          switch (ss) {
            case 0: ks = s.i; ms = s.j; break;
            case 1: ks = N + 1 - s.i; ms = s.j; break;
            case 2: ks = s.j; ms = s.i; break;
            default: ks = N + 1 - s.j; ms = s.i; break;
          }
          const size_t e = ((size_t)(s.p - 1) * 4 + ss) * hh * N + (size_t)(ks - 1) * N + (ms - 1);
          const size_t rd = (size_t)(di + hh - 1) + (size_t)nh * ((size_t)(dj + hh - 1) + (size_t)nh * (p - 1));
          const size_t rs =
              (size_t)(s.i + hh - 1) + (size_t)nh * ((size_t)(s.j + hh - 1) + (size_t)nh * (s.p - 1));
          double GIA[4], AIG[4], T[4];
          matmul22(&mv->matrixG[4 * rd], &mv->matrixIA[4 * rd], GIA);
          matmul22(&mv->matrixA[4 * rs], &mv->matrixIG[4 * rs], AIG);
          matmul22(GIA, AIG, T);
          xf[4 * e + 0] = T[0];  // T(1,1)
          xf[4 * e + 1] = T[2];  // T(1,2)
          xf[4 * e + 2] = T[1];  // T(2,1)
          xf[4 * e + 3] = T[3];  // T(2,2)
        }
  double *dxf = nullptr;
  // the transforms live after the FP64 mesh arrays in their own allocation
  CCS_TRY(h, cudaMalloc(&dxf, xf.size() * sizeof(double)));
  CCS_TRY(h, cudaMemcpyAsync(dxf, xf.data(), xf.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  dm->xf = dxf;
  dm->mm.s = dm->buf32;
  dm->mm.inv_s = dm->buf32 + np;
  dm->mm.lamx = dm->buf32 + o_lamx;
  dm->mm.lamy = dm->buf32 + o_lamy;
  dm->mm.ig = reinterpret_cast<const float4 *>(dm->buf32 + o_ig);
  dm->mm.phis = dm->buf32 + o_ig + 4 * np;
  dm->mm.fs = dm->buf32 + o_ig + 4 * np + nf;
  dm->mm.xf = dxf;
  dm->mm.push = dm->push;
  (void)nref;
  return CCS_OK;
}

static int mixed_handle_create(ccs_handle *h) {
  MixedLane *M = new MixedLane();
  h->mixed = M;
  const Layout &L = h->L;
  const size_t nf = (size_t)L.field;
  const size_t nref = (size_t)L.nh * L.nh * 6;
  CCS_TRY(h, cudaMalloc(&M->buf, 18 * nf * sizeof(float)));
  CCS_TRY(h, cudaMemsetAsync(M->buf, 0, 18 * nf * sizeof(float), h->stream));
  float *b = M->buf;
  for (int s = 0; s < 3; s++) {
    M->S[s].hp = b; b += nf;
    M->S[s].u = b; b += nf;
    M->S[s].v = b; b += nf;
  }
  for (int k = 0; k < 3; k++) { M->lo[k] = b; b += nf; }
  for (int k = 0; k < 3; k++) { M->acc[k] = b; b += nf; }
  for (int k = 0; k < 3; k++) { M->tend[k] = b; b += nf; }
  CCS_TRY(h, cudaMalloc(&M->staging, 22 * nref * sizeof(double)));
  for (int k = 0; k < 2; k++) {
    M->stage_in[k] = M->staging + 3 * k * nref;
    M->stage_out[k] = M->staging + (6 + 8 * k) * nref;
    CCS_TRY(h, cudaEventCreateWithFlags(&M->in_ready[k], cudaEventDisableTiming));
    CCS_TRY(h, cudaEventCreateWithFlags(&M->in_free[k], cudaEventDisableTiming));
    CCS_TRY(h, cudaEventCreateWithFlags(&M->out_ready[k], cudaEventDisableTiming));
    CCS_TRY(h, cudaEventCreateWithFlags(&M->out_free[k], cudaEventDisableTiming));
  }
  CCS_TRY(h, cudaStreamCreateWithFlags(&M->cin, cudaStreamNonBlocking));
  CCS_TRY(h, cudaStreamCreateWithFlags(&M->cout, cudaStreamNonBlocking));
  CCS_TRY(h, cudaMalloc(&h->d_partials, 2 * kDiagBlocks * sizeof(double)));
  int rc = build_work(h, kMxTiles[M->var], &M->d_work, &M->nwork);
  if (rc) return rc;
  M->grid = mixed_max_grid(M->var, h->cfg.device);
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

// (re)build the stage descriptors once phibar is known
static int mixed_build_stages(ccs_handle *h) {
  MixedLane *M = h->mixed;
  const ccs_config &c = h->cfg;
  const double a2 = c.radius * c.radius;
  MixedStage base{};
  base.L = h->L;
  base.m = h->mesh->mm;
  base.y0hp = M->S[0].hp; base.y0u = M->S[0].u; base.y0v = M->S[0].v;
  base.lohp = M->lo[0]; base.lou = M->lo[1]; base.lov = M->lo[2];
  base.acchp = M->acc[0]; base.accu = M->acc[1]; base.accv = M->acc[2];
  base.rdx = (float)(1. / c.dx); base.rdy = (float)(1. / c.dy);
  base.rdx60 = (float)(1. / (60. * c.dx)); base.rdy60 = (float)(1. / (60. * c.dy));
  base.phibar = (float)M->phibar;
  base.a2 = (float)a2;
  base.inv_a2 = (float)(1. / a2);
  base.eps_E = 1.e-2f;
  base.eps_F = (float)(1.e-2 / (a2 * a2));
  base.eps_P = (float)(1.e-2 / (a2 * a2));
  base.ediss = c.e_dissipation;
  base.op = h->op;
  {
    const double den = h->op == CCS_OP_CENTRAL2 ? 2. : h->op == CCS_OP_CENTRAL4 ? 12. : 60.;
    base.rdxc = (float)(1. / (den * c.dx));
    base.rdyc = (float)(1. / (den * c.dy));
  }
  auto mk = [&](int kind, int in, int out, double c1) {
    MixedStage s = base;
    s.kind = kind;
    s.in = M->S[in];
    s.out = M->S[out];
    s.c1 = (float)c1;
    return s;
  };
  M->h_stages.clear();
  const double dt = c.dt;
  if (c.scheme == CCS_RK4) {
    M->n_rk = 4;
    M->h_stages.push_back(mk(K_RK4_1, 0, 1, 0.5 * dt));
    M->h_stages.push_back(mk(K_RK4_2, 1, 2, 0.5 * dt));
    M->h_stages.push_back(mk(K_RK4_2, 2, 1, dt));
    M->h_stages.push_back(mk(K_RK4_4, 1, 0, dt));
  } else {
    M->n_rk = 3;
    M->h_stages.push_back(mk(K_RK3_1, 0, 1, dt));
    M->h_stages.push_back(mk(K_RK3_2, 1, 2, 0.25 * dt));
    M->h_stages.push_back(mk(K_RK3_3, 2, 0, 2. / 3. * dt));
  }
  MixedStage td = mk(K_TEND, 0, 0, 0.);
  td.thp = M->tend[0]; td.tu = M->tend[1]; td.tv = M->tend[2];
  M->h_stages.push_back(td);
  if (!M->d_stages) CCS_TRY(h, cudaMalloc(&M->d_stages, 8 * sizeof(MixedStage)));
  CCS_TRY(h, cudaMemcpyAsync(M->d_stages, M->h_stages.data(), M->h_stages.size() * sizeof(MixedStage),
                             cudaMemcpyHostToDevice, h->stream));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  if (M->g_step) {
    cudaGraphExecDestroy(M->g_step);
    M->g_step = nullptr;
  }
  return CCS_OK;
}

static void mixed_handle_destroy(ccs_handle *h) {
  MixedLane *M = h->mixed;
  if (!M) return;
  if (M->cin) cudaStreamSynchronize(M->cin);
  if (M->cout) cudaStreamSynchronize(M->cout);
  if (M->g_step) cudaGraphExecDestroy(M->g_step);
  if (M->buf) cudaFree(M->buf);
  for (int k = 0; k < 2; k++)
    for (cudaEvent_t e : {M->in_ready[k], M->in_free[k], M->out_ready[k], M->out_free[k]})
      if (e) cudaEventDestroy(e);
  if (M->cin) cudaStreamDestroy(M->cin);
  if (M->cout) cudaStreamDestroy(M->cout);
  if (M->staging) cudaFree(M->staging);
  if (M->d_stages) cudaFree(M->d_stages);
  if (M->d_work) cudaFree(M->d_work);
  delete M;
  h->mixed = nullptr;
}

// Copies n fields of `bytes` each (dst[q] <- src[q], NULL entries skipped), one
// cudaMemcpyAsync per run of fields whose destination and source both continue the
// previous field's: a caller whose host arrays are consecutive slices of one
// page-locked block gets one copy per direction, which the host link overlaps
// with the other direction better than many smaller copies.
static cudaError_t copy_field_runs(void *const *dst, const void *const *src, int n, size_t bytes,
                                   cudaMemcpyKind kind, cudaStream_t s) {
  int q = 0;
  while (q < n) {
    if (!dst[q] || !src[q]) {
      q++;
      continue;
    }
    int e = q + 1;
    while (e < n && dst[e] && src[e] && (char *)dst[e] == (char *)dst[e - 1] + bytes &&
           (const char *)src[e] == (const char *)src[e - 1] + bytes)
      e++;
    const cudaError_t err = cudaMemcpyAsync(dst[q], src[q], (size_t)(e - q) * bytes, kind, s);
    if (err != cudaSuccess) return err;
    q = e;
  }
  return cudaSuccess;
}

static int mixed_set_state(ccs_handle *h, const ccs_state_view *s, bool sync) {
  MixedLane *M = h->mixed;
  const Layout &L = h->L;
  const size_t nref = (size_t)L.nh * L.nh * 6;
  if (!M->have_phibar) {
    double phibar = h->cfg.phi_mean;
    if (!(phibar > 0.)) {
      double acc = 0.;
      for (int p = 0; p < 6; p++)
        for (int j = 1; j <= L.N; j++)
          for (int i = 1; i <= L.N; i++)
            acc += s->phi[(size_t)(i + L.h - 1) + (size_t)L.nh * ((size_t)(j + L.h - 1) + (size_t)L.nh * p)];
      phibar = acc / (6. * L.N * L.N);
    }
    M->phibar = phibar;
    M->have_phibar = true;
    int rc = mixed_build_stages(h);
    if (rc) return rc;
  }
  // copy into the next in slot once the import that last read it has run
  const int k = M->in_slot;
  M->in_slot ^= 1;
  double *st = M->stage_in[k];
  CCS_TRY(h, cudaStreamWaitEvent(M->cin, M->in_free[k], 0));
  void *const dst[3] = {st, st + nref, st + 2 * nref};
  const void *const src[3] = {s->phi, s->u, s->v};
  CCS_TRY(h, copy_field_runs(dst, src, 3, nref * sizeof(double), cudaMemcpyHostToDevice, M->cin));
  CCS_TRY(h, cudaEventRecord(M->in_ready[k], M->cin));
  CCS_TRY(h, cudaStreamWaitEvent(h->stream, M->in_ready[k], 0));
  const double a2 = h->cfg.radius * h->cfg.radius;
  CCS_TRY(h, launch_mixed_import(L, st, st + nref, st + 2 * nref, M->phibar, 1. / a2, M->S[0], M->lo[0],
                                 M->lo[1], M->lo[2], h->stream));
  CCS_TRY(h, cudaEventRecord(M->in_free[k], h->stream));
  if (sync) CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

static int mixed_get_state(ccs_handle *h, ccs_state_view *s, bool sync) {
  MixedLane *M = h->mixed;
  if (!M->have_phibar) return CCS_ERR_ARG;
  const Layout &L = h->L;
  const size_t nref = (size_t)L.nh * L.nh * 6;
  // export into the next out slot once the copies that last read it are done
  const int k = M->out_slot;
  M->out_slot ^= 1;
  double *out[8];
  for (int q = 0; q < 8; q++) out[q] = M->stage_out[k] + q * nref;
  const double a2 = h->cfg.radius * h->cfg.radius;
  CCS_TRY(h, cudaStreamWaitEvent(h->stream, M->out_free[k], 0));
  CCS_TRY(h, launch_mixed_export(L, M->S[0], M->lo[0], M->lo[1], M->lo[2], h->mesh->m64, M->phibar, a2, out,
                                 h->stream));
  CCS_TRY(h, cudaEventRecord(M->out_ready[k], h->stream));
  CCS_TRY(h, cudaStreamWaitEvent(M->cout, M->out_ready[k], 0));
  void *const dst[8] = {s->phiG, s->u, s->v, s->phi, s->uC, s->vC, s->zonal_wind, s->meridional_wind};
  const void *const src[8] = {out[0], out[1], out[2], out[3], out[4], out[5], out[6], out[7]};
  CCS_TRY(h, copy_field_runs(dst, src, 8, nref * sizeof(double), cudaMemcpyDeviceToHost, M->cout));
  CCS_TRY(h, cudaEventRecord(M->out_free[k], M->cout));
  if (sync) CCS_TRY(h, cudaStreamSynchronize(M->cout));
  return CCS_OK;
}

static bool mixed_has_stages(const ccs_handle *h) { return h->mixed->have_phibar; }

// one launch of the handle's mixed stage kernel instance (tile variant, operator
// family, E-flux option) over stage descriptor d
static cudaError_t mixed_launch(ccs_handle *h, const MixedStage *d) {
  MixedLane *M = h->mixed;
  return launch_mixed_stage(M->var, h->op != CCS_OP_WENO, h->cfg.e_dissipation != CCS_EDISS_ZERO, d, M->d_work,
                            M->nwork, M->grid, h->stream);
}

static int mixed_sync(ccs_handle *h) {
  MixedLane *M = h->mixed;
  CCS_TRY(h, cudaStreamSynchronize(M->cin));
  CCS_TRY(h, cudaStreamSynchronize(M->cout));
  return CCS_OK;
}

static int mixed_enqueue_step(ccs_handle *h) {
  MixedLane *M = h->mixed;
  for (int k = 0; k < M->n_rk; k++) {
    if (h->timing) CCS_TRY(h, cudaEventRecord(h->ev0, h->stream));
    CCS_TRY(h, mixed_launch(h, M->d_stages + k));
    if (h->timing) {
      CCS_TRY(h, cudaEventRecord(h->ev1, h->stream));
      CCS_TRY(h, cudaEventSynchronize(h->ev1));
      float ms = 0.f;
      CCS_TRY(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
      h->kernel_ms += ms;
      h->launches++;
    }
  }
  return CCS_OK;
}

static int mixed_step(ccs_handle *h, int nsteps, bool sync) {
  MixedLane *M = h->mixed;
  if (!M->have_phibar) return CCS_ERR_ARG;
  if (nsteps <= 0) return CCS_OK;
  if (h->timing) {
    for (int s = 0; s < nsteps; s++) {
      int rc = mixed_enqueue_step(h);
      if (rc) return rc;
    }
  } else {
    if (!M->g_step) {
      cudaGraph_t g = nullptr;
      CCS_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      int rc = mixed_enqueue_step(h);
      cudaError_t e = cudaStreamEndCapture(h->stream, &g);
      if (rc) return rc;
      CCS_TRY(h, e);
      e = cudaGraphInstantiate(&M->g_step, g, 0);
      cudaGraphDestroy(g);
      CCS_TRY(h, e);
    }
    for (int s = 0; s < nsteps; s++) CCS_TRY(h, cudaGraphLaunch(M->g_step, h->stream));
  }
  if (sync) CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

static int mixed_tend(ccs_handle *h, double *tp, double *tu, double *tv) {
  MixedLane *M = h->mixed;
  if (!M->have_phibar) return CCS_ERR_ARG;
  const Layout &L = h->L;
  const size_t nref = (size_t)L.nh * L.nh * 6;
  CCS_TRY(h, mixed_launch(h, M->d_stages + M->n_rk));
  const double a2 = h->cfg.radius * h->cfg.radius;
  CCS_TRY(h, cudaStreamSynchronize(M->cout));  // no copy may still read the out slots
  double *o = M->stage_out[0];
  CCS_TRY(h, launch_mixed_tend_export(L, M->tend[0], M->tend[1], M->tend[2], h->mesh->m64, a2, o, o + nref,
                                      o + 2 * nref, h->stream));
  double *dst[3] = {tp, tu, tv};
  for (int k = 0; k < 3; k++)
    if (dst[k])
      CCS_TRY(h, cudaMemcpyAsync(dst[k], o + k * nref, nref * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  return CCS_OK;
}

static int mixed_diag(ccs_handle *h, double *mass, double *energy) {
  MixedLane *M = h->mixed;
  if (!M->have_phibar) return CCS_ERR_ARG;
  const double a2 = h->cfg.radius * h->cfg.radius;
  CCS_TRY(h, launch_mixed_diag(h->L, M->S[0], M->lo[0], M->lo[1], M->lo[2], h->mesh->m64, M->phibar, a2,
                               h->d_partials, kDiagBlocks, h->stream));
  std::vector<double> part(2 * kDiagBlocks);
  CCS_TRY(h, cudaMemcpyAsync(part.data(), h->d_partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  double tm = 0., te = 0.;
  for (int b = 0; b < kDiagBlocks; b++) {
    tm += part[2 * b];
    te += part[2 * b + 1];
  }
  if (mass) *mass = tm;
  if (energy) *energy = te;
  return CCS_OK;
}

extern "C" int ccs_check_state(ccs_handle *h, int64_t *bad_cells) {
  if (!h) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  if (!h->d_bad) CCS_TRY(h, cudaMalloc(&h->d_bad, sizeof(unsigned long long)));
  CCS_TRY(h, cudaMemsetAsync(h->d_bad, 0, sizeof(unsigned long long), h->stream));
  const int64_t ncell = (int64_t)h->L.N * h->L.N * 6;
  const int grid = (int)std::min<int64_t>((ncell + 255) / 256, 4096);
  if (h->cfg.precision == CCS_MIXED) {
    MixedLane *M = h->mixed;
    if (!M->have_phibar) return CCS_ERR_ARG;
    health_kernel<float><<<grid, 256, 0, h->stream>>>(h->L, M->S[0].hp, M->S[0].u, M->S[0].v, M->phibar,
                                                       h->d_bad);
  } else {
    health_kernel<double><<<grid, 256, 0, h->stream>>>(h->L, h->S[0].phi, h->S[0].u, h->S[0].v, 0., h->d_bad);
  }
  CCS_TRY(h, cudaGetLastError());
  unsigned long long bad = 0;
  CCS_TRY(h, cudaMemcpyAsync(&bad, h->d_bad, sizeof(bad), cudaMemcpyDeviceToHost, h->stream));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  if (bad_cells) *bad_cells = (int64_t)bad;
  return bad ? CCS_ERR_NAN : CCS_OK;
}

extern "C" int ccs_courant(ccs_handle *h, double *courant) {
  if (!h || !courant) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  if (!h->d_lmax) CCS_TRY(h, cudaMalloc(&h->d_lmax, sizeof(unsigned long long)));
  CCS_TRY(h, cudaMemsetAsync(h->d_lmax, 0, sizeof(unsigned long long), h->stream));
  const int64_t ncell = (int64_t)(h->L.N + 2) * (h->L.N + 2) * 6;
  const int grid = (int)std::min<int64_t>((ncell + 255) / 256, 4096);
  const MeshF64 &m = h->mesh->m64;
  if (h->cfg.precision == CCS_MIXED) {
    MixedLane *M = h->mixed;
    if (!M->have_phibar) return CCS_ERR_ARG;
    courant_kernel<<<grid, 256, 0, h->stream>>>(h->L, M->S[0].hp, M->S[0].u, M->S[0].v, nullptr, nullptr, nullptr,
                                               m, M->phibar, h->cfg.radius * h->cfg.radius, h->d_lmax);
  } else {
    courant_kernel<<<grid, 256, 0, h->stream>>>(h->L, nullptr, nullptr, nullptr, h->S[0].phi, h->S[0].uC,
                                               h->S[0].vC, m, 0., 0., h->d_lmax);
  }
  CCS_TRY(h, cudaGetLastError());
  unsigned long long bits = 0;
  CCS_TRY(h, cudaMemcpyAsync(&bits, h->d_lmax, sizeof(bits), cudaMemcpyDeviceToHost, h->stream));
  CCS_TRY(h, cudaStreamSynchronize(h->stream));
  double lmax = 0.;
  std::memcpy(&lmax, &bits, sizeof(lmax));
  *courant = h->cfg.dt * lmax / std::min(h->cfg.dx, h->cfg.dy);
  return std::isfinite(*courant) ? CCS_OK : CCS_ERR_NAN;
}

// ---------------------------------------------------------------------------
// tile variants and the autotuner
// ---------------------------------------------------------------------------
namespace {
std::mutex g_tune_mutex;
std::map<std::tuple<int, int, int, int>, int> g_tune_cache;  // (device, lane, N, halo) -> variant
}  // namespace

static int lane_nvar(const ccs_handle *h) { return h->cfg.precision == CCS_MIXED ? MX_NVAR : F64_NVAR; }

// Switches the handle's stage kernel to tile variant var: new work list and grid;
// the captured step graphs are dropped and re-captured on the next step.
static int set_variant(ccs_handle *h, int var) {
  if (var < 0 || var >= lane_nvar(h)) return CCS_ERR_ARG;
  const int dev = h->cfg.device;
  if (h->cfg.precision == CCS_MIXED) {
    MixedLane *M = h->mixed;
    if (var == M->var && M->d_work) return CCS_OK;
    int rc = build_work(h, kMxTiles[var], &M->d_work, &M->nwork);
    if (rc) return rc;
    M->var = var;
    M->grid = mixed_max_grid(var, dev);
    if (M->g_step) {
      cudaGraphExecDestroy(M->g_step);
      M->g_step = nullptr;
    }
  } else {
    if (var == h->var && h->d_work) return CCS_OK;
    int rc = build_work(h, kF64Tiles[var], &h->d_work, &h->nwork);
    if (rc) return rc;
    h->var = var;
    h->grid = f64_max_grid(var, dev);
    if (h->g_step) cudaGraphExecDestroy(h->g_step);
    if (h->g_step_sw) cudaGraphExecDestroy(h->g_step_sw);
    h->g_step = h->g_step_sw = nullptr;
  }
  return CCS_OK;
}

// Mean time of one stage launch with the handle's current variant, over the RK
// stages before the last one, in step order.  Those stages read the state and
// write only stage scratch (the next stage's input and the RK accumulator); the
// last stage, which writes the state, is the only one left out, so timing leaves
// the state unchanged.
static int time_stages(ccs_handle *h, int reps, double *us) {
  const bool mx = h->cfg.precision == CCS_MIXED;
  const int nst = (mx ? h->mixed->n_rk : h->n_rk) - 1;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CCS_TRY(h, cudaEventCreate(&e0));
  CCS_TRY(h, cudaEventCreate(&e1));
  auto launch = [&](int k) -> cudaError_t {
    if (mx) {
      MixedLane *M = h->mixed;
      return mixed_launch(h, M->d_stages + k);
    }
    return launch_f64_stage(h->var, h->d_stages + k, h->d_work, h->nwork, h->grid, h->stream);
  };
  cudaError_t e = launch(0);  // warm-up
  for (int r = 0; r < reps && e == cudaSuccess; r++) {
    if (r == 0) e = cudaEventRecord(e0, h->stream);
    for (int k = 0; k < nst && e == cudaSuccess; k++) e = launch(k);
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, h->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CCS_TRY(h, e);
  *us = 1e3 * ms / (reps * nst);
  return CCS_OK;
}

extern "C" int ccs_set_variant(ccs_handle *h, int var) {
  if (!h) return CCS_ERR_ARG;
  cudaSetDevice(h->cfg.device);
  return set_variant(h, var);
}

extern "C" int ccs_get_variant(ccs_handle *h, int *var, int *tile_x, int *tile_y) {
  if (!h) return CCS_ERR_ARG;
  const bool mx = h->cfg.precision == CCS_MIXED;
  const int v = mx ? h->mixed->var : h->var;
  const TileShape ts = mx ? kMxTiles[v] : kF64Tiles[v];
  if (var) *var = v;
  if (tile_x) *tile_x = ts.tx;
  if (tile_y) *tile_y = ts.ty;
  return CCS_OK;
}

extern "C" int ccs_autotune(ccs_handle *h, int reps, int force, int *chosen, double *times_us) {
  NvtxRange nvtx("ccs_autotune");
  if (!h || reps < 1) return CCS_ERR_ARG;
  if (h->cfg.precision == CCS_MIXED && !h->mixed->have_phibar) return CCS_ERR_ARG;  // state not set
  cudaSetDevice(h->cfg.device);
  const int nvar = lane_nvar(h);
  if (times_us)
    for (int v = 0; v < CCS_MAX_VARIANTS; v++) times_us[v] = 0.;
  const auto key = std::make_tuple(h->cfg.device, h->cfg.precision, h->L.N, h->L.h);
  int best = -1;
  if (!force) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) best = it->second;
  }
  if (best < 0) {
    double best_us = 0.;
    for (int v = 0; v < nvar; v++) {
      int rc = set_variant(h, v);
      if (rc) return rc;
      double us = 0.;
      rc = time_stages(h, reps, &us);
      if (rc) return rc;
      if (times_us) times_us[v] = us;
      if (best < 0 || us < best_us) {
        best = v;
        best_us = us;
      }
    }
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = best;
  }
  int rc = set_variant(h, best);
  if (rc) return rc;
  if (chosen) *chosen = best;
  return CCS_OK;
}

// ---------------------------------------------------------------------------
// batches: one launch per lane and RK stage over the union of the members' tiles
// ---------------------------------------------------------------------------
struct BatchGroup {
  int lane = 0, scheme = 0, n_rk = 0, nmem = 0, var = 0;
  bool central = false;  // the members' spatial operator is a central difference
  bool ediss = false;    // the members reconstruct the E-flux dissipation
  std::vector<ccs_handle *> members;
  void *d_stages = nullptr;  // [n_rk + 1][nmem] F64Stage or MixedStage (last row: F64 final with sphere winds)
  WorkItem *d_work = nullptr;
  int nwork = 0, grid = 0;
  cudaStream_t stream = nullptr;  // groups are independent: each runs on its own stream
  cudaEvent_t done = nullptr;
};

struct ccs_batch {
  std::vector<BatchGroup> groups;
  std::vector<ccs_handle *> members;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  cudaEvent_t after = nullptr;  // end of the last enqueued step, for the members' streams
  int device = 0;
  cudaGraphExec_t g_step = nullptr, g_step_sw = nullptr;
  std::string err;
};

#define BATCH_TRY(b, call)                                                     \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      (b)->err = std::string(#call) + ": " + cudaGetErrorString(e_);           \
      return CCS_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

static int group_nvar(const BatchGroup &g) { return g.lane == CCS_FP64 ? F64_NVAR : MX_NVAR; }

// Stage k of group g (k = n_rk - 1 with with_sw: the FP64 final stage that also
// writes the sphere winds) as one launch over the work list of all its members.
static cudaError_t group_launch(BatchGroup &g, int k, bool with_sw) {
  if (g.lane == CCS_FP64) {
    const int row = (k == g.n_rk - 1 && with_sw) ? g.n_rk : k;
    return launch_f64_stage(g.var, (const F64Stage *)g.d_stages + (size_t)row * g.nmem, g.d_work, g.nwork, g.grid,
                            g.stream);
  }
  return launch_mixed_stage(g.var, g.central, g.ediss, (const MixedStage *)g.d_stages + (size_t)k * g.nmem,
                            g.d_work, g.nwork, g.grid, g.stream);
}

// (Re)builds group g's work list for tile variant var: every tile of the six panels
// of every member, member by member.
static int group_set_var(ccs_batch *b, BatchGroup &g, int var) {
  if (var < 0 || var >= group_nvar(g)) return CCS_ERR_ARG;
  const TileShape ts = g.lane == CCS_FP64 ? kF64Tiles[var] : kMxTiles[var];
  std::vector<WorkItem> work;
  for (int m = 0; m < g.nmem; m++) {
    const int N = g.members[m]->cfg.N;
    const int ntx = (N + ts.tx - 1) / ts.tx, nty = (N + ts.ty - 1) / ts.ty;
    for (int p = 0; p < 6; p++)
      for (int ty = 0; ty < nty; ty++)
        for (int tx = 0; tx < ntx; tx++)
          work.push_back(WorkItem{(int16_t)m, (int16_t)p, (int16_t)tx, (int16_t)ty});
  }
  if (g.d_work) {
    BATCH_TRY(b, cudaStreamSynchronize(g.stream));
    BATCH_TRY(b, cudaFree(g.d_work));
    g.d_work = nullptr;
  }
  BATCH_TRY(b, cudaMalloc(&g.d_work, work.size() * sizeof(WorkItem)));
  BATCH_TRY(b, cudaMemcpy(g.d_work, work.data(), work.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
  g.nwork = (int)work.size();
  g.var = var;
  g.grid = g.lane == CCS_FP64 ? f64_max_grid(var, b->device) : mixed_max_grid(var, b->device);
  return CCS_OK;
}

// One step of every group: the groups fork from the batch stream, run their RK
// stages on their own streams (an FP64 group is FP64-issue bound and a mixed group
// FP32 / latency bound, so they share the SMs well) and join back.
static int batch_enqueue(ccs_batch *b, bool with_sw) {
  BATCH_TRY(b, cudaEventRecord(b->fork, b->stream));
  for (auto &g : b->groups) {
    BATCH_TRY(b, cudaStreamWaitEvent(g.stream, b->fork, 0));
    for (int k = 0; k < g.n_rk; k++) BATCH_TRY(b, group_launch(g, k, with_sw));
    BATCH_TRY(b, cudaEventRecord(g.done, g.stream));
    BATCH_TRY(b, cudaStreamWaitEvent(b->stream, g.done, 0));
  }
  return CCS_OK;
}

extern "C" int ccs_debug_bounds(int *site, int64_t *index) {
  if (!site || !index) return CCS_ERR_ARG;
#ifndef CCS_BOUNDS
  *site = -1;
  *index = 0;
  return CCS_OK;
#else
  if (cudaDeviceSynchronize() != cudaSuccess) return CCS_ERR_CUDA;
  const unsigned long long a = f64_bounds_take(), b = mixed_bounds_take();
  const unsigned long long v = a ? a : b;
  *site = (int)(v >> 48);
  long long i = (long long)(v & 0xffffffffffffull);
  if (i & (1ll << 47)) i -= 1ll << 48;  // the index's sign
  *index = *site ? i : 0;
  return CCS_OK;
#endif
}

extern "C" int ccs_debug_bounds_selftest(void) {
#ifndef CCS_BOUNDS
  return CCS_ERR_UNSUPPORTED;
#else
  int site = 0;
  int64_t idx = 0;
  int rc = ccs_debug_bounds(&site, &idx);  // start clean
  if (rc) return rc;
  if (launch_bounds_selftest(7, 3, 999, 0) != cudaSuccess) return CCS_ERR_CUDA;
  if (launch_bounds_selftest(-2, 3, 998, 0) != cudaSuccess) return CCS_ERR_CUDA;  // the first hit stays
  if (launch_bounds_selftest(1, 3, 997, 0) != cudaSuccess) return CCS_ERR_CUDA;   // in range: no hit
  rc = ccs_debug_bounds(&site, &idx);
  if (rc) return rc;
  if (site != 999 || idx != 7) return CCS_ERR_CUDA;
  rc = ccs_debug_bounds(&site, &idx);
  if (rc) return rc;
  return site == 0 ? CCS_OK : CCS_ERR_CUDA;
#endif
}

// Fills batch b (already holding its members): one group per (lane, scheme,
// operator family, E-flux option), each with its own stream, stage table and work
// list.  A group runs one tile variant for all its members: the variant of its
// member with the most cells (that member's autotuned choice) until
// ccs_batch_autotune times the group's own work list.
static int batch_build(ccs_batch *b) {
  const int n = (int)b->members.size();
  BATCH_TRY(b, cudaSetDevice(b->device));
  BATCH_TRY(b, cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BATCH_TRY(b, cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  BATCH_TRY(b, cudaEventCreateWithFlags(&b->after, cudaEventDisableTiming));
  auto member_var = [](const ccs_handle *m) { return m->cfg.precision == CCS_MIXED ? m->mixed->var : m->var; };
  for (int lane = 0; lane < 2; lane++)
    for (int scheme = 0; scheme < 2; scheme++)
      for (int central = 0; central < 2; central++)
        for (int ediss = 0; ediss < 2; ediss++) {
          std::vector<ccs_handle *> mem;
          for (int k = 0; k < n; k++) {
            ccs_handle *h = b->members[k];
            if (h->cfg.precision == lane && h->cfg.scheme == scheme && (h->op != CCS_OP_WENO) == (central != 0) &&
                (h->cfg.e_dissipation != CCS_EDISS_ZERO) == (ediss != 0))
              mem.push_back(h);
          }
          if (mem.empty()) continue;
          b->groups.emplace_back();  // owned by the batch from here on, so a failure below frees it
          BatchGroup &g = b->groups.back();
          g.lane = lane;
          g.scheme = scheme;
          g.central = central != 0;
          g.ediss = ediss != 0;
          g.members = mem;
          g.nmem = (int)mem.size();
          g.n_rk = scheme == CCS_RK4 ? 4 : 3;
          BATCH_TRY(b, cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
          BATCH_TRY(b, cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming));
          ccs_handle *largest = mem[0];
          for (ccs_handle *h : mem)
            if (h->cfg.N > largest->cfg.N) largest = h;
          int rc = group_set_var(b, g, member_var(largest));
          if (rc) return rc;
          if (lane == CCS_FP64) {
            std::vector<F64Stage> st((size_t)(g.n_rk + 1) * g.nmem);
            for (int k = 0; k <= g.n_rk; k++)
              for (int m = 0; m < g.nmem; m++) st[(size_t)k * g.nmem + m] = g.members[m]->h_stages[k];
            BATCH_TRY(b, cudaMalloc(&g.d_stages, st.size() * sizeof(F64Stage)));
            BATCH_TRY(b, cudaMemcpy(g.d_stages, st.data(), st.size() * sizeof(F64Stage), cudaMemcpyHostToDevice));
          } else {
            std::vector<MixedStage> st((size_t)g.n_rk * g.nmem);
            for (int k = 0; k < g.n_rk; k++)
              for (int m = 0; m < g.nmem; m++) st[(size_t)k * g.nmem + m] = g.members[m]->mixed->h_stages[k];
            BATCH_TRY(b, cudaMalloc(&g.d_stages, st.size() * sizeof(MixedStage)));
            BATCH_TRY(b, cudaMemcpy(g.d_stages, st.data(), st.size() * sizeof(MixedStage), cudaMemcpyHostToDevice));
          }
        }
  return CCS_OK;
}

extern "C" int ccs_batch_create(ccs_handle *const *members, int n, ccs_batch **out) {
  if (!members || n < 1 || !out) return CCS_ERR_ARG;
  *out = nullptr;
  for (int k = 0; k < n; k++)
    if (!members[k]) return CCS_ERR_ARG;
  const int dev = members[0]->cfg.device;
  for (int k = 0; k < n; k++) {
    if (members[k]->cfg.device != dev) return CCS_ERR_ARG;
    if (members[k]->cfg.precision == CCS_MIXED && !members[k]->mixed->have_phibar) return CCS_ERR_ARG;
  }
  if (n > 32767) return CCS_ERR_ARG;
  ccs_batch *b = new ccs_batch();
  b->device = dev;
  b->members.assign(members, members + n);
  const int rc = batch_build(b);
  if (rc) {
    ccs_batch_destroy(b);
    return rc;
  }
  *out = b;
  return CCS_OK;
}

// Mean time of one stage launch of group g with its current variant: the stages
// before the last, which read the members' states and write only stage scratch.
static int group_time_stages(ccs_batch *b, BatchGroup &g, int reps, double *us) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BATCH_TRY(b, cudaEventCreate(&e0));
  cudaError_t e = cudaEventCreate(&e1);
  const int nst = g.n_rk - 1;
  if (e == cudaSuccess) e = group_launch(g, 0, false);  // warm-up
  if (e == cudaSuccess) e = cudaEventRecord(e0, g.stream);
  for (int r = 0; r < reps && e == cudaSuccess; r++)
    for (int k = 0; k < nst && e == cudaSuccess; k++) e = group_launch(g, k, false);
  if (e == cudaSuccess) e = cudaEventRecord(e1, g.stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  BATCH_TRY(b, e);
  *us = 1e3 * ms / (reps * nst);
  return CCS_OK;
}

extern "C" int ccs_batch_autotune(ccs_batch *b, int reps) {
  NvtxRange nvtx("ccs_batch_autotune");
  if (!b || reps < 1) return CCS_ERR_ARG;
  BATCH_TRY(b, cudaSetDevice(b->device));
  for (ccs_handle *h : b->members) BATCH_TRY(b, cudaStreamSynchronize(h->stream));  // pending uploads
  for (auto &g : b->groups) {
    int best = -1;
    double best_us = 0.;
    for (int v = 0; v < group_nvar(g); v++) {
      int rc = group_set_var(b, g, v);
      if (rc) return rc;
      double us = 0.;
      rc = group_time_stages(b, g, reps, &us);
      if (rc) return rc;
      if (best < 0 || us < best_us) {
        best = v;
        best_us = us;
      }
    }
    int rc = group_set_var(b, g, best);
    if (rc) return rc;
  }
  if (b->g_step) cudaGraphExecDestroy(b->g_step);
  if (b->g_step_sw) cudaGraphExecDestroy(b->g_step_sw);
  b->g_step = b->g_step_sw = nullptr;
  return CCS_OK;
}

extern "C" int ccs_batch_info(ccs_batch *b, int *launches_per_stage, int max_groups, int *lane, int *variant,
                              int *members) {
  if (!b || max_groups < 0) return CCS_ERR_ARG;
  if (launches_per_stage) *launches_per_stage = (int)b->groups.size();
  for (int q = 0; q < max_groups && q < (int)b->groups.size(); q++) {
    const BatchGroup &g = b->groups[q];
    if (lane) lane[q] = g.lane;
    if (variant) variant[q] = g.var;
    if (members) members[q] = g.nmem;
  }
  return CCS_OK;
}

static int batch_capture(ccs_batch *b, bool with_sw, cudaGraphExec_t *out) {
  cudaGraph_t g = nullptr;
  BATCH_TRY(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int rc = batch_enqueue(b, with_sw);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  BATCH_TRY(b, e);
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  BATCH_TRY(b, e);
  return CCS_OK;
}

static int batch_step(ccs_batch *b, int nsteps, bool sync) {
  NvtxRange nvtx("ccs_batch_step");
  if (!b || nsteps < 0) return CCS_ERR_ARG;
  if (nsteps == 0) return CCS_OK;
  BATCH_TRY(b, cudaSetDevice(b->device));
  if (!b->g_step) {
    int rc = batch_capture(b, false, &b->g_step);
    if (!rc) rc = batch_capture(b, true, &b->g_step_sw);
    if (rc) return rc;
  }
  // the step starts after the members' own pending work (an asynchronous upload and
  // its import, an asynchronous step) and the members' later work after the step
  for (ccs_handle *h : b->members) {
    if (!h->ev_order) BATCH_TRY(b, cudaEventCreateWithFlags(&h->ev_order, cudaEventDisableTiming));
    BATCH_TRY(b, cudaEventRecord(h->ev_order, h->stream));
    BATCH_TRY(b, cudaStreamWaitEvent(b->stream, h->ev_order, 0));
  }
  for (int s = 0; s < nsteps - 1; s++) BATCH_TRY(b, cudaGraphLaunch(b->g_step, b->stream));
  BATCH_TRY(b, cudaGraphLaunch(b->g_step_sw, b->stream));
  BATCH_TRY(b, cudaEventRecord(b->after, b->stream));
  for (ccs_handle *h : b->members) BATCH_TRY(b, cudaStreamWaitEvent(h->stream, b->after, 0));
  if (sync) BATCH_TRY(b, cudaStreamSynchronize(b->stream));
  for (ccs_handle *h : b->members) h->sphere_valid = true;
  return CCS_OK;
}

extern "C" int ccs_batch_step(ccs_batch *b, int nsteps) { return batch_step(b, nsteps, true); }
extern "C" int ccs_batch_step_async(ccs_batch *b, int nsteps) { return batch_step(b, nsteps, false); }
extern "C" void *ccs_batch_stream(ccs_batch *b) { return b ? (void *)b->stream : nullptr; }
extern "C" const char *ccs_batch_last_error(const ccs_batch *b) { return b ? b->err.c_str() : ""; }

extern "C" void ccs_batch_destroy(ccs_batch *b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->g_step) cudaGraphExecDestroy(b->g_step);
  if (b->g_step_sw) cudaGraphExecDestroy(b->g_step_sw);
  for (auto &g : b->groups) {
    if (g.d_stages) cudaFree(g.d_stages);
    if (g.d_work) cudaFree(g.d_work);
    if (g.done) cudaEventDestroy(g.done);
    if (g.stream) cudaStreamDestroy(g.stream);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->after) cudaEventDestroy(b->after);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}
