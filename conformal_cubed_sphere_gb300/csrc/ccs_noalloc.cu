// ccs_noalloc.cu -- ccs_diag_noalloc: total mass and energy of a state that already
// lives in device memory, for callers that must not allocate.
//
// Some host programs cannot call cudaMalloc: a model driver that runs inside another
// framework's memory pool, or under a device arena sized once at start-up, must not
// allocate behind that pool's back.  They hold the state on the device already and
// only want the diagnostic sums.  This entry point keeps its only scratch -- one
// partial sum pair per panel row -- in the file-scope array below, so it calls no
// cudaMalloc, cudaFree or allocating library routine.
#include <cuda_runtime.h>

#include <mutex>

#include "ccs_internal.h"

namespace {

// Largest panel size this entry point accepts: one (mass, energy) partial per panel
// row, 6 * 4096 rows -> 384 KiB of device memory, held by every GPU that loads the
// library until the process exits.
constexpr int kMaxN = CCS_NOALLOC_MAX_N;
static __device__ __align__(256) double g_row_partials[2 * 6 * kMaxN];

// Device addresses of g_row_partials, looked up once per device.
constexpr int kMaxDevices = 64;
double *g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// One block per panel row: the row's interior cells, i fastest (the reference's
// loop order of diag_mod.F90:10-53), reduced in a fixed tree order.
__global__ void row_sums_kernel(int N, int halo, const double *__restrict__ phiG, const double *__restrict__ phi,
                                const double *__restrict__ u, const double *__restrict__ v,
                                const double *__restrict__ uC, const double *__restrict__ vC,
                                const double *__restrict__ sqrtG, const double *__restrict__ phis,
                                double *__restrict__ partials) {
  __shared__ double sm[2][256];
  const int row = blockIdx.x;  // p * N + (j - 1)
  const int p = row / N, j = 1 + row % N;
  const int nh = N + 2 * halo;
  const size_t base = (size_t)halo + (size_t)nh * ((size_t)(j + halo - 1) + (size_t)nh * p);  // cell (1, j, p)
  double m = 0., e = 0.;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const size_t c = base + i;
    m += phiG[c];
    const double KE = 0.5 * phi[c] * (u[c] * uC[c] + v[c] * vC[c]);
    const double t = phi[c] + phis[c];
    e += sqrtG[c] * (KE + 0.5 * (t * t));
  }
  sm[0][threadIdx.x] = m;
  sm[1][threadIdx.x] = e;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sm[0][threadIdx.x] += sm[0][threadIdx.x + s];
      sm[1][threadIdx.x] += sm[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[2 * row] = sm[0][0];
    partials[2 * row + 1] = sm[1][0];
  }
}

// Sums the 6 N row partials in row order into out[0] (mass) and out[1] (energy).
__global__ void final_sum_kernel(int rows, const double *__restrict__ partials, double *__restrict__ out) {
  __shared__ double sm[2][256];
  double m = 0., e = 0.;
  const int per = (rows + blockDim.x - 1) / blockDim.x;
  const int beg = threadIdx.x * per;
  const int end = beg + per < rows ? beg + per : rows;
  for (int r = beg; r < end; r++) {
    m += partials[2 * r];
    e += partials[2 * r + 1];
  }
  sm[0][threadIdx.x] = m;
  sm[1][threadIdx.x] = e;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sm[0][threadIdx.x] += sm[0][threadIdx.x + s];
      sm[1][threadIdx.x] += sm[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sm[0][0];
    out[1] = sm[1][0];
  }
}

}  // namespace

// Set-up, once per device: the device address of g_row_partials (in host code the
// array's name is only a stand-in and must not be passed to a kernel).  Done by the
// first call on each device, with that device current; that first call should come
// before any stream capture, since it may load the module.
static int scratch_for_current_device(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CCS_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return CCS_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_row_partials) != cudaSuccess || !p) return CCS_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_ptr[dev];
  return CCS_OK;
}

// Launches kernel `fn` and returns that launch's own status (cudaLaunchKernel
// reports it directly, so an error left pending by unrelated earlier work of the
// caller is neither returned as this call's failure nor cleared).  A failed launch's
// error is taken back out of the runtime's last-error slot: it is reported through
// the return code.
static cudaError_t launch(const void *fn, dim3 grid, dim3 block, void **args, cudaStream_t s) {
  const cudaError_t e = cudaLaunchKernel(fn, grid, block, args, 0, s);
  if (e != cudaSuccess) cudaGetLastError();
  return e;
}

extern "C" int ccs_diag_noalloc(int N, int halo, const double *phiG, const double *phi, const double *u,
                                const double *v, const double *uC, const double *vC, const double *sqrtG,
                                const double *phis, double *mass_energy, void *stream) {
  if (N < 1 || halo < 3 || !phiG || !phi || !u || !v || !uC || !vC || !sqrtG || !phis || !mass_energy)
    return CCS_ERR_ARG;
  if (N > kMaxN) return CCS_ERR_TOO_LARGE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CCS_ERR_CUDA;
  if (s) {  // the scratch address below is the current device's: the stream must run there
    int sdev = -1;
    if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) {
      cudaGetLastError();
      return CCS_ERR_ARG;
    }
    if (sdev != dev) return CCS_ERR_ARG;
  }
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  // every partial the final sum reads is written earlier in the same call, so
  // nothing carries over from the previous call's contents
  int n = N, h = halo, rows = 6 * N;
  void *a1[] = {&n, &h, (void *)&phiG, (void *)&phi, (void *)&u, (void *)&v, (void *)&uC, (void *)&vC,
                (void *)&sqrtG, (void *)&phis, &scratch};
  if (launch((const void *)row_sums_kernel, dim3(6 * N), dim3(256), a1, s) != cudaSuccess) return CCS_ERR_CUDA;
  void *a2[] = {&rows, &scratch, &mass_energy};
  if (launch((const void *)final_sum_kernel, dim3(1), dim3(256), a2, s) != cudaSuccess) return CCS_ERR_CUDA;
  return CCS_OK;
}
