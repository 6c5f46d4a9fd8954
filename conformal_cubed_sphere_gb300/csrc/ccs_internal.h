// ccs_internal.h -- shared definitions of the cubed-sphere library (host + device).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <vector_types.h>

#include "../../include/ccs_gpu.h"

#if defined(__CUDACC__)
#define CCS_HD __host__ __device__ __forceinline__
#else
#define CCS_HD inline
#endif

namespace ccs {

// Device/host field layout.  A field holds the 6 panels of one instance, each a
// (N + 2h) x (N + 2h) halo'd block with rows of `pitch` elements: cell (i, j) of
// panel p (i, j in [1-h, N+h], p in [0, 6)) lives at
//   (i + h - 1) + pitch * (j + h - 1) + panel * p.
// With pitch == N + 2h this is exactly the reference's Fortran order.
struct Layout {
  int N, h, nh, pitch;
  int64_t panel;  // pitch * nh
  int64_t field;  // 6 * panel
  CCS_HD int64_t idx(int i, int j, int p) const {
    return (int64_t)(i + h - 1) + (int64_t)pitch * (j + h - 1) + panel * p;
  }
};

inline Layout make_layout(int N, int h, int pitch) {
  Layout L;
  L.N = N;
  L.h = h;
  L.nh = N + 2 * h;
  L.pitch = pitch;
  L.panel = (int64_t)pitch * L.nh;
  L.field = 6 * L.panel;
  return L;
}

struct GhostSrc {
  int p, i, j;
};
GhostSrc ghost_source(int N, int p, int side, int k, int m);
int ghost_source_side(int p, int side);
bool build_push_table(const Layout &L, std::vector<int32_t> &push);

// ---- FP64 lane ----------------------------------------------------------------

// Metric arrays of one grid, one array per matrix entry (structure of arrays).
// aig = matmul(A, IG) and gia = matmul(G, IA) are formed once at set-up exactly as
// covProjPlane2Sphere / covProjSphere2Plane form them on every call
// (projection_mod.F90:71,90), so applying them is bitwise the reference.
struct MeshF64 {
  const double *sqrtG, *phis, *f;
  const double *ig11, *ig12, *ig21, *ig22;
  const double *aig11, *aig12, *aig21, *aig22;
  const double *gia11, *gia12, *gia21, *gia22;
  const int32_t *push;  // ghost push table, see build_push_table
};

// One RK state slot of the FP64 lane: the prognostic triple and the diagnostic
// fields the operator reads, all on interior + edge-halo cells.
struct StateF64 {
  double *phiG, *u, *v, *phi, *uC, *vC;
};

// ---- mixed lane ----------------------------------------------------------------

// Panel-shared FP32 metric (the metric tensor of the cube map is the same on all
// six panels, halo included, up to rounding), non-dimensionalised by the radius:
// s = sqrtG / a^2, ig = IG a^2; these arrays hold one panel and are indexed with
// panel 0.  phis and f s are per panel.  xf holds, for every ghost push-table entry,
// the FP64 2x2 matrix G_h IA_h A_s IG_s taking the source cell's covariant wind to
// the receiving halo cell's covariant wind (P2SP, fill, SP2P of correct_bdy_ghost).
struct MeshMixed {
  const float *s, *inv_s;
  const float4 *ig;  // (IG11, IG12, IG21, IG22) * a^2 of each cell of the panel

  // static wave-speed metric of the faces: the x-face right of cell (i, j) has
  // (IG11(i,j) + IG11(i+1,j)) / 2, stored transposed at lamx[idx(j, i, 0)]; the
  // y-face above cell (i, j) has (IG22(i,j) + IG22(i,j+1)) / 2 at lamy[idx(i, j, 0)].
  // Both keep the face index in the row position, so a line sweep steps by the pitch.
  const float *lamx, *lamy;
  const float *phis, *fs;
  const double *xf;
  const int32_t *push;
};

struct StateMixed {
  float *hp, *u, *v;  // phi - phi_mean, u / a^2, v / a^2 (interior + edge halo)
};

}  // namespace ccs
