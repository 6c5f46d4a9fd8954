// ccs_mixed.cu -- mixed-precision lane: FP32 state and stencil arithmetic, FP64
// cross-panel vector transforms, FP64 import / export / diagnostics.
//
// State per cell: hp = phi - phibar (geopotential of the fluid depth minus a fixed
// mean), u~ = u / a^2, v~ = v / a^2 (covariant wind), FP32; the step-to-step state
// also carries an FP32 compensation term per field (Kahan update of the final RK
// stage).  Metric: the cube map's metric tensor is the same on all six panels
// (halo included), so one FP32 copy of s = sqrtG / a^2 and ig = IG a^2 serves
// every panel and stays L2-resident; phis and f s are per panel.
//
// The WENO-Z reconstructions are written in difference form: WENO is invariant
// under adding a constant to its five inputs, so every quantity of the flux
// formula of spatial_operators_mod.F90:101-179 is expressed through the
// differences d_k = Q_{k+1} - Q_k of neighbouring cells and the corrections
// D = Rec - Q_c.  The large mean parts (phibar of phit, phibar s of phitG) cancel
// before rounding instead of after; the weights are the reference's WENO-Z
// weights with eps rescaled to the non-dimensional fields.
#include "ccs_kernels.h"
#include "ccs_bounds.cuh"

namespace ccs {

namespace {

// A tile of 32 x TY cells (TY = 32 or 16) and 8 TY threads.  Phase 2 gives each of
// the TY rows four threads (segments of its 33 x-faces) and each of the 32 columns
// TY / 8 threads (segments of its TY + 1 y-faces); phase 3 gives each thread four cells.
template <int TY_>
struct MxTile {
  static constexpr int TX = 32, TY = TY_, NT = 8 * TY;
  static constexpr int RX = TX + 6, RY = TY + 6;  // halo'd tile
  static constexpr int SP = RX + 1;               // odd pitch: a warp reading one column hits 32 banks
  static constexpr int RN = RY * SP;
  static constexpr int NFL = TX + 1;              // x-faces per tile row
  static_assert(TY % 8 == 0 && TY <= 32, "column segments of eight faces");
};
constexpr int SP = 39;  // the smem row pitch, the same for every tile height

// a / b as a times the approximate reciprocal of b (rcp.approx.ftz.f32: one MUFU
// instruction, a few ulp).  Every denominator here is eps + beta >= eps (at least
// 1e-30 after the rescaling) or a sum of WENO weights >= 1, far from the range where
// the reciprocal would flush; the result equals __fdividef's on these operands
// without that intrinsic's range handling.
__device__ __forceinline__ float qdiv(float a, float b) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  return a * r;
}

// min(a, b, c) in one three-input min.f32 instruction
__device__ __forceinline__ float min3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Difference-form WENO-Z (spatial_operators_mod.F90:282-361) of one cell for both
// directions.  d0..d3 = Q(c-1)-Q(c-2), Q(c)-Q(c-1), Q(c+1)-Q(c), Q(c+2)-Q(c+1).
// Returns Dp = Rec+(c) - Q(c) (face c+1/2) and Dm = Rec-(c) - Q(c) (face c-1/2).
// The "-" smoothness indicators are the "+" ones mirrored (beta'_k = beta_{4-k}),
// so the three divisions tau5 / (eps + beta_k) are shared.
__device__ __forceinline__ void weno_d(float d0, float d1, float d2, float d3, float eps, float &Dp,
                                       float &Dm) {
  const float A1 = d1 - d0, A2 = d2 - d1, A3 = d3 - d2;
  const float B1 = fmaf(3.f, d1, -d0), B2 = d1 + d2, B3 = fmaf(-3.f, d2, d3);
  // 4 beta_k (eps is passed times 4 as well: the weights depend on ratios only)
  const float k133 = 13.f / 3.f;
  const float b1 = fmaf(k133 * A1, A1, B1 * B1);
  const float b2 = fmaf(k133 * A2, A2, B2 * B2);
  const float b3 = fmaf(k133 * A3, A3, B3 * B3);
  const float t40 = fabsf(b1 - b2), t41 = fabsf(b2 - b3), t5 = fabsf(b3 - b1);
  const float mn = min3(b1, b2, b3);
  const float r1 = qdiv(t5, eps + b1);
  const float r2 = qdiv(t5, eps + b2);
  const float r3 = qdiv(t5, eps + b3);
  // candidate corrections S_k - Q(c)
  const float p1 = fmaf(5.f / 6.f, d1, -(1.f / 3.f) * d0);
  const float p2 = fmaf(1.f / 6.f, d1, (1.f / 3.f) * d2);
  const float p3 = fmaf(2.f / 3.f, d2, -(1.f / 6.f) * d3);
  const float m1 = fmaf(-5.f / 6.f, d2, (1.f / 3.f) * d3);
  const float m2 = fmaf(-1.f / 6.f, d2, -(1.f / 3.f) * d1);
  const float m3 = fmaf(-2.f / 3.f, d1, (1.f / 6.f) * d0);
  // the two hard switches of the reference select fixed weights; computed
  // unconditionally and selected, so no branch diverges
  const float sa = fmaf(1.f / 3.f, p1, (2.f / 3.f) * p2), sb = fmaf(2.f / 3.f, p2, (1.f / 3.f) * p3);
  const float ta = fmaf(1.f / 3.f, m1, (2.f / 3.f) * m2), tb = fmaf(2.f / 3.f, m2, (1.f / 3.f) * m3);
  // (the reference's t > mn tests are the complements of t <= mn for finite data)
  const bool lo40 = t40 <= mn, lo41 = t41 <= mn, hi40 = !lo40, hi41 = !lo41;
  const bool lt40 = t40 < mn, lt41 = t41 < mn;
  {  // "+" weights
    const float a1 = fmaf(0.1f, r1, 0.1f), a2 = fmaf(0.6f, r2, 0.6f), a3 = fmaf(0.3f, r3, 0.3f);
    const float num = fmaf(a1, p1, fmaf(a2, p2, a3 * p3));
    float val = qdiv(num, a1 + a2 + a3);
    val = (hi40 && lt41) ? sb : val;
    Dp = (lo40 && hi41) ? sa : val;
  }
  {  // "-" weights: beta' = (b3, b2, b1), tau40' = t41, tau41' = t40
    const float a1 = fmaf(0.1f, r3, 0.1f), a2 = fmaf(0.6f, r2, 0.6f), a3 = fmaf(0.3f, r1, 0.3f);
    const float num = fmaf(a1, m1, fmaf(a2, m2, a3 * m3));
    float val = qdiv(num, a1 + a2 + a3);
    val = (hi41 && lt40) ? tb : val;
    Dm = (lo41 && hi40) ? ta : val;
  }
}

// weno_d for two fields at once (the mass flux and phitG of one line): the same
// operations, lane for lane, on float2 pairs, so that the FP32 adds, multiplies and
// FMAs issue as paired f32x2 instructions; divisions, comparisons and selections
// stay per lane.  Bit for bit the two scalar calls.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {  // RN(a - b): b (-1) is exact
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ float2 k2(float c) { return make_float2(c, c); }

__device__ __forceinline__ void weno_d2(float2 d0, float2 d1, float2 d2, float2 d3, float2 eps, float2 &Dp,
                                        float2 &Dm) {
  const float2 A1 = sub2(d1, d0), A2 = sub2(d2, d1), A3 = sub2(d3, d2);
  const float2 B1 = __ffma2_rn(k2(3.f), d1, sub2(k2(0.f), d0));
  const float2 B2 = __fadd2_rn(d1, d2), B3 = __ffma2_rn(k2(-3.f), d2, d3);
  const float k133 = 13.f / 3.f;
  const float2 b1 = __ffma2_rn(__fmul2_rn(k2(k133), A1), A1, __fmul2_rn(B1, B1));
  const float2 b2 = __ffma2_rn(__fmul2_rn(k2(k133), A2), A2, __fmul2_rn(B2, B2));
  const float2 b3 = __ffma2_rn(__fmul2_rn(k2(k133), A3), A3, __fmul2_rn(B3, B3));
  const float2 D12 = sub2(b1, b2), D23 = sub2(b2, b3), D31 = sub2(b3, b1);
  const float2 e1 = __fadd2_rn(eps, b1), e2 = __fadd2_rn(eps, b2), e3 = __fadd2_rn(eps, b3);
  const float2 p1 = __ffma2_rn(k2(5.f / 6.f), d1, __fmul2_rn(k2(-(1.f / 3.f)), d0));
  const float2 p2 = __ffma2_rn(k2(1.f / 6.f), d1, __fmul2_rn(k2(1.f / 3.f), d2));
  const float2 p3 = __ffma2_rn(k2(2.f / 3.f), d2, __fmul2_rn(k2(-(1.f / 6.f)), d3));
  const float2 m1 = __ffma2_rn(k2(-5.f / 6.f), d2, __fmul2_rn(k2(1.f / 3.f), d3));
  const float2 m2 = __ffma2_rn(k2(-1.f / 6.f), d2, __fmul2_rn(k2(-(1.f / 3.f)), d1));
  const float2 m3 = __ffma2_rn(k2(-2.f / 3.f), d1, __fmul2_rn(k2(1.f / 6.f), d0));
  const float2 sa = __ffma2_rn(k2(1.f / 3.f), p1, __fmul2_rn(k2(2.f / 3.f), p2));
  const float2 sb = __ffma2_rn(k2(2.f / 3.f), p2, __fmul2_rn(k2(1.f / 3.f), p3));
  const float2 ta = __ffma2_rn(k2(1.f / 3.f), m1, __fmul2_rn(k2(2.f / 3.f), m2));
  const float2 tb = __ffma2_rn(k2(2.f / 3.f), m2, __fmul2_rn(k2(1.f / 3.f), m3));
  float2 r1, r2, r3;
  bool lo40[2], lo41[2], hi40[2], hi41[2], lt40[2], lt41[2];
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const float t40 = fabsf(q ? D12.y : D12.x), t41 = fabsf(q ? D23.y : D23.x), t5 = fabsf(q ? D31.y : D31.x);
    const float mn = min3(q ? b1.y : b1.x, q ? b2.y : b2.x, q ? b3.y : b3.x);
    const float x1 = qdiv(t5, q ? e1.y : e1.x), x2 = qdiv(t5, q ? e2.y : e2.x),
                x3 = qdiv(t5, q ? e3.y : e3.x);
    if (q) { r1.y = x1; r2.y = x2; r3.y = x3; } else { r1.x = x1; r2.x = x2; r3.x = x3; }
    lo40[q] = t40 <= mn; lo41[q] = t41 <= mn; hi40[q] = !lo40[q]; hi41[q] = !lo41[q];
    lt40[q] = t40 < mn; lt41[q] = t41 < mn;
  }
  {  // "+" weights
    const float2 a1 = __ffma2_rn(k2(0.1f), r1, k2(0.1f)), a2 = __ffma2_rn(k2(0.6f), r2, k2(0.6f)),
                 a3 = __ffma2_rn(k2(0.3f), r3, k2(0.3f));
    const float2 num = __ffma2_rn(a1, p1, __ffma2_rn(a2, p2, __fmul2_rn(a3, p3)));
    const float2 den = __fadd2_rn(__fadd2_rn(a1, a2), a3);
    float vx = qdiv(num.x, den.x), vy = qdiv(num.y, den.y);
    vx = (hi40[0] && lt41[0]) ? sb.x : vx;
    vy = (hi40[1] && lt41[1]) ? sb.y : vy;
    Dp.x = (lo40[0] && hi41[0]) ? sa.x : vx;
    Dp.y = (lo40[1] && hi41[1]) ? sa.y : vy;
  }
  {  // "-" weights
    const float2 a1 = __ffma2_rn(k2(0.1f), r3, k2(0.1f)), a2 = __ffma2_rn(k2(0.6f), r2, k2(0.6f)),
                 a3 = __ffma2_rn(k2(0.3f), r1, k2(0.3f));
    const float2 num = __ffma2_rn(a1, m1, __ffma2_rn(a2, m2, __fmul2_rn(a3, m3)));
    const float2 den = __fadd2_rn(__fadd2_rn(a1, a2), a3);
    float vx = qdiv(num.x, den.x), vy = qdiv(num.y, den.y);
    vx = (hi41[0] && lt40[0]) ? tb.x : vx;
    vy = (hi41[1] && lt40[1]) ? tb.y : vy;
    Dm.x = (lo41[0] && hi40[0]) ? ta.x : vx;
    Dm.y = (lo41[1] && hi40[1]) ? ta.y : vy;
  }
}

// Square root of the face wave speed (a dissipation coefficient): the PTX
// approximate square root (one instruction, a few ulp; +0 -> +0) instead of the
// correctly rounded sequence.
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// 4-byte asynchronous copy global -> shared (cp.async, through L1), and the wait
// for every copy this thread has issued
__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// 60 dx times the 6th-order centred derivative (spatial_operators_mod.F90:165,169)
// of the values f[-3s .. 3s], the FMAs written out so that every build rounds the
// same way
__device__ __forceinline__ float diff6(const float *f, int s) {
  float t = fmaf(9.f, f[-2 * s], -f[-3 * s]);
  t = fmaf(-45.f, f[-s], t);
  t = fmaf(45.f, f[s], t);
  t = fmaf(-9.f, f[2 * s], t);
  return t + f[3 * s];
}

// The numerator of the centred difference of order op (2, 4, 6) of f[-3s .. 3s]
// around f[0] (spatial_operators_mod_2nd.F90:54-59, _4th.F90:58-63, _6th.F90:62-67);
// the caller multiplies by 1 / (2 dx), 1 / (12 dx) or 1 / (60 dx).
__device__ __forceinline__ float central(int op, const float *f, int s) {
  if (op == 2) return f[s] - f[-s];
  if (op == 4) {
    const float t = fmaf(-8.f, f[-s], f[-2 * s]);
    return fmaf(8.f, f[s], t) - f[2 * s];
  }
  return diff6(f, s);
}

template <class T>
struct SmemMx {
  // stage descriptors and work items of this tile and the next (double-buffered:
  // the next tile's descriptor is copied while this one computes)
  MixedStage stb[2];
  WorkItem wib[2];
  // cell quantities on the halo'd tile, [row][col] with pitch SP
  float F[T::RN], G[T::RN], E[T::RN], hs[T::RN], s[T::RN], uC[T::RN], vC[T::RN], u[T::RN], v[T::RN];
  float gx[2][T::TY][T::NFL];     // x-face (flux, E) values minus the value of the cell left of the face
  float gy[2][T::TY + 1][T::TX];  // y-face values minus the value of the cell below the face
};

__device__ __forceinline__ bool corner(int i, int j, int N) { return (i < 1 || i > N) && (j < 1 || j > N); }

// One tile line (a row for x-faces, a column for y-faces) from face f0 to f1:
// the cells' difference windows slide along the line so that each cell costs one
// new shared-memory value per field; the face between two cells is formed from
// the left cell's "+" and the right cell's "-" corrections in registers.
// EDISS: the E flux gets the Rusanov dissipation of the covariant wind along the
// line (u at x-faces, v at y-faces: CCS_EDISS_RECONSTRUCT), reconstructed like the
// other fields and paired with E in f32x2; its eps scales like the flux's (1e-2 / a^4).
template <bool XDIR, bool EDISS, class T>
__device__ __forceinline__ void tile_line(SmemMx<T> &S, const MixedStage &st, const float *__restrict__ Qflux,
                                          const float *__restrict__ cvel, const float *__restrict__ lam,
                                          const Layout &L, int line, int f0,
                                          int NFACE, int startg, int lineg) {
  const float phibar = st.phibar, epsF = 4.f * st.eps_F, epsE = 4.f * st.eps_E, epsP = 4.f * st.eps_P;
  const float *__restrict__ Uw = XDIR ? S.u : S.v;  // the wind component along the line
  const int stp = XDIR ? 1 : SP;
  const int base = XDIR ? (line + 3) * SP + 2 : 2 * SP + line + 3;  // cell ci = 0 of the line
  int o = base + (f0 - 2) * stp;
  if (!ccs_inb(o, T::RN, 111) || !ccs_inb(o + 3 * stp, T::RN, 112)) return;
  // window values at cells c-2 .. c+1 for c = f0
  float Fv[4], Ev[4], hv[4], sv[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    Fv[k] = Qflux[o + k * stp];
    Ev[k] = S.E[o + k * stp];
    hv[k] = S.hs[o + k * stp];
    sv[k] = S.s[o + k * stp];
  }
  float dF0 = Fv[1] - Fv[0], dF1 = Fv[2] - Fv[1], dF2 = Fv[3] - Fv[2];
  float dE0 = Ev[1] - Ev[0], dE1 = Ev[2] - Ev[1], dE2 = Ev[3] - Ev[2];
  float q0 = hv[0] * sv[0], q1 = hv[1] * sv[1], q2 = hv[2] * sv[2], q3 = hv[3] * sv[3];
  float dP0 = fmaf(phibar, sv[1] - sv[0], q1 - q0);
  float dP1 = fmaf(phibar, sv[2] - sv[1], q2 - q1);
  float dP2 = fmaf(phibar, sv[3] - sv[2], q3 - q2);
  float Flast = Fv[3], Elast = Ev[3], slast = sv[3], qlast = q3;
  float hc = hv[2], hc1 = hv[3];  // hs at c and c+1
  float pDFp = 0.f, pDEp = 0.f, pDPp = 0.f, pU = 0.f, pH = 0.f;
  float dU0 = 0.f, dU1 = 0.f, dU2 = 0.f, Ulast = 0.f, pDUp = 0.f;
  if constexpr (EDISS) {
    const float u0 = Uw[o], u1 = Uw[o + stp], u2 = Uw[o + 2 * stp], u3 = Uw[o + 3 * stp];
    dU0 = u1 - u0; dU1 = u2 - u1; dU2 = u3 - u2; Ulast = u3;
  }
  // face wave-speed metric, fetched one face ahead of its use by walking a pointer
  // along the line; faces of a partial tile beyond N are read (and not used) from
  // the 32 padding rows the metric arrays carry after each panel block
  // (both face metrics are stored with the face index in the row position, so the
  // threads of a warp, one line each, read consecutive addresses at every step)
  const float *lp = lam + L.idx(lineg, startg + f0, 0);
  const int lstride = L.pitch;
  const long long lam_n = L.panel + (long long)kLamPadRows * L.pitch;  // face-metric block + padding
  float lam_next = ccs_inb(lp - lam, lam_n, 115) ? __ldg(lp) : 0.f;
  for (int k = 0; k <= NFACE; k++) {
    const int ci = f0 + k;
    const float lam_cur = lam_next;
    if (k > 0 && k < NFACE) {
      lp += lstride;
      lam_next = ccs_inb(lp - lam, lam_n, 115) ? __ldg(lp) : 0.f;
    }
    const int on = base + (ci + 2) * stp;  // cell c+2
    if (!ccs_inb(on, T::RN, 113) || !ccs_inb(base + ci * stp, T::RN, 114)) break;
    const float Fn = Qflux[on], En = S.E[on], hn = S.hs[on], sn = S.s[on];
    const float qn = hn * sn;
    const float dF3 = Fn - Flast, dE3 = En - Elast, dP3 = fmaf(phibar, sn - slast, qn - qlast);
    float DFp, DFm, DEp, DEm, DPp, DPm;
    {
      float2 Dp2, Dm2;
      weno_d2(make_float2(dF0, dP0), make_float2(dF1, dP1), make_float2(dF2, dP2), make_float2(dF3, dP3),
              make_float2(epsF, epsP), Dp2, Dm2);
      DFp = Dp2.x; DPp = Dp2.y; DFm = Dm2.x; DPm = Dm2.y;
    }
    float DUp = 0.f, DUm = 0.f, Un = 0.f, dU3 = 0.f;
    if constexpr (EDISS) {
      Un = Uw[on];
      dU3 = Un - Ulast;
      float2 Dp2, Dm2;
      weno_d2(make_float2(dE0, dU0), make_float2(dE1, dU1), make_float2(dE2, dU2), make_float2(dE3, dU3),
              make_float2(epsE, epsF), Dp2, Dm2);
      DEp = Dp2.x; DUp = Dp2.y; DEm = Dm2.x; DUm = Dm2.y;
    } else {
      weno_d(dE0, dE1, dE2, dE3, epsE, DEp, DEm);
    }
    const float uc = cvel[base + ci * stp];
    if (k > 0) {
      const int fi = ci - 1;         // face between line cells ci-1 and ci
      const int fg = startg + fi;    // global index of the cell left of / below the face
      if (fg <= L.N) {
        const float uB = 0.5f * (pU + uc);
        const float pB = fmaf(0.5f, pH + hc, phibar);
        const float lm = fabsf(uB) + sqrt_approx(fmaxf(lam_cur * pB, 0.f));
        const float gF = 0.5f * fmaf(-lm, dP1 + DPm - pDPp, dF1 + pDFp + DFm);
        // (the wind is carried as u / a^2 and E unscaled: the dissipation takes a^2 back)
        const float gE = EDISS ? 0.5f * fmaf(-lm * st.a2, dU1 + DUm - pDUp, dE1 + pDEp + DEm)
                               : 0.5f * (dE1 + pDEp + DEm);
        if (XDIR) {
          if (ccs_inb((long long)line * T::NFL + fi, (long long)T::TY * T::NFL, 116)) {
            S.gx[0][line][fi] = gF;
            S.gx[1][line][fi] = gE;
          }
        } else if (ccs_inb((long long)fi * T::TX + line, (long long)(T::TY + 1) * T::TX, 117)) {
          S.gy[0][fi][line] = gF;
          S.gy[1][fi][line] = gE;
        }
      }
    }
    pDFp = DFp; pDEp = DEp; pDPp = DPp; pU = uc; pH = hc;
    dF0 = dF1; dF1 = dF2; dF2 = dF3;
    dE0 = dE1; dE1 = dE2; dE2 = dE3;
    dP0 = dP1; dP1 = dP2; dP2 = dP3;
    Flast = Fn; Elast = En; slast = sn; qlast = qn;
    hc = hc1; hc1 = hn;
    if constexpr (EDISS) {
      pDUp = DUp;
      dU0 = dU1; dU1 = dU2; dU2 = dU3;
      Ulast = Un;
    }
  }
}

// Phase 3 of a tile for stage kind KIND: the early global loads, the barrier after
// the line phase, the tendencies and the stage update.
template <int KIND, class T, bool CENTRAL>
__device__ __forceinline__ void tile_update(SmemMx<T> &S, const MixedStage &st, const Layout &L, int p, int i0,
                                            int j0, int lane, int warp) {
  constexpr int NT = T::NT;
  const int N = L.N;
  // Global operands of phase 3 for this thread's four cells, loaded before the
  // barrier so their latency overlaps the wait for the slowest line segment:
  // f s, 1/s, Y0, the accumulator (or the stage input's hp for RK3) and the
  // compensation terms, as the stage kind needs them.
  constexpr int kind = KIND;
  constexpr bool need_acc = kind == K_RK4_2 || kind == K_RK4_4;
  constexpr bool need_in = kind == K_RK3_2 || kind == K_RK3_3;
  constexpr bool need_lo = kind == K_RK4_4 || kind == K_RK3_3;
  float q_fs[4], q_is[4], q_y0[4][3], q_a[4][3], q_lo[4][3];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int i = i0 + lane, j = j0 + warp + (NT / 32) * k;
    q_fs[k] = q_is[k] = 0.f;
#pragma unroll
    for (int q = 0; q < 3; q++) q_y0[k][q] = q_a[k][q] = q_lo[k][q] = 0.f;
    if (i > N || j > N) continue;
    const int64_t c = L.idx(i, j, p);
    if (!ccs_inb(c, L.field, 121) || !ccs_inb(L.idx(i, j, 0), L.panel, 122)) continue;
    q_fs[k] = __ldg(st.m.fs + c);
    q_is[k] = __ldg(st.m.inv_s + L.idx(i, j, 0));
    if constexpr (kind == K_TEND) continue;
    q_y0[k][0] = st.y0hp[c]; q_y0[k][1] = st.y0u[c]; q_y0[k][2] = st.y0v[c];
    if (need_acc) { q_a[k][0] = st.acchp[c]; q_a[k][1] = st.accu[c]; q_a[k][2] = st.accv[c]; }
    if (need_in) q_a[k][0] = st.in.hp[c];
    if (need_lo) { q_lo[k][0] = st.lohp[c]; q_lo[k][1] = st.lou[c]; q_lo[k][2] = st.lov[c]; }
  }
  __syncthreads();

  // ---- phase 3: tendencies, stage update ---------------------------------------
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int li = lane, lj = warp + (NT / 32) * k;
    const int i = i0 + li, j = j0 + lj;
    if (i > N || j > N) continue;
    const int r = (lj + 3) * SP + li + 3;
    if (!ccs_inb(r - 3 * SP, T::RN, 131) || !ccs_inb(r + 3 * SP, T::RN, 132) ||
        !ccs_inb((long long)lj * T::NFL + li + 1, (long long)T::TY * T::NFL, 133) ||
        !ccs_inb((long long)(lj + 1) * T::TX + li, (long long)(T::TY + 1) * T::TX, 134) ||
        !ccs_inb(L.idx(i, j, p), L.field, 135))
      continue;
    float divx, dEdx, divy, dEdy, dvdx, dudy;
    if (!CENTRAL) {
      divx = (S.gx[0][lj][li + 1] - S.gx[0][lj][li] + (S.F[r] - S.F[r - 1])) * st.rdx;
      dEdx = (S.gx[1][lj][li + 1] - S.gx[1][lj][li] + (S.E[r] - S.E[r - 1])) * st.rdx;
      divy = (S.gy[0][lj + 1][li] - S.gy[0][lj][li] + (S.G[r] - S.G[r - SP])) * st.rdy;
      dEdy = (S.gy[1][lj + 1][li] - S.gy[1][lj][li] + (S.E[r] - S.E[r - SP])) * st.rdy;
      dvdx = diff6(S.v + r, 1) * st.rdx60;
      dudy = diff6(S.u + r, SP) * st.rdy60;
    } else {  // spatial_operators_mod_{2nd,4th,6th}.F90: centred differences of the cell values
      const int op = st.op;
      divx = central(op, S.F + r, 1) * st.rdxc;
      dEdx = central(op, S.E + r, 1) * st.rdxc;
      dvdx = central(op, S.v + r, 1) * st.rdxc;
      divy = central(op, S.G + r, SP) * st.rdyc;
      dEdy = central(op, S.E + r, SP) * st.rdyc;
      dudy = central(op, S.u + r, SP) * st.rdyc;
    }
    const int64_t c = L.idx(i, j, p);
    const float vort = dvdx - dudy + q_fs[k];
    const float tp = -(divx + divy) * q_is[k];
    const float tu = fmaf(vort, S.vC[r], -dEdx * st.inv_a2);
    const float tv = fmaf(-vort, S.uC[r], -dEdy * st.inv_a2);
    if (kind == K_TEND) {
      st.thp[c] = tp;
      st.tu[c] = tu;
      st.tv[c] = tv;
      continue;
    }
    const float y0p = q_y0[k][0], y0u = q_y0[k][1], y0v = q_y0[k][2];
    float ip, iu, iv;  // increments to Y0 (Y = Y0 + c1 k fused where the stage is linear)
    bool fin = false, lin = false;
    switch (kind) {
      case K_RK4_1:
        st.acchp[c] = tp; st.accu[c] = tu; st.accv[c] = tv;
        ip = tp; iu = tu; iv = tv;
        lin = true;
        break;
      case K_RK4_2:
        st.acchp[c] = fmaf(2.f, tp, q_a[k][0]);
        st.accu[c] = fmaf(2.f, tu, q_a[k][1]);
        st.accv[c] = fmaf(2.f, tv, q_a[k][2]);
        ip = tp; iu = tu; iv = tv;
        lin = true;
        break;
      case K_RK4_4: {
        const float k6 = st.c1 * (1.f / 6.f);
        ip = k6 * (q_a[k][0] + tp); iu = k6 * (q_a[k][1] + tu); iv = k6 * (q_a[k][2] + tv);
        fin = true;
        break;
      }
      case K_RK3_1:
        ip = tp; iu = tu; iv = tv;
        lin = true;
        break;
      case K_RK3_2:
        ip = fmaf(0.25f, q_a[k][0] - y0p, st.c1 * tp);
        iu = fmaf(0.25f, S.u[r] - y0u, st.c1 * tu);
        iv = fmaf(0.25f, S.v[r] - y0v, st.c1 * tv);
        break;
      default:  // K_RK3_3
        ip = fmaf(2.f / 3.f, q_a[k][0] - y0p, st.c1 * tp);
        iu = fmaf(2.f / 3.f, S.u[r] - y0u, st.c1 * tu);
        iv = fmaf(2.f / 3.f, S.v[r] - y0v, st.c1 * tv);
        fin = true;
        break;
    }
    float np, nu, nv;
    if (fin) {
      // compensated update of the step-to-step state (TwoSum)
      float lo[3] = {q_lo[k][0], q_lo[k][1], q_lo[k][2]};
      const float hi[3] = {y0p, y0u, y0v};
      const float inc[3] = {ip, iu, iv};
      float out[3];
#pragma unroll
      for (int q = 0; q < 3; q++) {
        const float y = inc[q] + lo[q];
        const float tt = hi[q] + y;
        const float bp = tt - hi[q];
        lo[q] = (hi[q] - (tt - bp)) + (y - bp);
        out[q] = tt;
      }
      np = out[0]; nu = out[1]; nv = out[2];
      st.lohp[c] = lo[0]; st.lou[c] = lo[1]; st.lov[c] = lo[2];
    } else if (lin) {
      np = fmaf(st.c1, ip, y0p); nu = fmaf(st.c1, iu, y0u); nv = fmaf(st.c1, iv, y0v);
    } else {
      np = y0p + ip; nu = y0u + iu; nv = y0v + iv;
    }
    st.out.hp[c] = np;
    st.out.u[c] = nu;
    st.out.v[c] = nv;
  }
  __syncthreads();

}

// resident CTAs per SM the register allocation targets (3: 80 registers)
#ifndef CCS_MIXED_MIN_CTAS
#define CCS_MIXED_MIN_CTAS 3
#endif
// halo'd-tile cells each thread loads per round in phase 1 (loads in flight); one
// cell per round measured fastest with three CTAs per SM
#ifndef CCS_MIXED_P1_UNROLL
#define CCS_MIXED_P1_UNROLL 1
#endif
constexpr int kP1Unroll = CCS_MIXED_P1_UNROLL;

// CENTRAL: the central-difference operators (no face phases); else WENO-Z.
// STG: the halo-staging schedule of phase 1 (kStageLoads or kStageAsync).
template <class T, bool CENTRAL, bool EDISS, int STG>
__global__ void __launch_bounds__(T::NT, CCS_MIXED_MIN_CTAS * 32 / T::TY)
mixed_stage_kernel(const MixedStage *__restrict__ stages, const WorkItem *__restrict__ work, int nwork) {
  constexpr int TX = T::TX, TY = T::TY, NT = T::NT, RX = T::RX, RY = T::RY;
  static_assert(T::SP == SP, "smem pitch");
  extern __shared__ __align__(16) float smem_f[];
  SmemMx<T> &S = *reinterpret_cast<SmemMx<T> *>(smem_f);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  constexpr int nwd = (int)(sizeof(MixedStage) / 4);  // descriptor words
  // the first work item's descriptor; each tile then copies the next one into the
  // other buffer asynchronously while it computes
  int buf = 0;
  if (blockIdx.x < nwork) {
    const WorkItem wi = work[blockIdx.x];
    const int *src = reinterpret_cast<const int *>(stages + wi.inst);
    int *dst = reinterpret_cast<int *>(&S.stb[0]);
    for (int k = tid; k < nwd; k += NT) dst[k] = src[k];
    if (tid == 0) S.wib[0] = wi;
  }
  __syncthreads();
  for (int w = blockIdx.x; w < nwork; w += gridDim.x, buf ^= 1) {
    const MixedStage &st = S.stb[buf];
    const WorkItem wi = S.wib[buf];
    const int wn = w + gridDim.x;
    if (tid == 0 && wn < nwork) S.wib[buf ^ 1] = work[wn];  // read by all after the phase-1 barrier
#ifdef CCS_BOUNDS
    {  // poison the tile arrays (checked build only)
      float *a = S.F;
      const int na = (int)((reinterpret_cast<const char *>(&S.gy[1][T::TY][T::TX - 1]) + sizeof(float) -
                            reinterpret_cast<const char *>(S.F)) / sizeof(float));
      for (int k = tid; k < na; k += NT) a[k] = __int_as_float(0x7fc00000);
      __syncthreads();
    }
#endif
    const Layout L = st.L;
    const int N = L.N, p = wi.panel;
    const int i0 = 1 + wi.tx * TX, j0 = 1 + wi.ty * TY;

    // ---- phase 1: cell quantities on the halo'd tile ------------------------
    if constexpr (STG == kStageAsync) {
      // the raw inputs of every cell this thread stages go straight into the tile
      // arrays by asynchronous copies, all in flight at once and none through
      // registers; after its own copies land, the thread turns each of its cells
      // into the cell quantities in place
      const float phibar = st.phibar, ha2 = 0.5f * st.a2;
      const float *__restrict__ ihp = st.in.hp, *__restrict__ iu = st.in.u, *__restrict__ iv = st.in.v;
      const MeshMixed m = st.m;
      for (int r = tid; r < RX * RY; r += NT) {
        const int li = r % RX, lj = r / RX;
        const int i = i0 - 3 + li, j = j0 - 3 + lj;
        const int64_t c = L.idx(i, j, p), cs = L.idx(i, j, 0);
        const int a = lj * SP + li;
        if (i <= N + 3 && j <= N + 3 && !corner(i, j, N) && ccs_inb(c, L.field, 101) &&
            ccs_inb(cs, L.panel, 102) && ccs_inb(a, T::RN, 103)) {
          const float *g = reinterpret_cast<const float *>(m.ig + cs);
          cp_async4(&S.F[a], ihp + c);
          cp_async4(&S.u[a], iu + c);
          cp_async4(&S.v[a], iv + c);
          cp_async4(&S.s[a], m.s + cs);
          cp_async4(&S.G[a], g);
          cp_async4(&S.E[a], g + 1);
          cp_async4(&S.uC[a], g + 2);
          cp_async4(&S.vC[a], g + 3);
          cp_async4(&S.hs[a], m.phis + c);
        }
      }
      cp_async_wait_all();
      for (int r = tid; r < RX * RY; r += NT) {
        const int li = r % RX, lj = r / RX;
        const int i = i0 - 3 + li, j = j0 - 3 + lj;
        const int a = lj * SP + li;
        if (!ccs_inb(a, T::RN, 103)) continue;
        float F = 0.f, G = 0.f, E = 0.f, hs = 0.f, sc = 1.f, uC = 0.f, vC = 0.f, u = 0.f, v = 0.f;
        if (i <= N + 3 && j <= N + 3 && !corner(i, j, N)) {
          const float hp = S.F[a];
          u = S.u[a];
          v = S.v[a];
          sc = S.s[a];
          const float4 g = make_float4(S.G[a], S.E[a], S.uC[a], S.vC[a]);
          uC = fmaf(g.x, u, g.y * v);
          vC = fmaf(g.z, u, g.w * v);
          const float mass = (phibar + hp) * sc;  // phiG / a^2
          F = mass * uC;
          G = mass * vC;
          hs = S.hs[a] + hp;
          E = fmaf(ha2, fmaf(u, uC, v * vC), hs);  // E - phibar
        }
        S.F[a] = F; S.G[a] = G; S.E[a] = E; S.hs[a] = hs; S.s[a] = sc;
        S.uC[a] = uC; S.vC[a] = vC; S.u[a] = u; S.v[a] = v;
      }
    } else {
      // each thread loads its cells' raw inputs into registers (coalesced rows of the
      // halo'd tile) and stores the derived cell quantities
      const float phibar = st.phibar, ha2 = 0.5f * st.a2;
      const float *__restrict__ ihp = st.in.hp, *__restrict__ iu = st.in.u, *__restrict__ iv = st.in.v;
      const MeshMixed m = st.m;
#pragma unroll kP1Unroll
      for (int r = tid; r < RX * RY; r += NT) {
        const int li = r % RX, lj = r / RX;
        const int i = i0 - 3 + li, j = j0 - 3 + lj;
        float F = 0.f, G = 0.f, E = 0.f, hs = 0.f, sc = 1.f, uC = 0.f, vC = 0.f, u = 0.f, v = 0.f;
        const int64_t c = L.idx(i, j, p), cs = L.idx(i, j, 0);
        if (i <= N + 3 && j <= N + 3 && !corner(i, j, N) && ccs_inb(c, L.field, 101) &&
            ccs_inb(cs, L.panel, 102)) {
          const float hp = __ldg(ihp + c);
          u = __ldg(iu + c);
          v = __ldg(iv + c);
          sc = __ldg(m.s + cs);
          const float4 g = __ldg(m.ig + cs);
          uC = fmaf(g.x, u, g.y * v);
          vC = fmaf(g.z, u, g.w * v);
          const float mass = (phibar + hp) * sc;  // phiG / a^2
          F = mass * uC;
          G = mass * vC;
          hs = __ldg(m.phis + c) + hp;
          E = fmaf(ha2, fmaf(u, uC, v * vC), hs);  // E - phibar
        }
        const int a = lj * SP + li;
        if (!ccs_inb(a, T::RN, 103)) continue;
        S.F[a] = F; S.G[a] = G; S.E[a] = E; S.hs[a] = hs; S.s[a] = sc;
        S.uC[a] = uC; S.vC[a] = vC; S.u[a] = u; S.v[a] = v;
      }
    }
    __syncthreads();

    if (wn < nwork) {  // the next tile's descriptor, landing during phases 2-4
      const int *src = reinterpret_cast<const int *>(stages + S.wib[buf ^ 1].inst);
      int *dst = reinterpret_cast<int *>(&S.stb[buf ^ 1]);
      for (int k = tid; k < nwd; k += NT) cp_async4(reinterpret_cast<float *>(dst + k),
                                                      reinterpret_cast<const float *>(src + k));
    }
    // ---- phase 2: lines -> face values (warps 0-3 rows, 4-7 columns) ---------
    if (!CENTRAL) {  // (the central-difference operators have no faces)
      // segment seg of a line covers faces 0-8 (seg 0) or 8 seg + 1 .. 8 seg + 8
      if (tid < 4 * TY) {
        const int line = tid % TY, seg = tid / TY;
        const int f0 = seg == 0 ? 0 : 1 + 8 * seg, nface = seg == 0 ? 9 : 8;
        if (j0 + line <= N) tile_line<true, EDISS>(S, st, S.F, S.uC, st.m.lamx, L, line, f0, nface, i0 - 1, j0 + line);
      } else {
        const int t = tid - 4 * TY, line = t % TX, seg = t / TX;
        const int f0 = seg == 0 ? 0 : 1 + 8 * seg, nface = seg == 0 ? 9 : 8;
        if (i0 + line <= N) tile_line<false, EDISS>(S, st, S.G, S.vC, st.m.lamy, L, line, f0, nface, j0 - 1, i0 + line);
      }
    }
    // phase 3 as an instance per stage kind: the stage kind is the same for every
    // work item of a launch (a batch groups its members by RK scheme and launches
    // one stage at a time), so the stage update carries no runtime branches and
    // loads only the operands its kind uses
    switch (st.kind) {
      case K_RK4_1: tile_update<K_RK4_1, T, CENTRAL>(S, st, L, p, i0, j0, lane, warp); break;
      case K_RK4_2: tile_update<K_RK4_2, T, CENTRAL>(S, st, L, p, i0, j0, lane, warp); break;
      case K_RK4_4: tile_update<K_RK4_4, T, CENTRAL>(S, st, L, p, i0, j0, lane, warp); break;
      case K_RK3_1: tile_update<K_RK3_1, T, CENTRAL>(S, st, L, p, i0, j0, lane, warp); break;
      case K_RK3_2: tile_update<K_RK3_2, T, CENTRAL>(S, st, L, p, i0, j0, lane, warp); break;
      case K_RK3_3: tile_update<K_RK3_3, T, CENTRAL>(S, st, L, p, i0, j0, lane, warp); break;
      default: tile_update<K_TEND, T, CENTRAL>(S, st, L, p, i0, j0, lane, warp); break;
    }

    // ---- phase 4: ghost push of the tile's edge strips ----------------------
    // hp copies; the covariant wind crosses the edge through the FP64 2x2
    // transform G_h IA_h A_s IG_s of the receiving halo cell.  Entries are dealt
    // out to threads in push-table order, so no lane idles behind an edge lane.
    if (st.kind != K_TEND) {
      const int h = L.h;
      // strips: 0 left (k = i), 1 right (k = N+1-i), 2 below (k = j), 3 above (k = N+1-j);
      // each tile pushes the strip cells it owns, strip by strip: entries [o_sd, o_sd+1)
      // cover the cross-edge cells x (i for left/right, j for below/above) times the
      // tile's cells m along the edge
      const int ie = min(i0 + TX - 1, N), je = min(j0 + TY - 1, N);
      const int xlo1 = max(i0, N - h + 1), xlo3 = max(j0, N - h + 1);
      const int na01 = je - j0 + 1, na23 = ie - i0 + 1;  // along-edge lengths
      const int o1 = max(min(ie, h) - i0 + 1, 0) * na01;
      const int o2 = o1 + max(ie - xlo1 + 1, 0) * na01;
      const int o3 = o2 + max(min(je, h) - j0 + 1, 0) * na23;
      const int o4 = o3 + max(je - xlo3 + 1, 0) * na23;
      for (int t = tid; t < o4; t += NT) {
        const int sd = (t >= o1) + (t >= o2) + (t >= o3);
        const int q = t - (sd == 0 ? 0 : sd == 1 ? o1 : sd == 2 ? o2 : o3);
        const int na = sd < 2 ? na01 : na23;
        const int xl = sd == 0 ? i0 : sd == 1 ? xlo1 : sd == 2 ? j0 : xlo3;
        const int x = xl + q / na, m = (sd < 2 ? j0 : i0) + q % na;
        const int k = (sd == 0 || sd == 2) ? x : N + 1 - x;
        const int i = sd < 2 ? x : m, j = sd < 2 ? m : x;
        const int64_t c = L.idx(i, j, p);
        const int64_t e = ((int64_t)p * 4 + sd) * h * N + (int64_t)(k - 1) * N + (m - 1);
        if (!ccs_inb(e, (long long)24 * h * N, 141) || !ccs_inb(c, L.field, 143)) continue;
        const int64_t d = st.m.push[e];
        if (!ccs_inb(d, L.field, 142)) continue;
        const double *X = st.m.xf + 4 * e;
        const float np = st.out.hp[c], nu = st.out.u[c], nv = st.out.v[c];
        const double ud = fma(X[0], (double)nu, X[1] * (double)nv);
        const double vd = fma(X[2], (double)nu, X[3] * (double)nv);
        st.out.hp[d] = np;
        st.out.u[d] = (float)ud;
        st.out.v[d] = (float)vd;
      }
    }
    cp_async_wait_all();  // this thread's copies of the next descriptor have landed
    __syncthreads();
  }
}

// ---- import / export between the reference FP64 layout and the lane state ----
__global__ void mixed_import_kernel(Layout L, const double *__restrict__ phi, const double *__restrict__ u,
                                    const double *__restrict__ v, double phibar, double inv_a2, StateMixed out,
                                    float *lohp, float *lou, float *lov) {
  const int nh = L.nh;
  const int64_t n = (int64_t)nh * nh * 6;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int ia = (int)(q % nh), ja = (int)((q / nh) % nh), p = (int)(q / ((int64_t)nh * nh));
    const int i = ia + 1 - L.h, j = ja + 1 - L.h;
    const int64_t c = L.idx(i, j, p);
    if ((i < 1 || i > L.N) && (j < 1 || j > L.N)) continue;
    const double hp = phi[q] - phibar, uu = u[q] * inv_a2, vv = v[q] * inv_a2;
    const float fh = (float)hp, fu = (float)uu, fv = (float)vv;
    out.hp[c] = fh;
    out.u[c] = fu;
    out.v[c] = fv;
    const bool interior = i >= 1 && i <= L.N && j >= 1 && j <= L.N;
    lohp[c] = interior ? (float)(hp - (double)fh) : 0.f;
    lou[c] = interior ? (float)(uu - (double)fu) : 0.f;
    lov[c] = interior ? (float)(vv - (double)fv) : 0.f;
  }
}

__global__ void mixed_export_kernel(Layout L, StateMixed st, const float *__restrict__ lohp,
                                    const float *__restrict__ lou, const float *__restrict__ lov, MeshF64 m,
                                    double phibar, double a2, double *phiG, double *u, double *v, double *phi,
                                    double *uC, double *vC, double *zonal, double *merid) {
  const int nh = L.nh;
  const int64_t n = (int64_t)nh * nh * 6;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int ia = (int)(q % nh), ja = (int)((q / nh) % nh), p = (int)(q / ((int64_t)nh * nh));
    const int i = ia + 1 - L.h, j = ja + 1 - L.h;
    const int64_t c = L.idx(i, j, p);
    if ((i < 1 || i > L.N) && (j < 1 || j > L.N)) continue;
    const bool interior = i >= 1 && i <= L.N && j >= 1 && j <= L.N;
    double hp = st.hp[c], uu = st.u[c], vv = st.v[c];
    if (interior) {
      hp += (double)lohp[c];
      uu += (double)lou[c];
      vv += (double)lov[c];
    }
    const double ph = phibar + hp, cu = uu * a2, cv = vv * a2;
    phi[q] = ph;
    phiG[q] = ph * m.sqrtG[c];
    u[q] = cu;
    v[q] = cv;
    uC[q] = m.ig11[c] * cu + m.ig12[c] * cv;
    vC[q] = m.ig21[c] * cu + m.ig22[c] * cv;
    zonal[q] = m.aig11[c] * cu + m.aig12[c] * cv;
    merid[q] = m.aig21[c] * cu + m.aig22[c] * cv;
  }
}

__global__ void mixed_tend_export_kernel(Layout L, const float *__restrict__ thp, const float *__restrict__ tu,
                                         const float *__restrict__ tv, MeshF64 m, double a2, double *op,
                                         double *ou, double *ov) {
  const int nh = L.nh;
  const int64_t n = (int64_t)nh * nh * 6;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int ia = (int)(q % nh), ja = (int)((q / nh) % nh), p = (int)(q / ((int64_t)nh * nh));
    const int i = ia + 1 - L.h, j = ja + 1 - L.h;
    const bool interior = i >= 1 && i <= L.N && j >= 1 && j <= L.N;
    if (!interior) {
      op[q] = 0.; ou[q] = 0.; ov[q] = 0.;
      continue;
    }
    const int64_t c = L.idx(i, j, p);
    op[q] = (double)thp[c] * m.sqrtG[c];
    ou[q] = (double)tu[c] * a2;
    ov[q] = (double)tv[c] * a2;
  }
}

// FP64 mass / energy of the mixed state (diag_mod.F90:10-53), block partials.
__global__ void mixed_diag_kernel(Layout L, StateMixed st, const float *__restrict__ lohp,
                                  const float *__restrict__ lou, const float *__restrict__ lov, MeshF64 m,
                                  double phibar, double a2, double *partials) {
  __shared__ double sm[2][256];
  const int64_t ncell = (int64_t)L.N * L.N * 6;
  const int64_t per = (ncell + gridDim.x - 1) / gridDim.x;
  const int64_t beg = blockIdx.x * per;
  int64_t end = beg + per;
  if (end > ncell) end = ncell;
  double ms = 0., en = 0.;
  for (int64_t q = beg + threadIdx.x; q < end; q += blockDim.x) {
    const int i = 1 + (int)(q % L.N), j = 1 + (int)((q / L.N) % L.N), p = (int)(q / ((int64_t)L.N * L.N));
    const int64_t c = L.idx(i, j, p);
    const double ph = phibar + ((double)st.hp[c] + (double)lohp[c]);
    const double cu = ((double)st.u[c] + (double)lou[c]) * a2, cv = ((double)st.v[c] + (double)lov[c]) * a2;
    const double uc = m.ig11[c] * cu + m.ig12[c] * cv, vc = m.ig21[c] * cu + m.ig22[c] * cv;
    const double sg = m.sqrtG[c];
    ms += ph * sg;
    const double t = ph + m.phis[c];
    en += sg * (0.5 * ph * (cu * uc + cv * vc) + 0.5 * (t * t));
  }
  sm[0][threadIdx.x] = ms;
  sm[1][threadIdx.x] = en;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sm[0][threadIdx.x] += sm[0][threadIdx.x + s];
      sm[1][threadIdx.x] += sm[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = sm[0][0];
    partials[2 * blockIdx.x + 1] = sm[1][0];
  }
}

}  // namespace

namespace {

using MxT0 = MxTile<32>;
using MxT1 = MxTile<16>;
static_assert(MxT0::TX == kMxTiles[0].tx && MxT0::TY == kMxTiles[0].ty, "tile table");
static_assert(MxT1::TX == kMxTiles[1].tx && MxT1::TY == kMxTiles[1].ty, "tile table");
static_assert(MxT0::TX == kMxTiles[2].tx && MxT0::TY == kMxTiles[2].ty, "tile table");
static_assert(MxT1::TX == kMxTiles[3].tx && MxT1::TY == kMxTiles[3].ty, "tile table");
static_assert(kMxStaging[0] == kStageLoads && kMxStaging[1] == kStageLoads && kMxStaging[2] == kStageAsync &&
                  kMxStaging[3] == kStageAsync,
              "staging table");

template <class T, int STG>
int mx_grid_for(int device) {  // the WENO instance bounds the occupancy of all
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  constexpr int smem = (int)sizeof(SmemMx<T>);
  cudaFuncSetAttribute(mixed_stage_kernel<T, false, false, STG>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, mixed_stage_kernel<T, false, false, STG>, T::NT, smem);
  if (per < 1) per = 1;
  return sms * per;
}

template <class T, bool CENTRAL, bool EDISS, int STG>
cudaError_t mx_launch(const MixedStage *d_stages, const WorkItem *d_work, int nwork, int grid, cudaStream_t s) {
  constexpr int smem = (int)sizeof(SmemMx<T>);
  static std::atomic<uint64_t> attr_done{0};
  const cudaError_t e = smem_attr_once((const void *)mixed_stage_kernel<T, CENTRAL, EDISS, STG>, smem, attr_done);
  if (e != cudaSuccess) return e;
  if (grid > nwork) grid = nwork;
  if (grid < 1) return cudaSuccess;
  mixed_stage_kernel<T, CENTRAL, EDISS, STG><<<grid, T::NT, smem, s>>>(d_stages, d_work, nwork);
  return cudaGetLastError();
}

template <class T, int STG>
cudaError_t mx_launch_any(bool central, bool ediss, const MixedStage *d_stages, const WorkItem *d_work, int nwork,
                          int grid, cudaStream_t s) {
  if (central) return mx_launch<T, true, false, STG>(d_stages, d_work, nwork, grid, s);  // no faces: no E term
  if (ediss) return mx_launch<T, false, true, STG>(d_stages, d_work, nwork, grid, s);
  return mx_launch<T, false, false, STG>(d_stages, d_work, nwork, grid, s);
}

}  // namespace

int mixed_max_grid(int var, int device) {
  switch (var) {
    case 1: return mx_grid_for<MxT1, kStageLoads>(device);
    case 2: return mx_grid_for<MxT0, kStageAsync>(device);
    case 3: return mx_grid_for<MxT1, kStageAsync>(device);
    default: return mx_grid_for<MxT0, kStageLoads>(device);
  }
}

cudaError_t launch_mixed_stage(int var, bool central, bool ediss, const MixedStage *d_stages,
                               const WorkItem *d_work, int nwork, int grid, cudaStream_t s) {
  switch (var) {
    case 1: return mx_launch_any<MxT1, kStageLoads>(central, ediss, d_stages, d_work, nwork, grid, s);
    case 2: return mx_launch_any<MxT0, kStageAsync>(central, ediss, d_stages, d_work, nwork, grid, s);
    case 3: return mx_launch_any<MxT1, kStageAsync>(central, ediss, d_stages, d_work, nwork, grid, s);
    default: return mx_launch_any<MxT0, kStageLoads>(central, ediss, d_stages, d_work, nwork, grid, s);
  }
}

static int ew_grid(const Layout &L) {
  const int64_t n = (int64_t)L.nh * L.nh * 6;
  int64_t g = (n + 255) / 256;
  if (g > 4096) g = 4096;
  return (int)g;
}

cudaError_t launch_mixed_import(const Layout &L, const double *phi, const double *u, const double *v,
                                double phibar, double inv_a2, StateMixed out, float *lohp, float *lou,
                                float *lov, cudaStream_t s) {
  mixed_import_kernel<<<ew_grid(L), 256, 0, s>>>(L, phi, u, v, phibar, inv_a2, out, lohp, lou, lov);
  return cudaGetLastError();
}

cudaError_t launch_mixed_export(const Layout &L, StateMixed st, const float *lohp, const float *lou,
                                const float *lov, const MeshF64 &m, double phibar, double a2, double *const out[8],
                                cudaStream_t s) {
  mixed_export_kernel<<<ew_grid(L), 256, 0, s>>>(L, st, lohp, lou, lov, m, phibar, a2, out[0], out[1], out[2],
                                                  out[3], out[4], out[5], out[6], out[7]);
  return cudaGetLastError();
}

cudaError_t launch_mixed_tend_export(const Layout &L, const float *thp, const float *tu, const float *tv,
                                     const MeshF64 &m, double a2, double *op, double *ou, double *ov,
                                     cudaStream_t s) {
  mixed_tend_export_kernel<<<ew_grid(L), 256, 0, s>>>(L, thp, tu, tv, m, a2, op, ou, ov);
  return cudaGetLastError();
}

cudaError_t launch_mixed_diag(const Layout &L, StateMixed st, const float *lohp, const float *lou,
                              const float *lov, const MeshF64 &m, double phibar, double a2, double *partials,
                              int nblocks, cudaStream_t s) {
  mixed_diag_kernel<<<nblocks, 256, 0, s>>>(L, st, lohp, lou, lov, m, phibar, a2, partials);
  return cudaGetLastError();
}

unsigned long long mixed_bounds_take() { return bounds_take_tu(); }

cudaError_t launch_bounds_selftest(long long i, long long n, int site, cudaStream_t s) {
#ifdef CCS_BOUNDS
  bounds_selftest_kernel<<<1, 32, 0, s>>>(i, n, site);
  return cudaGetLastError();
#else
  (void)i; (void)n; (void)site; (void)s;
  return cudaSuccess;
#endif
}

}  // namespace ccs
