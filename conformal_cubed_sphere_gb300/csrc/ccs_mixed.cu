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

namespace ccs {

namespace {

constexpr int TX = MX_TX, TY = MX_TY, NT = MX_THREADS;
constexpr int RX = TX + 6, RY = TY + 6;  // halo'd tile
constexpr int SP = RX + 1;               // odd pitch: a warp reading one column hits 32 banks
constexpr int RN = RY * SP;
constexpr int NFL = TX + 1;              // faces per tile line
static_assert(TX == 32 && TY == 32 && NT == 256, "lanes map to the 32 rows / columns of a tile");

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
  const float mn = fminf(b1, fminf(b2, b3));
  const float r1 = __fdividef(t5, eps + b1);
  const float r2 = __fdividef(t5, eps + b2);
  const float r3 = __fdividef(t5, eps + b3);
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
  const bool lo40 = t40 <= mn, lo41 = t41 <= mn, hi40 = t40 > mn, hi41 = t41 > mn;
  const bool lt40 = t40 < mn, lt41 = t41 < mn;
  {  // "+" weights
    const float a1 = fmaf(0.1f, r1, 0.1f), a2 = fmaf(0.6f, r2, 0.6f), a3 = fmaf(0.3f, r3, 0.3f);
    const float num = fmaf(a1, p1, fmaf(a2, p2, a3 * p3));
    float val = __fdividef(num, a1 + a2 + a3);
    val = (hi40 && lt41) ? sb : val;
    Dp = (lo40 && hi41) ? sa : val;
  }
  {  // "-" weights: beta' = (b3, b2, b1), tau40' = t41, tau41' = t40
    const float a1 = fmaf(0.1f, r3, 0.1f), a2 = fmaf(0.6f, r2, 0.6f), a3 = fmaf(0.3f, r1, 0.3f);
    const float num = fmaf(a1, m1, fmaf(a2, m2, a3 * m3));
    float val = __fdividef(num, a1 + a2 + a3);
    val = (hi41 && lt40) ? tb : val;
    Dm = (lo41 && hi40) ? ta : val;
  }
}

struct SmemMx {
  MixedStage st;  // this work item's stage descriptor
  // cell quantities on the halo'd tile, [row][col] with pitch SP
  float F[RN], G[RN], E[RN], hs[RN], s[RN], uC[RN], vC[RN], u[RN], v[RN];
  float gx[2][TY][NFL];  // x-face (flux, E) values minus the value of the cell left of the face
  float gy[2][NFL][TX];  // y-face values minus the value of the cell below the face
};

__device__ __forceinline__ bool corner(int i, int j, int N) { return (i < 1 || i > N) && (j < 1 || j > N); }

// One tile line (a row for x-faces, a column for y-faces) from face f0 to f1:
// the cells' difference windows slide along the line so that each cell costs one
// new shared-memory value per field; the face between two cells is formed from
// the left cell's "+" and the right cell's "-" corrections in registers.
template <bool XDIR>
__device__ __forceinline__ void tile_line(SmemMx &S, const float *__restrict__ Qflux, const float *__restrict__ cvel,
                                          const float *__restrict__ lam, const Layout &L, int lane, int f0,
                                          int NFACE, int startg, int lineg) {
  const MixedStage &st = S.st;
  const float phibar = st.phibar, epsF = 4.f * st.eps_F, epsE = 4.f * st.eps_E, epsP = 4.f * st.eps_P;
  const int stp = XDIR ? 1 : SP;
  const int base = XDIR ? (lane + 3) * SP + 2 : 2 * SP + lane + 3;  // cell ci = 0 of the line
  int o = base + (f0 - 2) * stp;
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
  // face wave-speed metric, fetched one face ahead of its use (the index is clamped
  // into the panel so the prefetch never leaves the array)
  auto lam_at = [&](int fi) -> float {
    int fg = startg + fi;
    fg = fg < 0 ? 0 : (fg > L.N ? L.N : fg);
    return __ldg(lam + (XDIR ? L.idx(fg, lineg, 0) : L.idx(lineg, fg, 0)));
  };
  float lam_next = lam_at(f0);
  for (int k = 0; k <= NFACE; k++) {
    const int ci = f0 + k;
    const float lam_cur = lam_next;
    if (k > 0 && k < NFACE) lam_next = lam_at(ci);
    const int on = base + (ci + 2) * stp;  // cell c+2
    const float Fn = Qflux[on], En = S.E[on], hn = S.hs[on], sn = S.s[on];
    const float qn = hn * sn;
    const float dF3 = Fn - Flast, dE3 = En - Elast, dP3 = fmaf(phibar, sn - slast, qn - qlast);
    float DFp, DFm, DEp, DEm, DPp, DPm;
    weno_d(dF0, dF1, dF2, dF3, epsF, DFp, DFm);
    weno_d(dE0, dE1, dE2, dE3, epsE, DEp, DEm);
    weno_d(dP0, dP1, dP2, dP3, epsP, DPp, DPm);
    const float uc = cvel[base + ci * stp];
    if (k > 0) {
      const int fi = ci - 1;         // face between line cells ci-1 and ci
      const int fg = startg + fi;    // global index of the cell left of / below the face
      if (fg <= L.N) {
        const float uB = 0.5f * (pU + uc);
        const float pB = phibar + 0.5f * (pH + hc);
        const float lm = fabsf(uB) + sqrtf(fmaxf(lam_cur * pB, 0.f));
        const float gF = 0.5f * (dF1 + pDFp + DFm - lm * (dP1 + DPm - pDPp));
        const float gE = 0.5f * (dE1 + pDEp + DEm);
        if (XDIR) {
          S.gx[0][lane][fi] = gF;
          S.gx[1][lane][fi] = gE;
        } else {
          S.gy[0][fi][lane] = gF;
          S.gy[1][fi][lane] = gE;
        }
      }
    }
    pDFp = DFp; pDEp = DEp; pDPp = DPp; pU = uc; pH = hc;
    dF0 = dF1; dF1 = dF2; dF2 = dF3;
    dE0 = dE1; dE1 = dE2; dE2 = dE3;
    dP0 = dP1; dP1 = dP2; dP2 = dP3;
    Flast = Fn; Elast = En; slast = sn; qlast = qn;
    hc = hc1; hc1 = hn;
  }
}

// resident CTAs per SM the register allocation targets (3: 80 registers)
#ifndef CCS_MIXED_MIN_CTAS
#define CCS_MIXED_MIN_CTAS 3
#endif

__global__ void __launch_bounds__(NT, CCS_MIXED_MIN_CTAS)
mixed_stage_kernel(const MixedStage *__restrict__ stages, const WorkItem *__restrict__ work, int nwork) {
  extern __shared__ __align__(16) float smem_f[];
  SmemMx &S = *reinterpret_cast<SmemMx *>(smem_f);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const WorkItem wi = work[w];
    {  // stage descriptor into shared memory
      const int nw = (int)(sizeof(MixedStage) / 4);
      const int *src = reinterpret_cast<const int *>(stages + wi.inst);
      int *dst = reinterpret_cast<int *>(&S.st);
      for (int k = tid; k < nw; k += NT) dst[k] = src[k];
    }
    __syncthreads();
    const MixedStage &st = S.st;
    const Layout L = st.L;
    const int N = L.N, p = wi.panel;
    const int i0 = 1 + wi.tx * TX, j0 = 1 + wi.ty * TY;

    // ---- phase 1: cell quantities on the halo'd tile ------------------------
    {
      const float phibar = st.phibar, ha2 = 0.5f * st.a2;
      const float *__restrict__ ihp = st.in.hp, *__restrict__ iu = st.in.u, *__restrict__ iv = st.in.v;
      const MeshMixed m = st.m;
#pragma unroll 2
      for (int r = tid; r < RX * RY; r += NT) {
        const int li = r % RX, lj = r / RX;
        const int i = i0 - 3 + li, j = j0 - 3 + lj;
        float F = 0.f, G = 0.f, E = 0.f, hs = 0.f, sc = 1.f, uC = 0.f, vC = 0.f, u = 0.f, v = 0.f;
        if (i <= N + 3 && j <= N + 3 && !corner(i, j, N)) {
          const int64_t c = L.idx(i, j, p), cs = L.idx(i, j, 0);
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
        S.F[a] = F; S.G[a] = G; S.E[a] = E; S.hs[a] = hs; S.s[a] = sc;
        S.uC[a] = uC; S.vC[a] = vC; S.u[a] = u; S.v[a] = v;
      }
    }
    __syncthreads();

    // ---- phase 2: lines -> face values (warps 0-3 rows, 4-7 columns) ---------
    {
      const int seg = warp & 3;
      const int f0 = seg == 0 ? 0 : 1 + 8 * seg;  // faces 0-8, 9-16, 17-24, 25-32
      const int nface = seg == 0 ? 9 : 8;
      if (warp < 4) {
        if (j0 + lane <= N) tile_line<true>(S, S.F, S.uC, st.m.lamx, L, lane, f0, nface, i0 - 1, j0 + lane);
      } else {
        if (i0 + lane <= N) tile_line<false>(S, S.G, S.vC, st.m.lamy, L, lane, f0, nface, j0 - 1, i0 + lane);
      }
    }
    __syncthreads();

    // ---- phase 3: tendencies, stage update, ghost push -------------------------
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int li = lane, lj = warp + 8 * k;
      const int i = i0 + li, j = j0 + lj;
      if (i > N || j > N) continue;
      const int r = (lj + 3) * SP + li + 3;
      const float divx = (S.gx[0][lj][li + 1] - S.gx[0][lj][li] + (S.F[r] - S.F[r - 1])) * st.rdx;
      const float dEdx = (S.gx[1][lj][li + 1] - S.gx[1][lj][li] + (S.E[r] - S.E[r - 1])) * st.rdx;
      const float divy = (S.gy[0][lj + 1][li] - S.gy[0][lj][li] + (S.G[r] - S.G[r - SP])) * st.rdy;
      const float dEdy = (S.gy[1][lj + 1][li] - S.gy[1][lj][li] + (S.E[r] - S.E[r - SP])) * st.rdy;
      const float *vv = S.v + r, *uu = S.u + r;
      const float dvdx = (-vv[-3] + 9.f * vv[-2] - 45.f * vv[-1] + 45.f * vv[1] - 9.f * vv[2] + vv[3]) * st.rdx60;
      const float dudy = (-uu[-3 * SP] + 9.f * uu[-2 * SP] - 45.f * uu[-SP] + 45.f * uu[SP] - 9.f * uu[2 * SP] +
                          uu[3 * SP]) *
                         st.rdy60;
      const int64_t c = L.idx(i, j, p), cs = L.idx(i, j, 0);
      const float vort = dvdx - dudy + __ldg(st.m.fs + c);
      const float tp = -(divx + divy) * __ldg(st.m.inv_s + cs);
      const float tu = fmaf(vort, S.vC[r], -dEdx * st.inv_a2);
      const float tv = fmaf(-vort, S.uC[r], -dEdy * st.inv_a2);
      if (st.kind == K_TEND) {
        st.thp[c] = tp;
        st.tu[c] = tu;
        st.tv[c] = tv;
        continue;
      }
      const float y0p = st.y0hp[c], y0u = st.y0u[c], y0v = st.y0v[c];
      float ip, iu, iv;  // increments to Y0
      bool fin = false;
      switch (st.kind) {
        case K_RK4_1:
          st.acchp[c] = tp; st.accu[c] = tu; st.accv[c] = tv;
          ip = st.c1 * tp; iu = st.c1 * tu; iv = st.c1 * tv;
          break;
        case K_RK4_2:
          st.acchp[c] = fmaf(2.f, tp, st.acchp[c]);
          st.accu[c] = fmaf(2.f, tu, st.accu[c]);
          st.accv[c] = fmaf(2.f, tv, st.accv[c]);
          ip = st.c1 * tp; iu = st.c1 * tu; iv = st.c1 * tv;
          break;
        case K_RK4_4: {
          const float k6 = st.c1 * (1.f / 6.f);
          ip = k6 * (st.acchp[c] + tp); iu = k6 * (st.accu[c] + tu); iv = k6 * (st.accv[c] + tv);
          fin = true;
          break;
        }
        case K_RK3_1:
          ip = st.c1 * tp; iu = st.c1 * tu; iv = st.c1 * tv;
          break;
        case K_RK3_2:
          ip = fmaf(0.25f, st.in.hp[c] - y0p, st.c1 * tp);
          iu = fmaf(0.25f, S.u[r] - y0u, st.c1 * tu);
          iv = fmaf(0.25f, S.v[r] - y0v, st.c1 * tv);
          break;
        default:  // K_RK3_3
          ip = fmaf(2.f / 3.f, st.in.hp[c] - y0p, st.c1 * tp);
          iu = fmaf(2.f / 3.f, S.u[r] - y0u, st.c1 * tu);
          iv = fmaf(2.f / 3.f, S.v[r] - y0v, st.c1 * tv);
          fin = true;
          break;
      }
      float np, nu, nv;
      if (fin) {
        // compensated update of the step-to-step state (TwoSum)
        float lo[3] = {st.lohp[c], st.lou[c], st.lov[c]};
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
      } else {
        np = y0p + ip; nu = y0u + iu; nv = y0v + iv;
      }
      st.out.hp[c] = np;
      st.out.u[c] = nu;
      st.out.v[c] = nv;
    }
    __syncthreads();

    // ---- phase 4: ghost push of the tile's edge strips ----------------------
    // hp copies; the covariant wind crosses the edge through the FP64 2x2
    // transform G_h IA_h A_s IG_s of the receiving halo cell.  Entries are dealt
    // out to threads in push-table order, so no lane idles behind an edge lane.
    if (st.kind != K_TEND) {
      const int h = L.h;
      // strips: 0 left (k = i), 1 right (k = N+1-i), 2 below (k = j), 3 above (k = N+1-j);
      // each tile pushes the strip cells it owns: cross-edge range [xlo, xhi]
      // (i for left/right, j for below/above) and along-edge range [alo, ahi]
      const int ie = min(i0 + TX - 1, N), je = min(j0 + TY - 1, N);
      int xlo[4], xhi[4], alo[4], ahi[4], off[5];
      xlo[0] = i0; xhi[0] = min(ie, h); alo[0] = j0; ahi[0] = je;
      xlo[1] = max(i0, N - h + 1); xhi[1] = ie; alo[1] = j0; ahi[1] = je;
      xlo[2] = j0; xhi[2] = min(je, h); alo[2] = i0; ahi[2] = ie;
      xlo[3] = max(j0, N - h + 1); xhi[3] = je; alo[3] = i0; ahi[3] = ie;
      off[0] = 0;
      for (int sd = 0; sd < 4; sd++) {
        const int nx = xhi[sd] - xlo[sd] + 1, na = ahi[sd] - alo[sd] + 1;
        off[sd + 1] = off[sd] + (nx > 0 && na > 0 ? nx * na : 0);
      }
      for (int t = tid; t < off[4]; t += NT) {
        int sd = 0;
        while (t >= off[sd + 1]) sd++;
        const int q = t - off[sd];
        const int na = ahi[sd] - alo[sd] + 1;
        const int x = xlo[sd] + q / na, m = alo[sd] + q % na;
        const int k = (sd == 0 || sd == 2) ? x : N + 1 - x;
        const int i = sd < 2 ? x : m, j = sd < 2 ? m : x;
        const int64_t c = L.idx(i, j, p);
        const int64_t e = ((int64_t)p * 4 + sd) * h * N + (int64_t)(k - 1) * N + (m - 1);
        const int64_t d = st.m.push[e];
        const double *T = st.m.xf + 4 * e;
        const float np = st.out.hp[c], nu = st.out.u[c], nv = st.out.v[c];
        const double ud = T[0] * (double)nu + T[1] * (double)nv;
        const double vd = T[2] * (double)nu + T[3] * (double)nv;
        st.out.hp[d] = np;
        st.out.u[d] = (float)ud;
        st.out.v[d] = (float)vd;
      }
    }
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

int mixed_smem_bytes() { return (int)sizeof(SmemMx); }

int mixed_max_grid(int device) {
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaFuncSetAttribute(mixed_stage_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mixed_smem_bytes());
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, mixed_stage_kernel, NT, mixed_smem_bytes());
  if (per < 1) per = 1;
  return sms * per;
}

cudaError_t launch_mixed_stage(const MixedStage *d_stages, const WorkItem *d_work, int nwork, int grid,
                               cudaStream_t s) {
  if (grid > nwork) grid = nwork;
  if (grid < 1) return cudaSuccess;
  mixed_stage_kernel<<<grid, NT, mixed_smem_bytes(), s>>>(d_stages, d_work, nwork);
  return cudaGetLastError();
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

}  // namespace ccs
