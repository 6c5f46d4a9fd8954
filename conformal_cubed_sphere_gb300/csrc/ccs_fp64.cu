// ccs_fp64.cu -- FP64 parity lane: one fused launch per RK stage.
//
// Built with -fmad=false: every operation below is a separately rounded IEEE
// double operation in the order of the Fortran source (left to right), so the
// result is bitwise the reference arithmetic (gfortran -fdefault-real-8 on x86-64
// emits no FMA).  `/` and sqrt are the IEEE-rounded CUDA double operations.
//
// A CTA owns a tile of F64_TX x F64_TY interior cells of one panel.  It stages the
// halo'd tile (3 cells each side) of the cell quantities of the spatial operator
// in shared memory, reconstructs every face value it needs (12 live WENO-Z calls
// per cell, spatial_operators_mod.F90:80-99), forms the Rusanov face fluxes
// (:101-149), the divergence / vorticity / tendencies (:151-179), applies the RK
// stage update (time_scheme_mod.F90:69-115) and the boundary correction
// (correct_bdy_ghost, :117-125): interior cells convert their new covariant wind
// to sphere components and back, and every cell within `halo` of a panel edge
// pushes its phiG and sphere wind into the halo cell that CubedSphereFillHalo
// (ghost_mod.f90:18-82) would fill from it, converting there with that cell's
// own metric.  The output slot never feeds the same launch, so one launch per
// stage is the whole grid-wide dependency.
#include "ccs_kernels.h"
#include "ccs_bounds.cuh"

namespace ccs {

namespace {

// a tile of TX x TY cells; phase 3 maps one thread to one cell
template <int TX_, int TY_>
struct F64Tile {
  static constexpr int TX = TX_, TY = TY_, NT = TX * TY;
  static constexpr int RX = TX + 6, RY = TY + 6, RN = RX * RY;
  static constexpr int NFX = TY * (TX + 1), NFY = (TY + 1) * TX, NF = NFX + NFY;
};
constexpr int NT = 256;
constexpr int NCELL_ARR = 11;

}  // namespace

// x / b for a divisor fixed in advance — the constants 3, 6, 12 of the reference
// (x/3., x/6., A*A*13./12.) and a grid's dx, dy, 60 dx, 60 dy — correctly rounded:
// q0 = RN(x y) with y = RN(1/b), the remainder
// r = x - q0 b is exact in one FMA, and q0 + r y rounded once is RN(x / b)
// (Markstein's correction, IBM J. Res. Dev. 34(1), 1990) when the quotient does not
// underflow.  Where the correction does not apply, q0 is already the IEEE result: a
// zero dividend keeps its sign, an infinite one stays infinite (the remainder would
// be inf - inf = NaN) and a NaN stays NaN.  The GPU test suite checks this against
// IEEE division.
__device__ __forceinline__ double ccs_div_const(double x, double b, double y) {
  const double q0 = x * y;
  const double r = fma(-q0, b, x);
  const double q1 = fma(r, y, q0);
  // x = +-0, +-inf or NaN, tested on the bits (the FP64 pipe is the lane's
  // bottleneck): with the sign shifted out, 0 - 1 wraps to the top of the range and
  // an all-ones exponent field is at least 0xffe0...
  const unsigned long long t = (unsigned long long)__double_as_longlong(x) << 1;
  return t - 1ull >= 0xffe0000000000000ull - 1ull ? q0 : q1;
}

// a / b for a divisor b shared by several quotients, from y = RN(1 / b) computed
// once: q0 = RN(a y), the exact remainder r = a - q0 b in one FMA, and q0 + r y
// rounded once, which is RN(a / b) when the quotient is a normal number (Markstein's
// correction, as in ccs_div_const).  The GPU test suite checks it against IEEE
// division on random operands.
__device__ __forceinline__ double ccs_div_by(double a, double b, double y) {
  const double q0 = a * y;
  const double r = fma(-q0, b, a);
  return fma(r, y, q0);
}

namespace {

// Comparisons of non-negative doubles on the integer pipes: for +0 and positive
// finite or infinite values the IEEE order is the order of the bit patterns read
// as signed integers, so these give the FP64 comparisons' results without issuing
// on the FP64 pipe (GB300 runs FP64 at 1/64 of the FP32 rate).  |x| is the bit
// pattern with the sign cleared.
__device__ __forceinline__ long long abs_bits(double x) {
  return __double_as_longlong(x) & 0x7fffffffffffffffLL;
}

// WENO_limiter, spatial_operators_mod.F90:282-361.
template <int DIR>
__device__ __forceinline__ double weno5z(double q0, double q1, double q2, double q3, double q4) {
  // q0..q4 = Q(1..5) = field(i-2 .. i+2)
  const double Qim2 = q0, Qim1 = q1, Qi = q2, Qip1 = q3, Qip2 = q4;
  double s0, s1, s2, a0, a1, a2, b0, b1, b2;
  const double y3 = 1. / 3., y6 = 1. / 6., y12 = 1. / 12.;
  if (DIR > 0) {
    s0 = ccs_div_const(Qim2, 3., y3) - 7. / 6. * Qim1 + 11. / 6. * Qi;
    s1 = ccs_div_const(-Qim1, 6., y6) + 5. / 6. * Qi + 1. / 3. * Qip1;
    s2 = ccs_div_const(Qi, 3., y3) + 5. / 6. * Qip1 - 1. / 6. * Qip2;
    a0 = Qim2 - 2. * Qim1 + Qi;
    a1 = Qim1 - 2. * Qi + Qip1;
    a2 = Qi - 2. * Qip1 + Qip2;
    b0 = Qim2 - 4. * Qim1 + 3. * Qi;
    b1 = Qim1 - Qip1;
    b2 = 3. * Qi - 4. * Qip1 + Qip2;
  } else {
    s0 = ccs_div_const(Qip2, 3., y3) - 7. / 6. * Qip1 + 11. / 6. * Qi;
    s1 = ccs_div_const(-Qip1, 6., y6) + 5. / 6. * Qi + 1. / 3. * Qim1;
    s2 = ccs_div_const(Qi, 3., y3) + 5. / 6. * Qim1 - 1. / 6. * Qim2;
    a0 = Qip2 - 2. * Qip1 + Qi;
    a1 = Qip1 - 2. * Qi + Qim1;
    a2 = Qi - 2. * Qim1 + Qim2;
    b0 = Qip2 - 4. * Qip1 + 3. * Qi;
    b1 = Qip1 - Qim1;
    b2 = 3. * Qi - 4. * Qim1 + Qim2;
  }
  const double be0 = ccs_div_const(a0 * a0 * 13., 12., y12) + b0 * b0 * 0.25;
  const double be1 = ccs_div_const(a1 * a1 * 13., 12., y12) + b1 * b1 * 0.25;
  const double be2 = ccs_div_const(a2 * a2 * 13., 12., y12) + b2 * b2 * 0.25;
  // the betas are sums of squares (never -0 or negative), the taus absolute values
  const long long t40 = abs_bits(be0 - be1), t41 = abs_bits(be1 - be2);
  const double tau5 = fabs(be2 - be0);
  long long mn = __double_as_longlong(be0);
  if (__double_as_longlong(be1) < mn) mn = __double_as_longlong(be1);
  if (__double_as_longlong(be2) < mn) mn = __double_as_longlong(be2);
  double w0, w1, w2;
  if (t40 <= mn && t41 > mn) {
    w0 = 1. / 3.; w1 = 2. / 3.; w2 = 0.;
  } else if (t40 > mn && t41 < mn) {
    w0 = 0.; w1 = 2. / 3.; w2 = 1. / 3.;
  } else {
    const double eps = 1.E-2;
    const double al0 = 0.1 * (1. + tau5 / (eps + be0));
    const double al1 = 0.6 * (1. + tau5 / (eps + be1));
    const double al2 = 0.3 * (1. + tau5 / (eps + be2));
    const double sum = ((0. + al0) + al1) + al2;
    // omega = alpha / sum(alpha): one IEEE reciprocal for the three quotients.  Each
    // alpha is at least its linear weight (0.1) and sum >= alpha, so the quotients lie
    // in (2^-1004, 1] whenever sum < 2^1000 (tested on the bits); a larger, infinite
    // or NaN sum takes IEEE division
    if (__double_as_longlong(sum) < 0x7e70000000000000LL) {
      const double ys = 1. / sum;
      w0 = ccs_div_by(al0, sum, ys); w1 = ccs_div_by(al1, sum, ys); w2 = ccs_div_by(al2, sum, ys);
    } else {
      w0 = al0 / sum; w1 = al1 / sum; w2 = al2 / sum;
    }
  }
  return ((0. + s0 * w0) + s1 * w1) + s2 * w2;
}

// Centred difference of cell values f[-3s .. 3s] around f[0], divided by the
// stencil's denominator times d: spatial_operators_mod_2nd.F90:54-59,
// spatial_operators_mod_4th.F90:58-63, spatial_operators_mod_6th.F90:62-67.
__device__ __forceinline__ double central_diff(int op, const double *f, int s, double d) {
  if (op == 2) return (f[s] - f[-s]) / (2. * d);
  if (op == 4) return (f[-2 * s] - 8. * f[-s] + 8. * f[s] - f[2 * s]) / (12. * d);
  return (-f[-3 * s] + 9. * f[-2 * s] - 45. * f[-s] + 45. * f[s] - 9. * f[2 * s] + f[3 * s]) / (60. * d);
}

template <int RN>
struct Smem {
  // cell quantities on the halo'd tile (row-major [RY][RX])
  double phit[RN], phitG[RN], E[RN], Fx[RN], Fy[RN], uC[RN], vC[RN], ig11[RN], ig22[RN], u[RN], v[RN];
};

__device__ __forceinline__ bool is_corner(int i, int j, int N) {
  return (i < 1 || i > N) && (j < 1 || j > N);
}

template <class T>
__global__ void __launch_bounds__(NT, 2)
f64_stage_kernel(const F64Stage *__restrict__ stages, const WorkItem *__restrict__ work, int nwork) {
  constexpr int TX = T::TX, TY = T::TY, RX = T::RX, RN = T::RN, NFX = T::NFX, NF = T::NF;
  static_assert(T::NT == NT, "phase 3 maps one thread to one cell");
  extern __shared__ __align__(16) double smem_raw[];
  Smem<RN> &S = *reinterpret_cast<Smem<RN> *>(smem_raw);
  double *rec = smem_raw + NCELL_ARR * RN;  // [nrec][NF]
  const int tid = threadIdx.x;

  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const WorkItem wi = work[w];
    const F64Stage &st = stages[wi.inst];
    const Layout L = st.L;
    const int N = L.N, p = wi.panel;
    const int i0 = 1 + wi.tx * TX, j0 = 1 + wi.ty * TY;
    const int nrec = st.ediss ? 8 : 6;
    const int op = st.op;  // uniform over the work item
#ifdef CCS_BOUNDS
    // poison the tile arrays: a read of a slot this tile never wrote shows up as NaN
    // in the result (checked build only)
    for (int k = tid; k < NCELL_ARR * RN + 8 * NF; k += NT) smem_raw[k] = __longlong_as_double(0x7ff8000000000000LL);
    __syncthreads();
#endif

    // ---- phase 1: cell quantities (spatial_operators_mod.F90:71-78) ----------
    for (int r = tid; r < RN; r += NT) {
      const int li = r % RX, lj = r / RX;
      const int i = i0 - 3 + li, j = j0 - 3 + lj;
      double phit = 0., phitG = 0., E = 0., Fx = 0., Fy = 0., uC = 0., vC = 0., g11 = 0., g22 = 0., u = 0.,
             v = 0.;
      const int64_t c = L.idx(i, j, p);
      if (i >= -2 && i <= N + 3 && j >= -2 && j <= N + 3 && !is_corner(i, j, N) && ccs_inb(c, L.field, 201)) {
        const double phiG = st.in.phiG[c], phi = st.in.phi[c];
        u = st.in.u[c];
        v = st.in.v[c];
        uC = st.in.uC[c];
        vC = st.in.vC[c];
        g11 = st.m.ig11[c];
        g22 = st.m.ig22[c];
        phit = phi + st.m.phis[c];
        phitG = phit * st.m.sqrtG[c];
        const double K = 0.5 * (u * uC + v * vC);
        E = phit + K;
        Fx = phiG * uC;
        Fy = phiG * vC;
      }
      S.phit[r] = phit; S.phitG[r] = phitG; S.E[r] = E; S.Fx[r] = Fx; S.Fy[r] = Fy;
      S.uC[r] = uC; S.vC[r] = vC; S.ig11[r] = g11; S.ig22[r] = g22; S.u[r] = u; S.v[r] = v;
    }
    __syncthreads();

    // ---- phase 2: face reconstructions (weno, :183-277) ---------------------
    // (the central-difference operators have no faces: straight to phase 3)
    if (op == CCS_OP_WENO) {
    for (int t = tid; t < nrec * NF; t += NT) {
      const int face = t % NF, q = t / NF;
      const double *fld;
      double val = 0.;
      if (face < NFX) {
        const int fi = face % (TX + 1), lj = face / (TX + 1);
        const int f = i0 - 1 + fi, j = j0 + lj;
        if (j <= N && f <= N && ccs_inb((lj + 3) * RX + fi + 5, RN, 211)) {
          fld = (q < 2) ? S.Fx : (q < 4) ? S.E : (q < 6) ? S.phitG : S.u;
          const double *row = fld + (lj + 3) * RX;
          if ((q & 1) == 0)  // "+" from cell f: field(f-2 .. f+2)
            val = weno5z<1>(row[fi], row[fi + 1], row[fi + 2], row[fi + 3], row[fi + 4]);
          else  // "-" from cell f+1: field(f-1 .. f+3)
            val = weno5z<-1>(row[fi + 1], row[fi + 2], row[fi + 3], row[fi + 4], row[fi + 5]);
        }
      } else {
        const int fy = face - NFX;
        const int li = fy % TX, fj = fy / TX;
        const int g = j0 - 1 + fj, i = i0 + li;
        if (i <= N && g <= N && ccs_inb(li + 3 + (fj + 5) * RX, RN, 212)) {
          fld = (q < 2) ? S.Fy : (q < 4) ? S.E : (q < 6) ? S.phitG : S.v;
          const double *col = fld + (li + 3);
          if ((q & 1) == 0)
            val = weno5z<1>(col[fj * RX], col[(fj + 1) * RX], col[(fj + 2) * RX], col[(fj + 3) * RX],
                            col[(fj + 4) * RX]);
          else
            val = weno5z<-1>(col[(fj + 1) * RX], col[(fj + 2) * RX], col[(fj + 3) * RX], col[(fj + 4) * RX],
                             col[(fj + 5) * RX]);
        }
      }
      if (ccs_inb(q * NF + face, 8 * NF, 213)) rec[q * NF + face] = val;
    }
    __syncthreads();

    // ---- phase 2b: Rusanov fluxes at faces (:101-149) ------------------------
    for (int face = tid; face < NF; face += NT) {
      const double Fp = rec[0 * NF + face], Fn = rec[1 * NF + face];
      const double Ep = rec[2 * NF + face], En = rec[3 * NF + face];
      const double Pp = rec[4 * NF + face], Pn = rec[5 * NF + face];
      double dp = 0., dn = 0.;  // never-written u_ext / v_ext slots (CCS_EDISS_ZERO)
      if (nrec == 8) {
        dp = rec[6 * NF + face];
        dn = rec[7 * NF + face];
      }
      double a, b, ga, gb, pa, pb;  // contravariant wind, IG diagonal, phit at the two cells
      if (face < NFX) {
        const int fi = face % (TX + 1), lj = face / (TX + 1);
        const int r = (lj + 3) * RX + fi + 2;  // cell f; cell f+1 is r + 1
        if (!ccs_inb(r + 1, RN, 214)) continue;
        a = S.uC[r + 1]; b = S.uC[r];
        ga = S.ig11[r + 1]; gb = S.ig11[r];
        pa = S.phit[r + 1]; pb = S.phit[r];
      } else {
        const int fy = face - NFX;
        const int li = fy % TX, fj = fy / TX;
        const int r = (fj + 2) * RX + li + 3;  // cell g; cell g+1 is r + RX
        if (!ccs_inb(r + RX, RN, 215)) continue;
        a = S.vC[r + RX]; b = S.vC[r];
        ga = S.ig22[r + RX]; gb = S.ig22[r];
        pa = S.phit[r + RX]; pb = S.phit[r];
      }
      const double uBdy = 0.5 * (a + b);
      const double phitBdy = 0.5 * (pa + pb);
      const double e1 = uBdy - sqrt(0.5 * (ga + gb) * phitBdy);
      const double e2 = uBdy + sqrt(0.5 * (ga + gb) * phitBdy);
      const double mx = abs_bits(e2) > abs_bits(e1) ? fabs(e2) : fabs(e1);
      rec[0 * NF + face] = 0.5 * (Fp + Fn - mx * (Pn - Pp));
      rec[1 * NF + face] = 0.5 * (Ep + En - mx * (dn - dp));
    }
    __syncthreads();
    }  // op == CCS_OP_WENO

    // ---- phase 3: tendencies, stage update, boundary correction --------------
    {
      const int li = tid % TX, lj = tid / TX;
      const int i = i0 + li, j = j0 + lj;
      const int64_t c = L.idx(i, j, p);
      const int rc = (lj + 3) * RX + li + 3;
      if (i <= N && j <= N && ccs_inb(c, L.field, 221) && ccs_inb(rc + 3 * RX, RN, 222) &&
          ccs_inb(NFX + (lj + 1) * TX + li, NF, 223)) {
        double dfluxdx, dEdx, dvdx, dfluxdy, dEdy, dudy;
        if (op == CCS_OP_WENO) {
          const double *FF = rec, *EF = rec + NF;
          const int xl = lj * (TX + 1) + li, xr = xl + 1;
          const int yb = NFX + lj * TX + li, yt = yb + TX;
          // divisions by dx, dy, 60 dx, 60 dy (spatial_operators_mod.F90:153-169) from
          // their reciprocals, corrected to the IEEE quotients (ccs_div_const)
          dfluxdx = ccs_div_const(FF[xr] - FF[xl], st.dx, st.rdx);
          dEdx = ccs_div_const(EF[xr] - EF[xl], st.dx, st.rdx);
          const double *vr = S.v + (lj + 3) * RX + li;  // v(i-3 .. i+3) at vr[0..6]
          dvdx = ccs_div_const(-vr[0] + 9. * vr[1] - 45. * vr[2] + 45. * vr[4] - 9. * vr[5] + vr[6], st.dx60,
                               st.rdx60);
          dfluxdy = ccs_div_const(FF[yt] - FF[yb], st.dy, st.rdy);
          dEdy = ccs_div_const(EF[yt] - EF[yb], st.dy, st.rdy);
          const double *uc = S.u + lj * RX + li + 3;  // u(j-3 .. j+3) at uc[k * RX]
          dudy = ccs_div_const(-uc[0] + 9. * uc[RX] - 45. * uc[2 * RX] + 45. * uc[4 * RX] - 9. * uc[5 * RX] +
                                   uc[6 * RX],
                               st.dy60, st.rdy60);
        } else {
          dfluxdx = central_diff(op, S.Fx + rc, 1, st.dx);
          dEdx = central_diff(op, S.E + rc, 1, st.dx);
          dvdx = central_diff(op, S.v + rc, 1, st.dx);
          dfluxdy = central_diff(op, S.Fy + rc, RX, st.dy);
          dEdy = central_diff(op, S.E + rc, RX, st.dy);
          dudy = central_diff(op, S.u + rc, RX, st.dy);
        }
        const double sqrtG = st.m.sqrtG[c];
        const double vort = dvdx - dudy + sqrtG * st.m.f[c];
        const double uCc = S.uC[rc], vCc = S.vC[rc];
        const double tp = -(dfluxdx + dfluxdy);
        const double tu = -dEdx + vort * vCc;
        const double tv = -dEdy - vort * uCc;

        if (st.kind == K_TEND) {
          st.tphiG[c] = tp;
          st.tu[c] = tu;
          st.tv[c] = tv;
        } else {
          const double y0p = st.y0phiG[c], y0u = st.y0u[c], y0v = st.y0v[c];
          double np, nu, nv;
          switch (st.kind) {
            case K_RK4_1:
              st.accphiG[c] = tp; st.accu[c] = tu; st.accv[c] = tv;
              np = y0p + st.c1 * tp; nu = y0u + st.c1 * tu; nv = y0v + st.c1 * tv;
              break;
            case K_RK4_2: {
              const double ap = st.accphiG[c] + 2. * tp;
              const double au = st.accu[c] + 2. * tu;
              const double av = st.accv[c] + 2. * tv;
              st.accphiG[c] = ap; st.accu[c] = au; st.accv[c] = av;
              np = y0p + st.c1 * tp; nu = y0u + st.c1 * tu; nv = y0v + st.c1 * tv;
              break;
            }
            case K_RK4_4: {
              const double kp = ccs_div_const(st.accphiG[c] + tp, 6., 1. / 6.);
              const double ku = ccs_div_const(st.accu[c] + tu, 6., 1. / 6.);
              const double kv = ccs_div_const(st.accv[c] + tv, 6., 1. / 6.);
              np = y0p + st.c1 * kp; nu = y0u + st.c1 * ku; nv = y0v + st.c1 * kv;
              break;
            }
            case K_RK3_1:
              np = y0p + st.c1 * tp; nu = y0u + st.c1 * tu; nv = y0v + st.c1 * tv;
              break;
            case K_RK3_2: {
              const double ycp = st.in.phiG[c], ycu = S.u[rc], ycv = S.v[rc];
              np = 0.75 * y0p + 0.25 * ycp + st.c1 * tp;
              nu = 0.75 * y0u + 0.25 * ycu + st.c1 * tu;
              nv = 0.75 * y0v + 0.25 * ycv + st.c1 * tv;
              break;
            }
            default: {  // K_RK3_3
              const double ycp = st.in.phiG[c], ycu = S.u[rc], ycv = S.v[rc];
              np = y0p / 3. + 2. / 3. * ycp + st.c1 * tp;
              nu = y0u / 3. + 2. / 3. * ycu + st.c1 * tu;
              nv = y0v / 3. + 2. / 3. * ycv + st.c1 * tv;
              break;
            }
          }
          // correct_bdy_ghost: P2SP (interior), SP2P, cov2contrav, phi = phiG / sqrtG
          const double zon = st.m.aig11[c] * nu + st.m.aig12[c] * nv;
          const double mer = st.m.aig21[c] * nu + st.m.aig22[c] * nv;
          const double u2 = st.m.gia11[c] * zon + st.m.gia12[c] * mer;
          const double v2 = st.m.gia21[c] * zon + st.m.gia22[c] * mer;
          st.out.phiG[c] = np;
          st.out.u[c] = u2;
          st.out.v[c] = v2;
          st.out.uC[c] = st.m.ig11[c] * u2 + st.m.ig12[c] * v2;
          st.out.vC[c] = st.m.ig21[c] * u2 + st.m.ig22[c] * v2;
          st.out.phi[c] = np / sqrtG;
          if (st.zonal) {
            st.zonal[c] = zon;
            st.merid[c] = mer;
          }
          // ghost push: this cell's value lands in the halo strip of each edge it is
          // within `halo` of (two strips near a panel corner)
          const int h = L.h;
          for (int side = 0; side < 4; side++) {
            int k, m;
            if (side == 0) { k = i; m = j; }
            else if (side == 1) { k = N + 1 - i; m = j; }
            else if (side == 2) { k = j; m = i; }
            else { k = N + 1 - j; m = i; }
            if (k > h) continue;
            const int64_t e = ((int64_t)p * 4 + side) * h * N + (int64_t)(k - 1) * N + (m - 1);
            if (!ccs_inb(e, (long long)24 * h * N, 224)) continue;
            const int64_t d = st.m.push[e];
            if (!ccs_inb(d, L.field, 225)) continue;
            const double ud = st.m.gia11[d] * zon + st.m.gia12[d] * mer;
            const double vd = st.m.gia21[d] * zon + st.m.gia22[d] * mer;
            st.out.phiG[d] = np;
            st.out.u[d] = ud;
            st.out.v[d] = vd;
            st.out.uC[d] = st.m.ig11[d] * ud + st.m.ig12[d] * vd;
            st.out.vC[d] = st.m.ig21[d] * ud + st.m.ig22[d] * vd;
            st.out.phi[d] = np / st.m.sqrtG[d];
            if (st.zonal) {
              st.zonal[d] = zon;
              st.merid[d] = mer;
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace

// test support: out[k] = ccs_div_const(x[k], b, 1/b) next to out[n + k] = x[k] / b
__global__ void div_const_check_kernel(const double *__restrict__ x, int64_t n, double b, double y,
                                       double *__restrict__ out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    out[k] = ccs_div_const(x[k], b, y);
    out[n + k] = x[k] / b;
  }
}

// test support: out[k] = ccs_div_by(a[k], b[k], 1 / b[k]) next to out[n + k] = a[k] / b[k]
__global__ void div_pairs_check_kernel(const double *__restrict__ a, const double *__restrict__ b, int64_t n,
                                       double *__restrict__ out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    out[k] = ccs_div_by(a[k], b[k], 1. / b[k]);
    out[n + k] = a[k] / b[k];
  }
}

cudaError_t launch_div_pairs_check(const double *a, const double *b, int64_t n, double *out, cudaStream_t s) {
  div_pairs_check_kernel<<<1024, 256, 0, s>>>(a, b, n, out);
  return cudaGetLastError();
}

unsigned long long f64_bounds_take() { return bounds_take_tu(); }

cudaError_t launch_div_const_check(const double *x, int64_t n, double b, double *out, cudaStream_t s) {
  div_const_check_kernel<<<1024, 256, 0, s>>>(x, n, b, 1. / b, out);
  return cudaGetLastError();
}

namespace {

using F64T0 = F64Tile<32, 8>;
using F64T1 = F64Tile<16, 16>;
using F64T2 = F64Tile<64, 4>;

template <class T>
constexpr int f64_smem_bytes() {  // sized for the E-reconstruction variant (8 face arrays)
  return (int)((NCELL_ARR * T::RN + 8 * T::NF) * sizeof(double));
}

template <class T>
int f64_grid_for(int device) {
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  constexpr int smem = f64_smem_bytes<T>();
  cudaFuncSetAttribute(f64_stage_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f64_stage_kernel<T>, NT, smem);
  if (per < 1) per = 1;
  return sms * per;
}

template <class T>
cudaError_t f64_launch(const F64Stage *d_stages, const WorkItem *d_work, int nwork, int grid, cudaStream_t s) {
  constexpr int smem = f64_smem_bytes<T>();
  static std::atomic<uint64_t> attr_done{0};
  const cudaError_t e = smem_attr_once((const void *)f64_stage_kernel<T>, smem, attr_done);
  if (e != cudaSuccess) return e;
  if (grid > nwork) grid = nwork;
  if (grid < 1) return cudaSuccess;
  f64_stage_kernel<T><<<grid, NT, smem, s>>>(d_stages, d_work, nwork);
  return cudaGetLastError();
}

static_assert(F64T0::TX == kF64Tiles[0].tx && F64T0::TY == kF64Tiles[0].ty, "tile table");
static_assert(F64T1::TX == kF64Tiles[1].tx && F64T1::TY == kF64Tiles[1].ty, "tile table");
static_assert(F64T2::TX == kF64Tiles[2].tx && F64T2::TY == kF64Tiles[2].ty, "tile table");

}  // namespace

int f64_max_grid(int var, int device) {
  switch (var) {
    case 1: return f64_grid_for<F64T1>(device);
    case 2: return f64_grid_for<F64T2>(device);
    default: return f64_grid_for<F64T0>(device);
  }
}

cudaError_t launch_f64_stage(int var, const F64Stage *d_stages, const WorkItem *d_work, int nwork, int grid,
                             cudaStream_t s) {
  switch (var) {
    case 1: return f64_launch<F64T1>(d_stages, d_work, nwork, grid, s);
    case 2: return f64_launch<F64T2>(d_stages, d_work, nwork, grid, s);
    default: return f64_launch<F64T0>(d_stages, d_work, nwork, grid, s);
  }
}

// ---- diagnostics: calc_total_mass / calc_total_energy (diag_mod.F90:10-53) ------
// Each block sums a contiguous range of interior cells in the reference's order
// (i fastest, then j, then panel); the host adds the block partials in order.
__global__ void f64_diag_kernel(Layout L, const double *__restrict__ phiG, const double *__restrict__ phi,
                                const double *__restrict__ u, const double *__restrict__ v,
                                const double *__restrict__ uC, const double *__restrict__ vC,
                                const double *__restrict__ sqrtG, const double *__restrict__ phis,
                                double *__restrict__ partials) {
  __shared__ double sm[2][256];
  const int64_t ncell = (int64_t)L.N * L.N * 6;
  const int64_t per = (ncell + gridDim.x - 1) / gridDim.x;
  const int64_t beg = blockIdx.x * per;
  int64_t end = beg + per;
  if (end > ncell) end = ncell;
  double m = 0., e = 0.;
  for (int64_t q = beg + threadIdx.x; q < end; q += blockDim.x) {
    const int i = 1 + (int)(q % L.N);
    const int j = 1 + (int)((q / L.N) % L.N);
    const int p = (int)(q / ((int64_t)L.N * L.N));
    const int64_t c = L.idx(i, j, p);
    m += phiG[c];
    const double KE = 0.5 * phi[c] * (u[c] * uC[c] + v[c] * vC[c]);
    const double t = phi[c] + phis[c];
    const double PE = 0.5 * (t * t);
    e += sqrtG[c] * (KE + PE);
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
    partials[2 * blockIdx.x] = sm[0][0];
    partials[2 * blockIdx.x + 1] = sm[1][0];
  }
}

cudaError_t launch_f64_diag(const Layout &L, const double *phiG, const double *phi, const double *u,
                            const double *v, const double *uC, const double *vC, const double *sqrtG,
                            const double *phis, double *partials, int nblocks, cudaStream_t s) {
  f64_diag_kernel<<<nblocks, 256, 0, s>>>(L, phiG, phi, u, v, uC, vC, sqrtG, phis, partials);
  return cudaGetLastError();
}

}  // namespace ccs
