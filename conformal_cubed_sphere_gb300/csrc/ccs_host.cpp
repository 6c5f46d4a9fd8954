// ccs_host.cpp -- host-side set-up of the cubed-sphere step: mesh-file samples,
// metric derivation (io_mod.read_mesh), the ghost-fill tables the kernels use,
// reference test cases and seeded initial states.  Runs once per run on the CPU.
#include "ccs_internal.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

namespace ccs {

// constants_mod.F90:6-12
static const double kPi = 3.14159265358979323846;
static const double kD2R = kPi / 180.;
static const double kR2D = 180. / kPi;
static const double kFillValue = -9999999999999999.;

// ---------------------------------------------------------------------------
// Ghost fill (ghost_mod.f90:18-82).  Sides: 0 = left (i = 1-k), 1 = right
// (i = N+k), 2 = below (j = 1-k), 3 = over (j = N+k); k = 1..h is the depth and
// m = 1..N runs along the edge.  ghost_source gives the interior cell whose value
// the reference copies to halo cell (p, side, k, m).
// ---------------------------------------------------------------------------
GhostSrc ghost_source(int N, int p, int side, int k, int m) {
  const int a = N - k + 1, b = N - m + 1;
  switch (p) {
    case 1:
      if (side == 0) return {4, a, m};
      if (side == 1) return {2, k, m};
      if (side == 2) return {6, m, a};
      return {5, m, k};
    case 2:
      if (side == 0) return {1, a, m};
      if (side == 1) return {3, k, m};
      if (side == 2) return {6, a, b};
      return {5, a, m};
    case 3:
      if (side == 0) return {2, a, m};
      if (side == 1) return {4, k, m};
      if (side == 2) return {6, b, k};
      return {5, b, a};
    case 4:
      if (side == 0) return {3, a, m};
      if (side == 1) return {1, k, m};
      if (side == 2) return {6, k, m};
      return {5, k, b};
    case 5:
      if (side == 0) return {4, b, a};
      if (side == 1) return {2, m, a};
      if (side == 2) return {1, m, a};
      return {3, b, a};
    default:
      if (side == 0) return {4, m, k};
      if (side == 1) return {2, b, k};
      if (side == 2) return {3, b, k};
      return {1, m, k};
  }
}

// Which edge strip of the source panel feeds halo strip (p, side): every one of
// the 24 interior edge strips is copied to exactly one halo strip.
int ghost_source_side(int p, int side) {
  static const int tab[6][4] = {
      {1, 0, 3, 2},  // panel 1: L<-P4 R, R<-P2 L, B<-P6 T, T<-P5 B
      {1, 0, 1, 1},  // panel 2: L<-P1 R, R<-P3 L, B<-P6 R, T<-P5 R
      {1, 0, 2, 3},  // panel 3: L<-P2 R, R<-P4 L, B<-P6 B, T<-P5 T
      {1, 0, 0, 0},  // panel 4: L<-P3 R, R<-P1 L, B<-P6 L, T<-P5 L
      {3, 3, 3, 3},  // panel 5: all from the top strips of P4, P2, P1, P3
      {2, 2, 2, 2},  // panel 6: all from the bottom strips of P4, P2, P3, P1
  };
  return tab[p - 1][side];
}

// Depth k and along-edge m of an interior cell inside edge strip `side`.
static inline void strip_coords(int N, int side, int i, int j, int *k, int *m) {
  switch (side) {
    case 0: *k = i; *m = j; break;
    case 1: *k = N + 1 - i; *m = j; break;
    case 2: *k = j; *m = i; break;
    default: *k = N + 1 - j; *m = i; break;
  }
}

// Push table for a layout: entry ((ps-1)*4 + s)*h*N + (k-1)*N + (m-1) is the
// linear index (within one field of `L`) of the halo cell that receives interior
// cell (k, m) of strip s of panel ps.  Returns false if the tables disagree.
bool build_push_table(const Layout &L, std::vector<int32_t> &push) {
  const int N = L.N, h = L.h;
  push.assign((size_t)24 * h * N, -1);
  for (int p = 1; p <= 6; p++)
    for (int side = 0; side < 4; side++)
      for (int k = 1; k <= h; k++)
        for (int m = 1; m <= N; m++) {
          const GhostSrc s = ghost_source(N, p, side, k, m);
          const int ss = ghost_source_side(p, side);
          int ks, ms;
          strip_coords(N, ss, s.i, s.j, &ks, &ms);
          if (ks != k || ms < 1 || ms > N) return false;
          int di, dj;
          switch (side) {
            case 0: di = 1 - k; dj = m; break;
            case 1: di = N + k; dj = m; break;
            case 2: di = m; dj = 1 - k; break;
            default: di = m; dj = N + k; break;
          }
          const size_t e = ((size_t)(s.p - 1) * 4 + ss) * h * N + (size_t)(ks - 1) * N + (ms - 1);
          if (push[e] != -1) return false;
          push[e] = (int32_t)L.idx(di, dj, p - 1);
        }
  for (int32_t v : push)
    if (v < 0) return false;
  return true;
}

// ---------------------------------------------------------------------------
// Fortran-order host arrays (ics:ice, jcs:jce, 1:6)
// ---------------------------------------------------------------------------
struct HArr {
  int N, h, nh;
  size_t at(int i, int j, int p) const {
    return (size_t)(i - (1 - h)) + (size_t)nh * ((size_t)(j - (1 - h)) + (size_t)nh * (size_t)(p - 1));
  }
};

static void fill_halo_host(int N, int h, double *field, int stride, int comp) {
  // generic over interleaved components: element (comp) of a `stride`-wide record
  HArr A{N, h, N + 2 * h};
  std::vector<double> inner((size_t)N * N * 6);
  auto in = [&](int i, int j, int p) -> double & {
    return inner[(size_t)(i - 1) + (size_t)N * ((size_t)(j - 1) + (size_t)N * (size_t)(p - 1))];
  };
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) in(i, j, p) = field[stride * A.at(i, j, p) + comp];
  for (int p = 1; p <= 6; p++)
    for (int side = 0; side < 4; side++)
      for (int k = 1; k <= h; k++)
        for (int m = 1; m <= N; m++) {
          const GhostSrc s = ghost_source(N, p, side, k, m);
          int di, dj;
          switch (side) {
            case 0: di = 1 - k; dj = m; break;
            case 1: di = N + k; dj = m; break;
            case 2: di = m; dj = 1 - k; break;
            default: di = m; dj = N + k; break;
          }
          field[stride * A.at(di, dj, p) + comp] = in(s.i, s.j, s.p);
        }
}

// CubedSphereFillJab (ghost_mod.f90:84-160): the same copy for the 3x2 Jacobian,
// with the local axes of the source panel re-expressed in the destination panel's
// axes.  The column map per halo strip: (c1, s1, c2, s2) meaning
// dest(:,1) = s1 * src(:,c1), dest(:,2) = s2 * src(:,c2).
static void fill_jab_host(int N, int h, double *jab) {
  static const int cmap[6][4][4] = {
      // panel 1: all strips copy unchanged
      {{1, 1, 2, 1}, {1, 1, 2, 1}, {1, 1, 2, 1}, {1, 1, 2, 1}},
      // panel 2: B: (-src2, src1); T: (src2, -src1)
      {{1, 1, 2, 1}, {1, 1, 2, 1}, {2, -1, 1, 1}, {2, 1, 1, -1}},
      // panel 3: B and T negate both columns
      {{1, 1, 2, 1}, {1, 1, 2, 1}, {1, -1, 2, -1}, {1, -1, 2, -1}},
      // panel 4: B: (src2, -src1); T: (-src2, src1)
      {{1, 1, 2, 1}, {1, 1, 2, 1}, {2, 1, 1, -1}, {2, -1, 1, 1}},
      // panel 5: L: (src2, -src1); R: (-src2, src1); B unchanged; T negated
      {{2, 1, 1, -1}, {2, -1, 1, 1}, {1, 1, 2, 1}, {1, -1, 2, -1}},
      // panel 6: L: (-src2, src1); R: (src2, -src1); B negated; T unchanged
      {{2, -1, 1, 1}, {2, 1, 1, -1}, {1, -1, 2, -1}, {1, 1, 2, 1}},
  };
  HArr A{N, h, N + 2 * h};
  std::vector<double> inner((size_t)6 * N * N * 6);
  auto in = [&](int r, int c, int i, int j, int p) -> double & {
    return inner[(size_t)(r - 1) + 3 * (size_t)(c - 1) +
                 6 * ((size_t)(i - 1) + (size_t)N * ((size_t)(j - 1) + (size_t)N * (size_t)(p - 1)))];
  };
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++)
        for (int c = 1; c <= 2; c++)
          for (int r = 1; r <= 3; r++) in(r, c, i, j, p) = jab[(r - 1) + 3 * (c - 1) + 6 * A.at(i, j, p)];
  for (int p = 1; p <= 6; p++)
    for (int side = 0; side < 4; side++)
      for (int k = 1; k <= h; k++)
        for (int m = 1; m <= N; m++) {
          const GhostSrc s = ghost_source(N, p, side, k, m);
          int di, dj;
          switch (side) {
            case 0: di = 1 - k; dj = m; break;
            case 1: di = N + k; dj = m; break;
            case 2: di = m; dj = 1 - k; break;
            default: di = m; dj = N + k; break;
          }
          const int *cm = cmap[p - 1][side];
          double *d = &jab[6 * A.at(di, dj, p)];
          for (int r = 1; r <= 3; r++) {
            const double v1 = in(r, cm[0], s.i, s.j, s.p);
            const double v2 = in(r, cm[2], s.i, s.j, s.p);
            d[(r - 1)] = cm[1] < 0 ? -v1 : v1;
            d[(r - 1) + 3] = cm[3] < 0 ? -v2 : v2;
          }
        }
}

// BRINV (math_mod.f90:451-525) for a 2x2 column-major matrix; false if singular.
static bool brinv2(const double *Ain, double *A) {
  const int n = 2;
  int IS[3] = {0, 0, 0}, JS[3] = {0, 0, 0};
  auto AA = [&](int i, int j) -> double & { return A[(i - 1) + n * (j - 1)]; };
  for (int k = 0; k < 4; k++) A[k] = Ain[k];
  for (int K = 1; K <= n; K++) {
    double D = 0.;
    for (int I = K; I <= n; I++)
      for (int J = K; J <= n; J++)
        if (std::fabs(AA(I, J)) > D) {
          D = std::fabs(AA(I, J));
          IS[K] = I;
          JS[K] = J;
        }
    if (D + 1.0 == 1.0) return false;
    for (int J = 1; J <= n; J++) std::swap(AA(K, J), AA(IS[K], J));
    for (int I = 1; I <= n; I++) std::swap(AA(I, K), AA(I, JS[K]));
    AA(K, K) = 1 / AA(K, K);
    for (int J = 1; J <= n; J++)
      if (J != K) AA(K, J) = AA(K, J) * AA(K, K);
    for (int I = 1; I <= n; I++)
      if (I != K)
        for (int J = 1; J <= n; J++)
          if (J != K) AA(I, J) = AA(I, J) - AA(I, K) * AA(K, J);
    for (int I = 1; I <= n; I++)
      if (I != K) AA(I, K) = -AA(I, K) * AA(K, K);
  }
  for (int K = n; K >= 1; K--) {
    for (int J = 1; J <= n; J++) std::swap(AA(K, J), AA(JS[K], J));
    for (int I = 1; I <= n; I++) std::swap(AA(I, K), AA(I, IS[K]));
  }
  return true;
}

}  // namespace ccs

using namespace ccs;

extern "C" int ccs_ghost_map(int N, int halo, int64_t *src_index) {
  if (N < 1 || halo < 1 || !src_index) return CCS_ERR_ARG;
  HArr A{N, halo, N + 2 * halo};
  const size_t n = (size_t)A.nh * A.nh * 6;
  for (size_t k = 0; k < n; k++) src_index[k] = -1;
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) src_index[A.at(i, j, p)] = (int64_t)A.at(i, j, p);
  // derive the forward map from the push table the kernels use
  Layout L = make_layout(N, halo, N + 2 * halo);
  std::vector<int32_t> push;
  if (!build_push_table(L, push)) return CCS_ERR_MESH;
  for (int ps = 1; ps <= 6; ps++)
    for (int s = 0; s < 4; s++)
      for (int k = 1; k <= halo; k++)
        for (int m = 1; m <= N; m++) {
          int i, j;
          switch (s) {
            case 0: i = k; j = m; break;
            case 1: i = N + 1 - k; j = m; break;
            case 2: i = m; j = k; break;
            default: i = m; j = N + 1 - k; break;
          }
          const int32_t dst = push[((size_t)(ps - 1) * 4 + s) * halo * N + (size_t)(k - 1) * N + (m - 1)];
          src_index[dst] = (int64_t)A.at(i, j, ps);  // Layout pitch == nh here
        }
  return CCS_OK;
}

// ---------------------------------------------------------------------------
// Cube-face maps in the face-local frame: face centre at (0,0,1), map coordinates
// X, Y in [-1, 1] along the local x and y axes.  Each returns the unit-sphere
// point and its derivatives with respect to X and Y.
// ---------------------------------------------------------------------------
namespace {

// f(0) .. f(n - 1) on the host's hardware threads (round robin); f must only write
// to the slots its argument owns.
template <class F>
void parallel_for(int n, F &&f) {
  const unsigned hw = std::thread::hardware_concurrency();
  const int nt = (int)std::max(1u, std::min(hw ? hw : 1u, 64u));
  if (nt == 1 || n < 2) {
    for (int r = 0; r < n; r++) f(r);
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; t++)
    pool.emplace_back([&, t]() {
      for (int r = t; r < n; r += nt) f(r);
    });
  for (auto &th : pool) th.join();
}


using cd = std::complex<double>;

// Equiangular gnomonic: angle coordinates (X, Y) * pi/4.
void gnomonic_local(double X, double Y, double P[3], double dX[3], double dY[3]) {
  const double al = X * (kPi / 4.), be = Y * (kPi / 4.);
  const double t = std::tan(al), u = std::tan(be);
  const double rho = std::sqrt(1. + t * t + u * u);
  const double r3 = rho * rho * rho;
  P[0] = t / rho; P[1] = u / rho; P[2] = 1. / rho;
  const double ca = (kPi / 4.) * (1. + t * t), cb = (kPi / 4.) * (1. + u * u);
  dX[0] = ca * (1. + u * u) / r3; dX[1] = -ca * t * u / r3; dX[2] = -ca * t / r3;
  dY[0] = -cb * t * u / r3; dY[1] = cb * (1. + t * t) / r3; dY[2] = -cb * u / r3;
}

// Conformal cubic map (the map of Rancic, Purser and Mesinger 1996 that the
// reference mesh generator evaluates with Purser's series library), built here
// from two automorphic functions of the face's symmetry group:
//   * the flat square S = [-1,1]^2 is tiled by the (2,4,4) reflection group whose
//     automorphic function is J_sq(z) = (wp(z)/e1)^2 = 4 (dn/sn)^4 (K z | m=1/2),
//     wp the Weierstrass function of the lattice 2Z + 2iZ (lemniscatic case);
//   * the spherical face, stereographically projected from the antipode of its
//     centre (w = (x + i y) / (1 + z)), is tiled by the octahedral (2,3,4) group
//     whose automorphic function is Klein's J_oct(w) = P^3 / (108 w^4 (w^4-1)^4),
//     P = w^8 + 14 w^4 + 1.
// Both send face centre -> infinity, edge midpoint -> 1, corner -> 0 and map each
// of the 8 symmetry triangles of a face one-to-one onto a half plane, so the
// conformal map is w = J_oct^-1(J_sq(z)).  J_oct is inverted by Newton's method
// with continuation along the ray from the face centre.

// sn, cn, dn of a real argument u in [0, K] for parameter m (AGM, A&S 16.4); for
// u > K/2 the quarter-period identities keep cn and dn accurate near u = K.
struct Jac { double sn, cn, dn; };
double agm(double a, double b) {
  for (int it = 0; it < 64 && std::fabs(a - b) > 1e-17 * a; it++) {
    const double an = 0.5 * (a + b);
    b = std::sqrt(a * b);
    a = an;
  }
  return 0.5 * (a + b);
}
Jac jac_small(double u, double m) {
  double a[20], c[20];
  a[0] = 1.;
  double b = std::sqrt(1. - m);
  c[0] = std::sqrt(m);
  int n = 0;
  while (std::fabs(c[n]) > 1e-18 && n < 18) {
    const double an = 0.5 * (a[n] + b);
    const double cn = 0.5 * (a[n] - b);
    b = std::sqrt(a[n] * b);
    n++;
    a[n] = an;
    c[n] = cn;
  }
  double phi = std::ldexp(a[n] * u, n);
  for (int k = n; k >= 1; k--) phi = 0.5 * (phi + std::asin(c[k] / a[k] * std::sin(phi)));
  Jac r;
  r.sn = std::sin(phi);
  r.cn = std::cos(phi);
  r.dn = std::sqrt(1. - m * r.sn * r.sn);
  return r;
}
Jac jac(double u, double m, double K) {
  if (u <= 0.5 * K) return jac_small(u, m);
  const Jac v = jac_small(K - u, m);  // sn(K-v) = cd v, cn(K-v) = k' sd v, dn(K-v) = k' nd v
  const double kp = std::sqrt(1. - m);
  return Jac{v.cn / v.dn, kp * v.sn / v.dn, kp / v.dn};
}

struct Conformal {
  double K;   // K(m = 1/2) = K'
  double c1;  // w ~ c1 z at the centre
  cd wc;      // corner of the fundamental triangle, w_c^4 = -7 + 4 sqrt 3
  Conformal() {
    K = kPi / (2. * agm(1., std::sqrt(0.5)));
    c1 = K / std::pow(432., 0.25);
    wc = cd(1., 1.) / (std::sqrt(3.) + 1.);
  }
  // sn, dn, cn of K z for z = x + i y with 0 <= x, y <= 1 (A&S 16.21.1-4)
  void sdc(cd z, cd *sn, cd *cn, cd *dn) const {
    const double m = 0.5;
    const Jac a = jac(K * z.real(), m, K), b = jac(K * z.imag(), 1. - m, K);
    const double den = b.cn * b.cn + m * a.sn * a.sn * b.sn * b.sn;
    *sn = cd(a.sn * b.dn, a.cn * a.dn * b.sn * b.cn) / den;
    *cn = cd(a.cn * b.cn, -a.sn * a.dn * b.sn * b.dn) / den;
    *dn = cd(a.dn * b.cn * b.dn, -m * a.sn * a.cn * b.sn) / den;
  }
  // P(w) = (w - wc)(w + wc)(w^2 + wc^2)(w^4 + 7 + 4 sqrt 3), factored so that the
  // zero at the corner keeps its relative accuracy
  cd P(cd w) const {
    const cd w2 = w * w;
    return (w - wc) * (w + wc) * (w2 + wc * wc) * (w2 * w2 + (7. + 4. * std::sqrt(3.)));
  }
  cd dP(cd w) const {
    const cd w3 = w * w * w;
    return 8. * w3 * w3 * w + 56. * w3;
  }
  cd Dn(cd w) const {
    const cd w4 = w * w * w * w, q = w4 - 1.;
    return 108. * w4 * (q * q) * (q * q);
  }
  cd dDn(cd w) const {
    const cd w3 = w * w * w, w4 = w3 * w, q = w4 - 1.;
    return 432. * w3 * (q * q * q) * (5. * w4 - 1.);
  }
  // solve J_oct(w) = J_sq(z) near w0; returns false if Newton does not converge.
  // Large |t| is solved in the form 1/J (the centre), small |t| as J (the corners).
  bool solve(cd z, cd w0, cd *w_out, cd *fprime) const {
    cd sn, cn, dn;
    sdc(z, &sn, &cn, &dn);
    const cd q = dn / sn;
    const cd q2 = q * q;
    const cd t = 4. * q2 * q2;  // J_sq
    const bool inv = std::abs(t) > 1.;
    const cd rt = inv ? 1. / t : t;
    cd w = w0;
    bool ok = false;
    int polish = -1;  // once |dw| is below 1e-12 |w|, two more steps reach the rounding floor
    for (int it = 0; it < 60; it++) {
      const cd p = P(w), d = Dn(w);
      cd F, dF;
      if (inv) {
        const cd p3 = p * p * p;
        F = d / p3 - rt;
        dF = (dDn(w) * p - 3. * d * dP(w)) / (p3 * p);
      } else {
        F = p * p * p / d - rt;
        dF = (3. * p * p * dP(w) * d - p * p * p * dDn(w)) / (d * d);
      }
      const cd dw = F / dF;
      w -= dw;
      if (!std::isfinite(w.real()) || !std::isfinite(w.imag())) return false;
      if (polish < 0 && std::abs(dw) <= 1e-12 * std::abs(w)) polish = 2;
      if (polish >= 0 && polish-- == 0) {
        ok = true;
        break;
      }
    }
    if (!ok) return false;
    // f'(z) = dJ_sq/dz / dJ_oct/dw, in the same (J or 1/J) form
    const cd p = P(w), d = Dn(w);
    if (inv) {
      const cd dsq = K * sn * sn * sn * cn / (dn * dn * dn * dn * dn);  // d(1/J_sq)/dz
      const cd doc = (dDn(w) * p - 3. * d * dP(w)) / (p * p * p * p);   // d(1/J_oct)/dw
      *fprime = dsq / doc;
    } else {
      const cd dsq = -16. * K * dn * dn * dn * cn / (sn * sn * sn * sn * sn);
      const cd doc = (3. * p * p * dP(w) * d - p * p * p * dDn(w)) / (d * d);
      *fprime = dsq / doc;
    }
    *w_out = w;
    return true;
  }
  // w and f' at z in the fundamental triangle 0 <= Im z <= Re z <= 1 (z != 0)
  bool fundamental(cd z, cd *w, cd *fp) const {
    const cd vmid(1., 0.), vcor(1., 1.);
    double tau = std::min(1., 0.05 / std::abs(z));
    cd cur = tau * z;
    cd wc_ = c1 * cur, fpc;
    if (!solve(cur, wc_, &wc_, &fpc)) return false;
    double h = 0.05;
    int guard = 0;
    while (tau < 1. && guard++ < 100000) {
      const double dv = std::min(std::abs(tau * z - vmid), std::abs(tau * z - vcor));
      const double hmax = std::max(1e-6, 0.25 * dv / std::abs(z));
      double hh = std::min(std::min(h, hmax), 1. - tau);
      const double tn = (1. - tau - hh < 1e-15) ? 1. : tau + hh;
      const cd zn = tn * z;
      const cd pred = wc_ + fpc * (zn - cur);
      cd wn, fpn;
      if (solve(zn, pred, &wn, &fpn) && std::abs(wn - pred) < 0.5 * std::abs(fpc * (zn - cur)) + 1e-14) {
        tau = tn;
        cur = zn;
        wc_ = wn;
        fpc = fpn;
        h = std::min(0.1, 1.5 * hh);
      } else {
        h = 0.5 * hh;
        if (h < 1e-9) return false;
      }
    }
    *w = wc_;
    *fp = fpc;
    return true;
  }
};

// Conformal map at face-local (X, Y): reduce to the fundamental triangle by the
// face's 8 symmetries (the map commutes with them), then map back the point and
// the real 2x2 Jacobian dw/d(X,Y).  `solve_fund` returns w and f' at a point of the
// fundamental triangle (a cache of solved points, or a direct solve).
template <class Fund>
bool conformal_local(const Conformal &C, double X, double Y, double P[3], double dX[3], double dY[3],
                     Fund &&solve_fund) {
  const double sx = X < 0 ? -1. : 1., sy = Y < 0 ? -1. : 1.;
  double a = std::fabs(X), b = std::fabs(Y);
  const bool swap = b > a;
  if (swap) std::swap(a, b);
  double u, v, J[2][2];  // J[r][c] = d(u,v)_r / d(X,Y)_c
  if (a == 0. && b == 0.) {
    u = v = 0.;
    J[0][0] = J[1][1] = C.c1;
    J[0][1] = J[1][0] = 0.;
  } else {
    cd w, fp;
    if (!solve_fund(a, b, &w, &fp)) return false;
    u = w.real();
    v = w.imag();
    J[0][0] = fp.real(); J[0][1] = -fp.imag();
    J[1][0] = fp.imag(); J[1][1] = fp.real();
  }
  if (swap) {  // reflection across the diagonal: M J M with M = [[0,1],[1,0]]
    std::swap(u, v);
    const double t00 = J[1][1], t01 = J[1][0], t10 = J[0][1], t11 = J[0][0];
    J[0][0] = t00; J[0][1] = t01; J[1][0] = t10; J[1][1] = t11;
  }
  // sign flips: M = diag(sx, sy)
  u *= sx;
  v *= sy;
  J[0][1] *= sx * sy;
  J[1][0] *= sx * sy;
  // inverse stereographic projection and its derivatives
  const double r2 = u * u + v * v, D = 1. + r2, D2 = D * D;
  P[0] = 2. * u / D;
  P[1] = 2. * v / D;
  P[2] = (1. - r2) / D;
  const double xu = 2. * (1. + v * v - u * u) / D2, xv = -4. * u * v / D2;
  const double yu = -4. * u * v / D2, yv = 2. * (1. + u * u - v * v) / D2;
  const double zu = -4. * u / D2, zv = -4. * v / D2;
  dX[0] = xu * J[0][0] + xv * J[1][0];
  dX[1] = yu * J[0][0] + yv * J[1][0];
  dX[2] = zu * J[0][0] + zv * J[1][0];
  dY[0] = xu * J[0][1] + xv * J[1][1];
  dY[1] = yu * J[0][1] + yv * J[1][1];
  dY[2] = zu * J[0][1] + zv * J[1][1];
  return true;
}

// global = R_p local with the panel frames of cuco.f90:89-105 (rotp0)
void rotate_panel(int p, const double *v, double *g) {
  switch (p) {
    case 1: g[0] = v[2]; g[1] = v[0]; g[2] = v[1]; break;
    case 2: g[0] = -v[0]; g[1] = v[2]; g[2] = v[1]; break;
    case 3: g[0] = -v[2]; g[1] = -v[0]; g[2] = v[1]; break;
    case 4: g[0] = v[0]; g[1] = -v[2]; g[2] = v[1]; break;
    case 5: g[0] = -v[1]; g[1] = v[0]; g[2] = v[2]; break;
    default: g[0] = v[1]; g[1] = v[0]; g[2] = -v[2]; break;
  }
}

}  // namespace

// Mesh-file samples at the cell centres: map coordinate of cell i is
// xm = ((2i - 1) dx / 2 - 45) * 2/90 with dx = 90/N degrees
// (mesh_generation/src/mesh_mod.f90:44-51); jab = dxc/dxm / 45 / D2R (:164).
extern "C" int ccs_mesh_generate(int N, int map, double *lon_deg, double *lat_deg, double *x, double *y,
                                 double *z, double *jab) {
  if (N < 1 || (map != CCS_MAP_GNOMONIC_EQUIANGULAR && map != CCS_MAP_CONFORMAL) || !lon_deg || !lat_deg || !x ||
      !y || !z || !jab)
    return CCS_ERR_ARG;
  const double dx_deg = 90. / N;
  const double scale = 1. / (45. * kD2R);
  std::vector<double> lp((size_t)N * N * 9);
  Conformal C;
  // cell i and N+1-i sit at opposite X: cache the fundamental-triangle solutions by
  // the pair (max, min) of distances-from-centre indices
  const int half = (N + 1) / 2;
  std::vector<cd> cw((size_t)half * half), cf((size_t)half * half);
  std::vector<char> have((size_t)half * half, 0);
  auto dist_index = [N](int i) { return (std::abs(2 * i - N - 1) - (N % 2 == 0 ? 1 : 0)) / 2; };
  auto local_x = [dx_deg](int i) { return ((2 * i - 1) * dx_deg / 2. - 45.) * (2. / 90.); };
  if (map == CCS_MAP_CONFORMAL) {
    // the fundamental-triangle argument of each key, taken from the first cell (in
    // row order) that needs it, then all keys solved on the host's threads
    std::vector<double> ka((size_t)half * half), kb((size_t)half * half);
    std::vector<size_t> keys;
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        double a = std::fabs(local_x(i)), b = std::fabs(local_x(j));
        if (b > a) std::swap(a, b);
        if (a == 0. && b == 0.) continue;  // the face centre needs no solve
        int ia = dist_index(i), ib = dist_index(j);
        if (ia < ib) std::swap(ia, ib);
        const size_t key = (size_t)ia * half + ib;
        if (have[key]) continue;
        have[key] = 1;
        ka[key] = a;
        kb[key] = b;
        keys.push_back(key);
      }
    std::vector<char> ok(keys.size(), 0);
    parallel_for((int)keys.size(), [&](int n) {
      const size_t key = keys[n];
      ok[n] = C.fundamental(cd(ka[key], kb[key]), &cw[key], &cf[key]) ? 1 : 0;
    });
    for (char o : ok)
      if (!o) return CCS_ERR_MESH;
  }
  std::vector<char> row_ok(N, 1);
  parallel_for(N, [&](int jr) {
    const int j = jr + 1;
    for (int i = 1; i <= N; i++) {
      const double X = local_x(i), Y = local_x(j);
      double *q = &lp[9 * ((size_t)(i - 1) + (size_t)N * (j - 1))];
      if (map == CCS_MAP_GNOMONIC_EQUIANGULAR) {
        gnomonic_local(X, Y, q, q + 3, q + 6);
        continue;
      }
      int ia = dist_index(i), ib = dist_index(j);
      if (ia < ib) std::swap(ia, ib);
      const size_t key = (size_t)ia * half + ib;
      auto fund = [&](double, double, cd *w, cd *fp) {
        *w = cw[key];
        *fp = cf[key];
        return true;
      };
      if (!conformal_local(C, X, Y, q, q + 3, q + 6, fund)) row_ok[jr] = 0;
    }
  });
  for (char o : row_ok)
    if (!o) return CCS_ERR_MESH;
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        const size_t s = (size_t)(i - 1) + (size_t)N * ((size_t)(j - 1) + (size_t)N * (size_t)(p - 1));
        const double *q = &lp[9 * ((size_t)(i - 1) + (size_t)N * (j - 1))];
        double g[3], ga[3], gb[3];
        rotate_panel(p, q, g);
        rotate_panel(p, q + 3, ga);
        rotate_panel(p, q + 6, gb);
        x[s] = g[0];
        y[s] = g[1];
        z[s] = g[2];
        // cart2sph (mesh_generation/src/math_mod.f90:29-38), written in degrees
        lon_deg[s] = std::atan2(g[1], g[0]) * kR2D;
        lat_deg[s] = std::atan2(g[2], std::sqrt(g[0] * g[0] + g[1] * g[1])) * kR2D;
        for (int r = 0; r < 3; r++) {
          jab[6 * s + r] = ga[r] * scale;
          jab[6 * s + 3 + r] = gb[r] * scale;
        }
      }
  return CCS_OK;
}

// io_mod.F90:119-220 and 295-306.
static int mesh_derive(int N, int halo, double radius, double omega, int flags, const double *lon_deg,
                       const double *lat_deg, const double *xc, const double *yc, const double *zc,
                       const double *jab_c, double *sqrtG, double *G, double *IG, double *A, double *IA, double *f,
                       double *lon_out, double *lat_out, double *sinlat_out, double *coslat_out);

extern "C" int ccs_mesh_derive(int N, int halo, double radius, double omega, const double *lon_deg,
                               const double *lat_deg, const double *xc, const double *yc, const double *zc,
                               const double *jab_c, double *sqrtG, double *G, double *IG, double *A, double *IA,
                               double *f, double *lon_out, double *lat_out, double *sinlat_out,
                               double *coslat_out) {
  return mesh_derive(N, halo, radius, omega, 0, lon_deg, lat_deg, xc, yc, zc, jab_c, sqrtG, G, IG, A, IA, f,
                     lon_out, lat_out, sinlat_out, coslat_out);
}

extern "C" int ccs_mesh_derive_ex(int N, int halo, double radius, double omega, int flags,
                                  const double *lon_deg, const double *lat_deg, const double *xc,
                                  const double *yc, const double *zc, const double *jab_c, double *sqrtG,
                                  double *G, double *IG, double *A, double *IA, double *f, double *lon_out,
                                  double *lat_out, double *sinlat_out, double *coslat_out) {
  if (flags & ~CCS_MESH_POLE_INVERSE) return CCS_ERR_ARG;
  return mesh_derive(N, halo, radius, omega, flags, lon_deg, lat_deg, xc, yc, zc, jab_c, sqrtG, G, IG, A, IA, f,
                     lon_out, lat_out, sinlat_out, coslat_out);
}

static int mesh_derive(int N, int halo, double radius, double omega, int flags, const double *lon_deg,
                       const double *lat_deg, const double *xc, const double *yc, const double *zc,
                       const double *jab_c, double *sqrtG, double *G, double *IG, double *A, double *IA, double *f,
                       double *lon_out, double *lat_out, double *sinlat_out, double *coslat_out) {
  if (N < 1 || halo < 1 || !lon_deg || !lat_deg || !xc || !yc || !zc || !jab_c || !sqrtG || !G || !IG || !A ||
      !IA || !f)
    return CCS_ERR_ARG;
  const int h = halo;
  HArr H{N, h, N + 2 * h};
  const size_t nc = (size_t)H.nh * H.nh * 6;
  std::vector<double> lon(nc, kFillValue), lat(nc, kFillValue), x(nc, 0.), y(nc, 0.), z(nc, 0.);
  std::vector<double> sinlon(nc), coslon(nc), sinlat(nc), coslat(nc), jab(6 * nc, 0.);
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        const size_t s = (size_t)(i - 1) + (size_t)N * ((size_t)(j - 1) + (size_t)N * (size_t)(p - 1));
        const size_t d = H.at(i, j, p);
        lon[d] = lon_deg[s] * kD2R;
        lat[d] = lat_deg[s] * kD2R;
        x[d] = xc[s] * radius;
        y[d] = yc[s] * radius;
        z[d] = zc[s] * radius;
        for (int q = 0; q < 6; q++) jab[6 * d + q] = jab_c[6 * s + q] * radius;
      }
  for (size_t k = 0; k < nc; k++) {
    sinlon[k] = std::sin(lon[k]);
    coslon[k] = std::cos(lon[k]);
    sinlat[k] = std::sin(lat[k]);
    coslat[k] = std::cos(lat[k]);
  }
  for (double *fld : {lon.data(), lat.data(), x.data(), y.data(), z.data(), sinlon.data(), coslon.data(),
                      sinlat.data(), coslat.data()})
    fill_halo_host(N, h, fld, 1, 0);
  fill_jab_host(N, h, jab.data());
  std::memset(sqrtG, 0, nc * sizeof(double));
  std::memset(G, 0, 4 * nc * sizeof(double));
  std::memset(IG, 0, 4 * nc * sizeof(double));
  std::memset(A, 0, 4 * nc * sizeof(double));
  std::memset(IA, 0, 4 * nc * sizeof(double));
  std::memset(f, 0, nc * sizeof(double));
  for (int p = 1; p <= 6; p++)
    for (int j = 1 - h; j <= N + h; j++)
      for (int i = 1 - h; i <= N + h; i++) {
        const size_t d = H.at(i, j, p);
        const double lo = lon[d], la = lat[d];
        if (!(lo != kFillValue && la != kFillValue)) continue;
        const double *J = &jab[6 * d];
        double S[6];
        S[0] = -std::sin(lo);
        S[1] = -std::cos(lo) * std::sin(la);
        S[2] = std::cos(lo);
        S[3] = -std::sin(lo) * std::sin(la);
        S[4] = 0.;
        S[5] = std::cos(la);
        double *g = &G[4 * d], *ig = &IG[4 * d], *a = &A[4 * d], *ia = &IA[4 * d];
        for (int c = 0; c < 2; c++)
          for (int r = 0; r < 2; r++) {
            double s = 0.;
            for (int k = 0; k < 3; k++) s = s + J[k + 3 * r] * J[k + 3 * c];
            g[r + 2 * c] = s;
          }
        if (!brinv2(g, ig)) return CCS_ERR_MESH;
        sqrtG[d] = std::sqrt(g[0] * g[3] - g[1] * g[2]);
        for (int c = 0; c < 2; c++)
          for (int r = 0; r < 2; r++) {
            double s = 0.;
            for (int k = 0; k < 3; k++) s = s + S[r + 2 * k] * J[k + 3 * c];
            a[r + 2 * c] = s;
          }
        if (std::fabs(la * kR2D) != 90 || (flags & CCS_MESH_POLE_INVERSE)) {
          if (!brinv2(a, ia)) return CCS_ERR_MESH;
        } else {
          double IA1[4];
          if (la * kR2D == 90) {
            IA1[0] = std::cos(lo); IA1[2] = -std::sin(lo); IA1[1] = std::sin(lo); IA1[3] = std::cos(lo);
          } else {
            IA1[0] = -std::cos(lo); IA1[2] = std::sin(lo); IA1[1] = std::sin(lo); IA1[3] = std::cos(lo);
          }
          const double I2[4] = {1., 0., 0., 1.};
          for (int c = 0; c < 2; c++)
            for (int r = 0; r < 2; r++) {
              double s = 0.;
              for (int k = 0; k < 2; k++) s = s + I2[r + 2 * k] * IA1[k + 2 * c];
              ia[r + 2 * c] = s * radius;
            }
        }
      }
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) f[H.at(i, j, p)] = 2. * omega * sinlat[H.at(i, j, p)];
  if (lon_out) std::memcpy(lon_out, lon.data(), nc * sizeof(double));
  if (lat_out) std::memcpy(lat_out, lat.data(), nc * sizeof(double));
  if (sinlat_out) std::memcpy(sinlat_out, sinlat.data(), nc * sizeof(double));
  if (coslat_out) std::memcpy(coslat_out, coslat.data(), nc * sizeof(double));
  return CCS_OK;
}

// ---------------------------------------------------------------------------
// Initial states
// ---------------------------------------------------------------------------
namespace {

struct Rng {  // splitmix64 + Box-Muller: identical streams on every platform
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double normal() {
    const double u1 = uniform(), u2 = uniform();
    return std::sqrt(-2. * std::log(u1)) * std::cos(2. * kPi * u2);
  }
};

// Real spherical-harmonic series sum_{l=1..L} sum_{m=0..l} Pbar_lm(sin lat) *
// (a_lm cos(m lon) + b_lm sin(m lon)), Pbar fully normalised, a,b ~ N(0,1) l^-2.
struct ShField {
  int L;
  std::vector<double> a, b;  // index l*(L+1)+m
  void draw(int lmax, Rng &rng) {
    L = lmax;
    a.assign((size_t)(L + 1) * (L + 1), 0.);
    b.assign((size_t)(L + 1) * (L + 1), 0.);
    for (int l = 1; l <= L; l++)
      for (int m = 0; m <= l; m++) {
        const double s = 1. / ((double)l * l);
        a[l * (L + 1) + m] = rng.normal() * s;
        b[l * (L + 1) + m] = m == 0 ? 0. : rng.normal() * s;
      }
  }
  // value and d/dlon at (lon, lat)
  void eval(double lon, double lat, double *val, double *dlon) const {
    const double mu = std::sin(lat), cl = std::cos(lat);
    thread_local std::vector<double> P;
    P.assign((size_t)(L + 1) * (L + 1), 0.);
    auto at = [&](int l, int m) -> double & { return P[(size_t)l * (L + 1) + m]; };
    at(0, 0) = 1.;
    for (int m = 1; m <= L; m++) at(m, m) = std::sqrt((2. * m + 1.) / (2. * m)) * cl * at(m - 1, m - 1);
    if (L >= 1) at(1, 1) = std::sqrt(3.) * cl;
    for (int m = 0; m < L; m++) at(m + 1, m) = std::sqrt(2. * m + 3.) * mu * at(m, m);
    for (int m = 0; m <= L; m++)
      for (int l = m + 2; l <= L; l++) {
        const double al = std::sqrt((4. * l * l - 1.) / ((double)l * l - (double)m * m));
        const double bl = std::sqrt(((l - 1.) * (l - 1.) - (double)m * m) / (4. * (l - 1.) * (l - 1.) - 1.));
        at(l, m) = al * (mu * at(l - 1, m) - bl * at(l - 2, m));
      }
    double v = 0., dv = 0.;
    for (int l = 1; l <= L; l++)
      for (int m = 0; m <= l; m++) {
        const double c = std::cos(m * lon), s = std::sin(m * lon);
        const double A = a[l * (L + 1) + m], B = b[l * (L + 1) + m];
        v += at(l, m) * (A * c + B * s);
        dv += at(l, m) * m * (-A * s + B * c);
      }
    *val = v;
    *dlon = dv;
  }
};

}  // namespace

extern "C" int ccs_initial_condition(int N, int halo, double radius, double gravity, double omega,
                                     const ccs_ic_params *prm, const double *lon, const double *lat,
                                     const double *sinlat, const double *coslat, double *phi, double *zonal,
                                     double *merid, double *phis) {
  if (N < 1 || halo < 1 || !prm || !lon || !lat || !sinlat || !coslat || !phi || !zonal || !merid || !phis)
    return CCS_ERR_ARG;
  HArr H{N, halo, N + 2 * halo};
  const size_t nc = (size_t)H.nh * H.nh * 6;
  const double pi = kPi;
  if (prm->kind == CCS_IC_CASE2) {
    // test_case_mod.F90:61-95
    const double gh0 = 29400.;
    const double u0 = 2. * pi * radius / (12. * 86400.);
    for (size_t k = 0; k < nc; k++) {
      phi[k] = gh0 - (radius * omega * u0 + u0 * u0 / 2.) * (sinlat[k] * sinlat[k]);
      zonal[k] = u0 * coslat[k];
      merid[k] = 0.;
      phis[k] = 0.;
    }
    return CCS_OK;
  }
  if (prm->kind == CCS_IC_CASE5) {
    // test_case_mod.F90:98-144
    const double hs0 = 2000., u0 = 20., alpha = 0., gh0 = 5960. * gravity;
    const double rr = pi / 9., lc = 1.5 * pi, tc = pi / 6.;
    for (size_t k = 0; k < nc; k++) {
      double lo = lon[k];
      const double la = lat[k];
      if (lo < 0) lo = 2. * pi + lo;
      const double dl = lo - lc, dt = la - tc;
      double r2 = dl * dl + dt * dt;
      if (rr * rr < r2) r2 = rr * rr;
      const double r = std::sqrt(r2);
      const double ghs = gravity * hs0 * (1. - r / rr);
      zonal[k] = u0 * (std::cos(la) * std::cos(alpha) + std::cos(lo) * std::sin(la) * std::sin(alpha));
      merid[k] = -u0 * std::sin(lo) * std::sin(alpha);
      const double t = -std::cos(lo) * std::cos(la) * std::sin(alpha) + std::sin(la) * std::cos(alpha);
      phi[k] = gh0 - (radius * omega * u0 + u0 * u0 / 2.) * (t * t) - ghs;
      phis[k] = ghs;
    }
    return CCS_OK;
  }
  if (prm->kind == CCS_IC_CASE6) {
    // test_case_mod.F90:147-204
    const double omg = 7.848e-6, R = 4., h0 = 8000.;
    for (size_t k = 0; k < nc; k++) {
      const double cl = coslat[k], sl = sinlat[k], lo = lon[k];
      const double u1 = cl, u2 = R * std::pow(cl, R - 1) * sl * sl * std::cos(R * lo);
      const double u3 = std::pow(cl, R + 1) * std::cos(R * lo);
      zonal[k] = radius * omg * (u1 + u2 - u3);
      merid[k] = -radius * omg * R * std::pow(cl, R - 1) * sl * std::sin(R * lo);
      const double AA1 = omg * 0.5 * (2. * omega + omg) * cl * cl;
      const double Ac = 0.25 * omg * omg;
      const double A21 = (R + 1.) * std::pow(cl, 2. * R + 2.);
      const double A22 = (2. * R * R - R - 2.) * std::pow(cl, 2. * R);
      const double A23 = 2. * R * R * std::pow(cl, 2. * R - 2);
      const double Ah = AA1 + Ac * (A21 + A22 - A23);
      const double Bc = 2. * (omega + omg) * omg / ((R + 1) * (R + 2)) * std::pow(cl, R);
      const double Bh = Bc * ((R * R + 2. * R + 2.) - (R + 1.) * (R + 1.) * cl * cl);
      const double CC = 0.25 * omg * omg * std::pow(cl, 2. * R);
      const double Ch = CC * ((R + 1.) * cl * cl - (R + 2.));
      phi[k] = gravity * h0 + radius * radius * (Ah + Bh * std::cos(R * lo) + Ch * std::cos(2.0 * R * lo));
      phis[k] = 0.;
    }
    return CCS_OK;
  }
  if (prm->kind != CCS_IC_SEEDED) return CCS_ERR_ARG;
  // Seeded state: h = h0 + SH perturbation (degrees 1..lmax_h, amplitude ~ l^-2,
  // scaled to h_rms RMS over the interior cells); winds non-divergent from an
  // independent streamfunction scaled to wind_max maximum interior speed;
  // orography from a third field (degrees 1..lmax_oro) scaled to oro_rms RMS and
  // clipped to [0, oro_max].  Corner blocks are set to 0.
  Rng rng{prm->seed * 0x2545F4914F6CDD1Dull + 0x1234567ull};
  ShField fh, fpsi, foro;
  fh.draw(prm->lmax_h > 0 ? prm->lmax_h : 12, rng);
  fpsi.draw(prm->lmax_psi > 0 ? prm->lmax_psi : 12, rng);
  const bool oro = prm->lmax_oro > 0;
  if (oro) foro.draw(prm->lmax_oro, rng);
  std::vector<double> hp(nc, 0.), us(nc, 0.), vs(nc, 0.), hs(nc, 0.);
  std::vector<char> live(nc, 0);
  // every cell's values depend on its own lon/lat only: the rows are shared out
  // among host threads (the reductions below stay sequential and in order)
  const int nrows = 6 * (N + 2 * halo);
  parallel_for(nrows, [&](int row) {
    const int p = 1 + row / (N + 2 * halo), j = 1 - halo + row % (N + 2 * halo);
    for (int i = 1 - halo; i <= N + halo; i++) {
      const bool ci = i < 1 || i > N, cj = j < 1 || j > N;
      if (ci && cj) continue;  // corner block
      const size_t k = H.at(i, j, p);
      live[k] = 1;
      double v, d;
      fh.eval(lon[k], lat[k], &v, &d);
      hp[k] = v;
      // u = -(1/a) dpsi/dlat (central difference, step 1e-5 rad); v = dpsi/dlon / (a cos lat)
      const double dl = 1e-5;
      double pp, pm, dd;
      fpsi.eval(lon[k], lat[k] + dl, &pp, &dd);
      fpsi.eval(lon[k], lat[k] - dl, &pm, &dd);
      double pc, dlon;
      fpsi.eval(lon[k], lat[k], &pc, &dlon);
      us[k] = -(pp - pm) / (2. * dl);
      vs[k] = dlon / std::cos(lat[k]);
      if (oro) {
        foro.eval(lon[k], lat[k], &v, &d);
        hs[k] = v;
      }
    }
  });
  double s2 = 0., vmax = 0., o2 = 0.;
  size_t cnt = 0;
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        const size_t k = H.at(i, j, p);
        s2 += hp[k] * hp[k];
        o2 += hs[k] * hs[k];
        const double sp = std::sqrt(us[k] * us[k] + vs[k] * vs[k]);
        if (sp > vmax) vmax = sp;
        cnt++;
      }
  const double hscale = s2 > 0 ? prm->h_rms / std::sqrt(s2 / cnt) : 0.;
  const double wscale = vmax > 0 ? prm->wind_max / vmax : 0.;
  const double oscale = o2 > 0 ? prm->oro_rms / std::sqrt(o2 / cnt) : 0.;
  for (size_t k = 0; k < nc; k++) {
    if (!live[k]) {
      phi[k] = 0.;
      zonal[k] = 0.;
      merid[k] = 0.;
      phis[k] = 0.;
      continue;
    }
    double ho = oro ? hs[k] * oscale : 0.;
    if (ho < 0.) ho = 0.;
    if (ho > prm->oro_max) ho = prm->oro_max;
    phis[k] = gravity * ho;
    phi[k] = gravity * (prm->h0 + hp[k] * hscale);
    zonal[k] = us[k] * wscale;
    merid[k] = vs[k] * wscale;
  }
  return CCS_OK;
}

extern "C" int ccs_state_from_sphere(int N, int halo, const ccs_mesh_view *m, ccs_state_view *s) {
  if (N < 1 || halo < 1 || !m || !s || !m->sqrtG || !m->matrixG || !m->matrixIA || !s->phi || !s->zonal_wind ||
      !s->meridional_wind || !s->phiG || !s->u || !s->v || !s->uC || !s->vC)
    return CCS_ERR_ARG;
  const size_t nc = (size_t)(N + 2 * halo) * (N + 2 * halo) * 6;
  for (size_t k = 0; k < nc; k++) s->phiG[k] = s->phi[k] * m->sqrtG[k];
  for (size_t k = 0; k < nc; k++) {
    const double *G = &m->matrixG[4 * k], *IA = &m->matrixIA[4 * k];
    double M[4];
    for (int c = 0; c < 2; c++)
      for (int r = 0; r < 2; r++) {
        double acc = 0.;
        for (int q = 0; q < 2; q++) acc = acc + G[r + 2 * q] * IA[q + 2 * c];
        M[r + 2 * c] = acc;
      }
    const double sv1 = s->zonal_wind[k], sv2 = s->meridional_wind[k];
    s->u[k] = M[0] * sv1 + M[2] * sv2;
    s->v[k] = M[1] * sv1 + M[3] * sv2;
    s->uC[k] = IA[0] * sv1 + IA[2] * sv2;
    s->vC[k] = IA[1] * sv1 + IA[3] * sv2;
  }
  return CCS_OK;
}

extern "C" double ccs_cfl_dt(int N, int halo, double cfl, double dx, double dy, const ccs_mesh_view *m,
                             const ccs_state_view *s) {
  if (N < 1 || halo < 1 || !m || !s) return -1.;
  HArr H{N, halo, N + 2 * halo};
  double lmax = 0.;
  for (int p = 1; p <= 6; p++)
    for (int j = 0; j <= N + 1; j++)
      for (int i = 0; i <= N + 1; i++) {
        if ((i < 1 || i > N) && (j < 1 || j > N)) continue;
        const size_t k = H.at(i, j, p);
        const double pt = s->phi[k] + m->phis[k];
        if (!(pt > 0.)) return -1.;
        const double lx = std::fabs(s->uC[k]) + std::sqrt(m->matrixIG[4 * k] * pt);
        const double ly = std::fabs(s->vC[k]) + std::sqrt(m->matrixIG[4 * k + 3] * pt);
        if (lx > lmax) lmax = lx;
        if (ly > lmax) lmax = ly;
      }
  if (!(lmax > 0.)) return -1.;
  return cfl * (dx < dy ? dx : dy) / lmax;
}

// ---- raw-binary mesh file --------------------------------------------------------
// A stand-in for the NetCDF mesh file of mesh_generation/src/output_mod.f90:25-86 and
// read_mesh (io_mod.F90:36-101), for machines without libnetcdf.  It holds the
// global attributes read_mesh reads (dx, dy in degrees; ids, ide, jds, jde, ifs,
// ife) and the cell-centre samples of lon, lat, x, y, z and jab that the time step
// uses, little-endian, Fortran order:
//   bytes  0-7   magic "CCSMESH" + '\1'
//          8-47  int32 version (1), N, map, ids, ide, jds, jde, ifs, ife, reserved (0)
//         48-63  float64 dx, dy (degrees)
//         64-    float64 lon, lat, x, y, z (N, N, 6) then jab (3, 2, N, N, 6)
namespace {

const char kMeshMagic[8] = {'C', 'C', 'S', 'M', 'E', 'S', 'H', '\1'};
constexpr int kMeshHeader = 64;

struct MeshHeader {
  int32_t version, N, map, ids, ide, jds, jde, ifs, ife, reserved;
  double dx, dy;
};

int read_mesh_header(FILE *fp, MeshHeader *hd) {
  char magic[8];
  if (fread(magic, 1, 8, fp) != 8 || std::memcmp(magic, kMeshMagic, 8) != 0) return CCS_ERR_IO;
  int32_t iv[10];
  double dv[2];
  if (fread(iv, sizeof(int32_t), 10, fp) != 10 || fread(dv, sizeof(double), 2, fp) != 2) return CCS_ERR_IO;
  hd->version = iv[0]; hd->N = iv[1]; hd->map = iv[2];
  hd->ids = iv[3]; hd->ide = iv[4]; hd->jds = iv[5]; hd->jde = iv[6]; hd->ifs = iv[7]; hd->ife = iv[8];
  hd->reserved = iv[9];
  hd->dx = dv[0]; hd->dy = dv[1];
  // version 1 only; the index attributes must describe the (2N+1)^2 x 6 grid
  if (hd->version != 1 || hd->N < 1 || hd->N > 8192) return CCS_ERR_IO;
  if (hd->ids != 1 || hd->jds != 1 || hd->ide != 2 * hd->N + 1 || hd->jde != 2 * hd->N + 1 || hd->ifs != 1 ||
      hd->ife != 6)
    return CCS_ERR_IO;
  return CCS_OK;
}

}  // namespace

extern "C" int ccs_mesh_save(const char *path, int N, int map, const double *lon_deg, const double *lat_deg,
                             const double *x, const double *y, const double *z, const double *jab) {
  if (!path || N < 1 || N > 8192 || !lon_deg || !lat_deg || !x || !y || !z || !jab) return CCS_ERR_ARG;
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return CCS_ERR_IO;
  const int32_t iv[10] = {1, N, map, 1, 2 * N + 1, 1, 2 * N + 1, 1, 6, 0};
  const double dv[2] = {90. / N, 90. / N};
  const size_t n = (size_t)N * N * 6;
  bool ok = std::fwrite(kMeshMagic, 1, 8, fp) == 8 && std::fwrite(iv, sizeof(int32_t), 10, fp) == 10 &&
            std::fwrite(dv, sizeof(double), 2, fp) == 2;
  const double *arr[5] = {lon_deg, lat_deg, x, y, z};
  for (int k = 0; k < 5 && ok; k++) ok = std::fwrite(arr[k], sizeof(double), n, fp) == n;
  if (ok) ok = std::fwrite(jab, sizeof(double), 6 * n, fp) == 6 * n;
  if (std::fclose(fp) != 0) ok = false;
  return ok ? CCS_OK : CCS_ERR_IO;
}

extern "C" int ccs_mesh_file_info(const char *path, int *N, int *map) {
  if (!path || !N) return CCS_ERR_ARG;
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return CCS_ERR_IO;
  MeshHeader hd{};
  const int rc = read_mesh_header(fp, &hd);
  std::fclose(fp);
  if (rc) return rc;
  *N = hd.N;
  if (map) *map = hd.map;
  return CCS_OK;
}

extern "C" int ccs_mesh_load(const char *path, int N, double *lon_deg, double *lat_deg, double *x, double *y,
                             double *z, double *jab) {
  if (!path || N < 1 || !lon_deg || !lat_deg || !x || !y || !z || !jab) return CCS_ERR_ARG;
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return CCS_ERR_IO;
  MeshHeader hd{};
  int rc = read_mesh_header(fp, &hd);
  if (!rc && hd.N != N) rc = CCS_ERR_ARG;
  if (!rc && std::fseek(fp, kMeshHeader, SEEK_SET) != 0) rc = CCS_ERR_IO;
  const size_t n = (size_t)N * N * 6;
  double *arr[5] = {lon_deg, lat_deg, x, y, z};
  for (int k = 0; k < 5 && !rc; k++)
    if (std::fread(arr[k], sizeof(double), n, fp) != n) rc = CCS_ERR_IO;
  if (!rc && std::fread(jab, sizeof(double), 6 * n, fp) != 6 * n) rc = CCS_ERR_IO;
  if (!rc && std::fgetc(fp) != EOF) rc = CCS_ERR_IO;  // trailing bytes: not this format
  std::fclose(fp);
  return rc;
}

// ---- checkpoint files -------------------------------------------------------------
// The reference writes NetCDF history only and has no restart reader.  A checkpoint
// here is the eight stat fields in the reference's layout behind a small header:
//   bytes 0-7   magic "CCSSTAT" + '\1'
//         8-23  int32 version (1), N, halo, number of fields (8)
//        24-    float64 phiG, u, v, phi, uC, vC, zonal, meridional ((N+2h)^2 * 6 each)
namespace {
const char kStateMagic[8] = {'C', 'C', 'S', 'S', 'T', 'A', 'T', '\1'};
}  // namespace

extern "C" int ccs_state_write(const char *path, int N, int halo, const ccs_state_view *s) {
  if (!path || N < 1 || halo < 1 || !s || !s->phiG || !s->u || !s->v || !s->phi || !s->uC || !s->vC ||
      !s->zonal_wind || !s->meridional_wind)
    return CCS_ERR_ARG;
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return CCS_ERR_IO;
  const size_t n = (size_t)(N + 2 * halo) * (N + 2 * halo) * 6;
  const int32_t iv[4] = {1, N, halo, 8};
  bool ok = std::fwrite(kStateMagic, 1, 8, fp) == 8 && std::fwrite(iv, sizeof(int32_t), 4, fp) == 4;
  const double *f[8] = {s->phiG, s->u, s->v, s->phi, s->uC, s->vC, s->zonal_wind, s->meridional_wind};
  for (int k = 0; k < 8 && ok; k++) ok = std::fwrite(f[k], sizeof(double), n, fp) == n;
  if (std::fclose(fp) != 0) ok = false;
  return ok ? CCS_OK : CCS_ERR_IO;
}

extern "C" int ccs_state_read(const char *path, int N, int halo, ccs_state_view *s) {
  if (!path || N < 1 || halo < 1 || !s || !s->phiG || !s->u || !s->v || !s->phi || !s->uC || !s->vC ||
      !s->zonal_wind || !s->meridional_wind)
    return CCS_ERR_ARG;
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return CCS_ERR_IO;
  char magic[8];
  int32_t iv[4];
  int rc = CCS_OK;
  if (std::fread(magic, 1, 8, fp) != 8 || std::memcmp(magic, kStateMagic, 8) != 0 ||
      std::fread(iv, sizeof(int32_t), 4, fp) != 4 || iv[0] != 1 || iv[3] != 8)
    rc = CCS_ERR_IO;
  else if (iv[1] != N || iv[2] != halo)
    rc = CCS_ERR_ARG;
  const size_t n = (size_t)(N + 2 * halo) * (N + 2 * halo) * 6;
  double *f[8] = {s->phiG, s->u, s->v, s->phi, s->uC, s->vC, s->zonal_wind, s->meridional_wind};
  for (int k = 0; k < 8 && !rc; k++)
    if (std::fread(f[k], sizeof(double), n, fp) != n) rc = CCS_ERR_IO;
  if (!rc && std::fgetc(fp) != EOF) rc = CCS_ERR_IO;
  std::fclose(fp);
  return rc;
}
