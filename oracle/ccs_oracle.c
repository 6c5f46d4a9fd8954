/*
 * ccs_oracle.c -- CPU FP64 restatement of the reference shallow-water step on the
 * conformal cubed sphere (DwyaneChou/Conformal_Cubed_Sphere, Fortran 90).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The
 * product path never calls it.
 *
 * PARITY UNPINNED: the reference is Fortran with a NetCDF dependency and has no
 * tests, fixtures or golden vectors; no Fortran compiler exists on the build or GPU
 * machines, so the restatement cannot be diffed against the reference binary.  It
 * is pinned instead by known-answer tests written against the reference source
 * (WENO on polynomials, ghost-map round trips, projection round trips, the steady
 * zonal flow of test case 2, the sphere-area check of read_mesh).
 *
 * Every routine follows the Fortran source operation by operation, left to right,
 * with no contraction (build with -ffp-contract=off): the reference is built with
 * -fdefault-real-8 and, on x86-64 without -march, gfortran emits no FMA.
 *
 * The spatial operator is the WENO-Z/Rusanov one of spatial_operators_mod.F90 by
 * default; orc_set_operator selects the central-difference modules
 * spatial_operators_mod_{2nd,4th,6th}.F90 instead (the reference picks one of them
 * at build time).
 *
 * Array layout is the reference's: Fortran column-major (i, j, panel) with
 * i, j in [1-h, N+h], panel in [1, 6]; 2x2 matrices (2,2,i,j,panel); the Jacobian
 * (3,2,i,j,panel); extended face arrays (2N+1, 2N+1, 6).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_FILL_VALUE (-9999999999999999.)

/* constants_mod.F90:6-12 (pi = 2*asin(1), D2R = pi/180, R2D = 180/pi) */
static const double ORC_PI = 3.14159265358979323846;
#define ORC_D2R (ORC_PI / 180.)
#define ORC_R2D (180. / ORC_PI)

typedef struct {
  double *phiG, *u, *v, *phi, *uC, *vC, *zonal, *merid, *phit;
} orc_state;

typedef struct {
  double *phiG, *u, *v;
} orc_tend;

typedef struct orc_ctx {
  int N, h, nh, ne;
  size_t ncell, next;
  double dx, dy;
  int e_diss; /* 0: never-written u/v face slots read as 0.0; 1: reconstructed */
  int op;     /* spatial operator: 0 WENO-Z/Rusanov, 2/4/6 central differences */
  /* mesh (owned copies) */
  double *sqrtG, *G, *IG, *A, *IA, *f, *phis;
  /* stat(-4:1), tend(-4:1): index = slot + 4 */
  orc_state stat[6];
  orc_tend tend[6];
  /* spatial_operator automatic arrays (spatial_operators_mod.F90:17-55) */
  double *E, *K, *flux_x, *flux_y, *vort, *phit, *phitG;
  double *dfluxdx, *dfluxdy, *dEdx, *dEdy, *dvdx, *dudy;
  double *fx_p, *fx_n, *fy_p, *fy_n, *E_p, *E_n, *pG_p, *pG_n, *ptG_p, *ptG_n;
  double *u_p, *u_n, *v_p, *v_n;
  double *fx_ext, *fy_ext, *E_ext, *pG_ext, *u_ext, *v_ext;
  /* fill_halo scratch */
  double *inner;
} orc_ctx;

/* Fortran index helpers: cell arrays (ics:ice, jcs:jce, 1:6) */
static inline size_t CI(const orc_ctx *c, int i, int j, int p) {
  return (size_t)(i - (1 - c->h)) + (size_t)c->nh * ((size_t)(j - (1 - c->h)) + (size_t)c->nh * (size_t)(p - 1));
}
/* extended arrays (ids:ide, jds:jde, 1:6) with ids = jds = 1 */
static inline size_t EI(const orc_ctx *c, int ie, int je, int p) {
  return (size_t)(ie - 1) + (size_t)c->ne * ((size_t)(je - 1) + (size_t)c->ne * (size_t)(p - 1));
}
/* 2x2 matrix element (r, col) of cell (i, j, p) */
static inline size_t MI(const orc_ctx *c, int r, int col, int i, int j, int p) {
  return (size_t)(r - 1) + 2 * (size_t)(col - 1) + 4 * CI(c, i, j, p);
}

static double *dalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* WENO_limiter: spatial_operators_mod.F90:282-361 (WENO-Z, eps = 1e-2,       */
/* linear weights (0.1, 0.6, 0.3), two hard branch switches).                 */
/* ------------------------------------------------------------------------- */
static inline double weno_limiter(const double Q[5], int dir) {
  const double weno_coef[3] = {0.1, 0.6, 0.3};
  const double eps = 1.E-2;
  const double Qim2 = Q[0], Qim1 = Q[1], Qi = Q[2], Qip1 = Q[3], Qip2 = Q[4];
  double st[3], cA[3], cB[3], beta[3], omega[3];
  if (dir > 0) {
    st[0] = Qim2 / 3. - 7. / 6. * Qim1 + 11. / 6. * Qi;
    st[1] = -Qim1 / 6. + 5. / 6. * Qi + 1. / 3. * Qip1;
    st[2] = Qi / 3. + 5. / 6. * Qip1 - 1. / 6. * Qip2;
    cA[0] = Qim2 - 2. * Qim1 + Qi;
    cA[1] = Qim1 - 2. * Qi + Qip1;
    cA[2] = Qi - 2. * Qip1 + Qip2;
    cB[0] = Qim2 - 4. * Qim1 + 3. * Qi;
    cB[1] = Qim1 - Qip1;
    cB[2] = 3. * Qi - 4. * Qip1 + Qip2;
  } else {
    st[0] = Qip2 / 3. - 7. / 6. * Qip1 + 11. / 6. * Qi;
    st[1] = -Qip1 / 6. + 5. / 6. * Qi + 1. / 3. * Qim1;
    st[2] = Qi / 3. + 5. / 6. * Qim1 - 1. / 6. * Qim2;
    cA[0] = Qip2 - 2. * Qip1 + Qi;
    cA[1] = Qip1 - 2. * Qi + Qim1;
    cA[2] = Qi - 2. * Qim1 + Qim2;
    cB[0] = Qip2 - 4. * Qip1 + 3. * Qi;
    cB[1] = Qip1 - Qim1;
    cB[2] = 3. * Qi - 4. * Qim1 + Qim2;
  }
  for (int k = 0; k < 3; k++) beta[k] = cA[k] * cA[k] * 13. / 12. + cB[k] * cB[k] * 0.25;
  const double tau40 = fabs(beta[0] - beta[1]);
  const double tau41 = fabs(beta[1] - beta[2]);
  const double tau5 = fabs(beta[2] - beta[0]);
  double mn = beta[0];
  if (beta[1] < mn) mn = beta[1];
  if (beta[2] < mn) mn = beta[2];
  if (tau40 <= mn && tau41 > mn) {
    omega[0] = 1. / 3.; omega[1] = 2. / 3.; omega[2] = 0.;
  } else if (tau40 > mn && tau41 < mn) {
    omega[0] = 0.; omega[1] = 2. / 3.; omega[2] = 1. / 3.;
  } else {
    double alpha[3];
    for (int k = 0; k < 3; k++) alpha[k] = weno_coef[k] * (1. + tau5 / (eps + beta[k]));
    double s = 0.;
    for (int k = 0; k < 3; k++) s = s + alpha[k];
    for (int k = 0; k < 3; k++) omega[k] = alpha[k] / s;
  }
  double q = 0.;
  for (int k = 0; k < 3; k++) q = q + st[k] * omega[k];
  return q;
}

double orc_weno_limiter(const double *Q, int dir) { return weno_limiter(Q, dir); }

/* weno sweep driver: spatial_operators_mod.F90:183-277 */
static void weno_sweep(const orc_ctx *c, double *fext, const double *field, int flux_dir, int axis) {
  const int N = c->N;
  for (int p = 1; p <= 6; p++) {
    if (axis == 1) {
#pragma omp parallel for schedule(static)
      for (int j = 1; j <= N; j++) {
        double Q[5];
        if (flux_dir > 0) {
          for (int i = 0; i <= N; i++) {
            for (int k = 0; k < 5; k++) Q[k] = field[CI(c, i - 2 + k, j, p)];
            fext[EI(c, 2 * i + 1, 2 * j, p)] = weno_limiter(Q, flux_dir);
          }
        } else {
          for (int i = 1; i <= N + 1; i++) {
            for (int k = 0; k < 5; k++) Q[k] = field[CI(c, i - 2 + k, j, p)];
            fext[EI(c, 2 * i - 1, 2 * j, p)] = weno_limiter(Q, flux_dir);
          }
        }
      }
    } else {
#pragma omp parallel for schedule(static)
      for (int i = 1; i <= N; i++) {
        double Q[5];
        if (flux_dir > 0) {
          for (int j = 0; j <= N; j++) {
            for (int k = 0; k < 5; k++) Q[k] = field[CI(c, i, j - 2 + k, p)];
            fext[EI(c, 2 * i, 2 * j + 1, p)] = weno_limiter(Q, flux_dir);
          }
        } else {
          for (int j = 1; j <= N + 1; j++) {
            for (int k = 0; k < 5; k++) Q[k] = field[CI(c, i, j - 2 + k, p)];
            fext[EI(c, 2 * i, 2 * j - 1, p)] = weno_limiter(Q, flux_dir);
          }
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------- */
/* CubedSphereFillHalo: ghost_mod.f90:18-82 (pure permutation copy of the 24  */
/* directed edge strips; the h x h corner blocks are not touched).            */
/* ------------------------------------------------------------------------- */
static void fill_halo_impl(int N, int h, double *field, double *inner) {
  const int nh = N + 2 * h;
#define F(i, j, p) field[(size_t)((i) - (1 - h)) + (size_t)nh * ((size_t)((j) - (1 - h)) + (size_t)nh * (size_t)((p) - 1))]
#define IN(i, j, p) inner[(size_t)((i) - 1) + (size_t)N * ((size_t)((j) - 1) + (size_t)N * (size_t)((p) - 1))]
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) IN(i, j, p) = F(i, j, p);
  const int ite = N, jte = N;
  for (int k = 1; k <= h; k++) {
    for (int m = 1; m <= N; m++) {
      /* panel 1 */
      F(1 - k, m, 1) = IN(ite - k + 1, m, 4);
      F(ite + k, m, 1) = IN(k, m, 2);
      F(m, 1 - k, 1) = IN(m, jte - k + 1, 6);
      F(m, jte + k, 1) = IN(m, k, 5);
      /* panel 2 */
      F(1 - k, m, 2) = IN(ite - k + 1, m, 1);
      F(ite + k, m, 2) = IN(k, m, 3);
      F(m, 1 - k, 2) = IN(ite - k + 1, jte - m + 1, 6);
      F(m, jte + k, 2) = IN(ite - k + 1, m, 5);
      /* panel 3 */
      F(1 - k, m, 3) = IN(ite - k + 1, m, 2);
      F(ite + k, m, 3) = IN(k, m, 4);
      F(m, 1 - k, 3) = IN(ite - m + 1, k, 6);
      F(m, jte + k, 3) = IN(ite - m + 1, jte - k + 1, 5);
      /* panel 4 */
      F(1 - k, m, 4) = IN(ite - k + 1, m, 3);
      F(ite + k, m, 4) = IN(k, m, 1);
      F(m, 1 - k, 4) = IN(k, m, 6);
      F(m, jte + k, 4) = IN(k, jte - m + 1, 5);
      /* panel 5 (top) */
      F(1 - k, m, 5) = IN(ite - m + 1, jte - k + 1, 4);
      F(ite + k, m, 5) = IN(m, jte - k + 1, 2);
      F(m, 1 - k, 5) = IN(m, jte - k + 1, 1);
      F(m, jte + k, 5) = IN(ite - m + 1, jte - k + 1, 3);
      /* panel 6 (bottom) */
      F(1 - k, m, 6) = IN(m, k, 4);
      F(ite + k, m, 6) = IN(ite - m + 1, k, 2);
      F(m, 1 - k, 6) = IN(ite - m + 1, k, 3);
      F(m, jte + k, 6) = IN(m, k, 1);
    }
  }
#undef F
#undef IN
}

void orc_fill_halo(int N, int h, double *field) {
  double *inner = dalloc((size_t)N * N * 6);
  fill_halo_impl(N, h, field, inner);
  free(inner);
}

/* CubedSphereFillJab: ghost_mod.f90:84-160 -- the same permutation applied to */
/* the 3x2 Jacobian with the column swaps / negations of each edge.           */
void orc_fill_jab(int N, int h, double *jab) {
  const int nh = N + 2 * h;
  double *inner = dalloc((size_t)6 * N * N * 6);
#define J(r, c, i, j, p) jab[(size_t)((r) - 1) + 3 * (size_t)((c) - 1) + 6 * ((size_t)((i) - (1 - h)) + (size_t)nh * ((size_t)((j) - (1 - h)) + (size_t)nh * (size_t)((p) - 1)))]
#define IN(r, c, i, j, p) inner[(size_t)((r) - 1) + 3 * (size_t)((c) - 1) + 6 * ((size_t)((i) - 1) + (size_t)N * ((size_t)((j) - 1) + (size_t)N * (size_t)((p) - 1)))]
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++)
        for (int c = 1; c <= 2; c++)
          for (int r = 1; r <= 3; r++) IN(r, c, i, j, p) = J(r, c, i, j, p);
  const int ite = N, jte = N;
  for (int k = 1; k <= h; k++) {
    for (int m = 1; m <= N; m++) {
      for (int r = 1; r <= 3; r++) {
        /* panel 1 */
        for (int c = 1; c <= 2; c++) {
          J(r, c, 1 - k, m, 1) = IN(r, c, ite - k + 1, m, 4);
          J(r, c, ite + k, m, 1) = IN(r, c, k, m, 2);
          J(r, c, m, 1 - k, 1) = IN(r, c, m, jte - k + 1, 6);
          J(r, c, m, jte + k, 1) = IN(r, c, m, k, 5);
        }
        /* panel 2 */
        for (int c = 1; c <= 2; c++) {
          J(r, c, 1 - k, m, 2) = IN(r, c, ite - k + 1, m, 1);
          J(r, c, ite + k, m, 2) = IN(r, c, k, m, 3);
        }
        J(r, 1, m, 1 - k, 2) = -IN(r, 2, ite - k + 1, jte - m + 1, 6);
        J(r, 2, m, 1 - k, 2) = IN(r, 1, ite - k + 1, jte - m + 1, 6);
        J(r, 1, m, jte + k, 2) = IN(r, 2, ite - k + 1, m, 5);
        J(r, 2, m, jte + k, 2) = -IN(r, 1, ite - k + 1, m, 5);
        /* panel 3 */
        for (int c = 1; c <= 2; c++) {
          J(r, c, 1 - k, m, 3) = IN(r, c, ite - k + 1, m, 2);
          J(r, c, ite + k, m, 3) = IN(r, c, k, m, 4);
        }
        J(r, 1, m, 1 - k, 3) = -IN(r, 1, ite - m + 1, k, 6);
        J(r, 2, m, 1 - k, 3) = -IN(r, 2, ite - m + 1, k, 6);
        J(r, 1, m, jte + k, 3) = -IN(r, 1, ite - m + 1, jte - k + 1, 5);
        J(r, 2, m, jte + k, 3) = -IN(r, 2, ite - m + 1, jte - k + 1, 5);
        /* panel 4 */
        for (int c = 1; c <= 2; c++) {
          J(r, c, 1 - k, m, 4) = IN(r, c, ite - k + 1, m, 3);
          J(r, c, ite + k, m, 4) = IN(r, c, k, m, 1);
        }
        J(r, 1, m, 1 - k, 4) = IN(r, 2, k, m, 6);
        J(r, 2, m, 1 - k, 4) = -IN(r, 1, k, m, 6);
        J(r, 1, m, jte + k, 4) = -IN(r, 2, k, jte - m + 1, 5);
        J(r, 2, m, jte + k, 4) = IN(r, 1, k, jte - m + 1, 5);
        /* panel 5 (top) */
        J(r, 1, 1 - k, m, 5) = IN(r, 2, ite - m + 1, jte - k + 1, 4);
        J(r, 2, 1 - k, m, 5) = -IN(r, 1, ite - m + 1, jte - k + 1, 4);
        J(r, 1, ite + k, m, 5) = -IN(r, 2, m, jte - k + 1, 2);
        J(r, 2, ite + k, m, 5) = IN(r, 1, m, jte - k + 1, 2);
        for (int c = 1; c <= 2; c++) J(r, c, m, 1 - k, 5) = IN(r, c, m, jte - k + 1, 1);
        J(r, 1, m, jte + k, 5) = -IN(r, 1, ite - m + 1, jte - k + 1, 3);
        J(r, 2, m, jte + k, 5) = -IN(r, 2, ite - m + 1, jte - k + 1, 3);
        /* panel 6 (bottom) */
        J(r, 1, 1 - k, m, 6) = -IN(r, 2, m, k, 4);
        J(r, 2, 1 - k, m, 6) = IN(r, 1, m, k, 4);
        J(r, 1, ite + k, m, 6) = IN(r, 2, ite - m + 1, k, 2);
        J(r, 2, ite + k, m, 6) = -IN(r, 1, ite - m + 1, k, 2);
        J(r, 1, m, 1 - k, 6) = -IN(r, 1, ite - m + 1, k, 3);
        J(r, 2, m, 1 - k, 6) = -IN(r, 2, ite - m + 1, k, 3);
        for (int c = 1; c <= 2; c++) J(r, c, m, jte + k, 6) = IN(r, c, m, k, 1);
      }
    }
  }
#undef J
#undef IN
  free(inner);
}

/* ------------------------------------------------------------------------- */
/* BRINV (math_mod.f90:451-525): full-pivot Gauss-Jordan inverse, here N = 2. */
/* Arrays are Fortran column-major a[(r-1) + N*(c-1)].  Returns L (0 = fail). */
/* ------------------------------------------------------------------------- */
static int brinv2(const double *Ain, double *A) {
  const int n = 2;
  int IS[3], JS[3];
#define AA(i, j) A[((i) - 1) + n * ((j) - 1)]
  for (int k = 0; k < 4; k++) A[k] = Ain[k];
  for (int K = 1; K <= n; K++) {
    double D = 0.;
    for (int I = K; I <= n; I++)
      for (int Jc = K; Jc <= n; Jc++)
        if (fabs(AA(I, Jc)) > D) { D = fabs(AA(I, Jc)); IS[K] = I; JS[K] = Jc; }
    if (D + 1.0 == 1.0) return 0;
    for (int Jc = 1; Jc <= n; Jc++) { double T = AA(K, Jc); AA(K, Jc) = AA(IS[K], Jc); AA(IS[K], Jc) = T; }
    for (int I = 1; I <= n; I++) { double T = AA(I, K); AA(I, K) = AA(I, JS[K]); AA(I, JS[K]) = T; }
    AA(K, K) = 1 / AA(K, K);
    for (int Jc = 1; Jc <= n; Jc++) if (Jc != K) AA(K, Jc) = AA(K, Jc) * AA(K, K);
    for (int I = 1; I <= n; I++)
      if (I != K)
        for (int Jc = 1; Jc <= n; Jc++)
          if (Jc != K) AA(I, Jc) = AA(I, Jc) - AA(I, K) * AA(K, Jc);
    for (int I = 1; I <= n; I++) if (I != K) AA(I, K) = -AA(I, K) * AA(K, K);
  }
  for (int K = n; K >= 1; K--) {
    for (int Jc = 1; Jc <= n; Jc++) { double T = AA(K, Jc); AA(K, Jc) = AA(JS[K], Jc); AA(JS[K], Jc) = T; }
    for (int I = 1; I <= n; I++) { double T = AA(I, K); AA(I, K) = AA(I, IS[K]); AA(I, IS[K]) = T; }
  }
#undef AA
  return 1;
}

/* ------------------------------------------------------------------------- */
/* Metric derivation: io_mod.F90:119-220 and 295-306.                          */
/* Inputs are the mesh-file samples at the N x N x 6 cell centres (the even   */
/* points of the extended grid, io_mod.F90:121-136): lon/lat in degrees,      */
/* x/y/z and jab on the unit sphere (jab per radian of the panel angle        */
/* coordinate).  Outputs are the reference's halo'd mesh arrays; the corner   */
/* blocks of the matrices are left at zero (the reference leaves them         */
/* uninitialised and never reads them).  Returns 0 on success, or -1 when a   */
/* matrix inversion fails (the reference stops there).                        */
/* ------------------------------------------------------------------------- */
int orc_derive_metrics(int N, int h, double radius, double omega,
                       const double *lon_deg, const double *lat_deg,
                       const double *xc, const double *yc, const double *zc, const double *jab_c,
                       double *sqrtG, double *G, double *IG, double *A, double *IA, double *f,
                       double *lon_out, double *lat_out, double *sinlat_out, double *coslat_out) {
  const int nh = N + 2 * h;
  const size_t nc = (size_t)nh * nh * 6;
  double *lon = dalloc(nc), *lat = dalloc(nc), *x = dalloc(nc), *y = dalloc(nc), *z = dalloc(nc);
  double *sinlon = dalloc(nc), *coslon = dalloc(nc), *sinlat = dalloc(nc), *coslat = dalloc(nc);
  double *jab = dalloc(6 * nc);
  int status = 0;
#define C3(i, j, p) ((size_t)((i) - (1 - h)) + (size_t)nh * ((size_t)((j) - (1 - h)) + (size_t)nh * (size_t)((p) - 1)))
#define S3(i, j, p) ((size_t)((i) - 1) + (size_t)N * ((size_t)((j) - 1) + (size_t)N * (size_t)((p) - 1)))
  for (size_t k = 0; k < nc; k++) { lon[k] = ORC_FILL_VALUE; lat[k] = ORC_FILL_VALUE; }
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        const size_t s = S3(i, j, p), d = C3(i, j, p);
        lon[d] = lon_deg[s] * ORC_D2R;  /* io_mod.F90:110 */
        lat[d] = lat_deg[s] * ORC_D2R;
        x[d] = xc[s] * radius;          /* io_mod.F90:113-115 */
        y[d] = yc[s] * radius;
        z[d] = zc[s] * radius;
        for (int q = 0; q < 6; q++) jab[6 * d + q] = jab_c[6 * s + q] * radius; /* :117 */
      }
  for (size_t k = 0; k < nc; k++) {
    sinlon[k] = sin(lon[k]); coslon[k] = cos(lon[k]);
    sinlat[k] = sin(lat[k]); coslat[k] = cos(lat[k]);
  }
  orc_fill_halo(N, h, lon); orc_fill_halo(N, h, lat);
  orc_fill_halo(N, h, x); orc_fill_halo(N, h, y); orc_fill_halo(N, h, z);
  orc_fill_halo(N, h, sinlon); orc_fill_halo(N, h, coslon);
  orc_fill_halo(N, h, sinlat); orc_fill_halo(N, h, coslat);
  orc_fill_jab(N, h, jab);
  memset(sqrtG, 0, nc * sizeof(double));
  memset(G, 0, 4 * nc * sizeof(double)); memset(IG, 0, 4 * nc * sizeof(double));
  memset(A, 0, 4 * nc * sizeof(double)); memset(IA, 0, 4 * nc * sizeof(double));
  memset(f, 0, nc * sizeof(double));
  for (int p = 1; p <= 6; p++)
    for (int j = 1 - h; j <= N + h; j++)
      for (int i = 1 - h; i <= N + h; i++) {
        const size_t d = C3(i, j, p);
        const double lo = lon[d], la = lat[d];
        if (!(lo != ORC_FILL_VALUE && la != ORC_FILL_VALUE)) continue;
        const double *J = &jab[6 * d]; /* J(r,c) = J[(r-1) + 3(c-1)] */
        double S[6];                   /* sph2cart_matrix(2,3), S(r,c) = S[(r-1) + 2(c-1)] */
        S[0] = -sin(lo);          /* dlondx */
        S[1] = -cos(lo) * sin(la); /* dlatdx */
        S[2] = cos(lo);           /* dlondy */
        S[3] = -sin(lo) * sin(la); /* dlatdy */
        S[4] = 0.;                /* dlondz */
        S[5] = cos(la);           /* dlatdz */
        double *g = &G[4 * d], *ig = &IG[4 * d], *a = &A[4 * d], *ia = &IA[4 * d];
        /* matmul(transpose(jab), jab): io_mod.F90:174 */
        for (int cc = 1; cc <= 2; cc++)
          for (int r = 1; r <= 2; r++) {
            double s = 0.;
            for (int k = 1; k <= 3; k++) s = s + J[(k - 1) + 3 * (r - 1)] * J[(k - 1) + 3 * (cc - 1)];
            g[(r - 1) + 2 * (cc - 1)] = s;
          }
        if (!brinv2(g, ig)) { status = -1; goto done; } /* :176-177 */
        sqrtG[d] = sqrt(g[0] * g[3] - g[1] * g[2]);     /* :179, det() math_mod.f90:327-347 */
        /* matmul(sph2cart_matrix, jab): :181 */
        for (int cc = 1; cc <= 2; cc++)
          for (int r = 1; r <= 2; r++) {
            double s = 0.;
            for (int k = 1; k <= 3; k++) s = s + S[(r - 1) + 2 * (k - 1)] * J[(k - 1) + 3 * (cc - 1)];
            a[(r - 1) + 2 * (cc - 1)] = s;
          }
        if (fabs(la * ORC_R2D) != 90) {
          if (!brinv2(a, ia)) { status = -1; goto done; }
        } else {
          /* pole special cases :189-216: IA = matmul(I, IA1) * radius */
          double IA1[4];
          if (la * ORC_R2D == 90) {
            IA1[0] = cos(lo); IA1[2] = -sin(lo); IA1[1] = sin(lo); IA1[3] = cos(lo);
          } else {
            IA1[0] = -cos(lo); IA1[2] = sin(lo); IA1[1] = sin(lo); IA1[3] = cos(lo);
          }
          const double I2[4] = {1., 0., 0., 1.};
          for (int cc = 1; cc <= 2; cc++)
            for (int r = 1; r <= 2; r++) {
              double s = 0.;
              for (int k = 1; k <= 2; k++) s = s + I2[(r - 1) + 2 * (k - 1)] * IA1[(k - 1) + 2 * (cc - 1)];
              ia[(r - 1) + 2 * (cc - 1)] = s * radius;
            }
        }
      }
  /* f = 2 Omega sin(lat) on the interior (:295-301) */
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) f[C3(i, j, p)] = 2. * omega * sinlat[C3(i, j, p)];
  if (lon_out) memcpy(lon_out, lon, nc * sizeof(double));
  if (lat_out) memcpy(lat_out, lat, nc * sizeof(double));
  if (sinlat_out) memcpy(sinlat_out, sinlat, nc * sizeof(double));
  if (coslat_out) memcpy(coslat_out, coslat, nc * sizeof(double));
done:
#undef C3
#undef S3
  free(lon); free(lat); free(x); free(y); free(z);
  free(sinlon); free(coslon); free(sinlat); free(coslat); free(jab);
  return status;
}

/* ------------------------------------------------------------------------- */
/* context                                                                    */
/* ------------------------------------------------------------------------- */
static void state_alloc(orc_state *s, size_t n) {
  s->phiG = dalloc(n); s->u = dalloc(n); s->v = dalloc(n); s->phi = dalloc(n);
  s->uC = dalloc(n); s->vC = dalloc(n); s->zonal = dalloc(n); s->merid = dalloc(n); s->phit = dalloc(n);
}
static void state_free(orc_state *s) {
  free(s->phiG); free(s->u); free(s->v); free(s->phi); free(s->uC); free(s->vC);
  free(s->zonal); free(s->merid); free(s->phit);
}

orc_ctx *orc_create(int N, int h, double dx, double dy,
                    const double *sqrtG, const double *G, const double *IG,
                    const double *A, const double *IA, const double *f, const double *phis) {
  if (N < 1 || h < 3) return NULL;
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  c->N = N; c->h = h; c->nh = N + 2 * h; c->ne = 2 * N + 1;
  c->ncell = (size_t)c->nh * c->nh * 6;
  c->next = (size_t)c->ne * c->ne * 6;
  c->dx = dx; c->dy = dy;
  const size_t n = c->ncell, ne = c->next;
  c->sqrtG = dalloc(n); c->G = dalloc(4 * n); c->IG = dalloc(4 * n); c->A = dalloc(4 * n);
  c->IA = dalloc(4 * n); c->f = dalloc(n); c->phis = dalloc(n);
  memcpy(c->sqrtG, sqrtG, n * sizeof(double));
  memcpy(c->G, G, 4 * n * sizeof(double)); memcpy(c->IG, IG, 4 * n * sizeof(double));
  memcpy(c->A, A, 4 * n * sizeof(double)); memcpy(c->IA, IA, 4 * n * sizeof(double));
  memcpy(c->f, f, n * sizeof(double)); memcpy(c->phis, phis, n * sizeof(double));
  for (int s = 0; s < 6; s++) {
    state_alloc(&c->stat[s], n);
    c->tend[s].phiG = dalloc(n); c->tend[s].u = dalloc(n); c->tend[s].v = dalloc(n);
  }
  c->E = dalloc(n); c->K = dalloc(n); c->flux_x = dalloc(n); c->flux_y = dalloc(n);
  c->vort = dalloc(n); c->phit = dalloc(n); c->phitG = dalloc(n);
  c->dfluxdx = dalloc(n); c->dfluxdy = dalloc(n); c->dEdx = dalloc(n); c->dEdy = dalloc(n);
  c->dvdx = dalloc(n); c->dudy = dalloc(n);
  c->fx_p = dalloc(ne); c->fx_n = dalloc(ne); c->fy_p = dalloc(ne); c->fy_n = dalloc(ne);
  c->E_p = dalloc(ne); c->E_n = dalloc(ne); c->pG_p = dalloc(ne); c->pG_n = dalloc(ne);
  c->ptG_p = dalloc(ne); c->ptG_n = dalloc(ne);
  c->u_p = dalloc(ne); c->u_n = dalloc(ne); c->v_p = dalloc(ne); c->v_n = dalloc(ne);
  c->fx_ext = dalloc(ne); c->fy_ext = dalloc(ne); c->E_ext = dalloc(ne); c->pG_ext = dalloc(ne);
  c->u_ext = dalloc(ne); c->v_ext = dalloc(ne);
  c->inner = dalloc((size_t)N * N * 6);
  return c;
}

void orc_destroy(orc_ctx *c) {
  if (!c) return;
  free(c->sqrtG); free(c->G); free(c->IG); free(c->A); free(c->IA); free(c->f); free(c->phis);
  for (int s = 0; s < 6; s++) {
    state_free(&c->stat[s]);
    free(c->tend[s].phiG); free(c->tend[s].u); free(c->tend[s].v);
  }
  double *bufs[] = {c->E, c->K, c->flux_x, c->flux_y, c->vort, c->phit, c->phitG, c->dfluxdx, c->dfluxdy,
                    c->dEdx, c->dEdy, c->dvdx, c->dudy, c->fx_p, c->fx_n, c->fy_p, c->fy_n, c->E_p, c->E_n,
                    c->pG_p, c->pG_n, c->ptG_p, c->ptG_n, c->u_p, c->u_n, c->v_p, c->v_n, c->fx_ext,
                    c->fy_ext, c->E_ext, c->pG_ext, c->u_ext, c->v_ext, c->inner};
  for (size_t k = 0; k < sizeof(bufs) / sizeof(bufs[0]); k++) free(bufs[k]);
  free(c);
}

void orc_set_e_dissipation(orc_ctx *c, int mode) { c->e_diss = mode; }

/* 0 selects spatial_operators_mod.F90 (WENO-Z + Rusanov); 2, 4 and 6 select the
   central-difference modules spatial_operators_mod_{2nd,4th,6th}.F90.  Returns 0,
   or -1 for any other value (the operator is left unchanged). */
int orc_set_operator(orc_ctx *c, int op) {
  if (op != 0 && op != 2 && op != 4 && op != 6) return -1;
  c->op = op;
  return 0;
}

static orc_state *slot_state(orc_ctx *c, int slot) { return &c->stat[slot + 4]; }
static orc_tend *slot_tend(orc_ctx *c, int slot) { return &c->tend[slot + 4]; }

/* field ids: 0 phiG 1 u 2 v 3 phi 4 uC 5 vC 6 zonal 7 meridional 8 phit */
static double *state_field(orc_state *s, int id) {
  switch (id) {
    case 0: return s->phiG; case 1: return s->u; case 2: return s->v; case 3: return s->phi;
    case 4: return s->uC; case 5: return s->vC; case 6: return s->zonal; case 7: return s->merid;
    default: return s->phit;
  }
}

void orc_set_field(orc_ctx *c, int slot, int id, const double *src) {
  memcpy(state_field(slot_state(c, slot), id), src, c->ncell * sizeof(double));
}
void orc_get_field(orc_ctx *c, int slot, int id, double *dst) {
  memcpy(dst, state_field(slot_state(c, slot), id), c->ncell * sizeof(double));
}
void orc_get_tend(orc_ctx *c, int slot, int id, double *dst) {
  orc_tend *t = slot_tend(c, slot);
  const double *s = id == 0 ? t->phiG : (id == 1 ? t->u : t->v);
  memcpy(dst, s, c->ncell * sizeof(double));
}

/* ------------------------------------------------------------------------- */
/* spatial_operator: spatial_operators_mod.F90:13-181                         */
/* ------------------------------------------------------------------------- */
/* Central-difference operators: spatial_operators_mod_2nd.F90:13-70,
   spatial_operators_mod_4th.F90:13-74, spatial_operators_mod_6th.F90:13-81.
   Same prologue as the WENO operator (:38-45 there), then every derivative is a
   centred difference of the cell values, evaluated left to right as written. */
static double cd_diff(int op, const double *f, size_t k, ptrdiff_t s, double d) {
  if (op == 2) return (f[k + s] - f[k - s]) / (2. * d);
  if (op == 4) return (f[k - 2 * s] - 8. * f[k - s] + 8. * f[k + s] - f[k + 2 * s]) / (12. * d);
  return (-f[k - 3 * s] + 9. * f[k - 2 * s] - 45. * f[k - s] + 45. * f[k + s] - 9. * f[k + 2 * s] + f[k + 3 * s]) /
         (60. * d);
}

static void spatial_operator_cd(orc_ctx *c, const orc_state *st, orc_tend *td) {
  const int N = c->N, op = c->op;
  const size_t n = c->ncell;
  const ptrdiff_t sx = 1, sy = c->nh;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < n; k++) {
    c->phit[k] = st->phi[k] + c->phis[k];
    c->K[k] = 0.5 * (st->u[k] * st->uC[k] + st->v[k] * st->vC[k]);
    c->E[k] = c->phit[k] + c->K[k];
    c->flux_x[k] = st->phiG[k] * st->uC[k];
    c->flux_y[k] = st->phiG[k] * st->vC[k];
  }
  for (int p = 1; p <= 6; p++) {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        const size_t k = CI(c, i, j, p);
        c->dfluxdx[k] = cd_diff(op, c->flux_x, k, sx, c->dx);
        c->dEdx[k] = cd_diff(op, c->E, k, sx, c->dx);
        c->dvdx[k] = cd_diff(op, st->v, k, sx, c->dx);
        c->dfluxdy[k] = cd_diff(op, c->flux_y, k, sy, c->dy);
        c->dEdy[k] = cd_diff(op, c->E, k, sy, c->dy);
        c->dudy[k] = cd_diff(op, st->u, k, sy, c->dy);
        c->vort[k] = c->dvdx[k] - c->dudy[k] + c->sqrtG[k] * c->f[k];
        td->phiG[k] = -(c->dfluxdx[k] + c->dfluxdy[k]);
        td->u[k] = -c->dEdx[k] + c->vort[k] * st->vC[k];
        td->v[k] = -c->dEdy[k] - c->vort[k] * st->uC[k];
      }
  }
}

static void spatial_operator(orc_ctx *c, const orc_state *st, orc_tend *td) {
  if (c->op != 0) {
    spatial_operator_cd(c, st, td);
    return;
  }
  const int N = c->N;
  const size_t n = c->ncell;
  const double dx = c->dx, dy = c->dy;
  /* :71-78 whole-array prologue */
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < n; k++) {
    c->phit[k] = st->phi[k] + c->phis[k];
    c->phitG[k] = c->phit[k] * c->sqrtG[k];
    c->K[k] = 0.5 * (st->u[k] * st->uC[k] + st->v[k] * st->vC[k]);
    c->E[k] = c->phit[k] + c->K[k];
    c->flux_x[k] = st->phiG[k] * st->uC[k];
    c->flux_y[k] = st->phiG[k] * st->vC[k];
  }
  /* :80-99 (the phiG reconstructions are commented out in the reference) */
  weno_sweep(c, c->fx_p, c->flux_x, 1, 1);
  weno_sweep(c, c->fx_n, c->flux_x, -1, 1);
  weno_sweep(c, c->E_p, c->E, 1, 1);
  weno_sweep(c, c->E_n, c->E, -1, 1);
  weno_sweep(c, c->ptG_p, c->phitG, 1, 1);
  weno_sweep(c, c->ptG_n, c->phitG, -1, 1);
  weno_sweep(c, c->v_p, st->v, 1, 1);
  weno_sweep(c, c->v_n, st->v, -1, 1);
  weno_sweep(c, c->fy_p, c->flux_y, 1, 2);
  weno_sweep(c, c->fy_n, c->flux_y, -1, 2);
  weno_sweep(c, c->E_p, c->E, 1, 2);
  weno_sweep(c, c->E_n, c->E, -1, 2);
  weno_sweep(c, c->ptG_p, c->phitG, 1, 2);
  weno_sweep(c, c->ptG_n, c->phitG, -1, 2);
  weno_sweep(c, c->u_p, st->u, 1, 2);
  weno_sweep(c, c->u_n, st->u, -1, 2);
  if (c->e_diss == 1) {
    /* intended-physics option: fill the face slots the reference never writes */
    weno_sweep(c, c->u_p, st->u, 1, 1);
    weno_sweep(c, c->u_n, st->u, -1, 1);
    weno_sweep(c, c->v_p, st->v, 1, 2);
    weno_sweep(c, c->v_n, st->v, -1, 2);
  }
  /* :101-124 x faces */
  for (int p = 1; p <= 6; p++) {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= N; j++)
      for (int i = 0; i <= N; i++) {
        const int ip1 = 2 * i + 1, jc = 2 * j;
        const double uBdy = 0.5 * (st->uC[CI(c, i + 1, j, p)] + st->uC[CI(c, i, j, p)]);
        const double phitBdy = 0.5 * (c->phit[CI(c, i + 1, j, p)] + c->phit[CI(c, i, j, p)]);
        const double ig = 0.5 * (c->IG[MI(c, 1, 1, i + 1, j, p)] + c->IG[MI(c, 1, 1, i, j, p)]);
        const double e1 = uBdy - sqrt(ig * phitBdy);
        const double e2 = uBdy + sqrt(0.5 * (c->IG[MI(c, 1, 1, i + 1, j, p)] + c->IG[MI(c, 1, 1, i, j, p)]) * phitBdy);
        double mx = fabs(e1);
        if (fabs(e2) > mx) mx = fabs(e2);
        const size_t e = EI(c, ip1, jc, p);
        c->fx_ext[e] = 0.5 * (c->fx_p[e] + c->fx_n[e] - mx * (c->ptG_n[e] - c->ptG_p[e]));
        c->E_ext[e] = 0.5 * (c->E_p[e] + c->E_n[e] - mx * (c->u_n[e] - c->u_p[e]));
        c->v_ext[e] = 0.5 * (c->v_p[e] + c->v_n[e] - copysign(1., uBdy) * (c->v_n[e] - c->v_p[e]));
      }
  }
  /* :126-149 y faces */
  for (int p = 1; p <= 6; p++) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        const int ic = 2 * i, jp1 = 2 * j + 1;
        const double vBdy = 0.5 * (st->vC[CI(c, i, j + 1, p)] + st->vC[CI(c, i, j, p)]);
        const double phitBdy = 0.5 * (c->phit[CI(c, i, j + 1, p)] + c->phit[CI(c, i, j, p)]);
        const double e1 = vBdy - sqrt(0.5 * (c->IG[MI(c, 2, 2, i, j + 1, p)] + c->IG[MI(c, 2, 2, i, j, p)]) * phitBdy);
        const double e2 = vBdy + sqrt(0.5 * (c->IG[MI(c, 2, 2, i, j + 1, p)] + c->IG[MI(c, 2, 2, i, j, p)]) * phitBdy);
        double my = fabs(e1);
        if (fabs(e2) > my) my = fabs(e2);
        const size_t e = EI(c, ic, jp1, p);
        c->fy_ext[e] = 0.5 * (c->fy_p[e] + c->fy_n[e] - my * (c->ptG_n[e] - c->ptG_p[e]));
        c->E_ext[e] = 0.5 * (c->E_p[e] + c->E_n[e] - my * (c->v_n[e] - c->v_p[e]));
        c->u_ext[e] = 0.5 * (c->u_p[e] + c->u_n[e] - copysign(1., vBdy) * (c->u_n[e] - c->u_p[e]));
      }
  }
  /* :151-175 divergence and vorticity */
  for (int p = 1; p <= 6; p++) {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        const int ic = 2 * i, jc = 2 * j, ip1 = 2 * i + 1, im1 = 2 * i - 1, jp1 = 2 * j + 1, jm1 = 2 * j - 1;
        const size_t k = CI(c, i, j, p);
        c->dfluxdx[k] = (c->fx_ext[EI(c, ip1, jc, p)] - c->fx_ext[EI(c, im1, jc, p)]) / dx;
        c->dEdx[k] = (c->E_ext[EI(c, ip1, jc, p)] - c->E_ext[EI(c, im1, jc, p)]) / dx;
        c->dvdx[k] = (-st->v[CI(c, i - 3, j, p)] + 9. * st->v[CI(c, i - 2, j, p)] - 45. * st->v[CI(c, i - 1, j, p)] +
                      45. * st->v[CI(c, i + 1, j, p)] - 9. * st->v[CI(c, i + 2, j, p)] + st->v[CI(c, i + 3, j, p)]) /
                     (60. * dx);
        c->dfluxdy[k] = (c->fy_ext[EI(c, ic, jp1, p)] - c->fy_ext[EI(c, ic, jm1, p)]) / dy;
        c->dEdy[k] = (c->E_ext[EI(c, ic, jp1, p)] - c->E_ext[EI(c, ic, jm1, p)]) / dy;
        c->dudy[k] = (-st->u[CI(c, i, j - 3, p)] + 9. * st->u[CI(c, i, j - 2, p)] - 45. * st->u[CI(c, i, j - 1, p)] +
                      45. * st->u[CI(c, i, j + 1, p)] - 9. * st->u[CI(c, i, j + 2, p)] + st->u[CI(c, i, j + 3, p)]) /
                     (60. * dy);
        c->vort[k] = c->dvdx[k] - c->dudy[k] + c->sqrtG[k] * c->f[k];
      }
  }
  /* :177-179 tendencies (interior; the reference's halo values are undefined) */
  for (int p = 1; p <= 6; p++) {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        const size_t k = CI(c, i, j, p);
        td->phiG[k] = -(c->dfluxdx[k] + c->dfluxdy[k]);
        td->u[k] = -c->dEdx[k] + c->vort[k] * st->vC[k];
        td->v[k] = -c->dEdy[k] - c->vort[k] * st->uC[k];
      }
  }
}

void orc_spatial_operator(orc_ctx *c, int stat_slot, int tend_slot) {
  spatial_operator(c, slot_state(c, stat_slot), slot_tend(c, tend_slot));
}

/* ------------------------------------------------------------------------- */
/* wind conversions: spatial_operators_mod.F90:364-410, projection_mod.F90    */
/* ------------------------------------------------------------------------- */
/* matmul(X, Y) of two 2x2 matrices as gfortran inlines it: c = 0; c += ...   */
static inline void matmul22(const double *X, const double *Y, double *M) {
  for (int cc = 0; cc < 2; cc++)
    for (int r = 0; r < 2; r++) {
      double s = 0.;
      for (int k = 0; k < 2; k++) s = s + X[r + 2 * k] * Y[k + 2 * cc];
      M[r + 2 * cc] = s;
    }
}

/* convert_wind_P2SP on the interior (covProjPlane2Sphere, projection_mod.F90:79-96) */
static void convert_wind_P2SP(orc_ctx *c, orc_state *s) {
  const int N = c->N;
  for (int p = 1; p <= 6; p++) {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= N; j++)
      for (int i = 1; i <= N; i++) {
        const size_t k = CI(c, i, j, p);
        double M[4];
        matmul22(&c->A[4 * k], &c->IG[4 * k], M);
        s->zonal[k] = M[0] * s->u[k] + M[2] * s->v[k];
        s->merid[k] = M[1] * s->u[k] + M[3] * s->v[k];
      }
  }
}

/* convert_wind_SP2P on the full array (covProjSphere2Plane, projection_mod.F90:60-77) */
static void convert_wind_SP2P(orc_ctx *c, orc_state *s) {
  const size_t n = c->ncell;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < n; k++) {
    double M[4];
    matmul22(&c->G[4 * k], &c->IA[4 * k], M);
    s->u[k] = M[0] * s->zonal[k] + M[2] * s->merid[k];
    s->v[k] = M[1] * s->zonal[k] + M[3] * s->merid[k];
  }
}

/* convert_wind_cov2contrav on the full array (cov2contrav, projection_mod.F90:138-148) */
static void convert_wind_cov2contrav(orc_ctx *c, orc_state *s) {
  const size_t n = c->ncell;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < n; k++) {
    const double *ig = &c->IG[4 * k];
    s->uC[k] = ig[0] * s->u[k] + ig[2] * s->v[k];
    s->vC[k] = ig[1] * s->u[k] + ig[3] * s->v[k];
  }
}

/* correct_bdy_ghost: time_scheme_mod.F90:117-125 */
static void correct_bdy_ghost(orc_ctx *c, orc_state *s) {
  convert_wind_P2SP(c, s);
  fill_halo_impl(c->N, c->h, s->phiG, c->inner); /* fill_ghost ghost_mod.f90:163-170 */
  fill_halo_impl(c->N, c->h, s->zonal, c->inner);
  fill_halo_impl(c->N, c->h, s->merid, c->inner);
  convert_wind_SP2P(c, s);
  convert_wind_cov2contrav(c, s);
}

static void finish_update(orc_ctx *c, orc_state *nw) {
  correct_bdy_ghost(c, nw);
  const size_t n = c->ncell;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < n; k++) nw->phi[k] = nw->phiG[k] / c->sqrtG[k];
}

/* update_stat: time_scheme_mod.F90:69-83 */
static void update_stat(orc_ctx *c, orc_state *nw, const orc_state *old, const orc_tend *t, double inc_t) {
  const size_t n = c->ncell;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < n; k++) {
    nw->phiG[k] = old->phiG[k] + inc_t * t->phiG[k];
    nw->u[k] = old->u[k] + inc_t * t->u[k];
    nw->v[k] = old->v[k] + inc_t * t->v[k];
  }
  finish_update(c, nw);
}

/* RK4: time_scheme_mod.F90:13-44 (stat(1) from stat(0)) */
void orc_rk4(orc_ctx *c, double dt) {
  orc_state *old = slot_state(c, 0), *nw = slot_state(c, 1);
  spatial_operator(c, old, slot_tend(c, -1));
  update_stat(c, slot_state(c, -2), old, slot_tend(c, -1), 0.5 * dt);
  spatial_operator(c, slot_state(c, -2), slot_tend(c, -2));
  update_stat(c, slot_state(c, -3), old, slot_tend(c, -2), 0.5 * dt);
  spatial_operator(c, slot_state(c, -3), slot_tend(c, -3));
  update_stat(c, slot_state(c, -4), old, slot_tend(c, -3), dt);
  spatial_operator(c, slot_state(c, -4), slot_tend(c, -4));
  orc_tend *t1 = slot_tend(c, -1), *t2 = slot_tend(c, -2), *t3 = slot_tend(c, -3), *t4 = slot_tend(c, -4);
  orc_tend *tn = slot_tend(c, 1);
  const size_t n = c->ncell;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < n; k++) {
    tn->phiG[k] = (t1->phiG[k] + 2. * t2->phiG[k] + 2. * t3->phiG[k] + t4->phiG[k]) / 6.;
    tn->u[k] = (t1->u[k] + 2. * t2->u[k] + 2. * t3->u[k] + t4->u[k]) / 6.;
    tn->v[k] = (t1->v[k] + 2. * t2->v[k] + 2. * t3->v[k] + t4->v[k]) / 6.;
  }
  update_stat(c, nw, old, tn, dt);
}

/* RK3_TVD: time_scheme_mod.F90:46-67, 85-115 */
void orc_rk3_tvd(orc_ctx *c, double dt) {
  orc_state *old = slot_state(c, 0), *nw = slot_state(c, 1);
  spatial_operator(c, old, slot_tend(c, -1));
  update_stat(c, slot_state(c, -2), old, slot_tend(c, -1), dt);
  spatial_operator(c, slot_state(c, -2), slot_tend(c, -2));
  {
    orc_state *s1 = slot_state(c, -2), *o = slot_state(c, -3);
    orc_tend *t = slot_tend(c, -2);
    const size_t n = c->ncell;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; k++) {
      o->phiG[k] = 0.75 * old->phiG[k] + 0.25 * s1->phiG[k] + 0.25 * dt * t->phiG[k];
      o->u[k] = 0.75 * old->u[k] + 0.25 * s1->u[k] + 0.25 * dt * t->u[k];
      o->v[k] = 0.75 * old->v[k] + 0.25 * s1->v[k] + 0.25 * dt * t->v[k];
    }
    finish_update(c, o);
  }
  spatial_operator(c, slot_state(c, -3), slot_tend(c, -3));
  {
    orc_state *s2 = slot_state(c, -3);
    orc_tend *t = slot_tend(c, -3);
    const size_t n = c->ncell;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; k++) {
      nw->phiG[k] = old->phiG[k] / 3. + 2. / 3. * s2->phiG[k] + 2. / 3. * dt * t->phiG[k];
      nw->u[k] = old->u[k] / 3. + 2. / 3. * s2->u[k] + 2. / 3. * dt * t->u[k];
      nw->v[k] = old->v[k] / 3. + 2. / 3. * s2->v[k] + 2. / 3. * dt * t->v[k];
    }
    finish_update(c, nw);
  }
}

/* copyStat(stat(0), stat(1)): stat_mod.F90:51-65 (ccsm.F90:66) */
void orc_copy_new_to_old(orc_ctx *c) {
  orc_state *o = slot_state(c, 0), *nw = slot_state(c, 1);
  for (int id = 0; id < 9; id++) memcpy(state_field(o, id), state_field(nw, id), c->ncell * sizeof(double));
}

/* the time loop of ccsm.F90:50-67 without output: scheme 0 = RK4, 1 = RK3_TVD */
void orc_run(orc_ctx *c, int scheme, double dt, int nsteps) {
  for (int it = 0; it < nsteps; it++) {
    if (scheme == 1) orc_rk3_tvd(c, dt); else orc_rk4(c, dt);
    orc_copy_new_to_old(c);
  }
}

/* initTestCase tail: test_case_mod.F90:38-48.  Given phi, zonal and meridional */
/* wind of stat(slot) on the full array, set phiG, u, v, uC, vC.               */
void orc_init_from_sphere(orc_ctx *c, int slot) {
  orc_state *s = slot_state(c, slot);
  const size_t n = c->ncell;
  for (size_t k = 0; k < n; k++) s->phiG[k] = s->phi[k] * c->sqrtG[k];
  for (size_t k = 0; k < n; k++) {
    double M[4];
    matmul22(&c->G[4 * k], &c->IA[4 * k], M);
    const double sv1 = s->zonal[k], sv2 = s->merid[k];
    s->u[k] = M[0] * sv1 + M[2] * sv2;
    s->v[k] = M[1] * sv1 + M[3] * sv2;
    const double *ia = &c->IA[4 * k];
    s->uC[k] = ia[0] * sv1 + ia[2] * sv2;
    s->vC[k] = ia[1] * sv1 + ia[3] * sv2;
  }
}

/* interior P2SP of a slot (ccsm.F90:56 before history output) */
void orc_p2sp(orc_ctx *c, int slot) { convert_wind_P2SP(c, slot_state(c, slot)); }

/* calc_total_mass / calc_total_energy: diag_mod.F90:10-53 (sequential sums) */
double orc_total_mass(orc_ctx *c, int slot) {
  orc_state *s = slot_state(c, slot);
  double t = 0.;
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= c->N; j++)
      for (int i = 1; i <= c->N; i++) t = t + s->phiG[CI(c, i, j, p)];
  return t;
}

double orc_total_energy(orc_ctx *c, int slot) {
  orc_state *s = slot_state(c, slot);
  double t = 0.;
  for (int p = 1; p <= 6; p++)
    for (int j = 1; j <= c->N; j++)
      for (int i = 1; i <= c->N; i++) {
        const size_t k = CI(c, i, j, p);
        const double KE = 0.5 * s->phi[k] * (s->u[k] * s->uC[k] + s->v[k] * s->vC[k]);
        const double PE = 0.5 * ((s->phi[k] + c->phis[k]) * (s->phi[k] + c->phis[k]));
        t = t + c->sqrtG[k] * (KE + PE);
      }
  return t;
}
