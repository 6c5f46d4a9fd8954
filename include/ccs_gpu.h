/*
 * ccs_gpu.h -- C ABI of the GB300 (sm_103a) shallow-water step on the conformal
 * cubed sphere.  Drop-in for the FP64 CPU step of DwyaneChou/Conformal_Cubed_Sphere.
 *
 * The reference has no FFI of its own: its host driver calls Fortran module
 * procedures that share module globals (bounds, mesh, stat, tend, dt).  Each entry
 * point below names the Fortran procedure or call site it replaces, so that a
 * Fortran ISO_C_BINDING interface (or a ctypes / cgo stub) binds one-to-one.
 *
 * Conventions
 *  - Every array is FP64, Fortran column-major, exactly as the reference stores it
 *    (stat_mod.F90:7-17, mesh_mod.F90:17-33): cell fields are (ics:ice, jcs:jce, 1:6)
 *    with ics = jcs = 1 - halo and ice = jce = N + halo; 2x2 metric matrices are
 *    (2, 2, ics:ice, ics:ice, 1:6); the Jacobian is (3, 2, ics:ice, ics:ice, 1:6).
 *  - The caller owns host arrays.  The library copies in (ccs_init, ccs_set_state)
 *    and out (ccs_get_state, ccs_spatial_operator) and keeps no host pointer past a
 *    call.  It owns its device buffers until ccs_destroy.
 *  - Every function returns a status code (CCS_OK = 0) and never exits the process;
 *    a Fortran shim maps non-zero codes to its own `stop`, as io_mod.F90:604-612 and
 *    parameters_mod.F90:146 do.
 *  - A handle is not re-entrant.  Separate handles run on separate CUDA streams and
 *    are independent.
 */
#ifndef CCS_GPU_H
#define CCS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CCS_ABI_VERSION 1

/* status codes */
enum {
  CCS_OK = 0,
  CCS_ERR_ARG = 1,         /* bad argument, bounds or configuration */
  CCS_ERR_CUDA = 2,        /* a CUDA runtime call failed (ccs_last_error has the text) */
  CCS_ERR_NAN = 3,         /* non-finite or negative-depth state detected by the health check */
  CCS_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
  CCS_ERR_UNSUPPORTED = 5, /* option not available in this build */
  CCS_ERR_MESH = 6,        /* singular metric (io_mod.F90:176-188 stops here) */
  CCS_ERR_NOMEM = 7,       /* device or host allocation failed */
  CCS_ERR_NODEVICE = 8,    /* no CUDA device visible */
  CCS_ERR_TOO_LARGE = 9,   /* size above a fixed capacity (ccs_diag_noalloc) */
  CCS_ERR_IO = 10          /* mesh file missing, unreadable, truncated or not in this format */
};

/* integral_scheme (parameters_mod.F90:402-408) */
enum { CCS_RK4 = 0, CCS_RK3_TVD = 1 };

/* arithmetic lane */
enum {
  CCS_FP64 = 0, /* the reference arithmetic, operation for operation (parity lane) */
  CCS_MIXED = 1 /* FP32 state and stencil arithmetic, FP64 metric and edge transforms */
};

/* The E-flux dissipation of spatial_operators_mod.F90:119,144 reads face slots of
 * u_ext / v_ext that the reference never writes (u is reconstructed only at
 * y-faces, v only at x-faces).  ZERO reads them as 0.0, i.e. E at a face is the
 * plain average of its two reconstructions (what a freshly zeroed scratch gives).
 * RECONSTRUCT fills them with WENO reconstructions of u at x-faces and v at y-faces
 * (both lanes). */
enum { CCS_EDISS_ZERO = 0, CCS_EDISS_RECONSTRUCT = 1 };

/* spatial operator.  The reference ships four interchangeable modules of the same
 * name and compiles one of them: spatial_operators_mod.F90 (WENO-Z reconstruction
 * with Rusanov face fluxes, the default) and the centred-difference modules
 * spatial_operators_mod_2nd.F90, _4th.F90 and _6th.F90.  The CENTRAL values are the
 * order of accuracy. */
enum { CCS_OP_WENO = 0, CCS_OP_CENTRAL2 = 2, CCS_OP_CENTRAL4 = 4, CCS_OP_CENTRAL6 = 6 };

/* cube-to-sphere map used by the host mesh generator: the conformal cubic map of
 * the reference mesh generator (gen_method 'Rancic', mesh_generation/src/
 * mesh_mod.f90:150-171) or the equiangular gnomonic map */
enum { CCS_MAP_GNOMONIC_EQUIANGULAR = 0, CCS_MAP_CONFORMAL = 1 };

typedef struct ccs_config {
  int N;             /* cells along a panel edge: its = 1, ite = N (io_mod.F90:49-52) */
  int halo;          /* xhalo = yhalo (parameters_mod.F90:98-99); at least 3 */
  int scheme;        /* CCS_RK4 or CCS_RK3_TVD */
  int precision;     /* CCS_FP64 or CCS_MIXED */
  int e_dissipation; /* CCS_EDISS_ZERO (reference dataflow) or CCS_EDISS_RECONSTRUCT */
  int device;        /* CUDA device ordinal */
  double dx, dy;     /* cell widths in radians (io_mod.F90:54-55) */
  double dt;         /* time step in seconds (parameters_mod.F90:13) */
  double radius;     /* sphere radius a (m); the reference fixes 6371229 */
  double gravity;    /* g (m s-2) */
  double omega;      /* rotation rate (s-1) */
  double phi_mean;   /* mixed lane: reference geopotential; <= 0 means the mean of
                        the interior phi at ccs_set_state */
} ccs_config;

/* The metric arrays the step reads: mesh_mod.F90:17-33 after io_mod.read_mesh. */
typedef struct ccs_mesh_view {
  const double *sqrtG;    /* (ics:ice, ics:ice, 6) */
  const double *matrixG;  /* (2, 2, ics:ice, ics:ice, 6) */
  const double *matrixIG; /* (2, 2, ...) */
  const double *matrixA;  /* (2, 2, ...) */
  const double *matrixIA; /* (2, 2, ...) */
  const double *f;        /* (ics:ice, ics:ice, 6); interior values used */
  const double *phis;     /* (ics:ice, ics:ice, 6) surface geopotential */
} ccs_mesh_view;

/* stat_field (stat_mod.F90:7-17).  On input phiG, u, v, phi, uC, vC are required and
 * zonal_wind / meridional_wind are optional (kept for ccs_get_state before a step);
 * phit is never read.  On output every non-NULL pointer except phit is written
 * (the reference step never assigns stat%phit). */
typedef struct ccs_state_view {
  double *phiG, *u, *v, *phi, *uC, *vC, *zonal_wind, *meridional_wind, *phit;
} ccs_state_view;

typedef struct ccs_handle ccs_handle;
typedef struct ccs_batch ccs_batch;

/* ---- lifecycle ---------------------------------------------------------- */

/* Replaces read_mesh (io_mod.F90:15-307) + initStat/initTend (stat_mod.F90:22,
 * tend_mod.F90:17) on the device side: validates the configuration, uploads the
 * metric arrays and allocates the state slots. */
int ccs_init(const ccs_config *cfg, const ccs_mesh_view *mesh, ccs_handle **out);

/* Same, but shares the device mesh of `mesh_owner` (an ensemble member on the same
 * grid).  `cfg` must agree with the owner on N, halo, dx, dy and device. */
int ccs_init_shared(const ccs_config *cfg, ccs_handle *mesh_owner, ccs_handle **out);

/* Releases everything.  Members sharing a mesh keep it alive until the last one
 * is destroyed. */
void ccs_destroy(ccs_handle *h);

/* ---- state -------------------------------------------------------------- */

/* Uploads stat(old) (initTestCase output, test_case_mod.F90:13-58, or a restart). */
int ccs_set_state(ccs_handle *h, const ccs_state_view *s);

/* Downloads stat(old) after the last completed step (what ccsm.F90:66 leaves in
 * stat(old) and stat(new)). */
int ccs_get_state(ccs_handle *h, ccs_state_view *s);

/* ---- the step ----------------------------------------------------------- */

/* Replaces the time loop body of ccsm.F90:50-67 `nsteps` times:
 * call RK4(stat(new), stat(old)) (time_scheme_mod.F90:13-44) or RK3_TVD
 * (time_scheme_mod.F90:46-67), then copyStat(stat(old), stat(new)).
 * Synchronous: returns after the device finished. */
int ccs_step(ccs_handle *h, int nsteps);

/* Same, enqueued on the handle's stream; ccs_sync waits for it. */
int ccs_step_async(ccs_handle *h, int nsteps);
int ccs_sync(ccs_handle *h);

/* ccs_set_state / ccs_get_state without the final wait: the copies and conversion
 * kernels are enqueued in order with the handle's steps, and the host arrays must
 * stay valid (and, for set, unchanged) until ccs_sync returns.  On the mixed lane
 * the copies run on two copy streams with double-buffered device staging, so a loop
 * of set_async / step_async / get_async overlaps the upload of one state and the
 * download of the previous result with the step in between; pass page-locked host
 * arrays for the copies to be asynchronous.  Fields whose host arrays are
 * consecutive slices of one block (each nh*nh*6 doubles, in the order phi, u, v for
 * set and phiG, u, v, phi, uC, vC, zonal_wind, meridional_wind for get) move in one
 * copy per run; the host link overlaps one large upload and one large download
 * better than many smaller copies.  No counterpart in the reference. */
int ccs_set_state_async(ccs_handle *h, const ccs_state_view *s);
int ccs_get_state_async(ccs_handle *h, ccs_state_view *s);

/* Selects the spatial operator of the handle's steps (default CCS_OP_WENO): the
 * choice the reference makes at build time by compiling one of its four
 * spatial_operators_mod sources.  Both lanes (the FP64 lane operation for
 * operation, the mixed lane in FP32 like its WENO operator); a batch copies its
 * members' operators when it is created.  No counterpart call in the reference. */
int ccs_set_operator(ccs_handle *h, int op);

/* ---- kernel variants and the autotuner (no counterpart in the reference) ----
 * Each lane's stage kernel comes in variants: FP64 lane tile shapes (cells per
 * work item) 0: 32x8, 1: 16x16, 2: 64x4; mixed lane tile shape and halo-staging
 * schedule 0: 32x32 and 1: 32x16 with per-thread loads (each thread loads its
 * cells' raw inputs into registers and stores the derived quantities), 2: 32x32
 * and 3: 32x16 with asynchronous copies (the raw inputs of all of a thread's cells
 * go into shared memory at once, then are derived in place).  Every variant
 * computes the same per-cell arithmetic, so results do not depend on the choice.  ccs_autotune times the handle's RK stages before the last one (they write
 * only stage scratch, so the state is unchanged), `reps` rounds with each variant
 * after one warm-up launch, and keeps the fastest mean stage time; the choice is cached per (device, lane, N,
 * halo) for the process, and later calls with force = 0 reuse it without timing.
 * The state must be set first.  chosen (may be NULL) receives the variant,
 * times_us (may be NULL, CCS_MAX_VARIANTS entries) the mean launch times in
 * microseconds (0 where nothing was timed).  A batch groups its members by
 * variant, so tune members before ccs_batch_create. */
#define CCS_MAX_VARIANTS 4
int ccs_autotune(ccs_handle *h, int reps, int force, int *chosen, double *times_us);
int ccs_set_variant(ccs_handle *h, int variant);
int ccs_get_variant(ccs_handle *h, int *variant, int *tile_x, int *tile_y);

/* spatial_operator(stat(old), tend) (spatial_operators_mod.F90:13-181): the
 * tendencies of phiG, u, v of the current state, interior cells (halo and corner
 * entries of the outputs are set to 0).  Any output pointer may be NULL. */
int ccs_spatial_operator(ccs_handle *h, double *tend_phiG, double *tend_u, double *tend_v);

/* Health check of the current state: the number of interior cells whose depth is
 * not positive (NaN included) or whose covariant wind is not finite, in bad_cells
 * (may be NULL); returns CCS_ERR_NAN when there is one, CCS_OK otherwise.  The
 * reference has no such check (a blown-up run goes on with NaNs). */
int ccs_check_state(ccs_handle *h, int64_t *bad_cells);

/* Courant number of the handle's current state: dt * max over interior and
 * edge-halo cells of max(|uC| + sqrt(IG11 phit), |vC| + sqrt(IG22 phit)) /
 * min(dx, dy), phit = phi + phis, evaluated on the device in FP64 (the largest
 * wave speed ccs_cfl_dt takes on the host).  A cell with non-positive phit or a
 * non-finite value makes it +inf and the call return CCS_ERR_NAN.  No counterpart in
 * the reference (its time step is a namelist constant). */
int ccs_courant(ccs_handle *h, double *courant);

/* calc_total_mass / calc_total_energy (diag_mod.F90:10-53) of the current state,
 * as FP64 sums on the device. */
int ccs_diag(ccs_handle *h, double *total_mass, double *total_energy);

/* Total mass and energy, like ccs_diag, of a state that already lives in device
 * memory, without allocating anything.  This entry point has no counterpart in the
 * reference.  It serves callers that cannot call cudaMalloc: a model driver that
 * runs inside another framework's memory pool, or under a device arena sized once
 * at start-up, must not allocate behind that pool's back.  All array arguments are
 * device pointers in the reference layout (ics:ice, jcs:jce, 6); mass_energy is a
 * device pointer to two doubles; stream is a cudaStream_t of the current device
 * (NULL for the legacy default stream; a stream of another device returns
 * CCS_ERR_ARG) and the call returns once the work is enqueued, with the status of
 * its own launches only.  Its scratch is a fixed device array sized for N up to
 * CCS_NOALLOC_MAX_N (larger N returns CCS_ERR_TOO_LARGE); every GPU that loads the
 * library holds that array until exit.  The first call on a device looks up the
 * array's device address, so make it before any stream capture.  All calls share
 * the array: calls that overlap on the GPU race, so order them on one stream. */
#define CCS_NOALLOC_MAX_N 4096
int ccs_diag_noalloc(int N, int halo, const double *phiG, const double *phi, const double *u,
                     const double *v, const double *uC, const double *vC, const double *sqrtG,
                     const double *phis, double *mass_energy, void *stream);

/* ---- ensembles and uneven batches ---------------------------------------- */

/* Groups handles (any mix of N, dt and lanes) so that each RK stage of all members
 * runs as one launch per group over a shared work list, captured in a CUDA graph.
 * The members of a group share the lane, the RK scheme, the operator family (WENO-Z
 * or central differences) and the E-flux option: an ensemble, or an uneven mix of
 * resolutions on both lanes, runs one launch per lane and RK stage.  A group runs
 * one tile variant for all its members, at first the variant of its member with the
 * most cells (tune members before creating the batch), or the one
 * ccs_batch_autotune picks by timing the group's own work list.  A batch step is
 * ordered after each member's pending work on its own stream (an asynchronous
 * upload and its import, an asynchronous step), and each member's later work after
 * the batch step, so the members' *_async calls and ccs_batch_step_async compose in
 * call order.  The batch keeps each member's operator as it was at creation, and
 * the members must outlive it (ccs_batch_destroy first).  The reference advances
 * one grid per program run (ccsm.F90:50-67); batches have no counterpart there. */
int ccs_batch_create(ccs_handle *const *members, int n, ccs_batch **out);
int ccs_batch_step(ccs_batch *b, int nsteps);
/* Same, enqueued on the batch's stream (ccs_batch_stream) without waiting. */
int ccs_batch_step_async(ccs_batch *b, int nsteps);
void *ccs_batch_stream(ccs_batch *b);
/* Times every tile variant of each group on the group's work list (the RK stages
 * before the last, which leave the members' states unchanged; `reps` rounds after
 * one warm-up launch) and keeps the fastest per group.  Results do not depend on
 * the variant. */
int ccs_batch_autotune(ccs_batch *b, int reps);
/* launches_per_stage (may be NULL): the number of groups, one launch each per RK
 * stage; for the first max_groups groups, lane (CCS_FP64 / CCS_MIXED), tile variant
 * and member count (each array may be NULL). */
int ccs_batch_info(ccs_batch *b, int *launches_per_stage, int max_groups, int *lane, int *variant, int *members);
/* Text of the last CUDA error a batch call met ("" if none). */
const char *ccs_batch_last_error(const ccs_batch *b);
void ccs_batch_destroy(ccs_batch *b);

/* ---- introspection -------------------------------------------------------- */

/* CubedSphereFillHalo (ghost_mod.f90:18-82) as an index map: for every cell of a
 * (ics:ice, jcs:jce, 6) array, the 0-based linear index (same layout) of the cell
 * whose value the fill copies there; interior cells map to themselves and the
 * never-filled corner blocks to -1.  Computed from the tables the kernels use. */
int ccs_ghost_map(int N, int halo, int64_t *src_index);

/* Device time spent in this handle's stage kernels since the last reset, measured
 * with CUDA events on the handle's stream when timing is enabled. */
int ccs_timing(ccs_handle *h, int enable, int reset, double *kernel_ms, int64_t *launches);

/* Self-check of the FP64 lane's division by the constants 3, 6 and 12: for each
 * x[k] the device computes the correctly rounded quotient the kernels use (fast[k])
 * and the IEEE quotient x[k] / b (ieee[k]); they must agree bit for bit.  Runs on
 * device 0 with temporary buffers. */
int ccs_selftest_div(const double *x, int64_t n, double b, double *fast, double *ieee);

/* Self-check of the FP64 lane's division by a divisor several quotients share (the
 * WENO-Z weights alpha_k / sum(alpha)): for each pair the device computes the
 * quotient the kernels use, from the divisor's IEEE reciprocal and one FMA
 * correction (fast[k]), and the IEEE quotient a[k] / b[k] (ieee[k]); they must agree
 * bit for bit when the quotient is a normal number.  Runs on device 0 with temporary
 * buffers. */
int ccs_selftest_div_pairs(const double *a, const double *b, int64_t n, double *fast, double *ieee);

/* Bounds-checked build (libccs_gpu.so built with -DCCS_BOUNDS, build.build_bounds):
 * the kernels check their array indices and skip, instead of performing, any access
 * outside its array, recording the first such index.  ccs_debug_bounds waits for
 * the current device, returns the first recorded check site (0: none) and index
 * since its last call and clears them; in the normal build it sets *site = -1.
 * ccs_debug_bounds_selftest checks the recording path with a kernel that tests an
 * out-of-range index and accesses nothing (CCS_ERR_UNSUPPORTED in the normal
 * build).  No counterpart in the reference (its DEBUG builds add -fcheck=all,
 * CMakeLists.txt:9,17). */
int ccs_debug_bounds(int *site, int64_t *index);
int ccs_debug_bounds_selftest(void);

/* The CUDA stream (a cudaStream_t) every launch of this handle is ordered on, so
 * that a caller can place its own events or copies before and after a step. */
void *ccs_stream(ccs_handle *h);

const char *ccs_strerror(int status);
const char *ccs_last_error(const ccs_handle *h);
int ccs_abi_version(void);

/* ---- host mesh and initial state (run once at set-up, CPU only) ---------- */

/* Mesh-file contents at the N x N x 6 cell centres (the even points of the
 * extended grid written by mesh_generation/src/output_mod.f90:25-86): lon/lat in
 * degrees, x/y/z on the unit sphere, jab (3, 2, N, N, 6) the derivative of x/y/z
 * with respect to the panel angle coordinates in radians
 * (mesh_generation/src/mesh_mod.f90:164).  Panel numbering and orientation follow
 * mesh_generation/src/cuco.f90:17-36. */
int ccs_mesh_generate(int N, int map, double *lon_deg, double *lat_deg, double *x,
                      double *y, double *z, double *jab);

/* Raw-binary mesh file, for machines without libnetcdf: the global attributes that
 * read_mesh takes from the NetCDF mesh file (io_mod.F90:36-47: dx, dy in degrees,
 * ids, ide, jds, jde, ifs, ife) and the cell-centre samples of its lon, lat, x, y, z
 * and jab variables (:87-101), little-endian, Fortran order, in the layout of
 * ccs_mesh_generate.  Header: 8-byte magic "CCSMESH\1", ten int32 (version 1, N, map,
 * ids, ide, jds, jde, ifs, ife, 0), two float64 (dx, dy); then lon, lat, x, y, z
 * (N*N*6 float64 each) and jab (6*N*N*6).  ccs_mesh_file_info reads N (and the map
 * id, if map is non-NULL) so the caller can size the arrays for ccs_mesh_load;
 * ccs_mesh_load fails with CCS_ERR_ARG when the file's N differs from N, and with
 * CCS_ERR_IO on a missing, short, over-long or foreign file. */
int ccs_mesh_save(const char *path, int N, int map, const double *lon_deg, const double *lat_deg,
                  const double *x, const double *y, const double *z, const double *jab);
int ccs_mesh_file_info(const char *path, int *N, int *map);
int ccs_mesh_load(const char *path, int N, double *lon_deg, double *lat_deg, double *x, double *y,
                  double *z, double *jab);

/* Checkpoint files (the reference writes NetCDF history only and has no restart):
 * the eight stat fields phiG, u, v, phi, uC, vC, zonal_wind, meridional_wind in the
 * reference's layout behind a header (magic "CCSSTAT\1", int32 version 1, N, halo,
 * 8).  ccs_state_read fails with CCS_ERR_ARG when the file's N or halo differ and
 * CCS_ERR_IO on a missing, short, over-long or foreign file.  Writing the state of an
 * FP64-lane handle and setting it again resumes the run bit for bit. */
int ccs_state_write(const char *path, int N, int halo, const ccs_state_view *s);
int ccs_state_read(const char *path, int N, int halo, ccs_state_view *s);

/* io_mod.F90:119-220, 295-306: halo fill of the samples and per-cell G = J^T J,
 * G^-1, sqrt(det G), A = S J, A^-1 (pole cases included), f = 2 Omega sin(lat).
 * Outputs are (ics:ice, ics:ice, 6) / (2, 2, ...) arrays; corner-block matrices are
 * 0.  lon/lat/sinlat/coslat outputs (radians) may be NULL. */
int ccs_mesh_derive(int N, int halo, double radius, double omega,
                    const double *lon_deg, const double *lat_deg, const double *x,
                    const double *y, const double *z, const double *jab, double *sqrtG,
                    double *matrixG, double *matrixIG, double *matrixA, double *matrixIA,
                    double *f, double *lon, double *lat, double *sinlat, double *coslat);

/* ccs_mesh_derive with options.  CCS_MESH_POLE_INVERSE: at a cell centred on a pole
 * (odd N) A^-1 is the inverse of A, like at every other cell, instead of the
 * reference's analytic formula (io_mod.F90:190-210), which multiplies the
 * longitude rotation by the radius where every other A^-1 scales as 1/radius and
 * makes an odd-N run blow up in its first step.  Not the reference's arithmetic:
 * off by default (ccs_mesh_derive). */
enum { CCS_MESH_POLE_INVERSE = 1 };
int ccs_mesh_derive_ex(int N, int halo, double radius, double omega, int flags,
                       const double *lon_deg, const double *lat_deg, const double *x,
                       const double *y, const double *z, const double *jab, double *sqrtG,
                       double *matrixG, double *matrixIG, double *matrixA, double *matrixIA,
                       double *f, double *lon, double *lat, double *sinlat, double *coslat);

/* Initial states: the reference test cases of test_case_mod.F90 (2: steady zonal
 * geostrophic flow :61-95, 5: isolated mountain :98-144, 6: Rossby-Haurwitz wave
 * :147-204) and a seeded random state of spherical harmonics. */
enum { CCS_IC_CASE2 = 2, CCS_IC_CASE5 = 5, CCS_IC_CASE6 = 6, CCS_IC_SEEDED = 100 };

typedef struct ccs_ic_params {
  int kind;          /* CCS_IC_* */
  int lmax_h;        /* seeded: height perturbation degrees 1..lmax_h (12) */
  int lmax_psi;      /* seeded: streamfunction degrees 1..lmax_psi (12) */
  int lmax_oro;      /* seeded: orography degrees 1..lmax_oro (8); 0 = flat */
  uint64_t seed;     /* seeded: PRNG seed (member k of an ensemble uses seed + k) */
  double h0;         /* seeded: mean depth (m), 8000 */
  double h_rms;      /* seeded: perturbation RMS over the interior cells (m), 200 */
  double wind_max;   /* seeded: maximum interior wind speed (m/s), 40 */
  double oro_rms;    /* seeded: orography field RMS before clipping (m), 1000 */
  double oro_max;    /* seeded: orography clipped to [0, oro_max] (m), 2000 */
} ccs_ic_params;

/* phi (geopotential of the fluid depth), zonal / meridional wind and phis on the
 * full halo'd array, evaluated at each cell's own lon/lat as initTestCase does
 * (halo cells carry their source cell's lon/lat). */
int ccs_initial_condition(int N, int halo, double radius, double gravity, double omega,
                          const ccs_ic_params *p, const double *lon, const double *lat,
                          const double *sinlat, const double *coslat, double *phi,
                          double *zonal_wind, double *meridional_wind, double *phis);

/* test_case_mod.F90:38-48: phiG = phi sqrtG, (u, v) = G IA (zonal, meridional),
 * (uC, vC) = IA (zonal, meridional) over the full array.  Reads s->phi,
 * s->zonal_wind, s->meridional_wind; writes s->phiG, u, v, uC, vC. */
int ccs_state_from_sphere(int N, int halo, const ccs_mesh_view *mesh, ccs_state_view *s);

/* CFL-limited step: cfl * min(dx, dy) / max over interior and edge-halo cells of
 * max(|uC| + sqrt(IG11 phit), |vC| + sqrt(IG22 phit)), phit = phi + phis. */
double ccs_cfl_dt(int N, int halo, double cfl, double dx, double dy, const ccs_mesh_view *mesh,
                  const ccs_state_view *s);

#ifdef __cplusplus
}
#endif

#endif /* CCS_GPU_H */
