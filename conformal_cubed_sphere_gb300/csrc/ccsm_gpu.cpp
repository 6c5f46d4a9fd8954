// ccsm_gpu.cpp -- the reference's model program (dynamic_core/src/ccsm.F90) as a
// C++ host driver over the C ABI of libccs_gpu.so: mesh, initial state, time loop
// with history output times and the mass / energy change ratios, with the step
// itself on the GPU.  It is the host side a non-Python caller writes: every call
// below is an entry point of include/ccs_gpu.h.
//
//   ccsm_gpu --N 48 [--halo 3] [--mesh-file F] [--precision fp64|mixed]
//            [--scheme RK4|RK3_TVD] [--case 2|5|6|seeded] [--seed K] [--lmax-oro L]
//            [--dt S | --cfl C] [--radius A] [--run-days D] [--run-hours H] [--run-minutes M]
//            [--run-seconds S] [--history-interval S] [--energy-of-new-state]
//            [--autotune] [--max-courant C] [--out FILE] [--history PREFIX] [--plan]
//            [--namelist namelist.input] [--mesh-namelist FILE]
//
// Time settings follow parameters_mod.F90 (defaults :118-128; nsteps = total run
// time / dt truncated, :149); an output happens after step `it` when
// mod(it*dt, history_interval) == 0 and it*dt >= history_interval (ccsm.F90:55).
// The energy of an output line is that of the state before the last step, as
// ccsm.F90:60 computes it from stat(old), unless --energy-of-new-state.  --out
// writes phiG, u, v of the final state (FP64, the reference's array layout, one
// field after the other).  --plan prints the time settings and output steps and
// exits without touching a GPU.  Every output time runs the health check
// (ccs_check_state) and stops on a state with non-positive depth or non-finite wind;
// with --max-courant it also stops when the state's Courant number (ccs_courant)
// exceeds C.  --namelist reads the dynamic core's namelist.input
// (parameters_mod.F90:87-113: time_settings, case_select, domain; a mesh_file that
// exists is read as a raw-binary mesh file) and --mesh-namelist the mesh
// generator's (N = 90 / dx, mesh_generation/src/parameters_mod.f90:40-50); options
// after them override what they set.  --history PREFIX writes the state of every
// history time, the initial one included, as checkpoint files PREFIX_NNNN.ccsstate
// (ccs_state_write; the place of history_write_stat, ccsm.F90:44,60, whose NetCDF
// output needs a library this program does not link).
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "ccs_gpu.h"

namespace {

struct Options {
  int N = 48, halo = 3, precision = CCS_FP64, scheme = CCS_RK4, ic = CCS_IC_SEEDED, lmax_oro = 0;
  uint64_t seed = 1;
  double dt = 0., cfl = 0.5, radius = 6371229.;  // a of constants_mod.F90:9
  double max_courant = 0.;                       // 0: no Courant check
  int run_days = 1, run_hours = 0, run_minutes = 0, run_seconds = 0, history_interval = 360;
  bool energy_new = false, autotune = false, plan = false;
  std::string mesh_file, out, history;
};

// constants_mod.F90:6-12
const double kGravity = 9.80616, kOmega = 7.292e-5;

int fail(const char *what, int rc) {
  std::fprintf(stderr, "ccsm_gpu: %s: %s (%d)\n", what, ccs_strerror(rc), rc);
  return 1;
}

// Fortran namelist file -> {group: {key: value}}, names lower-cased, quotes of
// string values removed, `!` comments dropped.
using Namelist = std::map<std::string, std::map<std::string, std::string>>;

std::string lower(std::string t) {
  for (char &c : t) c = (char)std::tolower((unsigned char)c);
  return t;
}

std::string trim(const std::string &t) {
  size_t a = t.find_first_not_of(" \t\r"), b = t.find_last_not_of(" \t\r");
  return a == std::string::npos ? std::string() : t.substr(a, b - a + 1);
}

bool read_namelist(const std::string &path, Namelist &out) {
  std::ifstream f(path);
  if (!f) return false;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string text = ss.str();
  size_t i = 0;
  while ((i = text.find('&', i)) != std::string::npos) {
    size_t e = i + 1;
    while (e < text.size() && (std::isalnum((unsigned char)text[e]) || text[e] == '_')) e++;
    const std::string group = lower(text.substr(i + 1, e - i - 1));
    std::vector<std::string> toks;
    std::string cur;
    char q = 0;
    size_t j = e;
    for (; j < text.size(); j++) {
      const char ch = text[j];
      if (q) {
        cur += ch;
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
        cur += ch;
      } else if (ch == '!') {
        while (j < text.size() && text[j] != '\n') j++;
        toks.push_back(cur);
        cur.clear();
      } else if (ch == '/') {
        break;
      } else if (ch == ',' || ch == '\n') {
        toks.push_back(cur);
        cur.clear();
      } else {
        cur += ch;
      }
    }
    toks.push_back(cur);
    auto &g = out[group];
    for (const std::string &t : toks) {
      const size_t eq = t.find('=');
      if (eq == std::string::npos) continue;
      std::string v = trim(t.substr(eq + 1));
      if (v.size() >= 2 && (v[0] == '\'' || v[0] == '"') && v.back() == v[0]) v = v.substr(1, v.size() - 2);
      g[lower(trim(t.substr(0, eq)))] = v;
    }
    i = j + 1;
  }
  return true;
}

// a Fortran real (1.5, 6.0d2, 3E1) as a double
double fnum(std::string t) {
  for (char &c : t)
    if (c == 'd' || c == 'D') c = 'e';
  return std::atof(t.c_str());
}

bool file_exists(const std::string &path) {
  std::ifstream f(path);
  return (bool)f;
}

bool parse(int argc, char **argv, Options &o) {
  for (int k = 1; k < argc; k++) {
    const std::string a = argv[k];
    auto val = [&](const char *name) -> const char * {
      if (k + 1 >= argc) {
        std::fprintf(stderr, "ccsm_gpu: %s needs a value\n", name);
        std::exit(2);
      }
      return argv[++k];
    };
    if (a == "--N") o.N = std::atoi(val("--N"));
    else if (a == "--halo") o.halo = std::atoi(val("--halo"));
    else if (a == "--mesh-file") o.mesh_file = val("--mesh-file");
    else if (a == "--precision") o.precision = std::string(val("--precision")) == "mixed" ? CCS_MIXED : CCS_FP64;
    else if (a == "--scheme") o.scheme = std::string(val("--scheme")) == "RK3_TVD" ? CCS_RK3_TVD : CCS_RK4;
    else if (a == "--case") {
      const std::string c = val("--case");
      o.ic = c == "2" ? CCS_IC_CASE2 : c == "5" ? CCS_IC_CASE5 : c == "6" ? CCS_IC_CASE6 : CCS_IC_SEEDED;
    } else if (a == "--seed") o.seed = std::strtoull(val("--seed"), nullptr, 10);
    else if (a == "--lmax-oro") o.lmax_oro = std::atoi(val("--lmax-oro"));
    else if (a == "--dt") o.dt = std::atof(val("--dt"));
    else if (a == "--radius") o.radius = std::atof(val("--radius"));
    else if (a == "--cfl") o.cfl = std::atof(val("--cfl"));
    else if (a == "--run-days") o.run_days = std::atoi(val("--run-days"));
    else if (a == "--run-hours") o.run_hours = std::atoi(val("--run-hours"));
    else if (a == "--run-minutes") o.run_minutes = std::atoi(val("--run-minutes"));
    else if (a == "--run-seconds") o.run_seconds = std::atoi(val("--run-seconds"));
    else if (a == "--history-interval") o.history_interval = std::atoi(val("--history-interval"));
    else if (a == "--energy-of-new-state") o.energy_new = true;
    else if (a == "--autotune") o.autotune = true;
    else if (a == "--max-courant") o.max_courant = std::atof(val("--max-courant"));
    else if (a == "--out") o.out = val("--out");
    else if (a == "--history") o.history = val("--history");
    else if (a == "--plan") o.plan = true;
    else if (a == "--namelist") {
      const std::string path = val("--namelist");
      Namelist nml;
      if (!read_namelist(path, nml)) {
        std::fprintf(stderr, "ccsm_gpu: cannot read namelist %s\n", path.c_str());
        return false;
      }
      auto &ts = nml["time_settings"];
      if (ts.count("dt")) o.dt = fnum(ts["dt"]);
      if (ts.count("run_days")) o.run_days = std::atoi(ts["run_days"].c_str());
      if (ts.count("run_hours")) o.run_hours = std::atoi(ts["run_hours"].c_str());
      if (ts.count("run_minutes")) o.run_minutes = std::atoi(ts["run_minutes"].c_str());
      if (ts.count("run_seconds")) o.run_seconds = std::atoi(ts["run_seconds"].c_str());
      if (ts.count("history_interval")) o.history_interval = std::atoi(ts["history_interval"].c_str());
      if (ts.count("integral_scheme")) {
        const std::string sc = trim(ts["integral_scheme"]);
        if (sc != "RK4" && sc != "RK3_TVD") {  // parameters_mod.F90:146 stops here
          std::fprintf(stderr, "ccsm_gpu: unknown integral scheme %s\n", sc.c_str());
          return false;
        }
        o.scheme = sc == "RK3_TVD" ? CCS_RK3_TVD : CCS_RK4;
      }
      auto &cs = nml["case_select"];
      if (cs.count("case_num")) {
        const int c = std::atoi(cs["case_num"].c_str());
        o.ic = c == 2 ? CCS_IC_CASE2 : c == 5 ? CCS_IC_CASE5 : c == 6 ? CCS_IC_CASE6 : o.ic;
      }
      auto &dom = nml["domain"];
      if (dom.count("xhalo")) o.halo = std::atoi(dom["xhalo"].c_str());
      if (dom.count("mesh_file")) {
        const std::string mf = trim(dom["mesh_file"]);
        int fn = 0, fmap = 0;
        // the reference's own mesh_file is NetCDF (io_mod.F90:37): only a raw-binary
        // mesh file is read, anything else leaves the mesh to the generator
        if (!file_exists(mf))
          std::fprintf(stderr, "ccsm_gpu: mesh_file '%s' not found: the mesh is generated\n", mf.c_str());
        else if (ccs_mesh_file_info(mf.c_str(), &fn, &fmap) != CCS_OK)
          std::fprintf(stderr, "ccsm_gpu: mesh_file '%s' is not a raw-binary mesh file: the mesh is generated\n",
                       mf.c_str());
        else
          o.mesh_file = mf;
      }
    } else if (a == "--mesh-namelist") {
      const std::string path = val("--mesh-namelist");
      Namelist nml;
      if (!read_namelist(path, nml)) {
        std::fprintf(stderr, "ccsm_gpu: cannot read namelist %s\n", path.c_str());
        return false;
      }
      auto &dom = nml["domain"];
      const double dx = dom.count("dx") ? fnum(dom["dx"]) : 1.;
      const double n = 90. / dx;
      if (!(dx > 0.) || std::fabs(n - std::round(n)) > 1e-9) {
        std::fprintf(stderr, "ccsm_gpu: dx = %g degrees does not divide a panel edge\n", dx);
        return false;
      }
      o.N = (int)std::lround(n);
    }
    else {
      std::fprintf(stderr, "ccsm_gpu: unknown option %s\n", a.c_str());
      return false;
    }
  }
  return true;
}

struct Arrays {  // the reference's mesh and stat arrays, Fortran order
  std::vector<double> sqrtG, G, IG, A, IA, f, phis, lon, lat, sinlat, coslat;
  std::vector<double> phiG, u, v, phi, uC, vC, zonal, merid, phit;
  explicit Arrays(size_t nc)
      : sqrtG(nc), G(4 * nc), IG(4 * nc), A(4 * nc), IA(4 * nc), f(nc), phis(nc), lon(nc), lat(nc), sinlat(nc),
        coslat(nc), phiG(nc), u(nc), v(nc), phi(nc), uC(nc), vC(nc), zonal(nc), merid(nc), phit(nc) {}
  ccs_mesh_view mesh() {
    return ccs_mesh_view{sqrtG.data(), G.data(), IG.data(), A.data(), IA.data(), f.data(), phis.data()};
  }
  ccs_state_view state() {
    return ccs_state_view{phiG.data(), u.data(), v.data(), phi.data(), uC.data(), vC.data(),
                          zonal.data(), merid.data(), phit.data()};
  }
};

}  // namespace

int main(int argc, char **argv) {
  Options o;
  if (!parse(argc, argv, o)) return 2;
  // time settings (parameters_mod.F90:135, 149) and output steps (ccsm.F90:55)
  const int total = o.run_days * 86400 + o.run_hours * 3600 + o.run_minutes * 60 + o.run_seconds;

  int rc = 0;
  if (!o.mesh_file.empty()) {
    int fmap = 0;
    if ((rc = ccs_mesh_file_info(o.mesh_file.c_str(), &o.N, &fmap))) return fail("ccs_mesh_file_info", rc);
  }
  const int N = o.N, h = o.halo;
  if (N < 1 || h < 3) {
    std::fprintf(stderr, "ccsm_gpu: need N >= 1 and halo >= 3\n");
    return 2;
  }
  const size_t ns = (size_t)N * N * 6, nc = (size_t)(N + 2 * h) * (N + 2 * h) * 6;
  std::vector<double> flon(ns), flat(ns), fx(ns), fy(ns), fz(ns), fjab(6 * ns);
  if (!o.mesh_file.empty())
    rc = ccs_mesh_load(o.mesh_file.c_str(), N, flon.data(), flat.data(), fx.data(), fy.data(), fz.data(),
                       fjab.data());
  else
    rc = ccs_mesh_generate(N, CCS_MAP_CONFORMAL, flon.data(), flat.data(), fx.data(), fy.data(), fz.data(),
                           fjab.data());
  if (rc) return fail("mesh", rc);
  Arrays a(nc);
  rc = ccs_mesh_derive(N, h, o.radius, kOmega, flon.data(), flat.data(), fx.data(), fy.data(), fz.data(),
                       fjab.data(), a.sqrtG.data(), a.G.data(), a.IG.data(), a.A.data(), a.IA.data(), a.f.data(),
                       a.lon.data(), a.lat.data(), a.sinlat.data(), a.coslat.data());
  if (rc) return fail("ccs_mesh_derive", rc);
  // initTestCase
  ccs_ic_params p{};
  p.kind = o.ic;
  p.lmax_h = 12;
  p.lmax_psi = 12;
  p.lmax_oro = o.lmax_oro;
  p.seed = o.seed;
  p.h0 = 8000.;
  p.h_rms = 200.;
  p.wind_max = 40.;
  p.oro_rms = 1000.;
  p.oro_max = 2000.;
  rc = ccs_initial_condition(N, h, o.radius, kGravity, kOmega, &p, a.lon.data(), a.lat.data(), a.sinlat.data(),
                             a.coslat.data(), a.phi.data(), a.zonal.data(), a.merid.data(), a.phis.data());
  if (rc) return fail("ccs_initial_condition", rc);
  ccs_mesh_view mv = a.mesh();
  ccs_state_view sv = a.state();
  if ((rc = ccs_state_from_sphere(N, h, &mv, &sv))) return fail("ccs_state_from_sphere", rc);
  const double dx = (90. / N) * (std::acos(-1.) / 180.);
  const double dt = o.dt > 0. ? o.dt : ccs_cfl_dt(N, h, o.cfl, dx, dx, &mv, &sv);
  const int nsteps = (int)(total / dt);
  const int total_output_num = (int)(nsteps * dt / o.history_interval);
  std::vector<int> outputs;
  for (int it = 1; it <= nsteps; it++) {
    const double t = it * dt;
    if (std::fmod(t, (double)o.history_interval) == 0. && t >= o.history_interval) outputs.push_back(it);
  }
  std::printf(" Temporal integration scheme is %s\n", o.scheme == CCS_RK4 ? "RK4" : "RK3_TVD");
  std::printf(" N %d halo %d dt %.17g nsteps %d outputs %zu\n", N, h, dt, nsteps, outputs.size());
  if (o.plan) {
    for (int it : outputs) std::printf(" output step %d\n", it);
    return 0;
  }

  ccs_config cfg{};
  cfg.N = N;
  cfg.halo = h;
  cfg.scheme = o.scheme;
  cfg.precision = o.precision;
  cfg.e_dissipation = CCS_EDISS_ZERO;
  cfg.device = 0;
  cfg.dx = dx;
  cfg.dy = dx;
  cfg.dt = dt;
  cfg.radius = o.radius;
  cfg.gravity = kGravity;
  cfg.omega = kOmega;
  cfg.phi_mean = 0.;
  ccs_handle *hd = nullptr;
  if ((rc = ccs_init(&cfg, &mv, &hd))) return fail("ccs_init", rc);
  auto done = [&](int code) {
    ccs_destroy(hd);
    return code;
  };
  if ((rc = ccs_set_state(hd, &sv))) return done(fail("ccs_set_state", rc));
  if (o.autotune) {
    int chosen = 0;
    if ((rc = ccs_autotune(hd, 3, 0, &chosen, nullptr))) return done(fail("ccs_autotune", rc));
  }
  double mass0 = 0., energy0 = 0.;
  if ((rc = ccs_diag(hd, &mass0, &energy0))) return done(fail("ccs_diag", rc));
  // history output (ccsm.F90:44,60): the state as ccs_get_state gives it
  auto write_history = [&](int idx) -> int {
    if (o.history.empty()) return 0;
    int r = ccs_get_state(hd, &sv);
    if (r) return fail("ccs_get_state", r);
    char name[32];
    std::snprintf(name, sizeof(name), "_%04d.ccsstate", idx);
    if ((r = ccs_state_write((o.history + name).c_str(), N, h, &sv))) return fail("ccs_state_write", r);
    return 0;
  };
  if (write_history(1)) return done(1);
  std::printf(" output index/total, MCR, ECR : %d / %d   %.17g %.17g\n", 0, total_output_num, 0., 0.);
  int stepped = 0;
  for (size_t k = 0; k < outputs.size(); k++) {
    const int it = outputs[k];
    double mass = 0., energy = 0., tmp = 0.;
    if (o.energy_new) {
      if ((rc = ccs_step(hd, it - stepped))) return done(fail("ccs_step", rc));
      if ((rc = ccs_diag(hd, &mass, &energy))) return done(fail("ccs_diag", rc));
    } else {
      if (it - stepped > 1 && (rc = ccs_step(hd, it - stepped - 1))) return done(fail("ccs_step", rc));
      if ((rc = ccs_diag(hd, &tmp, &energy))) return done(fail("ccs_diag", rc));  // stat(old)
      if ((rc = ccs_step(hd, 1))) return done(fail("ccs_step", rc));
      if ((rc = ccs_diag(hd, &mass, &tmp))) return done(fail("ccs_diag", rc));
    }
    stepped = it;
    int64_t nbad = 0;
    if (ccs_check_state(hd, &nbad) == CCS_ERR_NAN) {
      std::fprintf(stderr, "ccsm_gpu: step %d: %lld cells with non-positive depth or non-finite wind\n", it,
                   (long long)nbad);
      return done(1);
    }
    if (o.max_courant > 0.) {
      double courant = 0.;
      rc = ccs_courant(hd, &courant);
      if (rc && rc != CCS_ERR_NAN) return done(fail("ccs_courant", rc));
      if (!(courant <= o.max_courant)) {
        std::fprintf(stderr, "ccsm_gpu: step %d: Courant number %.4g above %.4g\n", it, courant, o.max_courant);
        return done(1);
      }
    }
    if (write_history((int)k + 2)) return done(1);  // history_write_stat(stat(new), output_idx)
    std::printf(" output index/total, MCR, ECR : %zu / %d   %.17g %.17g\n", k + 1, total_output_num,
                (mass - mass0) / mass0, (energy - energy0) / energy0);
  }
  if (nsteps > stepped && (rc = ccs_step(hd, nsteps - stepped))) return done(fail("ccs_step", rc));
  if (!o.out.empty()) {
    if ((rc = ccs_get_state(hd, &sv))) return done(fail("ccs_get_state", rc));
    FILE *fp = std::fopen(o.out.c_str(), "wb");
    if (!fp) return done(fail("--out", CCS_ERR_IO));
    bool ok = std::fwrite(a.phiG.data(), sizeof(double), nc, fp) == nc &&
              std::fwrite(a.u.data(), sizeof(double), nc, fp) == nc &&
              std::fwrite(a.v.data(), sizeof(double), nc, fp) == nc;
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) return done(fail("--out", CCS_ERR_IO));
  }
  std::printf(" steps %d done\n", nsteps);
  return done(0);
}
