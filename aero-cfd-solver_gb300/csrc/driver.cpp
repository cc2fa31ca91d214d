// driver.cpp -- case-level driver of the device path (include/aero_driver.h): the "cuda"
// branch of run_case / run_euler_airfoil_case with the reference's outputs.
#include "../../include/aero_batch.h"
#include "../../include/aero_driver.h"
#include "../../include/aero_gb300.h"
#include "../../include/aero_mesh.h"

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace fs = std::filesystem;

namespace {

thread_local std::string g_driver_error;
// State file: this magic, int64 cell count, int64 components (5), then [N][5] doubles in the
// reference's cell order and AoS layout, host byte order (little-endian on the targets).
constexpr char kStateMagic[16] = {'A', 'E', 'R', 'O', '-', 'S', 'T', 'A', 'T', 'E', '-', 'v', '1', 0, 0, 0};
const char* kVersion = "0.1.1";  // version string written to run.log (version.hpp of the reference)

// ---------------------------------------------------------------------------------------
// case file (residual_stub.cpp:148-296)
// ---------------------------------------------------------------------------------------
std::string trim(const std::string& v) {
  size_t b = 0, e = v.size();
  while (b < e && std::isspace(static_cast<unsigned char>(v[b]))) ++b;
  while (e > b && std::isspace(static_cast<unsigned char>(v[e - 1]))) --e;
  return v.substr(b, e - b);
}

std::string lower(std::string v) {
  std::transform(v.begin(), v.end(), v.begin(), [](unsigned char c) { return static_cast<char>(std::tolower(c)); });
  return v;
}

using KV = std::unordered_map<std::string, std::string>;

KV parse_kv(const fs::path& path) {
  KV kv;
  std::ifstream in(path);
  std::string line;
  while (std::getline(in, line)) {
    const std::string s = trim(line);
    if (s.empty() || s[0] == '#') continue;
    size_t sep = s.find('=');
    if (sep == std::string::npos) sep = s.find(':');
    if (sep == std::string::npos) continue;
    const std::string k = trim(s.substr(0, sep));
    if (!k.empty()) kv[k] = trim(s.substr(sep + 1));
  }
  return kv;
}

std::string get_s(const KV& kv, const char* key, const std::string& fb) {
  auto it = kv.find(key);
  return (it == kv.end() || it->second.empty()) ? fb : it->second;
}
bool has(const KV& kv, const char* key) { return kv.count(key) != 0; }
float get_f(const KV& kv, const char* key, float fb) {
  auto it = kv.find(key);
  if (it == kv.end()) return fb;
  try {
    return std::stof(it->second);
  } catch (...) {
    return fb;
  }
}
int get_i(const KV& kv, const char* key, int fb) {
  auto it = kv.find(key);
  if (it == kv.end()) return fb;
  try {
    return std::stoi(it->second);
  } catch (...) {
    return fb;
  }
}
bool on_off(const std::string& v, bool fb) {
  const std::string n = lower(trim(v));
  if (n == "on" || n == "true" || n == "yes" || n == "1") return true;
  if (n == "off" || n == "false" || n == "no" || n == "0") return false;
  return fb;
}

// Float-valued settings are parsed as float (std::stof) like the reference and widened.
void map_case(const KV& kv, aero_case_desc* c, aero_airfoil_mesh_cfg* m) {
  aero_case_defaults(c);
  auto F = [&](const char* key, double cur) { return static_cast<double>(get_f(kv, key, static_cast<float>(cur))); };
  c->iterations = get_i(kv, "iterations", c->iterations);
  c->min_iterations = get_i(kv, "min_iterations", c->min_iterations);
  c->cfl_start = F("cfl_start", c->cfl_start);
  c->cfl_max = F("cfl_max", c->cfl_max);
  c->cfl_ramp_iters = get_i(kv, "cfl_ramp_iters", c->cfl_ramp_iters);
  c->residual_reduction_target = F("residual_reduction_target", c->residual_reduction_target);
  c->force_stability_tol = F("force_stability_tol", c->force_stability_tol);
  c->force_stability_window = get_i(kv, "force_stability_window", c->force_stability_window);
  c->force_mean_drift_tol = F("force_mean_drift_tol", c->force_mean_drift_tol);
  c->startup_first_order_iters = get_i(kv, "startup_first_order_iters", c->startup_first_order_iters);
  c->rk_stages = get_i(kv, "rk_stages", c->rk_stages);
  c->local_time_stepping = on_off(get_s(kv, "local_time_stepping", c->local_time_stepping ? "on" : "off"),
                                  c->local_time_stepping != 0);
  c->gamma = F("gamma", c->gamma);
  c->gas_constant = F("gas_constant", c->gas_constant);
  c->mach = F("mach", c->mach);
  c->aoa_deg = F("aoa_deg", c->aoa_deg);
  c->p_inf = F("p_inf", c->p_inf);
  c->t_inf = F("t_inf", c->t_inf);
  c->rho_inf = F("rho_inf", c->rho_inf);
  c->x_ref = F("x_ref", c->x_ref);
  c->y_ref = F("y_ref", c->y_ref);
  {
    const std::string f = lower(trim(get_s(kv, "flux", "rusanov")));
    if (f == "hllc") c->flux = AERO_FLUX_HLLC;
    else if (f == "rusanov") c->flux = AERO_FLUX_RUSANOV;
    const std::string l = lower(trim(get_s(kv, "limiter", "minmod")));
    if (l == "venkat" || l == "venkatakrishnan") c->limiter = AERO_LIMITER_VENKAT;
    else if (l == "minmod") c->limiter = AERO_LIMITER_MINMOD;
  }
  const bool has_lmf = has(kv, "low_mach_fix");
  const bool lmf = on_off(get_s(kv, "low_mach_fix", c->low_mach_fix ? "on" : "off"), c->low_mach_fix != 0);
  const bool has_pc = has(kv, "precond") || has(kv, "precond_on");
  const std::string pct = has(kv, "precond") ? get_s(kv, "precond", "on") : get_s(kv, "precond_on", "on");
  c->precond_on = has_pc ? on_off(pct, c->precond_on != 0) : lmf;
  c->precond_mach_ref = static_cast<double>(get_f(kv, "precond_mach_ref", get_f(kv, "mach_ref", static_cast<float>(c->precond_mach_ref))));
  c->precond_mach_min = F("precond_mach_min", c->precond_mach_min);
  c->precond_beta_min = F("precond_beta_min", c->precond_beta_min);
  c->precond_beta_max = F("precond_beta_max", c->precond_beta_max);
  c->precond_farfield_bc = on_off(get_s(kv, "precond_farfield_bc", c->precond_farfield_bc ? "on" : "off"),
                                  c->precond_farfield_bc != 0);
  const float stab_fb = get_f(kv, "stabilization_mach_floor", static_cast<float>(c->stab_floor_target));
  c->stab_floor_start = get_f(kv, "stabilization_mach_floor_start", stab_fb);
  c->stab_floor_target = get_f(kv, "stabilization_mach_floor_target", stab_fb);
  c->stab_floor_k_start = F("stabilization_mach_floor_k_start", c->stab_floor_k_start);
  c->stab_floor_k_target = F("stabilization_mach_floor_k_target", c->stab_floor_k_target);
  c->stab_ramp_iters = get_i(kv, "stabilization_ramp_iters", c->stab_ramp_iters);
  c->low_mach_fix = has_lmf ? lmf : c->precond_on;
  c->mach_cutoff = F("mach_cutoff", c->mach_cutoff);
  c->all_speed_flux_fix = on_off(get_s(kv, "all_speed_flux_fix", c->all_speed_flux_fix ? "on" : "off"),
                                 c->all_speed_flux_fix != 0);
  c->all_speed_mach_cutoff = F("all_speed_mach_cutoff", c->all_speed_mach_cutoff);
  if (c->all_speed_mach_cutoff <= 0.0) c->all_speed_mach_cutoff = static_cast<double>(0.25f);
  c->all_speed_f_min = static_cast<double>(get_f(kv, "all_speed_f_min", get_f(kv, "all_speed_theta_min", static_cast<float>(c->all_speed_f_min))));
  if (c->all_speed_f_min <= 0.0) c->all_speed_f_min = static_cast<double>(0.05f);
  c->all_speed_f_min = std::clamp(static_cast<float>(c->all_speed_f_min), 1.0e-6f, 1.0f);
  c->all_speed_ramp_start_iter = std::max(get_i(kv, "all_speed_ramp_start_iter", c->all_speed_ramp_start_iter), 0);
  c->all_speed_ramp_iters = std::max(get_i(kv, "all_speed_ramp_iters", c->all_speed_ramp_iters), 0);
  c->all_speed_staged_controller = on_off(get_s(kv, "all_speed_staged_controller", c->all_speed_staged_controller ? "on" : "off"),
                                          c->all_speed_staged_controller != 0);
  c->all_speed_stage_a_min_iters = std::max(get_i(kv, "all_speed_stage_a_min_iters", c->all_speed_stage_a_min_iters), 0);
  c->all_speed_stage_a_max_iters = std::max(get_i(kv, "all_speed_stage_a_max_iters", c->all_speed_stage_a_max_iters), 0);
  c->all_speed_stage_f_min_high = F("all_speed_stage_f_min_high", c->all_speed_stage_f_min_high);
  c->all_speed_stage_f_min_mid = F("all_speed_stage_f_min_mid", c->all_speed_stage_f_min_mid);
  c->all_speed_stage_f_min_low = F("all_speed_stage_f_min_low", c->all_speed_stage_f_min_low);
  c->all_speed_pjump_wall_target = F("all_speed_pjump_wall_target", c->all_speed_pjump_wall_target);
  c->all_speed_pjump_spike_factor = F("all_speed_pjump_spike_factor", c->all_speed_pjump_spike_factor);
  c->all_speed_pjump_hold_iters = std::max(get_i(kv, "all_speed_pjump_hold_iters", c->all_speed_pjump_hold_iters), 1);
  c->all_speed_freeze_iters = std::max(get_i(kv, "all_speed_freeze_iters", c->all_speed_freeze_iters), 0);
  c->all_speed_cfl_drop_factor = F("all_speed_cfl_drop_factor", c->all_speed_cfl_drop_factor);
  c->all_speed_cfl_restore_factor = F("all_speed_cfl_restore_factor", c->all_speed_cfl_restore_factor);
  c->all_speed_cfl_min_scale = F("all_speed_cfl_min_scale", c->all_speed_cfl_min_scale);
  c->aoa0_symmetry_enforce = on_off(get_s(kv, "aoa0_symmetry_enforce", c->aoa0_symmetry_enforce ? "on" : "off"),
                                    c->aoa0_symmetry_enforce != 0);
  c->aoa0_symmetry_enforce_interval = std::max(get_i(kv, "aoa0_symmetry_enforce_interval", c->aoa0_symmetry_enforce_interval), 0);
  if (c->force_mean_drift_tol <= 0.0) c->force_mean_drift_tol = c->force_stability_tol;
  const std::string prec = lower(trim(get_s(kv, "precision", "fp32")));
  c->precision = (prec == "fp64" || prec == "double") ? AERO_PRECISION_FP64 : AERO_PRECISION_FP32;
  const std::string ord = lower(trim(get_s(kv, "ordering", "morton")));
  c->ordering = ord == "none" ? AERO_ORDER_NONE : (ord == "rcm" ? AERO_ORDER_RCM : AERO_ORDER_MORTON);
  const std::string pp = lower(trim(get_s(kv, "precond_precision", "auto")));
  c->precond_fp64 = (pp == "fp64" || pp == "double")      ? 1
                    : (pp == "fp32" || pp == "float")       ? -1
                    : (pp == "ff" || pp == "double-float") ? 2
                                                            : 0;

  std::memset(m, 0, sizeof(*m));
  const std::string src = get_s(kv, "airfoil_source", "naca4");
  if (src == "file") throw std::invalid_argument("airfoil_source=file is not supported by the device driver");
  std::snprintf(m->naca_code, sizeof(m->naca_code), "%s", get_s(kv, "naca_code", "0012").c_str());
  m->chord = get_f(kv, "chord", 1.0f);
  c->chord = m->chord;
  m->num_circumferential = get_i(kv, "num_circumferential", 160);
  m->num_radial = get_i(kv, "num_radial", 48);
  m->farfield_radius = get_f(kv, "farfield_radius", 15.0f);
  m->radial_stretch = get_f(kv, "radial_stretch", 1.4f);
}

bool env_flag_on(const char* name) {
  const char* v = std::getenv(name);
  if (v == nullptr) return false;
  const std::string t(v);
  return t == "1" || t == "true" || t == "TRUE" || t == "on" || t == "ON";
}

// ---------------------------------------------------------------------------------------
// host numerics for end-of-run statistics (double), restating the reference formulas
// ---------------------------------------------------------------------------------------
struct P {
  double r, u, v, p;
};
P c2p(const double* u, double g) {  // euler_flux.cpp:115-127
  P w;
  w.r = std::max(u[0], 1.0e-8);
  const double inv = 1.0 / w.r;
  w.u = u[1] * inv;
  w.v = u[2] * inv;
  const double ke = 0.5 * w.r * (w.u * w.u + w.v * w.v);
  w.p = std::max((g - 1.0) * (u[4] - ke), 1.0e-8);
  return w;
}
double sos(const P& w, double g) { return std::sqrt(std::max(g * w.p / std::max(w.r, 1.0e-8), 0.0)); }
double lmach(const P& w, double g) { return std::sqrt(w.u * w.u + w.v * w.v) / std::max(sos(w, g), 1.0e-8); }

struct PcCfg {
  bool on;
  double mref, mmin, bmin, bmax;
};
double beta_of(const P& w, double g, const PcCfg& pc) {  // preconditioning.cpp:24-32
  if (!pc.on) return 1.0;
  const double t = std::max({lmach(w, g), pc.mref, pc.mmin, 1.0e-8});
  const double bmin = std::max(pc.bmin, 1.0e-4), bmax = std::max(bmin, pc.bmax);
  return std::clamp(t, bmin, bmax);
}
double psr(double un, double a, double as) {  // boundary_conditions.cpp:14-25
  const double b = std::clamp(as, 1.0e-4, 1.0), b2 = b * b, o = 1.0 - b2;
  const double ut = 0.5 * (1.0 + b2) * un;
  const double ct = 0.5 * std::sqrt(std::max(o * o * un * un + 4.0 * b2 * a * a, 0.0));
  return std::max({std::abs(un), std::abs(ut - ct), std::abs(ut + ct), 1.0e-8});
}
struct Scaling {
  double beta, face_mach, low_mach, base, floor, stab, scale;
};
// compute_acoustic_scaling_info (euler_solver.cpp:392-416)
Scaling scaling(const P& l, const P& r, double g, const PcCfg& pc, bool lmf, double cutoff, double floor_m) {
  Scaling s;
  s.face_mach = 0.5 * (lmach(l, g) + lmach(r, g));
  const P avg{0.5 * (l.r + r.r), 0.5 * (l.u + r.u), 0.5 * (l.v + r.v), 0.5 * (l.p + r.p)};
  s.beta = beta_of(avg, g, pc);
  s.base = pc.on ? std::clamp(s.beta, 1.0e-4, 1.0) : 1.0;
  s.low_mach = 1.0;
  if (lmf && cutoff > 0.0) {  // compute_low_mach_dissipation_scale (euler_flux.cpp:154-175)
    const double al = std::max(sos(l, g), 1.0e-8), ar = std::max(sos(r, g), 1.0e-8);
    const double fm = 0.5 * (std::sqrt(l.u * l.u + l.v * l.v) / al + std::sqrt(r.u * r.u + r.v * r.v) / ar);
    s.low_mach = std::clamp(std::max(fm, std::max(pc.mref, 1.0e-8)) / std::max(cutoff, 1.0e-8), 1.0e-4, 1.0);
  }
  s.base = std::clamp(std::min(s.base, s.low_mach), 1.0e-4, 1.0);
  s.floor = std::clamp(floor_m, 0.0, 1.0);
  const double d = s.face_mach - s.floor;
  const double meff = 0.5 * (s.face_mach + s.floor + std::sqrt(d * d + 1.0e-12));
  s.stab = std::clamp(meff, 1.0e-4, 1.0);
  s.scale = std::max(s.base, s.stab);
  return s;
}
// compute_all_speed_hllc_pressure_scale (euler_flux.cpp:177-201)
double as_pressure_scale(const P& l, const P& r, double nx, double ny, double g, bool on, double cutoff,
                         double fmin, double w) {
  if (!on) return 1.0;
  const double unl = l.u * nx + l.v * ny, unr = r.u * nx + r.v * ny;
  const double al = std::max(sos(l, g), 1.0e-8), ar = std::max(sos(r, g), 1.0e-8);
  const double m = std::max(0.5 * (std::sqrt(l.u * l.u + l.v * l.v) / al + std::sqrt(r.u * r.u + r.v * r.v) / ar), 1.0e-6);
  double mn = std::max(0.5 * (std::abs(unl) / al + std::abs(unr) / ar), 1.0e-6);
  mn = std::max(std::min(mn, m), 1.0e-6);
  const double cut = std::max(cutoff, 1.0e-6), tf = std::clamp(fmin, 1.0e-6, 1.0);
  const double tn = std::clamp(mn / cut, tf, 1.0), mr = std::clamp(m / cut, 0.0, 1.0), gate = mr * mr;
  const double tc = (1.0 - gate) * tn + gate, ww = std::clamp(w, 0.0, 1.0);
  return std::clamp((1.0 - ww) + ww * tc, tf, 1.0);
}

double quantile(const std::vector<double>& s, double q) {  // euler_solver.cpp:364-374
  if (s.empty()) return 1.0;
  const double qc = std::clamp(q, 0.0, 1.0);
  const double idx = qc * static_cast<double>(s.size() - 1);
  const size_t i0 = static_cast<size_t>(std::floor(idx));
  const size_t i1 = std::min(i0 + 1, s.size() - 1);
  const double t = idx - static_cast<double>(i0);
  return (1.0 - t) * s[i0] + t * s[i1];
}

// Wall faces in the order of the wall-vertex walk (forces.cpp:39-132).
std::vector<int> order_wall(const std::vector<int>& faces, const std::vector<int>& fv, const std::vector<double>& pts,
                            const std::vector<double>& fc) {
  if (faces.size() <= 2) return faces;
  std::map<std::pair<int, int>, int> e2f;
  std::map<int, std::vector<int>> nb;
  auto key = [](int a, int b) { return a < b ? std::make_pair(a, b) : std::make_pair(b, a); };
  for (int f : faces) {
    const int a = fv[2 * f], b = fv[2 * f + 1];
    e2f.emplace(key(a, b), f);
    nb[a].push_back(b);
    nb[b].push_back(a);
  }
  int start = -1;
  double bx = -1.0e30, by = -1.0e30;
  for (const auto& kv : nb) {
    const double x = static_cast<float>(pts[3 * kv.first]), y = static_cast<float>(pts[3 * kv.first + 1]);
    if (x > bx || (std::abs(x - bx) < 1.0e-8 && y > by)) {
      bx = x;
      by = y;
      start = kv.first;
    }
  }
  std::vector<int> out;
  if (start >= 0 && nb[start].size() >= 2) {
    const auto& fn = nb[start];
    int next = fn[0];
    if (pts[3 * fn[1] + 1] - pts[3 * start + 1] > pts[3 * fn[0] + 1] - pts[3 * start + 1]) next = fn[1];
    int prev = start, cur = next;
    for (size_t step = 0; step < faces.size(); ++step) {
      auto it = e2f.find(key(prev, cur));
      if (it == e2f.end()) {
        out.clear();
        break;
      }
      out.push_back(it->second);
      int nxt = -1;
      for (int cnd : nb[cur]) {
        if (cnd != prev) {
          nxt = cnd;
          break;
        }
      }
      if (nxt < 0) {
        out.clear();
        break;
      }
      prev = cur;
      cur = nxt;
      if (prev == start) break;
    }
  }
  if (out.size() != faces.size()) {
    out = faces;
    std::sort(out.begin(), out.end(), [&](int a, int b) {
      return std::atan2(fc[3 * a + 1], fc[3 * a]) > std::atan2(fc[3 * b + 1], fc[3 * b]);
    });
  }
  return out;
}

template <class T>
void write_array(std::ofstream& o, const std::vector<T>& v) {
  for (size_t i = 0; i < v.size(); ++i) {
    if (i) o << ' ';
    if constexpr (std::is_same_v<T, unsigned char>) o << static_cast<int>(v[i]);
    else o << v[i];
  }
}

// Driver options beyond the reference's case keys (no reference counterpart): a state to
// start from, a state dump after the run, and the VTU encoding.
struct DriverOpts {
  std::string restart_in;   // path of a state file (aero_state_write format); empty: free stream
  std::string restart_out;  // file name in out_dir for the final state; empty: none
  bool vtu_binary = false;  // VTU arrays as raw appended binary instead of ASCII
};

DriverOpts map_opts(const KV& kv, const fs::path& case_dir) {
  DriverOpts o;
  const std::string in = trim(get_s(kv, "restart_in", ""));
  if (!in.empty()) o.restart_in = fs::path(in).is_absolute() ? in : (case_dir / in).string();
  o.restart_out = trim(get_s(kv, "restart_out", ""));
  const std::string vf = lower(trim(get_s(kv, "vtu_format", "ascii")));
  if (vf != "ascii" && vf != "binary") throw std::invalid_argument("vtu_format must be ascii or binary");
  o.vtu_binary = vf == "binary";
  return o;
}

// Appended raw binary data of a VTU file: each array is a UInt32 byte count followed by its
// bytes; DataArray elements give their offsets from the start of the appended block.
struct Appended {
  std::string bytes;
  template <class T>
  size_t add(const std::vector<T>& v) {
    const size_t off = bytes.size();
    const uint32_t nb = static_cast<uint32_t>(v.size() * sizeof(T));
    bytes.append(reinterpret_cast<const char*>(&nb), sizeof(nb));
    if (nb) bytes.append(reinterpret_cast<const char*>(v.data()), nb);
    return off;
  }
};

struct MeshHolder {
  aero_mesh* m = nullptr;
  ~MeshHolder() { aero_mesh_free(m); }
};
struct CtxHolder {
  aero_ctx* c = nullptr;
  ~CtxHolder() { aero_destroy(c); }
};

void check(int rc, aero_ctx* ctx, const char* what) {
  if (rc == AERO_OK) return;
  throw std::runtime_error(std::string(what) + ": " + aero_last_error(ctx));
}

// The reference O-grid of a run with the auxiliary arrays its outputs use (euler_solver.cpp:474).
struct EulerMesh {
  MeshHolder mh;
  aero_mesh_sizes sz{};
  aero_mesh_desc md{};
  std::vector<double> pts;
  std::vector<int> fv, conn, offs, ff, wall;
  std::vector<unsigned char> types;
  int N = 0, F = 0;
};

void build_mesh(const aero_airfoil_mesh_cfg& mc, EulerMesh* em) {
  if (aero_mesh_ogrid_reference(mc.naca_code, mc.num_circumferential, mc.num_radial, mc.farfield_radius,
                                mc.radial_stretch, mc.chord, &em->mh.m) != AERO_OK)
    throw std::invalid_argument(aero_mesh_last_error());
  MeshHolder& mh = em->mh;
  aero_mesh_sizes& sz = em->sz;
  aero_mesh_get_sizes(mh.m, &sz);
  aero_mesh_desc& md = em->md;
  aero_mesh_describe(mh.m, &md);
  std::vector<double> pts(3 * static_cast<size_t>(sz.num_points));
  std::vector<int> fv(2 * static_cast<size_t>(sz.num_faces)), conn(sz.conn_length), offs(sz.num_cells),
      ff(std::max(sz.num_farfield_faces, 1));
  std::vector<unsigned char> types(sz.num_cells);
  aero_mesh_get_aux(mh.m, pts.data(), fv.data(), conn.data(), offs.data(), types.data(), ff.data());
  ff.resize(sz.num_farfield_faces);
  const int N = sz.num_cells, F = sz.num_faces;
  const std::vector<int> wall(md.wall_faces, md.wall_faces + md.num_wall_faces);
  if (wall.empty()) throw std::runtime_error("Wall patch face set is empty.");
  em->pts = std::move(pts);
  em->fv = std::move(fv);
  em->conn = std::move(conn);
  em->offs = std::move(offs);
  em->ff = std::move(ff);
  em->types = std::move(types);
  em->wall = wall;
  em->N = N;
  em->F = F;
}

// One run's settings as run_euler_airfoil_case resolves them (euler_solver.cpp:463-566), its
// output directory and driver options.
struct EulerCase {
  aero_case_desc cfg{};
  bool pc_req = false, pc_env = false, pc_forced_off = false;
  double g = 0, rho_inf = 0, alpha = 0, a_inf = 0, v_inf = 0, u_inf_x = 0, u_inf_y = 0, q_inf = 0;
  double chord = 0, s_ref = 0, pressure_ref = 0;
  PcCfg pc{};
  double ks = 0, kt = 0, stab_start = 0, stab_target = 0;
  fs::path out_dir;
  DriverOpts opts;
};

// Resolves the case and writes the outputs known before the iterations:
// boundary_faces_debug.txt and effective_config_snapshot.txt.
EulerCase prepare_case(const aero_case_desc& cfg_in, const aero_airfoil_mesh_cfg& mc, const EulerMesh& em,
                       const fs::path& out_dir, const DriverOpts& opts) {
  if (cfg_in.iterations <= 0) throw std::invalid_argument("Euler iterations must be positive.");
  if (cfg_in.rk_stages != 1 && cfg_in.rk_stages != 3)
    throw std::invalid_argument("Euler pseudo-time rk_stages must be 1 or 3.");
  const aero_mesh_desc& md = em.md;
  const int F = em.F;
  const std::vector<int>& wall = em.wall;
  const std::vector<int>& ff = em.ff;
  aero_case_desc cfg = cfg_in;
  const bool pc_req = cfg.precond_on != 0;
  const bool pc_env = env_flag_on("AERO_ENABLE_EXPERIMENTAL_PRECOND");
  const bool pc_forced_off = pc_req && !pc_env;
  if (pc_forced_off) {
    cfg.precond_on = 0;
    std::cerr << "preconditioning forced off (experimental)\n";
  }
  cfg.diagnostics = 1;
  const double g = cfg.gamma;
  double rho_inf = cfg.rho_inf;
  if (rho_inf <= 0.0) rho_inf = cfg.p_inf / (cfg.gas_constant * cfg.t_inf);
  if (!(rho_inf > 0.0)) throw std::invalid_argument("Invalid freestream density. Set rho_inf or p_inf/T_inf.");
  const double pi = 3.14159265358979323846, alpha = cfg.aoa_deg * (pi / 180.0);
  const double a_inf = std::sqrt(g * cfg.p_inf / rho_inf), v_inf = std::max(cfg.mach, 0.0) * a_inf;
  const double u_inf_x = v_inf * std::cos(alpha), u_inf_y = v_inf * std::sin(alpha);
  const double q_inf = 0.5 * rho_inf * v_inf * v_inf + 1.0e-12;
  const double chord = std::max(mc.chord, 1.0e-8), s_ref = chord;
  const double pressure_ref = std::max(rho_inf * a_inf * a_inf, 1.0e-12);
  const double minf = std::max(cfg.mach, 1.0e-4);
  PcCfg pc{cfg.precond_on != 0,
           std::max(cfg.precond_mach_ref > 0.0 ? cfg.precond_mach_ref : minf, 1.0e-4),
           std::max(cfg.precond_mach_min > 0.0 ? cfg.precond_mach_min : 1.0e-6, 1.0e-6),
           std::max(cfg.precond_beta_min > 0.0 ? cfg.precond_beta_min : std::max(1.0e-4, std::min(1.0e-3, 0.1 * minf)), 1.0e-4),
           0.0};
  pc.bmax = std::max(cfg.precond_beta_max, pc.bmin);
  const double ks = cfg.stab_floor_k_start >= 0.0 ? cfg.stab_floor_k_start : cfg.stab_floor_start / minf;
  const double kt = cfg.stab_floor_k_target >= 0.0 ? cfg.stab_floor_k_target : cfg.stab_floor_target / minf;
  const double stab_start = std::clamp(std::max(ks, 0.0) * minf, 0.0, 1.0);
  const double stab_target = std::clamp(std::max(kt, 0.0) * minf, 0.0, 1.0);

  fs::create_directories(out_dir);
  // boundary_faces_debug.txt (euler_solver.cpp:252-301)
  {
    std::vector<int> wall_bc, ff_bc;
    for (int f = 0; f < F; ++f) {
      if (md.face_neighbor[f] >= 0) continue;
      (md.face_bc[f] == AERO_BC_WALL ? wall_bc : ff_bc).push_back(f);
    }
    auto stats = [&](const std::vector<int>& fs_, const char* name, std::ofstream& o) {
      int first = -1, last = -1;
      double x0 = 0, x1 = 0, y0 = 0, y1 = 0, ds = 0, nxs = 0, nys = 0;
      if (!fs_.empty()) {
        first = last = fs_.front();
        x0 = y0 = 1e300;
        x1 = y1 = -1e300;
      }
      for (int f : fs_) {
        first = std::min(first, f);
        last = std::max(last, f);
        x0 = std::min(x0, md.face_center[3 * f]);
        x1 = std::max(x1, md.face_center[3 * f]);
        y0 = std::min(y0, md.face_center[3 * f + 1]);
        y1 = std::max(y1, md.face_center[3 * f + 1]);
        ds += md.face_area[f];
        nxs += md.face_normal[3 * f] * md.face_area[f];
        nys += md.face_normal[3 * f + 1] * md.face_area[f];
      }
      o << name << "," << fs_.size() << "," << first << "," << last << "," << static_cast<float>(x0) << ","
        << static_cast<float>(x1) << "," << static_cast<float>(y0) << "," << static_cast<float>(y1) << ","
        << static_cast<float>(ds) << "," << static_cast<float>(nxs) << "," << static_cast<float>(nys) << "\n";
    };
    std::ofstream o(out_dir / "boundary_faces_debug.txt", std::ios::trunc);
    o << "boundary_patch_id,name,start_face,face_count\n";
    o << "0,wall," << wall.front() << "," << wall.size() << "\n";
    if (!ff.empty()) o << "1,farfield," << ff.front() << "," << ff.size() << "\n";
    o << "\n";
    o << "set,count,first_face,last_face,x_min,x_max,y_min,y_max,sum_ds,sum_nx_ds,sum_ny_ds\n";
    stats(wall, "wall_patch", o);
    stats(wall_bc, "wall_bc_type", o);
    stats(ff, "farfield_patch", o);
    stats(ff_bc, "farfield_bc_type", o);
    o << "\n";
    o << "wall_patch_vs_bc_mismatch_faces=0\n";
    o << "farfield_patch_vs_bc_mismatch_faces=0\n";
    o << "normal_normalized_faces=0\n";
    o << "normal_invalid_faces=0\n";
    o << "normal_max_norm_deviation=0\n";
  }
  // effective_config_snapshot.txt (euler_solver.cpp:650-715)
  {
    std::ofstream o(out_dir / "effective_config_snapshot.txt", std::ios::trunc);
    auto fl = [](double x) { return static_cast<float>(x); };
    o << "iterations=" << cfg.iterations << "\nmin_iterations=" << cfg.min_iterations << "\naoa_deg=" << fl(cfg.aoa_deg)
      << "\nmach_inf=" << fl(cfg.mach) << "\ngamma=" << fl(g) << "\nu_inf=" << fl(u_inf_x) << "\nv_inf=" << fl(u_inf_y)
      << "\nrho_inf=" << fl(rho_inf) << "\na_inf=" << fl(a_inf) << "\nq_inf=" << fl(q_inf)
      << "\ncfl_start=" << fl(cfg.cfl_start) << "\ncfl_max=" << fl(cfg.cfl_max) << "\ncfl_ramp_iters=" << cfg.cfl_ramp_iters
      << "\nall_speed_flux_fix=" << cfg.all_speed_flux_fix << "\nall_speed_mach_cutoff=" << fl(cfg.all_speed_mach_cutoff)
      << "\nall_speed_f_min=" << fl(std::clamp(cfg.all_speed_f_min, 1.0e-6, 1.0))
      << "\nall_speed_ramp_start_iter=" << cfg.all_speed_ramp_start_iter
      << "\nall_speed_ramp_iters=" << cfg.all_speed_ramp_iters
      << "\nall_speed_staged_controller=" << cfg.all_speed_staged_controller
      << "\nforce_stability_tol=" << fl(cfg.force_stability_tol) << "\nforce_stability_window=" << cfg.force_stability_window
      << "\nforce_mean_drift_tol=" << fl(cfg.force_mean_drift_tol)
      << "\nresidual_reduction_target=" << fl(cfg.residual_reduction_target)
      << "\nprecond_requested=" << (pc_req ? 1 : 0) << "\nprecond_experimental_env_enabled=" << (pc_env ? 1 : 0)
      << "\nprecond_forced_off=" << (pc_forced_off ? 1 : 0) << "\nprecond_effective=" << (pc.on ? 1 : 0)
      << "\nprecond_mach_ref_effective=" << fl(pc.mref) << "\nprecond_mach_min=" << fl(pc.mmin)
      << "\nprecond_beta_min_effective=" << fl(pc.bmin) << "\nprecond_beta_max_effective=" << fl(pc.bmax)
      << "\nprecond_farfield_bc=" << cfg.precond_farfield_bc
      << "\nstabilization_mach_floor_start_effective=" << fl(stab_start)
      << "\nstabilization_mach_floor_target_effective=" << fl(stab_target)
      << "\nstabilization_ramp_iters_effective=" << std::max(cfg.stab_ramp_iters, 0)
      << "\nprecision=" << (cfg.precision == AERO_PRECISION_FP64 ? "fp64" : "fp32") << "\n";
  }
  EulerCase ec;
  ec.cfg = cfg;
  ec.pc_req = pc_req;
  ec.pc_env = pc_env;
  ec.pc_forced_off = pc_forced_off;
  ec.g = g;
  ec.rho_inf = rho_inf;
  ec.alpha = alpha;
  ec.a_inf = a_inf;
  ec.v_inf = v_inf;
  ec.u_inf_x = u_inf_x;
  ec.u_inf_y = u_inf_y;
  ec.q_inf = q_inf;
  ec.chord = chord;
  ec.s_ref = s_ref;
  ec.pressure_ref = pressure_ref;
  ec.pc = pc;
  ec.ks = ks;
  ec.kt = kt;
  ec.stab_start = stab_start;
  ec.stab_target = stab_target;
  ec.out_dir = out_dir;
  ec.opts = opts;
  return ec;
}

// residuals.csv, forces.csv and euler_diagnostics.csv of the executed iterations
// (euler_solver.cpp:723-738, 1161-1203).
void write_history(const EulerCase& ec, const EulerMesh& em, const std::vector<aero_iter_record>& hist) {
  const aero_mesh_desc& md = em.md;
  const std::vector<int>& wall = em.wall;
  const fs::path& out_dir = ec.out_dir;
  const aero_case_desc& cfg = ec.cfg;
  const double q_inf = ec.q_inf, rho_inf = ec.rho_inf, v_inf = ec.v_inf, s_ref = ec.s_ref, chord = ec.chord;
  const double pressure_ref = ec.pressure_ref;
  auto fl = [](double x) { return static_cast<float>(x); };
  std::ofstream rcsv(out_dir / "residuals.csv", std::ios::trunc);
  std::ofstream fcsv(out_dir / "forces.csv", std::ios::trunc);
  std::ofstream dcsv(out_dir / "euler_diagnostics.csv", std::ios::trunc);
  if (!rcsv || !fcsv || !dcsv) throw std::runtime_error("Failed to open Euler CSV outputs.");
  rcsv << "iter,residual_l1,residual_l2,residual_linf,residual_ratio\n";
  fcsv << "iter,cl,cd,cm,lift,drag,moment,dcl,dcd,dcm,mean_dcl,mean_dcd,mean_dcm,"
          "force_window_stable,force_mean_drift_stable,force_physical_converged\n";
  dcsv << "iter,residual_ratio,force_window_stable,integrated_wall_faces,wall_patch_faces,"
          "wall_patch_bc_mismatch,sum_wall_ds,sum_nA_x,sum_nA_y,sum_nA_mag,max_wall_un,"
          "max_wall_mass_flux_n,max_farfield_abs_dp,max_farfield_abs_drho,max_farfield_abs_du,"
          "max_farfield_abs_dv,max_farfield_abs_dw,wall_cp_min,wall_cp_max,wall_cp_nonfinite,"
          "q_inf,rho_inf,V_inf,S_ref,chord,Fx_gauge,Fy_gauge,Fx_abs,Fy_abs,L,D,Cl,Cd,Cm,"
          "cl_abs,cd_abs,cm_abs,dcl,dcd,dcm,force_mean_drift_stable,force_physical_converged,"
          "mean_dcl,mean_dcd,mean_dcm,cd_sign_flip,p_jump_energy_nd,p_jump_energy_wall_nd,"
          "all_speed_stage,all_speed_flux_fix_effective,all_speed_f_min_effective,"
          "all_speed_ramp_weight_effective,all_speed_freeze_counter,all_speed_controller_action,"
          "cfl_scale_effective,cd_times_mach,p_fluct_nd_max,p_fluct_nd_wall,p_fluct_nd_farfield,"
          "num_faces_first_order_fallback,num_faces_diffusive_fallback,first_failure_face,"
          "first_failure_owner,first_failure_neighbor\n";
  double sum_wall_ds = 0.0;
  for (int f : wall) sum_wall_ds += md.face_area[f];
  for (size_t k = 0; k < hist.size(); ++k) {
    const aero_iter_record& r = hist[k];
    const bool ws = r.flags & AERO_REC_FORCE_WINDOW_STABLE, ds = r.flags & AERO_REC_FORCE_DRIFT_STABLE;
    const bool flip = k > 0 && ((hist[k - 1].cd >= 0.0) != (r.cd >= 0.0));
    rcsv << r.iter << "," << fl(r.residual_l1) << "," << fl(r.residual_l2) << "," << fl(r.residual_linf) << ","
         << fl(r.residual_ratio) << "\n";
    fcsv << r.iter << "," << fl(r.cl) << "," << fl(r.cd) << "," << fl(r.cm) << "," << fl(r.lift) << ","
         << fl(r.drag) << "," << fl(r.moment) << "," << fl(r.dcl) << "," << fl(r.dcd) << "," << fl(r.dcm) << ","
         << fl(r.mean_dcl) << "," << fl(r.mean_dcd) << "," << fl(r.mean_dcm) << "," << ws << "," << ds << ","
         << (ws && ds) << "\n";
    const char* stage = (r.flags & AERO_REC_STAGE_A) ? "A" : ((r.flags & AERO_REC_STAGE_B) ? "B" : "single");
    dcsv << r.iter << "," << fl(r.residual_ratio) << "," << ws << "," << wall.size() << "," << wall.size() << ",0,"
         << fl(sum_wall_ds) << "," << fl(r.sum_nax) << "," << fl(r.sum_nay) << ","
         << fl(std::sqrt(r.sum_nax * r.sum_nax + r.sum_nay * r.sum_nay)) << "," << fl(r.max_wall_un) << ","
         << fl(r.max_wall_mass_flux) << "," << fl(r.max_farfield_abs_dp) << "," << fl(r.max_farfield_abs_drho) << ","
         << fl(r.max_farfield_abs_du) << "," << fl(r.max_farfield_abs_dv) << ",0," << fl(r.wall_cp_min) << ","
         << fl(r.wall_cp_max) << "," << r.wall_cp_nonfinite << "," << fl(q_inf) << "," << fl(rho_inf) << ","
         << fl(v_inf) << "," << fl(s_ref) << "," << fl(chord) << "," << fl(r.fx_gauge) << "," << fl(r.fy_gauge)
         << "," << fl(r.fx_abs) << "," << fl(r.fy_abs) << "," << fl(r.lift) << "," << fl(r.drag) << ","
         << fl(r.cl) << "," << fl(r.cd) << "," << fl(r.cm) << "," << fl(r.cl_abs) << "," << fl(r.cd_abs) << ","
         << fl(r.cm_abs) << "," << fl(r.dcl) << "," << fl(r.dcd) << "," << fl(r.dcm) << "," << ds << ","
         << (ws && ds) << "," << fl(r.mean_dcl) << "," << fl(r.mean_dcd) << "," << fl(r.mean_dcm) << ","
         << flip << "," << fl(r.p_jump_energy_nd) << "," << fl(r.p_jump_energy_wall_nd) << "," << stage << ","
         << ((r.flags & AERO_REC_ALL_SPEED_FIX) ? 1 : 0) << "," << fl(r.all_speed_f_min) << ","
         << fl(r.all_speed_ramp_weight) << ",0," << r.controller_action << "," << fl(r.cfl_scale) << ","
         << fl(r.cd * std::max(cfg.mach, 0.0)) << "," << fl(r.max_abs_dp_domain / pressure_ref) << ","
         << fl(r.max_abs_dp_wall / pressure_ref) << "," << fl(r.max_farfield_abs_dp / pressure_ref) << ","
         << r.first_order_fallback_faces << "," << r.diffusive_fallback_faces << ",-1,-1,-1\n";
  }
}

// Appends a chunk of records to a run's history; the record of a non-finite trap is not kept
// (the reference stops before writing it). Returns whether the run stopped.
bool take_records(const aero_iter_record* recs, int done, int chunk, std::vector<aero_iter_record>* hist,
                  bool* nonfinite) {
  for (int k = 0; k < done; ++k) {
    const aero_iter_record& r = recs[k];
    if (r.flags & AERO_REC_NONFINITE) {
      std::cerr << "non_finite_trap iter=" << r.iter << " location=conserved\n";
      *nonfinite = true;
      return true;
    }
    hist->push_back(r);
    if (r.flags & AERO_REC_CONVERGED) return true;
  }
  return done < chunk;
}

// The outputs of the final state (euler_solver.cpp:1217-1477): fields, acoustic-scale
// statistics, wall_flux.csv, dissipation_debug.csv, cp_wall.csv, the state dump, the VTU
// file and run.log, and the summary dict's values.
void write_final(const EulerCase& ec, const EulerMesh& em, const std::vector<double>& U, const std::vector<double>& R,
                 const std::vector<aero_iter_record>& hist, bool nonfinite, aero_run_summary* summary) {
  const aero_mesh_desc& md = em.md;
  const int N = em.N, F = em.F;
  const std::vector<int>& wall = em.wall;
  const std::vector<int>& fv = em.fv;
  const std::vector<int>& conn = em.conn;
  const std::vector<int>& offs = em.offs;
  const std::vector<unsigned char>& types = em.types;
  const std::vector<double>& pts = em.pts;
  const aero_mesh_sizes& sz = em.sz;
  const fs::path& out_dir = ec.out_dir;
  const DriverOpts& opts = ec.opts;
  const aero_case_desc& cfg = ec.cfg;
  const double g = ec.g, rho_inf = ec.rho_inf, alpha = ec.alpha, u_inf_x = ec.u_inf_x, u_inf_y = ec.u_inf_y;
  const double q_inf = ec.q_inf, v_inf = ec.v_inf, s_ref = ec.s_ref, chord = ec.chord, pressure_ref = ec.pressure_ref;
  const double ks = ec.ks, kt = ec.kt, stab_start = ec.stab_start, stab_target = ec.stab_target;
  const bool pc_req = ec.pc_req;
  const PcCfg& pc = ec.pc;
  auto fl = [](double x) { return static_cast<float>(x); };
  std::vector<float> rho(N), uu(N), vv(N), pp(N), mach(N), rmag(N);
  double bmin = 1e300, bmax = -1e300, bsum = 0, mmin = 1e300, mmax = -1e300, msum = 0;
  std::vector<P> prim(N);
  for (int c = 0; c < N; ++c) {
    const P w = c2p(&U[5 * static_cast<size_t>(c)], g);
    prim[c] = w;
    rho[c] = fl(w.r);
    uu[c] = fl(w.u);
    vv[c] = fl(w.v);
    pp[c] = fl(w.p);
    const double m = std::sqrt(w.u * w.u + w.v * w.v) / std::max(sos(w, g), 1.0e-8);
    mach[c] = fl(m);
    const double b = beta_of(w, g, pc);
    bmin = std::min(bmin, b);
    bmax = std::max(bmax, b);
    bsum += b;
    mmin = std::min(mmin, m);
    mmax = std::max(mmax, m);
    msum += m;
    const double inv = 1.0 / std::max(md.cell_volume[c], 1.0e-12);
    double m2 = 0.0;
    for (int k = 0; k < 5; ++k) m2 += (R[5 * c + k] * inv) * (R[5 * c + k] * inv);
    rmag[c] = fl(std::sqrt(m2));
  }
  const aero_iter_record& last = hist.back();
  const double stab_final = last.stab_mach_floor;
  const bool lmf = cfg.low_mach_fix != 0;
  // acoustic-scale statistics over all faces (euler_solver.cpp:1262-1302)
  const P pinf = c2p(std::array<double, 5>{rho_inf, rho_inf * u_inf_x, rho_inf * u_inf_y, 0.0,
                                           std::max(cfg.p_inf, 1.0e-8) / (g - 1.0) +
                                               0.5 * rho_inf * (u_inf_x * u_inf_x + u_inf_y * u_inf_y)}.data(), g);
  double asmin = 1e300, asmax = -1e300, assum = 0, afmin = 1e300, afmax = -1e300, afsum = 0;
  std::vector<unsigned char> wall_cell(N, 0);
  for (int f : wall) wall_cell[md.face_owner[f]] = 1;
  for (int f = 0; f < F; ++f) {
    const P& l = prim[md.face_owner[f]];
    const P r = md.face_neighbor[f] >= 0 ? prim[md.face_neighbor[f]] : (md.face_bc[f] == AERO_BC_WALL ? l : pinf);
    const Scaling s = scaling(l, r, g, pc, lmf, cfg.mach_cutoff, stab_final);
    asmin = std::min(asmin, s.base);
    asmax = std::max(asmax, s.base);
    assum += s.base;
    afmin = std::min(afmin, s.scale);
    afmax = std::max(afmax, s.scale);
    afsum += s.scale;
  }
  // wall_flux.csv (euler_solver.cpp:1304-1331): the slip-wall flux has no mass component
  {
    std::ofstream o(out_dir / "wall_flux.csv", std::ios::trunc);
    o << "face,x,y,mass_flux_n\n";
    for (int f = 0; f < F; ++f) {
      if (md.face_neighbor[f] >= 0 || md.face_bc[f] != AERO_BC_WALL) continue;
      o << f << "," << fl(md.face_center[3 * f]) << "," << fl(md.face_center[3 * f + 1]) << ",0\n";
    }
  }
  // wall-adjacent statistics and dissipation_debug.csv (euler_solver.cpp:1333-1465)
  std::vector<int> wadj;
  for (int f = 0; f < F; ++f) {
    const int o = md.face_owner[f], b = md.face_neighbor[f];
    if (b >= 0 && (wall_cell[o] || wall_cell[b])) wadj.push_back(f);
  }
  std::vector<double> sa, ss, sf;
  for (int f : wadj) {
    const Scaling s = scaling(prim[md.face_owner[f]], prim[md.face_neighbor[f]], g, pc, lmf, cfg.mach_cutoff, stab_final);
    sa.push_back(s.base);
    ss.push_back(s.stab);
    sf.push_back(s.scale);
  }
  std::sort(sa.begin(), sa.end());
  std::sort(ss.begin(), ss.end());
  std::sort(sf.begin(), sf.end());
  {
    std::ofstream o(out_dir / "dissipation_debug.csv", std::ios::trunc);
    o << "face,region,x,y,area,mach_local,un_abs,a,beta,low_mach_scale,acoustic_scale,"
         "s_stab,acoustic_scale_final,stabilization_m0,all_speed_pressure_scale,"
         "smax_physical,smax_dissipation\n";
    const bool asf = last.flags & AERO_REC_ALL_SPEED_FIX;
    auto row = [&](int f, const char* region, const P& l, const P& r) {
      const double nx = md.face_normal[3 * f], ny = md.face_normal[3 * f + 1];
      const double unl = l.u * nx + l.v * ny, unr = r.u * nx + r.v * ny;
      const double al = sos(l, g), ar = sos(r, g);
      const double ml = std::sqrt(l.u * l.u + l.v * l.v) / std::max(al, 1.0e-8);
      const double mr = std::sqrt(r.u * r.u + r.v * r.v) / std::max(ar, 1.0e-8);
      const Scaling s = scaling(l, r, g, pc, lmf, cfg.mach_cutoff, stab_final);
      const double ps = as_pressure_scale(l, r, nx, ny, g, asf, cfg.all_speed_mach_cutoff, last.all_speed_f_min,
                                          last.all_speed_ramp_weight);
      o << f << "," << region << "," << fl(md.face_center[3 * f]) << "," << fl(md.face_center[3 * f + 1]) << ","
        << fl(md.face_area[f]) << "," << fl(0.5 * (ml + mr)) << "," << fl(0.5 * (std::abs(unl) + std::abs(unr))) << ","
        << fl(0.5 * (al + ar)) << "," << fl(s.beta) << "," << fl(s.low_mach) << "," << fl(s.base) << "," << fl(s.stab)
        << "," << fl(s.scale) << "," << fl(s.floor) << "," << fl(ps) << ","
        << fl(std::max(std::abs(unl) + al, std::abs(unr) + ar)) << ","
        << fl(std::max(psr(unl, al, s.scale), psr(unr, ar, s.scale))) << "\n";
    };
    for (size_t i = 0; i < wadj.size() && i < 10; ++i)
      row(wadj[i], "wall_adjacent_interior", prim[md.face_owner[wadj[i]]], prim[md.face_neighbor[wadj[i]]]);
    int nfar = 0;
    for (int f = 0; f < F && nfar < 10; ++f) {
      if (md.face_neighbor[f] >= 0 || md.face_bc[f] != AERO_BC_FARFIELD) continue;
      row(f, "farfield_boundary", prim[md.face_owner[f]], pinf);
      ++nfar;
    }
  }
  // cp_wall.csv (forces.cpp:177-206)
  {
    const std::vector<int> ordered = order_wall(wall, fv, pts, std::vector<double>(md.face_center, md.face_center + 3 * static_cast<size_t>(F)));
    std::ofstream o(out_dir / "cp_wall.csv", std::ios::trunc);
    o << "s,x,y,Cp\n";
    double s = 0.0;
    for (int f : ordered) {
      o << fl(s) << "," << fl(md.face_center[3 * f]) << "," << fl(md.face_center[3 * f + 1]) << ","
        << fl((prim[md.face_owner[f]].p - cfg.p_inf) / q_inf) << "\n";
      s += md.face_area[f];
    }
  }
  if (!opts.restart_out.empty()) {
    if (aero_state_write((out_dir / opts.restart_out).string().c_str(), N, U.data()) != AERO_OK)
      throw std::runtime_error(std::string("restart_out: ") + aero_driver_last_error());
  }
  // field_0000.vtu (io_vtk_stub.cpp:95-166)
  if (opts.vtu_binary) {
    std::ofstream o(out_dir / "field_0000.vtu", std::ios::trunc | std::ios::binary);
    if (!o) throw std::runtime_error("Failed to write Euler VTU output.");
    std::vector<float> pf(pts.begin(), pts.end());
    Appended ap;
    auto da = [&](const char* type, const char* name, int ncomp, size_t off) {
      o << "        <DataArray type=\"" << type << "\"";
      if (name) o << " Name=\"" << name << "\"";
      if (ncomp > 1) o << " NumberOfComponents=\"" << ncomp << "\"";
      o << " format=\"appended\" offset=\"" << off << "\"/>\n";
    };
    o << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\" "
         "header_type=\"UInt32\">\n  <UnstructuredGrid>\n    <Piece NumberOfPoints=\"" << sz.num_points
      << "\" NumberOfCells=\"" << N << "\">\n      <Points>\n";
    da("Float32", nullptr, 3, ap.add(pf));
    o << "      </Points>\n      <Cells>\n";
    da("Int32", "connectivity", 1, ap.add(conn));
    da("Int32", "offsets", 1, ap.add(offs));
    da("UInt8", "types", 1, ap.add(types));
    o << "      </Cells>\n      <PointData/>\n      <CellData Scalars=\"rho\">\n";
    const std::pair<const char*, const std::vector<float>*> arrays[] = {
        {"rho", &rho}, {"u", &uu}, {"v", &vv}, {"p", &pp}, {"Mach", &mach}, {"residual_magnitude", &rmag}};
    for (const auto& a : arrays) da("Float32", a.first, 1, ap.add(*a.second));
    o << "      </CellData>\n    </Piece>\n  </UnstructuredGrid>\n  <AppendedData encoding=\"raw\">\n   _";
    o.write(ap.bytes.data(), static_cast<std::streamsize>(ap.bytes.size()));
    o << "\n  </AppendedData>\n</VTKFile>\n";
  } else {
    std::ofstream o(out_dir / "field_0000.vtu", std::ios::trunc);
    if (!o) throw std::runtime_error("Failed to write Euler VTU output.");
    std::vector<float> pf(pts.begin(), pts.end());
    o << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
         "  <UnstructuredGrid>\n    <Piece NumberOfPoints=\"" << sz.num_points << "\" NumberOfCells=\"" << N << "\">\n"
         "      <Points>\n        <DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">";
    write_array(o, pf);
    o << "</DataArray>\n      </Points>\n      <Cells>\n        <DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">";
    write_array(o, conn);
    o << "</DataArray>\n        <DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">";
    write_array(o, offs);
    o << "</DataArray>\n        <DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">";
    write_array(o, types);
    o << "</DataArray>\n      </Cells>\n      <PointData/>\n      <CellData Scalars=\"rho\">\n";
    const std::pair<const char*, const std::vector<float>*> arrays[] = {
        {"rho", &rho}, {"u", &uu}, {"v", &vv}, {"p", &pp}, {"Mach", &mach}, {"residual_magnitude", &rmag}};
    for (const auto& a : arrays) {
      o << "        <DataArray type=\"Float32\" Name=\"" << a.first << "\" format=\"ascii\">";
      write_array(o, *a.second);
      o << "</DataArray>\n";
    }
    o << "      </CellData>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n";
  }

  // run.log (residual_stub.cpp:607-762)
  const fs::path log_path = out_dir / "run.log";
  {
    std::ofstream o(log_path, std::ios::trunc);
    const bool ws = last.flags & AERO_REC_FORCE_WINDOW_STABLE, ds = last.flags & AERO_REC_FORCE_DRIFT_STABLE;
    const double nmag = std::sqrt(last.sum_nax * last.sum_nax + last.sum_nay * last.sum_nay);
    auto q = [&](const std::vector<double>& v, double p) { return v.empty() ? 1.0 : quantile(v, p); };
    o << "AeroCFD Euler airfoil 2D\nversion=" << kVersion << "\ncase_path=" << summary->run_log
      << "\nbackend=cuda\ncase_type=euler_airfoil_2d\nnum_cells=" << N << "\nnum_faces=" << F
      << "\niterations=" << hist.size() << "\nresidual_l1=" << fl(last.residual_l1) << "\nresidual_l2="
      << fl(last.residual_l2) << "\nresidual_linf=" << fl(last.residual_linf) << "\ncl=" << fl(last.cl)
      << "\ncd=" << fl(last.cd) << "\ncm=" << fl(last.cm) << "\naoa_deg=" << fl(cfg.aoa_deg)
      << "\naoa_rad=" << fl(alpha) << "\nu_inf=" << fl(u_inf_x) << "\nv_inf=" << fl(u_inf_y)
      << "\nwall_faces_integrated=" << wall.size() << "\nnormal_is_unit=1\nsum_nA_x=" << fl(last.sum_nax)
      << "\nsum_nA_y=" << fl(last.sum_nay) << "\nsum_nA_mag=" << fl(nmag) << "\nFx_abs=" << fl(last.fx_abs)
      << "\nFy_abs=" << fl(last.fy_abs) << "\nFx_gauge=" << fl(last.fx_gauge) << "\nFy_gauge=" << fl(last.fy_gauge)
      << "\nq_inf=" << fl(q_inf) << "\nV_inf=" << fl(v_inf) << "\nrho_inf=" << fl(rho_inf) << "\nS_ref=" << fl(s_ref)
      << "\nchord=" << fl(chord) << "\nFx=" << fl(last.fx_gauge) << "\nFy=" << fl(last.fy_gauge) << "\nL="
      << fl(last.lift) << "\nD=" << fl(last.drag) << "\ncl_abs=" << fl(last.cl_abs) << "\ncd_abs=" << fl(last.cd_abs)
      << "\ncm_abs=" << fl(last.cm_abs) << "\nflux=" << (cfg.flux == AERO_FLUX_HLLC ? "hllc" : "rusanov")
      << "\nlimiter=" << (cfg.limiter == AERO_LIMITER_VENKAT ? "venkat" : "minmod")
      << "\nlow_mach_fix=" << (cfg.low_mach_fix ? "on" : "off") << "\nmach_cutoff=" << fl(cfg.mach_cutoff)
      << "\nall_speed_flux_fix=" << (cfg.all_speed_flux_fix ? "on" : "off")
      << "\nall_speed_mach_cutoff=" << fl(cfg.all_speed_mach_cutoff) << "\nall_speed_f_min=" << fl(cfg.all_speed_f_min)
      << "\nall_speed_ramp_start_iter=" << cfg.all_speed_ramp_start_iter
      << "\nall_speed_ramp_iters=" << cfg.all_speed_ramp_iters
      << "\nall_speed_staged_controller=" << (cfg.all_speed_staged_controller ? "on" : "off")
      << "\nall_speed_stage_a_min_iters=" << cfg.all_speed_stage_a_min_iters
      << "\nall_speed_stage_a_max_iters=" << cfg.all_speed_stage_a_max_iters
      << "\nall_speed_stage_f_min_high=" << fl(cfg.all_speed_stage_f_min_high)
      << "\nall_speed_stage_f_min_mid=" << fl(cfg.all_speed_stage_f_min_mid)
      << "\nall_speed_stage_f_min_low=" << fl(cfg.all_speed_stage_f_min_low)
      << "\nall_speed_pjump_wall_target=" << fl(cfg.all_speed_pjump_wall_target)
      << "\nall_speed_pjump_spike_factor=" << fl(cfg.all_speed_pjump_spike_factor)
      << "\nall_speed_pjump_hold_iters=" << cfg.all_speed_pjump_hold_iters
      << "\nall_speed_freeze_iters=" << cfg.all_speed_freeze_iters
      << "\nall_speed_cfl_drop_factor=" << fl(cfg.all_speed_cfl_drop_factor)
      << "\nall_speed_cfl_restore_factor=" << fl(cfg.all_speed_cfl_restore_factor)
      << "\nall_speed_cfl_min_scale=" << fl(cfg.all_speed_cfl_min_scale)
      << "\naoa0_symmetry_enforce=" << (cfg.aoa0_symmetry_enforce ? "on" : "off")
      << "\naoa0_symmetry_enforce_interval=" << cfg.aoa0_symmetry_enforce_interval
      << "\nprecond=" << (pc_req ? "on" : "off") << "\nprecond_mach_ref=" << fl(cfg.precond_mach_ref)
      << "\nprecond_mach_min=" << fl(cfg.precond_mach_min) << "\nprecond_beta_min=" << fl(cfg.precond_beta_min)
      << "\nprecond_beta_max=" << fl(cfg.precond_beta_max)
      << "\nprecond_farfield_bc=" << (cfg.precond_farfield_bc ? "on" : "off")
      << "\nstabilization_mach_floor_start=" << fl(cfg.stab_floor_start)
      << "\nstabilization_mach_floor_target=" << fl(cfg.stab_floor_target)
      << "\nstabilization_mach_floor_k_start=" << fl(cfg.stab_floor_k_start)
      << "\nstabilization_mach_floor_k_target=" << fl(cfg.stab_floor_k_target)
      << "\nstabilization_ramp_iters=" << cfg.stab_ramp_iters
      << "\nprecond_mach_ref_effective=" << fl(pc.mref) << "\nprecond_beta_min_effective=" << fl(pc.bmin)
      << "\nprecond_beta_max_effective=" << fl(pc.bmax)
      << "\nstabilization_mach_floor_start_effective=" << fl(stab_start)
      << "\nstabilization_mach_floor_target_effective=" << fl(stab_target)
      << "\nstabilization_mach_floor_k_start_effective=" << fl(std::max(ks, 0.0))
      << "\nstabilization_mach_floor_k_target_effective=" << fl(std::max(kt, 0.0))
      << "\nstabilization_ramp_iters_effective=" << std::max(cfg.stab_ramp_iters, 0)
      << "\nstabilization_mach_floor_final=" << fl(stab_final) << "\nbeta_min=" << fl(bmin) << "\nbeta_max="
      << fl(bmax) << "\nbeta_mean=" << fl(bsum / N) << "\nmach_local_min=" << fl(mmin) << "\nmach_local_max="
      << fl(mmax) << "\nmach_local_mean=" << fl(msum / N) << "\nacoustic_scale_min=" << fl(asmin)
      << "\nacoustic_scale_max=" << fl(asmax) << "\nacoustic_scale_mean=" << fl(assum / F)
      << "\nacoustic_scale_final_min=" << fl(afmin) << "\nacoustic_scale_final_max=" << fl(afmax)
      << "\nacoustic_scale_final_mean=" << fl(afsum / F)
      << "\nwall_adjacent_acoustic_scale_min=" << fl(sa.empty() ? 1.0 : sa.front())
      << "\nwall_adjacent_acoustic_scale_p01=" << fl(q(sa, 0.01))
      << "\nwall_adjacent_acoustic_scale_p50=" << fl(q(sa, 0.5))
      << "\nwall_adjacent_stabilization_scale_min=" << fl(ss.empty() ? 1.0 : ss.front())
      << "\nwall_adjacent_stabilization_scale_p01=" << fl(q(ss, 0.01))
      << "\nwall_adjacent_stabilization_scale_p50=" << fl(q(ss, 0.5))
      << "\nwall_adjacent_acoustic_scale_final_min=" << fl(sf.empty() ? 1.0 : sf.front())
      << "\nwall_adjacent_acoustic_scale_final_p01=" << fl(q(sf, 0.01))
      << "\nwall_adjacent_acoustic_scale_final_p50=" << fl(q(sf, 0.5))
      << "\ndissipation_debug_csv=" << (out_dir / "dissipation_debug.csv").string()
      << "\nstartup_first_order_iters=" << cfg.startup_first_order_iters << "\nrk_stages=" << cfg.rk_stages
      << "\nlocal_time_stepping=" << (cfg.local_time_stepping ? "on" : "off")
      << "\nforce_stability_window=" << cfg.force_stability_window
      << "\nforce_mean_drift_tol=" << fl(cfg.force_mean_drift_tol)
      << "\nforce_window_stable_final=" << (nonfinite ? 0 : ws) << "\nforce_mean_drift_stable_final=" << (nonfinite ? 0 : ds)
      << "\nforce_physical_converged_final=" << (nonfinite ? 0 : (ws && ds))
      << "\nforce_mean_dcl_final=" << fl(last.mean_dcl) << "\nforce_mean_dcd_final=" << fl(last.mean_dcd)
      << "\nforce_mean_dcm_final=" << fl(last.mean_dcm)
      << "\npressure_fluctuation_nd_max_final=" << fl(last.max_abs_dp_domain / pressure_ref)
      << "\npressure_fluctuation_nd_wall_final=" << fl(last.max_abs_dp_wall / pressure_ref)
      << "\npressure_fluctuation_nd_farfield_final=" << fl(last.max_farfield_abs_dp / pressure_ref)
      << "\ncd_times_mach_final=" << fl(last.cd * std::max(cfg.mach, 0.0)) << "\nmax_wall_mass_flux=0"
      << "\nprecision=" << (cfg.precision == AERO_PRECISION_FP64 ? "fp64" : "fp32") << "\n";
  }
  std::snprintf(summary->status, sizeof(summary->status), "ok");
  std::snprintf(summary->backend, sizeof(summary->backend), "cuda");
  std::snprintf(summary->case_type, sizeof(summary->case_type), "euler_airfoil_2d");
  std::snprintf(summary->run_log, sizeof(summary->run_log), "%s", log_path.string().c_str());
  summary->iterations = static_cast<int>(hist.size());
  summary->residual_l1 = fl(last.residual_l1);
  summary->residual_l2 = fl(last.residual_l2);
  summary->residual_linf = fl(last.residual_linf);
  summary->cl = fl(last.cl);
  summary->cd = fl(last.cd);
  summary->cm = fl(last.cm);
}

// run_euler_airfoil_case (euler_solver.cpp:463-1487) on the device.
void run_euler(const aero_case_desc& cfg_in, const aero_airfoil_mesh_cfg& mc, const fs::path& out_dir,
               const DriverOpts& opts, aero_run_summary* summary) {
  if (cfg_in.iterations <= 0) throw std::invalid_argument("Euler iterations must be positive.");
  if (cfg_in.rk_stages != 1 && cfg_in.rk_stages != 3)
    throw std::invalid_argument("Euler pseudo-time rk_stages must be 1 or 3.");
  EulerMesh em;
  build_mesh(mc, &em);
  const EulerCase ec = prepare_case(cfg_in, mc, em, out_dir, opts);
  const int N = em.N;
  CtxHolder ch;
  check(aero_create(&em.md, &ec.cfg, &ch.c), nullptr, "aero_create");
  if (!opts.restart_in.empty()) {  // start from a dumped state instead of the free stream
    std::vector<double> u0(5 * static_cast<size_t>(N));
    if (aero_state_read(opts.restart_in.c_str(), N, u0.data()) != AERO_OK)
      throw std::invalid_argument(std::string("restart_in: ") + aero_driver_last_error());
    check(aero_set_state(ch.c, u0.data()), ch.c, "aero_set_state");
  }
  std::vector<aero_iter_record> recs(512), hist;
  int remaining = ec.cfg.iterations;
  bool stop = false, nonfinite = false;
  while (remaining > 0 && !stop) {
    const int chunk = std::min(remaining, static_cast<int>(recs.size()));
    int done = 0;
    const int rc = aero_run(ch.c, chunk, recs.data(), &done);
    if (rc != AERO_ERR_NONFINITE) check(rc, ch.c, "aero_run");
    stop = take_records(recs.data(), done, chunk, &hist, &nonfinite);
    remaining -= done;
  }
  if (hist.empty()) throw std::runtime_error("Euler run produced no iterations.");
  write_history(ec, em, hist);
  std::vector<double> U(5 * static_cast<size_t>(N)), R(5 * static_cast<size_t>(N)), SR(N);
  check(aero_get_state(ch.c, U.data()), ch.c, "aero_get_state");
  check(aero_get_last_residual(ch.c, R.data(), SR.data()), ch.c, "aero_get_last_residual");
  write_final(ec, em, U, R, hist, nonfinite, summary);
}

// A sweep of the base case over angles of attack (and Mach numbers): every case runs in one
// batched context on the base case's mesh, and each writes the outputs of a single run into
// out_root/run_NNN (python/cfd/sweep.py:41-56 runs them one after another). The cases'
// results are those of single runs: a batch reproduces them bit for bit.
void run_sweep(const aero_case_desc& base, const aero_airfoil_mesh_cfg& mc, int n, const double* aoa,
               const double* mach, const fs::path& out_root, const DriverOpts& opts, const std::string& case_path,
               aero_run_summary* summaries) {
  if (n <= 0) throw std::invalid_argument("a sweep needs at least one case");
  EulerMesh em;
  build_mesh(mc, &em);
  const int N = em.N;
  fs::create_directories(out_root);
  std::vector<EulerCase> cases;
  std::vector<aero_case_desc> cds;
  for (int k = 0; k < n; ++k) {
    aero_case_desc c = base;
    c.aoa_deg = static_cast<double>(static_cast<float>(aoa[k]));  // case values are floats
    if (mach) c.mach = static_cast<double>(static_cast<float>(mach[k]));
    char name[32];
    std::snprintf(name, sizeof(name), "run_%03d", k);
    cases.push_back(prepare_case(c, mc, em, out_root / name, opts));
    cds.push_back(cases.back().cfg);
  }
  std::vector<aero_mesh_desc> mds(static_cast<size_t>(n), em.md);
  CtxHolder ch;
  check(aero_batch_create(n, mds.data(), cds.data(), &ch.c), nullptr, "aero_batch_create");
  if (!opts.restart_in.empty()) {
    std::vector<double> u0(5 * static_cast<size_t>(N));
    if (aero_state_read(opts.restart_in.c_str(), N, u0.data()) != AERO_OK)
      throw std::invalid_argument(std::string("restart_in: ") + aero_driver_last_error());
    for (int k = 0; k < n; ++k) check(aero_batch_set_state(ch.c, k, u0.data()), ch.c, "aero_batch_set_state");
  }
  const int cap = 512;
  std::vector<aero_iter_record> recs(static_cast<size_t>(n) * cap);
  std::vector<int> done(n);
  std::vector<std::vector<aero_iter_record>> hist(n);
  std::vector<char> stopped(n, 0), nonfinite(n, 0);
  int remaining = base.iterations;
  auto running = [&] { return std::count(stopped.begin(), stopped.end(), 0) > 0; };
  while (remaining > 0 && running()) {
    const int chunk = std::min(remaining, cap);
    const int rc = aero_batch_run(ch.c, chunk, recs.data(), done.data());
    if (rc != AERO_ERR_NONFINITE) check(rc, ch.c, "aero_batch_run");
    for (int k = 0; k < n; ++k) {
      if (stopped[k]) continue;
      bool nf = false;
      stopped[k] = take_records(recs.data() + static_cast<size_t>(k) * chunk, done[k], chunk, &hist[k], &nf);
      nonfinite[k] = nf;
    }
    remaining -= chunk;
  }
  std::ofstream sweep_csv(out_root / "sweep_summary.csv", std::ios::trunc);
  sweep_csv << "run,aoa_deg,mach,iterations,residual_l2,cl,cd,cm,status\n";
  for (int k = 0; k < n; ++k) {
    if (hist[k].empty()) throw std::runtime_error("sweep case " + std::to_string(k) + " produced no iterations.");
    write_history(cases[k], em, hist[k]);
    std::vector<double> U(5 * static_cast<size_t>(N)), R(5 * static_cast<size_t>(N)), SR(N);
    check(aero_batch_get_state(ch.c, k, U.data()), ch.c, "aero_batch_get_state");
    check(aero_batch_get_last_residual(ch.c, k, R.data(), SR.data()), ch.c, "aero_batch_get_last_residual");
    aero_run_summary& sm = summaries[k];
    std::memset(&sm, 0, sizeof(sm));
    std::snprintf(sm.run_log, sizeof(sm.run_log), "%s", case_path.c_str());  // case_path for run.log
    write_final(cases[k], em, U, R, hist[k], nonfinite[k] != 0, &sm);
    const aero_iter_record& last = hist[k].back();
    sweep_csv << k << "," << static_cast<float>(cases[k].cfg.aoa_deg) << "," << static_cast<float>(cases[k].cfg.mach)
              << "," << hist[k].size() << "," << static_cast<float>(last.residual_l2) << ","
              << static_cast<float>(last.cl) << "," << static_cast<float>(last.cd) << ","
              << static_cast<float>(last.cm) << "," << (nonfinite[k] ? "nonfinite" : "ok") << "\n";
  }
}

template <class Fn>
int guard(Fn&& fn) {
  try {
    fn();
    return AERO_OK;
  } catch (const std::invalid_argument& e) {
    g_driver_error = e.what();
    return AERO_ERR_INVALID;
  } catch (const std::bad_alloc&) {
    g_driver_error = "host allocation failed";
    return AERO_ERR_NOMEM;
  } catch (const std::exception& e) {
    g_driver_error = e.what();
    return AERO_ERR_CUDA;
  }
}

}  // namespace

extern "C" {

const char* aero_driver_last_error(void) { return g_driver_error.c_str(); }

int aero_normalize_backend(const char* backend, char* normalized, int len) {
  std::string b = lower(backend ? backend : "");
  if (b.empty()) b = "cpu";
  if (normalized && len > 0) std::snprintf(normalized, static_cast<size_t>(len), "%s", b.c_str());
  if (b != "cpu" && b != "cuda") {
    g_driver_error = "Unsupported backend. Use 'cpu' or 'cuda'.";
    return AERO_ERR_INVALID;
  }
  if (b == "cpu") {
    g_driver_error = "backend 'cpu' is the reference library's CPU path; this library implements backend 'cuda'";
    return AERO_ERR_INVALID;
  }
  if (!aero_cuda_available()) {
    g_driver_error =
        "CUDA backend requested but unavailable. A compute capability 10.3 (GB300) device must be visible.";
    return AERO_ERR_CUDA;
  }
  return AERO_OK;
}

int aero_parse_case(const char* case_path, aero_case_desc* cfg, aero_airfoil_mesh_cfg* mesh, char* case_type,
                    int case_type_len) {
  if (!case_path || !cfg || !mesh) {
    g_driver_error = "aero_parse_case: null argument";
    return AERO_ERR_INVALID;
  }
  return guard([&] {
    const KV kv = parse_kv(case_path);
    map_case(kv, cfg, mesh);
    if (case_type && case_type_len > 0)
      std::snprintf(case_type, static_cast<size_t>(case_type_len), "%s",
                    get_s(kv, "case_type", "scalar_advect_demo").c_str());
  });
}

int aero_run_euler_airfoil_case(const aero_case_desc* cfg, const aero_airfoil_mesh_cfg* mesh, const char* out_dir,
                                aero_run_summary* out) {
  if (!cfg || !mesh || !out_dir || !out) {
    g_driver_error = "aero_run_euler_airfoil_case: null argument";
    return AERO_ERR_INVALID;
  }
  return guard([&] {
    std::memset(out, 0, sizeof(*out));
    run_euler(*cfg, *mesh, out_dir, DriverOpts{}, out);
  });
}

int aero_state_write(const char* path, int num_cells, const double* conserved) {
  if (!path || !conserved || num_cells <= 0) {
    g_driver_error = "aero_state_write: bad argument";
    return AERO_ERR_INVALID;
  }
  return guard([&] {
    std::ofstream o(path, std::ios::binary | std::ios::trunc);
    if (!o) throw std::invalid_argument(std::string("cannot write ") + path);
    const int64_t head[2] = {num_cells, 5};
    o.write(kStateMagic, sizeof(kStateMagic));
    o.write(reinterpret_cast<const char*>(head), sizeof(head));
    o.write(reinterpret_cast<const char*>(conserved), static_cast<std::streamsize>(sizeof(double) * 5 * num_cells));
    if (!o) throw std::invalid_argument(std::string("cannot write ") + path);
  });
}

int aero_state_read(const char* path, int num_cells, double* conserved) {
  if (!path || !conserved || num_cells <= 0) {
    g_driver_error = "aero_state_read: bad argument";
    return AERO_ERR_INVALID;
  }
  return guard([&] {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::invalid_argument(std::string("cannot read ") + path);
    char magic[sizeof(kStateMagic)];
    int64_t head[2] = {0, 0};
    in.read(magic, sizeof(magic));
    in.read(reinterpret_cast<char*>(head), sizeof(head));
    if (!in || std::memcmp(magic, kStateMagic, sizeof(magic)) != 0)
      throw std::invalid_argument(std::string(path) + " is not a state file");
    if (head[0] != num_cells || head[1] != 5)
      throw std::invalid_argument("state file holds " + std::to_string(head[0]) + " cells, the mesh has " +
                                  std::to_string(num_cells));
    in.read(reinterpret_cast<char*>(conserved), static_cast<std::streamsize>(sizeof(double) * 5 * num_cells));
    if (!in) throw std::invalid_argument(std::string(path) + " is truncated");
  });
}

int aero_run_case(const char* case_path, const char* out_dir, const char* backend, aero_run_summary* out) {
  if (!case_path || !out_dir || !out) {
    g_driver_error = "aero_run_case: null argument";
    return AERO_ERR_INVALID;
  }
  char nb[16];
  const int rc = aero_normalize_backend(backend, nb, sizeof(nb));
  if (rc != AERO_OK) return rc;
  return guard([&] {
    fs::create_directories(out_dir);
    const KV kv = parse_kv(case_path);
    const std::string case_type = get_s(kv, "case_type", "scalar_advect_demo");
    if (case_type != "euler_airfoil_2d")
      throw std::invalid_argument("case_type '" + case_type + "' is not served by the device Euler path");
    aero_case_desc c;
    aero_airfoil_mesh_cfg m;
    map_case(kv, &c, &m);
    const DriverOpts opts = map_opts(kv, fs::path(case_path).parent_path());
    std::memset(out, 0, sizeof(*out));
    std::snprintf(out->run_log, sizeof(out->run_log), "%s", case_path);  // case_path for run.log
    run_euler(c, m, out_dir, opts, out);
  });
}

int aero_run_sweep(const char* case_path, int n_cases, const double* aoa_deg, const double* mach,
                   const char* out_root, const char* backend, aero_run_summary* summaries) {
  if (!case_path || !out_root || !aoa_deg || !summaries || n_cases <= 0) {
    g_driver_error = "aero_run_sweep: bad argument";
    return AERO_ERR_INVALID;
  }
  char nb[16];
  const int rc = aero_normalize_backend(backend, nb, sizeof(nb));
  if (rc != AERO_OK) return rc;
  return guard([&] {
    const KV kv = parse_kv(case_path);
    const std::string case_type = get_s(kv, "case_type", "scalar_advect_demo");
    if (case_type != "euler_airfoil_2d")
      throw std::invalid_argument("case_type '" + case_type + "' is not served by the device Euler path");
    aero_case_desc c;
    aero_airfoil_mesh_cfg m;
    map_case(kv, &c, &m);
    const DriverOpts opts = map_opts(kv, fs::path(case_path).parent_path());
    run_sweep(c, m, n_cases, aoa_deg, mach, out_root, opts, case_path, summaries);
  });
}

}  // extern "C"
