// aero_oracle.hpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of AeroCFD's 2D Euler residual-and-update path, templated on the
// arithmetic type so the same code is
//   * the reference itself at Real=float, Acc=float (checked bitwise against the
//     compiled reference library and against committed golden vectors),
//   * the FP64 oracle at Real=double, Acc=double,
//   * the FP32-bulk / FP64-accumulate oracle at Real=float, Acc=double (the RK
//     stage combination, the preconditioned residual and the conserved state are
//     carried in double; everything else runs in float).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
// file; the product library never links it.
//
// Every function keeps the operation order and branch structure of the reference
// function it restates (cited per function, paths relative to the reference
// project root), so that at Real=float the results are bit-identical when both are
// compiled with -ffp-contract=off.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <deque>
#include <limits>
#include <vector>

namespace aero_oracle {

// ---------------------------------------------------------------------------
// Constants (src/cfd_core/numerics/euler_flux.cpp:9-14, reconstruction.cpp:15-18,
// residual_assembly.cpp:9-11, boundary_conditions.cpp:7, preconditioning.cpp:7).
// In float mode they are the reference's float literals; in double mode the same
// decimal values as doubles.
// ---------------------------------------------------------------------------
template <class R>
struct K {
  static constexpr R rho_floor = R(1.0e-8);
  static constexpr R p_floor = R(1.0e-8);
  static constexpr R wave_floor = R(1.0e-8);
  static constexpr R low_mach_min = R(1.0e-4);
  static constexpr R all_speed_floor = R(1.0e-6);
  static constexpr R smooth_eps = R(1.0e-6);
  static constexpr R vol_floor = R(1.0e-12);
  static constexpr R pi = R(3.14159265358979323846);
};

template <class R>
struct Prim {
  R rho = R(1), u = R(0), v = R(0), w = R(0), p = R(1);
};
template <class R>
struct Cons {
  R rho = R(1), ru = R(0), rv = R(0), rw = R(0), rE = R(1);
};
template <class R>
using V5 = std::array<R, 5>;
template <class R>
using V3 = std::array<R, 3>;

enum FluxScheme : int { kRusanov = 0, kHllc = 1 };
enum Limiter : int { kMinmod = 0, kVenkat = 1 };
enum Bc : int { kInterior = 0, kFarfield = 1, kSlipWall = 2 };

template <class R>
V5<R> as_array(const Cons<R>& c) {
  return {c.rho, c.ru, c.rv, c.rw, c.rE};
}

template <class R>
bool all_finite(const V5<R>& v) {
  for (R x : v) {
    if (!std::isfinite(x)) return false;
  }
  return true;
}

// euler_flux.cpp:101-113
template <class R>
Cons<R> prim_to_cons(const Prim<R>& w, R gamma) {
  Cons<R> c;
  c.rho = std::max(w.rho, K<R>::rho_floor);
  c.ru = c.rho * w.u;
  c.rv = c.rho * w.v;
  c.rw = c.rho * w.w;
  const R ke = R(0.5) * c.rho * (w.u * w.u + w.v * w.v + w.w * w.w);
  const R p = std::max(w.p, K<R>::p_floor);
  c.rE = p / (gamma - R(1)) + ke;
  return c;
}

// euler_flux.cpp:115-127
template <class R>
Prim<R> cons_to_prim(const Cons<R>& c, R gamma) {
  Prim<R> w;
  w.rho = std::max(c.rho, K<R>::rho_floor);
  const R inv = R(1) / w.rho;
  w.u = c.ru * inv;
  w.v = c.rv * inv;
  w.w = c.rw * inv;
  const R ke = R(0.5) * w.rho * (w.u * w.u + w.v * w.v + w.w * w.w);
  w.p = std::max((gamma - R(1)) * (c.rE - ke), K<R>::p_floor);
  return w;
}

// euler_flux.cpp:129-144
template <class R>
void enforce_physical(Cons<R>* s, R gamma) {
  s->rho = std::max(s->rho, K<R>::rho_floor);
  const R inv = R(1) / s->rho;
  const R u = s->ru * inv, v = s->rv * inv, w = s->rw * inv;
  const R ke = R(0.5) * s->rho * (u * u + v * v + w * w);
  s->rE = std::max(s->rE, ke + K<R>::p_floor / (gamma - R(1)));
  const R p = (gamma - R(1)) * (s->rE - ke);
  if (p < K<R>::p_floor) s->rE = ke + K<R>::p_floor / (gamma - R(1));
}

// euler_flux.cpp:150-152
template <class R>
R sound_speed(const Prim<R>& w, R gamma) {
  return std::sqrt(std::max(gamma * w.p / std::max(w.rho, K<R>::rho_floor), R(0)));
}

template <class R>
R normal_velocity(const Prim<R>& w, const V3<R>& n) {
  return w.u * n[0] + w.v * n[1] + w.w * n[2];
}

template <class R>
R speed(const Prim<R>& w) {
  return std::sqrt(w.u * w.u + w.v * w.v + w.w * w.w);
}

// euler_flux.cpp:28-39
template <class R>
V5<R> physical_flux(const Cons<R>& c, const Prim<R>& w, const V3<R>& n) {
  const R un = normal_velocity(w, n);
  return {c.rho * un, c.ru * un + n[0] * w.p, c.rv * un + n[1] * w.p, c.rw * un + n[2] * w.p,
          (c.rE + w.p) * un};
}

// euler_flux.cpp:45-51
template <class R>
R with_sign_floor(R x) {
  if (std::abs(x) >= K<R>::wave_floor) return x;
  return (x >= R(0)) ? K<R>::wave_floor : -K<R>::wave_floor;
}

template <class R>
struct Speeds {
  R lm, lp, sr;
};

// euler_flux.cpp:58-74 (also boundary_conditions.cpp:14-25 for the radius)
template <class R>
Speeds<R> precond_speeds(R un, R a, R acoustic_scale) {
  const R beta = std::clamp(acoustic_scale, K<R>::low_mach_min, R(1));
  const R b2 = beta * beta;
  const R omb2 = R(1) - b2;
  const R ut = R(0.5) * (R(1) + b2) * un;
  const R disc = omb2 * omb2 * un * un + R(4) * b2 * a * a;
  const R ct = R(0.5) * std::sqrt(std::max(disc, R(0)));
  Speeds<R> s;
  s.lm = ut - ct;
  s.lp = ut + ct;
  s.sr = std::max({std::abs(un), std::abs(s.lm), std::abs(s.lp), K<R>::wave_floor});
  return s;
}

// euler_flux.cpp:154-175
template <class R>
R low_mach_dissipation_scale(const Cons<R>& l, const Cons<R>& r, R gamma, bool enable,
                             R cutoff, R mach_ref) {
  if (!enable || cutoff <= R(0)) return R(1);
  const Prim<R> pl = cons_to_prim(l, gamma), pr = cons_to_prim(r, gamma);
  const R al = std::max(sound_speed(pl, gamma), K<R>::wave_floor);
  const R ar = std::max(sound_speed(pr, gamma), K<R>::wave_floor);
  const R ml = speed(pl) / al;
  const R mr = speed(pr) / ar;
  const R face_mach = R(0.5) * (ml + mr);
  const R mstar = std::max(face_mach, std::max(mach_ref, K<R>::wave_floor));
  const R ratio = mstar / std::max(cutoff, K<R>::wave_floor);
  return std::clamp(ratio, K<R>::low_mach_min, R(1));
}

// euler_flux.cpp:81-98 + 177-201
template <class R>
R all_speed_pressure_scale(const Cons<R>& l, const Cons<R>& r, const V3<R>& n, R gamma,
                           bool enable, R cutoff, R f_min, R ramp_weight) {
  if (!enable) return R(1);
  const Prim<R> pl = cons_to_prim(l, gamma), pr = cons_to_prim(r, gamma);
  const R unl = normal_velocity(pl, n), unr = normal_velocity(pr, n);
  const R al = std::max(sound_speed(pl, gamma), K<R>::wave_floor);
  const R ar = std::max(sound_speed(pr, gamma), K<R>::wave_floor);
  const R vl = speed(pl), vr = speed(pr);
  const R mach = std::max(R(0.5) * (vl / al + vr / ar), K<R>::all_speed_floor);
  R mach_n = std::max(R(0.5) * (std::abs(unl) / al + std::abs(unr) / ar), K<R>::all_speed_floor);
  mach_n = std::min(mach_n, mach);
  mach_n = std::max(mach_n, K<R>::all_speed_floor);
  const R cut = std::max(cutoff, K<R>::all_speed_floor);
  const R theta_floor = std::clamp(f_min, K<R>::all_speed_floor, R(1));
  const R theta_n = std::clamp(mach_n / cut, theta_floor, R(1));
  const R ratio = std::clamp(mach / cut, R(0), R(1));
  const R gate = ratio * ratio;
  const R theta_corr = (R(1) - gate) * theta_n + gate;
  const R wgt = std::clamp(ramp_weight, R(0), R(1));
  const R theta_eff = (R(1) - wgt) + wgt * theta_corr;
  return std::clamp(theta_eff, theta_floor, R(1));
}

// euler_flux.cpp:203-239
template <class R>
V5<R> rusanov(const Cons<R>& l, const Cons<R>& r, const V3<R>& n, R gamma, R* mws,
              R acoustic_scale) {
  const Prim<R> pl = cons_to_prim(l, gamma), pr = cons_to_prim(r, gamma);
  const R unl = normal_velocity(pl, n), unr = normal_velocity(pr, n);
  const R al = sound_speed(pl, gamma), ar = sound_speed(pr, gamma);
  const R smax_phys = std::max(std::abs(unl) + al, std::abs(unr) + ar);
  const Speeds<R> sl = precond_speeds(unl, al, acoustic_scale);
  const Speeds<R> sr = precond_speeds(unr, ar, acoustic_scale);
  const R sdiss = std::max(sl.sr, sr.sr);
  if (mws) *mws = std::max(smax_phys, K<R>::wave_floor);
  const V5<R> fl = physical_flux(l, pl, n), fr = physical_flux(r, pr, n);
  const V5<R> ul = as_array(l), ur = as_array(r);
  V5<R> f{};
  for (int k = 0; k < 5; ++k) f[k] = R(0.5) * (fl[k] + fr[k]) - R(0.5) * sdiss * (ur[k] - ul[k]);
  return f;
}

// euler_flux.cpp:241-364
template <class R>
V5<R> hllc(const Cons<R>& l, const Cons<R>& r, const V3<R>& n, R gamma, R* mws, R acoustic_scale,
           bool as_fix, R as_cutoff, R as_fmin, R as_ramp, bool* fallback) {
  if (fallback) *fallback = false;
  const Prim<R> pl = cons_to_prim(l, gamma), pr = cons_to_prim(r, gamma);
  const R unl = normal_velocity(pl, n), unr = normal_velocity(pr, n);
  const R al = sound_speed(pl, gamma), ar = sound_speed(pr, gamma);
  const R pscale = all_speed_pressure_scale(l, r, n, gamma, as_fix, as_cutoff, as_fmin, as_ramp);
  const R pavg = R(0.5) * (pl.p + pr.p);
  const R plc = pavg + pscale * (pl.p - pavg);
  const R prc = pavg + pscale * (pr.p - pavg);
  const Speeds<R> spl = precond_speeds(unl, al, acoustic_scale);
  const Speeds<R> spr = precond_speeds(unr, ar, acoustic_scale);
  const R s_l = std::min(spl.lm, spr.lm);
  const R s_r = std::max(spl.lp, spr.lp);
  const R s_l_phys = std::min(unl - al, unr - ar);
  const R s_r_phys = std::max(unl + al, unr + ar);
  if (mws) *mws = std::max(std::max(std::abs(s_l_phys), std::abs(s_r_phys)), K<R>::wave_floor);

  auto diffusive = [&]() {
    if (fallback) *fallback = true;
    return rusanov(l, r, n, gamma, mws, acoustic_scale);
  };
  if (std::abs(s_r - s_l) < K<R>::wave_floor) return diffusive();

  const V5<R> ul = as_array(l), ur = as_array(r);
  const V5<R> fl = physical_flux(l, pl, n), fr = physical_flux(r, pr, n);
  if (s_l >= R(0)) return fl;
  if (s_r <= R(0)) return fr;

  const R rhol = std::max(pl.rho, K<R>::rho_floor);
  const R rhor = std::max(pr.rho, K<R>::rho_floor);
  const R denom = rhol * (s_l - unl) - rhor * (s_r - unr);
  if (std::abs(denom) < K<R>::wave_floor) return diffusive();
  const R s_m = (prc - plc + rhol * unl * (s_l - unl) - rhor * unr * (s_r - unr)) / denom;

  auto star = [&](const Cons<R>& c, const Prim<R>& w, R pcorr, R s_k, R un_k) {
    V5<R> st = as_array(c);
    const R rho_k = std::max(w.rho, K<R>::rho_floor);
    const R skun = s_k - un_k;
    const R sksm = s_k - s_m;
    if (std::abs(skun) < K<R>::wave_floor || std::abs(sksm) < K<R>::wave_floor) return st;
    const R rho_star = rho_k * skun / sksm;
    const R shift = s_m - un_k;
    st[0] = rho_star;
    st[1] = rho_star * (w.u + shift * n[0]);
    st[2] = rho_star * (w.v + shift * n[1]);
    st[3] = rho_star * (w.w + shift * n[2]);
    const R e_total = c.rE / rho_k;
    const R p_term = pcorr / with_sign_floor(rho_k * skun);
    st[4] = rho_star * (e_total + shift * (s_m + p_term));
    return st;
  };
  const V5<R> usl = star(l, pl, plc, s_l, unl);
  const V5<R> usr = star(r, pr, prc, s_r, unr);
  if (!all_finite(usl) || !all_finite(usr) || usl[0] <= R(0) || usr[0] <= R(0)) return diffusive();

  V5<R> f{};
  if (s_m >= R(0)) {
    for (int k = 0; k < 5; ++k) f[k] = fl[k] + s_l * (usl[k] - ul[k]);
  } else {
    for (int k = 0; k < 5; ++k) f[k] = fr[k] + s_r * (usr[k] - ur[k]);
  }
  if (!all_finite(f)) return diffusive();
  return f;
}

// Numerics switches of one residual evaluation
// (src/cfd_core/include/cfd_core/solvers/euler/residual_assembly.hpp:12-31,
//  preconditioning.hpp:9-15).
template <class R>
struct Numerics {
  R gamma = R(1.4);
  Cons<R> farfield;
  int flux = kHllc;
  int limiter = kMinmod;
  bool second_order = true;
  bool low_mach_fix = false;
  R mach_cutoff = R(0.3);
  R stab_mach_floor = R(0);
  bool precond_farfield_bc = false;
  bool precond = false;
  R pc_mach_ref = R(0.15), pc_mach_min = R(1.0e-3), pc_beta_min = R(0.2), pc_beta_max = R(1);
  bool as_fix = false;
  R as_cutoff = R(0.25), as_fmin = R(0.05), as_ramp = R(1);
};

// euler_flux.cpp:366-395
template <class R>
V5<R> face_flux(const Cons<R>& l, const Cons<R>& r, const V3<R>& n, const Numerics<R>& nm, R* mws,
                R acoustic_scale, bool* fallback) {
  if (nm.flux == kHllc)
    return hllc(l, r, n, nm.gamma, mws, acoustic_scale, nm.as_fix, nm.as_cutoff, nm.as_fmin,
                nm.as_ramp, fallback);
  if (fallback) *fallback = false;
  return rusanov(l, r, n, nm.gamma, mws, acoustic_scale);
}

// preconditioning.cpp:17-22
template <class R>
R local_mach(const Prim<R>& w, R gamma) {
  const R a = std::max(sound_speed(w, gamma), K<R>::wave_floor);
  return speed(w) / a;
}

// preconditioning.cpp:9-15 + 24-32
template <class R>
R cell_beta(const Prim<R>& w, const Numerics<R>& nm) {
  if (!nm.precond) return R(1);
  const R m = local_mach(w, nm.gamma);
  const R target = std::max({m, nm.pc_mach_ref, nm.pc_mach_min, K<R>::wave_floor});
  const R bmin = std::max(nm.pc_beta_min, K<R>::low_mach_min);
  const R bmax = std::max(bmin, nm.pc_beta_max);
  return std::clamp(target, bmin, bmax);
}

// preconditioning.cpp:34-49
template <class R>
R face_beta(const Cons<R>& l, const Cons<R>& r, const Numerics<R>& nm) {
  if (!nm.precond) return R(1);
  const Prim<R> pl = cons_to_prim(l, nm.gamma), pr = cons_to_prim(r, nm.gamma);
  const Prim<R> avg{R(0.5) * (pl.rho + pr.rho), R(0.5) * (pl.u + pr.u), R(0.5) * (pl.v + pr.v),
                    R(0.5) * (pl.w + pr.w), R(0.5) * (pl.p + pr.p)};
  return cell_beta(avg, nm);
}

// residual_assembly.cpp:16-20
template <class R>
R smooth_max(R a, R b) {
  const R d = a - b;
  return R(0.5) * (a + b + std::sqrt(d * d + K<R>::smooth_eps * K<R>::smooth_eps));
}

// residual_assembly.cpp:31-51
template <class R>
R face_acoustic_scale(const Numerics<R>& nm, const Cons<R>& l, const Cons<R>& r, R fbeta) {
  R s = R(1);
  if (nm.precond) s = std::clamp(fbeta, K<R>::low_mach_min, R(1));
  if (nm.low_mach_fix) {
    const R lm = low_mach_dissipation_scale(l, r, nm.gamma, true, nm.mach_cutoff, nm.pc_mach_ref);
    s = std::min(s, lm);
  }
  s = std::clamp(s, K<R>::low_mach_min, R(1));
  const Prim<R> pl = cons_to_prim(l, nm.gamma), pr = cons_to_prim(r, nm.gamma);
  const R fm = R(0.5) * (local_mach(pl, nm.gamma) + local_mach(pr, nm.gamma));
  const R floor_m = std::clamp(nm.stab_mach_floor, R(0), R(1));
  const R meff = smooth_max(fm, floor_m);
  const R stab = std::clamp(meff, K<R>::low_mach_min, R(1));
  return std::max(s, stab);
}

// boundary_conditions.cpp:27-78
template <class R>
Cons<R> precond_farfield_state(const Cons<R>& in, const Cons<R>& ff, const V3<R>& n, R gamma,
                               R acoustic_scale) {
  const Prim<R> pi = cons_to_prim(in, gamma), pf = cons_to_prim(ff, gamma);
  const R uni = normal_velocity(pi, n), unf = normal_velocity(pf, n);
  const R ai = std::max(sound_speed(pi, gamma), K<R>::rho_floor);
  const R af = std::max(sound_speed(pf, gamma), K<R>::rho_floor);
  const R rho_ref = std::max(R(0.5) * (pi.rho + pf.rho), K<R>::rho_floor);
  const R a_ref = std::max(R(0.5) * (ai + af), K<R>::rho_floor);
  const R a_t = std::max(std::clamp(acoustic_scale, K<R>::low_mach_min, R(1)) * a_ref,
                         K<R>::all_speed_floor);
  if (std::abs(uni) >= a_t) return (uni >= R(0)) ? in : ff;
  const R rp = uni + pi.p / (rho_ref * a_t);
  const R rm = unf - pf.p / (rho_ref * a_t);
  const R unb = R(0.5) * (rp + rm);
  const R pb = std::max(R(0.5) * rho_ref * a_t * (rp - rm), K<R>::rho_floor);
  const V3<R> ti{pi.u - uni * n[0], pi.v - uni * n[1], pi.w - uni * n[2]};
  const V3<R> tf{pf.u - unf * n[0], pf.v - unf * n[1], pf.w - unf * n[2]};
  const bool inflow = unb < R(0);
  const V3<R>& t = inflow ? tf : ti;
  const R rho_b = inflow ? pf.rho : pi.rho;
  const R p_b0 = inflow ? pf.p : pi.p;
  const R a_b = inflow ? af : ai;
  Prim<R> b;
  b.rho = std::max(rho_b + (pb - p_b0) / std::max(a_b * a_b, K<R>::rho_floor), K<R>::rho_floor);
  b.u = unb * n[0] + t[0];
  b.v = unb * n[1] + t[1];
  b.w = unb * n[2] + t[2];
  b.p = pb;
  return prim_to_cons(b, gamma);
}

// boundary_conditions.cpp:81-123
template <class R>
V5<R> boundary_flux(int bc, const Cons<R>& in, const V3<R>& n, const Numerics<R>& nm,
                    R acoustic_scale, R* mws, bool* fallback) {
  if (fallback) *fallback = false;
  if (bc == kSlipWall) {
    const Prim<R> w = cons_to_prim(in, nm.gamma);
    const R un = normal_velocity(w, n);
    const R a = sound_speed(w, nm.gamma);
    *mws = precond_speeds(un, a, acoustic_scale).sr;
    return {R(0), w.p * n[0], w.p * n[1], w.p * n[2], R(0)};
  }
  const Cons<R> bs = nm.precond_farfield_bc
                         ? precond_farfield_state(in, nm.farfield, n, nm.gamma, acoustic_scale)
                         : nm.farfield;
  return face_flux(in, bs, n, nm, mws, acoustic_scale, fallback);
}

// ---------------------------------------------------------------------------
// Mesh in the reference layout (src/cfd_core/include/cfd_core/mesh.hpp:14-35),
// restricted to what the path reads; the arithmetic type is the caller's.
// ---------------------------------------------------------------------------
template <class R>
struct Mesh {
  int num_cells = 0;
  int num_faces = 0;
  std::vector<int> owner, neighbor, bc;  // bc: 0 interior, 1 farfield, 2 wall
  std::vector<R> normal;                 // 3 per face, unit, out of owner
  std::vector<R> center;                 // 3 per face
  std::vector<R> area;                   // per face
  std::vector<R> volume;                 // per cell
  std::vector<R> cell_center;            // 3 per cell
  std::vector<int> wall_faces;           // faces of the "wall" patch in patch order
};

template <class R>
V3<R> face_normal(const Mesh<R>& m, int f) {
  return {m.normal[3 * f], m.normal[3 * f + 1], m.normal[3 * f + 2]};
}

template <class R>
R prim_var(const Prim<R>& w, int v) {
  switch (v) {
    case 0: return w.rho;
    case 1: return w.u;
    case 2: return w.v;
    case 3: return w.w;
    default: return w.p;
  }
}
template <class R>
void set_prim_var(Prim<R>* w, int v, R x) {
  switch (v) {
    case 0: w->rho = x; break;
    case 1: w->u = x; break;
    case 2: w->v = x; break;
    case 3: w->w = x; break;
    default: w->p = x; break;
  }
}

// reconstruction.cpp:73-119. Layout [cell][var][comp], 2 components.
template <class R>
std::vector<R> green_gauss(const Mesh<R>& m, const std::vector<Prim<R>>& w) {
  std::vector<R> g(static_cast<size_t>(m.num_cells) * 10, R(0));
  for (int f = 0; f < m.num_faces; ++f) {
    const int o = m.owner[f], nb = m.neighbor[f];
    for (int v = 0; v < 5; ++v) {
      const R qo = prim_var(w[o], v);
      R qf = qo;
      if (nb >= 0) qf = R(0.5) * (qo + prim_var(w[nb], v));
      for (int c = 0; c < 2; ++c) {
        const R nA = m.normal[3 * f + c] * m.area[f];
        g[(o * 5 + v) * 2 + c] += qf * nA;
        if (nb >= 0) g[(nb * 5 + v) * 2 + c] -= qf * nA;
      }
    }
  }
  for (int c = 0; c < m.num_cells; ++c) {
    const R inv = R(1) / std::max(m.volume[c], K<R>::vol_floor);
    for (int k = 0; k < 10; ++k) g[c * 10 + k] *= inv;
  }
  return g;
}

// reconstruction.cpp:121-146
template <class R>
R limit(int lim, R a, R b) {
  if (lim == kVenkat) {
    if (a * b <= R(0)) return R(0);
    const R eps2 = R(1.0e-12) * (R(1) + a * a + b * b);
    const R num = (b * b + R(2) * a * b + eps2) * a;
    const R den = a * a + R(2) * b * b + a * b + eps2;
    if (std::abs(den) <= R(1.0e-20)) return R(0);
    const R x = num / den;
    if (!std::isfinite(x)) return R(0);
    if (a > R(0)) return std::clamp(x, R(0), a);
    return std::clamp(x, a, R(0));
  }
  if (a * b <= R(0)) return R(0);
  return (std::abs(a) < std::abs(b)) ? a : b;
}

// reconstruction.cpp:148-219
template <class R>
void muscl(const Mesh<R>& m, const std::vector<Prim<R>>& w, const std::vector<R>& g, int f,
           int lim, Prim<R>* L, Prim<R>* Rt) {
  const int o = m.owner[f], nb = m.neighbor[f];
  const R dox = m.center[3 * f] - m.cell_center[3 * o];
  const R doy = m.center[3 * f + 1] - m.cell_center[3 * o + 1];
  const R dnx = m.center[3 * f] - m.cell_center[3 * nb];
  const R dny = m.center[3 * f + 1] - m.cell_center[3 * nb + 1];
  *L = w[o];
  *Rt = w[nb];
  for (int v = 0; v < 5; ++v) {
    const R qo = prim_var(w[o], v), qn = prim_var(w[nb], v);
    const R dc = qn - qo;
    R d_o = R(0), d_n = R(0);
    d_o += g[(o * 5 + v) * 2 + 0] * dox;
    d_n += g[(nb * 5 + v) * 2 + 0] * dnx;
    d_o += g[(o * 5 + v) * 2 + 1] * doy;
    d_n += g[(nb * 5 + v) * 2 + 1] * dny;
    set_prim_var(L, v, qo + limit(lim, d_o, dc));
    set_prim_var(Rt, v, qn + limit(lim, d_n, -dc));
  }
  L->rho = std::max(L->rho, K<R>::rho_floor);
  Rt->rho = std::max(Rt->rho, K<R>::rho_floor);
  L->p = std::max(L->p, K<R>::p_floor);
  Rt->p = std::max(Rt->p, K<R>::p_floor);
}

// residual_assembly.cpp:53-58
template <class R>
bool valid_prim(const Prim<R>& w) {
  return std::isfinite(w.rho) && std::isfinite(w.u) && std::isfinite(w.v) && std::isfinite(w.w) &&
         std::isfinite(w.p) && w.rho > K<R>::rho_floor && w.p > K<R>::p_floor;
}

struct AssemblyDiag {
  int first_order_fallback = 0;
  int diffusive_fallback = 0;
  int first_failure_face = -1;
  int first_failure_owner = -1;
  int first_failure_neighbor = -1;
};

// residual_assembly.cpp:73-182. res, sr must be sized 5N and N; they are zeroed here.
// fscale (optional, test metric only) receives per cell and component sum_faces |F_k A|.
template <class R>
void assemble(const Mesh<R>& m, const std::vector<Prim<R>>& w, const std::vector<R>& g,
              const Numerics<R>& nm, std::vector<R>* res, std::vector<R>* sr, AssemblyDiag* diag,
              std::vector<double>* fscale = nullptr) {
  res->assign(static_cast<size_t>(m.num_cells) * 5, R(0));
  sr->assign(static_cast<size_t>(m.num_cells), R(0));
  if (fscale) fscale->assign(static_cast<size_t>(m.num_cells) * 5, 0.0);
  AssemblyDiag dg;
  for (int f = 0; f < m.num_faces; ++f) {
    const int o = m.owner[f], nb = m.neighbor[f];
    const V3<R> n = face_normal(m, f);
    const R area = m.area[f];
    V5<R> flux{};
    R mws = R(0);
    bool fb = false;
    if (nb >= 0) {
      Prim<R> L = w[o], Rt = w[nb];
      if (nm.second_order) {
        muscl(m, w, g, f, nm.limiter, &L, &Rt);
        if (!valid_prim(L) || !valid_prim(Rt)) {
          if (dg.first_failure_face < 0) {
            dg.first_failure_face = f;
            dg.first_failure_owner = o;
            dg.first_failure_neighbor = nb;
          }
          L = w[o];
          Rt = w[nb];
          ++dg.first_order_fallback;
        }
      }
      const Cons<R> cl = prim_to_cons(L, nm.gamma), cr = prim_to_cons(Rt, nm.gamma);
      const R fb_beta = face_beta(cl, cr, nm);
      const R as = face_acoustic_scale(nm, cl, cr, fb_beta);
      flux = face_flux(cl, cr, n, nm, &mws, as, &fb);
    } else {
      const Cons<R> in = prim_to_cons(w[o], nm.gamma);
      const int bc = m.bc[f];
      Cons<R> ex = nm.farfield;
      R fb_beta;
      if (bc == kSlipWall) {
        fb_beta = face_beta(in, in, nm);
        ex = in;
      } else {
        fb_beta = face_beta(in, nm.farfield, nm);
      }
      const R as = face_acoustic_scale(nm, in, ex, fb_beta);
      flux = boundary_flux(bc, in, n, nm, as, &mws, &fb);
    }
    if (fb) ++dg.diffusive_fallback;
    const R wave = mws * area;
    (*sr)[o] += wave;
    for (int k = 0; k < 5; ++k) {
      const R fa = flux[k] * area;
      (*res)[5 * o + k] += fa;
      if (nb >= 0) (*res)[5 * nb + k] -= fa;
      if (fscale) {
        (*fscale)[5 * o + k] += std::abs(static_cast<double>(fa));
        if (nb >= 0) (*fscale)[5 * nb + k] += std::abs(static_cast<double>(fa));
      }
    }
    if (nb >= 0) (*sr)[nb] += wave;
  }
  if (diag) *diag = dg;
}

// preconditioning.cpp:51-76 (computed in the accumulator type A)
template <class R, class A>
void precondition_residual(const std::vector<Prim<R>>& w, const Numerics<R>& nm,
                           std::vector<A>* res) {
  if (!nm.precond) return;
  Numerics<A> na;
  na.gamma = A(nm.gamma);
  na.precond = true;
  na.pc_mach_ref = A(nm.pc_mach_ref);
  na.pc_mach_min = A(nm.pc_mach_min);
  na.pc_beta_min = A(nm.pc_beta_min);
  na.pc_beta_max = A(nm.pc_beta_max);
  for (size_t c = 0; c < w.size(); ++c) {
    const Prim<A> p{A(w[c].rho), A(w[c].u), A(w[c].v), A(w[c].w), A(w[c].p)};
    const A beta = cell_beta(p, na);
    const A b2 = beta * beta;
    const A rho = std::max(p.rho, K<A>::rho_floor);
    const A inv_rho = A(1) / rho;
    A* r = res->data() + 5 * c;
    const A ud = p.u * r[1] + p.v * r[2] + p.w * r[3];
    r[4] = b2 * r[4] + (b2 - A(1)) * inv_rho * ud;
  }
}

// The same energy row in float with fused multiply-adds (the FP32-bulk mode's arithmetic):
// ud = fma(u, r1, v r2), r4 = fma(b2, r4, (b2 - 1) / rho * ud).
template <class A>
void precondition_residual_fma(const std::vector<Prim<float>>& w, const Numerics<float>& nm, std::vector<A>* res) {
  if (!nm.precond) return;
  for (size_t c = 0; c < w.size(); ++c) {
    const float beta = cell_beta(w[c], nm);
    const float b2 = beta * beta;
    const float inv_rho = 1.0f / std::max(w[c].rho, K<float>::rho_floor);
    A* r = res->data() + 5 * c;
    const float ud = std::fma(w[c].u, float(r[1]), w[c].v * float(r[2]));
    r[4] = A(std::fma(b2, float(r[4]), (b2 - 1.0f) * inv_rho * ud));
  }
}

// The FP32-bulk mode's low-Mach energy row (preconditioning.cpp:51-76): beta from the float
// state, N = b2 (r4 rho) + (b2 - 1)(u r1 + v r2) formed in double with one fused
// multiply-add (the device forms the same sum in double-float arithmetic), then
// r4 = float(N) / rho in float.
template <class A>
void precondition_residual_row64(const std::vector<Prim<float>>& w, const Numerics<float>& nm,
                                 std::vector<A>* res) {
  if (!nm.precond) return;
  for (size_t c = 0; c < w.size(); ++c) {
    const float beta = cell_beta(w[c], nm);
    const float rho = std::max(w[c].rho, K<float>::rho_floor);
    A* r = res->data() + 5 * c;
    const double b2 = double(beta) * double(beta);
    const double rr = double(float(r[4])) * double(rho);
    const double ud = double(w[c].u) * double(float(r[1])) + double(w[c].v) * double(float(r[2]));
    const double n = std::fma(b2, rr, (b2 - 1.0) * ud);
    r[4] = A(float(n) / rho);
  }
}

// time_integrator.cpp:31-59
template <class R>
std::vector<R> dt_over_volume(const std::vector<R>& sr, R cfl, bool local) {
  std::vector<R> dt(sr.size(), R(0));
  if (sr.empty()) return dt;
  if (local) {
    for (size_t c = 0; c < sr.size(); ++c) dt[c] = cfl / std::max(sr[c], K<R>::wave_floor);
    return dt;
  }
  R g = std::numeric_limits<R>::max();
  for (R s : sr) g = std::min(g, cfl / std::max(s, K<R>::wave_floor));
  if (!std::isfinite(g)) g = R(0);
  std::fill(dt.begin(), dt.end(), g);
  return dt;
}

// time_integrator.cpp:61-104, in the accumulator type A.
template <class A>
void rk_stage(int stage, const std::vector<A>& un, const std::vector<A>& us,
              const std::vector<A>& rp, const std::vector<A>& dtv, A gamma, std::vector<A>* out) {
  const size_t n = dtv.size();
  out->assign(n * 5, A(0));
  const A third = A(1) / A(3), two_thirds = A(2) / A(3);
  for (size_t c = 0; c < n; ++c) {
    Cons<A> s{us[5 * c], us[5 * c + 1], us[5 * c + 2], us[5 * c + 3], us[5 * c + 4]};
    const A d = dtv[c];
    s.rho -= d * rp[5 * c];
    s.ru -= d * rp[5 * c + 1];
    s.rv -= d * rp[5 * c + 2];
    s.rw -= d * rp[5 * c + 3];
    s.rE -= d * rp[5 * c + 4];
    if (stage >= 1) {
      const A* b = un.data() + 5 * c;
      const A cb = (stage == 1) ? A(0.75) : third;
      const A cs = (stage == 1) ? A(0.25) : two_thirds;
      s.rho = cb * b[0] + cs * s.rho;
      s.ru = cb * b[1] + cs * s.ru;
      s.rv = cb * b[2] + cs * s.rv;
      s.rw = cb * b[3] + cs * s.rw;
      s.rE = cb * b[4] + cs * s.rE;
    }
    enforce_physical(&s, gamma);
    A* o = out->data() + 5 * c;
    o[0] = s.rho;
    o[1] = s.ru;
    o[2] = s.rv;
    o[3] = s.rw;
    o[4] = s.rE;
  }
}

// euler_solver.cpp:309-339
template <class R>
struct Norms {
  R l1 = R(0), l2 = R(0), linf = R(0);
};
template <class R>
Norms<R> residual_norms(const Mesh<R>& m, const std::vector<R>& res, std::vector<R>* mag) {
  double l1 = 0.0, l2s = 0.0, linf = 0.0;
  if (mag) mag->assign(static_cast<size_t>(m.num_cells), R(0));
  for (int c = 0; c < m.num_cells; ++c) {
    const R inv = R(1) / std::max(m.volume[c], K<R>::vol_floor);
    double cm2 = 0.0;
    for (int k = 0; k < 5; ++k) {
      const R val = res[5 * c + k] * inv;
      const double a = std::abs(static_cast<double>(val));
      l1 += a;
      l2s += a * a;
      linf = std::max(linf, a);
      cm2 += static_cast<double>(val) * static_cast<double>(val);
    }
    if (mag) (*mag)[c] = static_cast<R>(std::sqrt(cm2));
  }
  Norms<R> out;
  out.l1 = static_cast<R>(l1);
  out.l2 = static_cast<R>(std::sqrt(l2s / std::max(1, m.num_cells * 5)));
  out.linf = static_cast<R>(linf);
  return out;
}

// Freestream reference for forces (src/cfd_core/include/cfd_core/post/forces.hpp:9-17).
template <class R>
struct Reference {
  R rho_inf = R(1.225), p_inf = R(101325), aoa_deg = R(0), speed_inf = R(1), chord = R(1);
  R x_ref = R(0.25), y_ref = R(0);
};

template <class R>
struct Forces {
  R fx = 0, fy = 0, lift = 0, drag = 0, moment = 0, cl = 0, cd = 0, cm = 0;
};
template <class R>
struct ForceDiag {
  R sum_nax = 0, sum_nay = 0, fx_abs = 0, fy_abs = 0, fx_gauge = 0, fy_gauge = 0;
};

// forces.cpp:208-249
template <class R>
ForceDiag<R> force_diagnostics(const Mesh<R>& m, const std::vector<R>& p, const Reference<R>& ref) {
  ForceDiag<R> d;
  for (int f : m.wall_faces) {
    const R nax = -m.normal[3 * f] * m.area[f];
    const R nay = -m.normal[3 * f + 1] * m.area[f];
    const R pc = p[m.owner[f]];
    const R gp = pc - ref.p_inf;
    d.sum_nax += nax;
    d.sum_nay += nay;
    d.fx_abs -= pc * nax;
    d.fy_abs -= pc * nay;
    d.fx_gauge -= gp * nax;
    d.fy_gauge -= gp * nay;
  }
  return d;
}

// forces.cpp:251-294
template <class R>
Forces<R> integrate_forces(const Mesh<R>& m, const std::vector<R>& p, const Reference<R>& ref,
                           bool gauge) {
  const ForceDiag<R> d = force_diagnostics(m, p, ref);
  const R q = R(0.5) * ref.rho_inf * ref.speed_inf * ref.speed_inf + R(1.0e-12);
  const R alpha = ref.aoa_deg * (K<R>::pi / R(180));
  const R ca = std::cos(alpha), sa = std::sin(alpha);
  const R chord = std::max(ref.chord, R(1.0e-8));
  const R s_ref = chord * R(1);
  Forces<R> out;
  out.fx = gauge ? d.fx_gauge : d.fx_abs;
  out.fy = gauge ? d.fy_gauge : d.fy_abs;
  for (int f : m.wall_faces) {
    const R pc = p[m.owner[f]];
    const R pr = gauge ? (pc - ref.p_inf) : pc;
    const R nax = -m.normal[3 * f] * m.area[f];
    const R nay = -m.normal[3 * f + 1] * m.area[f];
    const R dfx = -pr * nax;
    const R dfy = -pr * nay;
    const R x = m.center[3 * f] - ref.x_ref;
    const R y = m.center[3 * f + 1] - ref.y_ref;
    out.moment += x * dfy - y * dfx;
  }
  out.drag = out.fx * ca + out.fy * sa;
  out.lift = -out.fx * sa + out.fy * ca;
  out.cd = out.drag / (q * s_ref);
  out.cl = out.lift / (q * s_ref);
  out.cm = out.moment / (q * s_ref * chord);
  return out;
}

// convergence_monitor.cpp:13-127
template <class R>
struct Monitor {
  R residual_target = R(1.0e-3), stab_tol = R(2.0e-5), drift_tol = R(2.0e-5);
  int window = 6, min_iterations = 40;
  R initial_l2 = R(-1);
  bool has_prev = false;
  Forces<R> prev;
  std::deque<Forces<R>> hist;

  void init() {
    if (drift_tol <= R(0)) drift_tol = stab_tol;
  }
  R update_residual(R l2) {
    const R b = std::max(l2, R(1.0e-20));
    if (initial_l2 < R(0)) initial_l2 = b;
    return b / std::max(initial_l2, R(1.0e-20));
  }
  V3<R> update_forces(const Forces<R>& f) {
    V3<R> d{R(0), R(0), R(0)};
    if (has_prev) d = {std::abs(f.cl - prev.cl), std::abs(f.cd - prev.cd), std::abs(f.cm - prev.cm)};
    prev = f;
    has_prev = true;
    const int req = std::max(window, 1);
    hist.push_back(f);
    while (static_cast<int>(hist.size()) > 2 * req) hist.pop_front();
    return d;
  }
  bool stable() const {
    const int req = std::max(window, 1);
    if (static_cast<int>(hist.size()) < req) return false;
    const int b = static_cast<int>(hist.size()) - req;
    R l0 = hist[b].cl, l1 = l0, d0 = hist[b].cd, d1 = d0, m0 = hist[b].cm, m1 = m0;
    for (int i = b; i < static_cast<int>(hist.size()); ++i) {
      l0 = std::min(l0, hist[i].cl);
      l1 = std::max(l1, hist[i].cl);
      d0 = std::min(d0, hist[i].cd);
      d1 = std::max(d1, hist[i].cd);
      m0 = std::min(m0, hist[i].cm);
      m1 = std::max(m1, hist[i].cm);
    }
    return (l1 - l0) <= stab_tol && (d1 - d0) <= stab_tol && (m1 - m0) <= stab_tol;
  }
  bool drift(V3<R>* out) const {
    const int req = std::max(window, 1);
    if (static_cast<int>(hist.size()) < 2 * req) return false;
    const int pb = static_cast<int>(hist.size()) - 2 * req;
    const int cb = static_cast<int>(hist.size()) - req;
    R a[3] = {0, 0, 0}, c[3] = {0, 0, 0};
    for (int i = pb; i < cb; ++i) {
      a[0] += hist[i].cl;
      a[1] += hist[i].cd;
      a[2] += hist[i].cm;
    }
    for (int i = cb; i < static_cast<int>(hist.size()); ++i) {
      c[0] += hist[i].cl;
      c[1] += hist[i].cd;
      c[2] += hist[i].cm;
    }
    const R inv = R(1) / static_cast<R>(req);
    for (int k = 0; k < 3; ++k) (*out)[k] = std::abs(c[k] * inv - a[k] * inv);
    return true;
  }
  bool drift_stable() const {
    V3<R> d;
    if (!drift(&d)) return false;
    return d[0] <= drift_tol && d[1] <= drift_tol && d[2] <= drift_tol;
  }
  bool converged(int iter, R ratio) const {
    if (iter + 1 < min_iterations) return false;
    if (ratio > residual_target) return false;
    return stable() && drift_stable();
  }
};

}  // namespace aero_oracle
