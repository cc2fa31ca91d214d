// aero_oracle_driver.hpp -- TEST INFRASTRUCTURE ONLY.
//
// The pseudo-time iteration loop of run_euler_airfoil_case
// (src/cfd_core/solvers/euler_solver.cpp:463-1208) restated on an injected mesh.
// R is the residual (bulk) type, A the type of the conserved state across RK stages,
// of the norms/forces and of the controller scalars. <float,float> is the reference,
// <double,double> the FP64 oracle, <float,double> the FP32-bulk / FP64-accumulate oracle,
// whose residual preconditioning is float with fused multiply-adds, as the device forms it.
#pragma once

#include "aero_oracle.hpp"
#include "../include/aero_gb300.h"

#include <string>
#include <type_traits>

namespace aero_oracle {

// euler_solver.cpp:69-79
template <class A>
A schedule_cfl(A start, A mx, int ramp, int iter, A scale) {
  A base;
  if (ramp <= 0) {
    base = mx;
  } else {
    const A t = std::min(A(1), static_cast<A>(iter + 1) / static_cast<A>(std::max(ramp, 1)));
    base = start + t * (mx - start);
  }
  return base * scale;
}

// euler_solver.cpp:93-104
template <class A>
A schedule_stab_floor(A start, A target, int ramp, int iter) {
  const A m0s = std::clamp(start, A(0), A(1));
  const A m0t = std::clamp(target, A(0), A(1));
  if (ramp <= 0) return m0t;
  const A t = std::clamp(static_cast<A>(std::max(iter, 0)) / static_cast<A>(std::max(ramp, 1)),
                         A(0), A(1));
  return m0s + t * (m0t - m0s);
}

// euler_solver.cpp:106-112
template <class A>
A schedule_all_speed_ramp(int on, int len, int iter) {
  if (len <= 0) return (iter >= on) ? A(1) : A(0);
  const A x = static_cast<A>(iter - on) / static_cast<A>(std::max(len, 1));
  return std::clamp(x, A(0), A(1));
}

// Float screen of the FP32-bulk mode: true when enforce_physical is provably the identity.
inline bool positivity_safe(const Cons<double>& s, float gm1) {
  const float r = static_cast<float>(s.rho);
  if (!(r > 2.0e-8f)) return false;
  const float inv = 1.0f / r;
  const float u = static_cast<float>(s.ru) * inv, v = static_cast<float>(s.rv) * inv;
  const float ke = 0.5f * r * (u * u + v * v);
  const float e = static_cast<float>(s.rE) - ke;
  return e > 1.0e-3f * static_cast<float>(s.rE) && gm1 * e > 2.0e-8f;
}

// Float-float arithmetic of the FP32-bulk mode's conserved state: hi is the float image,
// lo the remainder. Knuth's error-free two-sum, so that s + e == a + b exactly.
inline void two_sum(float a, float b, float* s, float* e) {
  const float x = a + b;
  const float bb = x - a;
  *e = (a - (x - bb)) + (b - bb);
  *s = x;
}
inline void ff_add(float hi, float lo, float d, float* nh, float* nl) {
  float s, e;
  two_sum(hi, d, &s, &e);
  two_sum(s, lo + e, nh, nl);
}
inline void ff_split(double u, float* hi, float* lo) {
  *hi = static_cast<float>(u);
  *lo = static_cast<float>(u - static_cast<double>(*hi));
}

// RK3 stage of the FP32-bulk mode in delta form: delta' = b (delta - dt R) with b = 1, 1/4,
// 2/3 (the RK3 weights sum to one). Intermediate stage states are float, hi + delta' with hi
// the float image of U_n, clamped in float; the last stage adds delta' to the float-float
// pair (hi, lo) of U_n and clamps in double only when the float screen cannot prove the clamp
// is the identity. *us receives the stage state (the float state widened, or hi + lo).
inline void rk_stage_delta(int stage, bool last, std::vector<float>* uhi, std::vector<float>* ulo,
                           const std::vector<double>& rp, const std::vector<float>& dt, double gamma,
                           std::vector<float>* delta, std::vector<double>* us) {
  const size_t n = dt.size();
  const float b = (stage == 1) ? 0.25f : 2.0f / 3.0f;
  const float gm1 = static_cast<float>(gamma - 1.0);
  const float gf = static_cast<float>(gamma);
  for (size_t c = 0; c < n; ++c) {
    float d[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int k : {0, 1, 2, 4}) {
      const float t = dt[c] * static_cast<float>(rp[5 * c + k]);
      d[k] = (stage == 0) ? -t : b * ((*delta)[5 * c + k] - t);
    }
    float* hi = uhi->data() + 5 * c;
    float* lo = ulo->data() + 5 * c;
    double* o = us->data() + 5 * c;
    if (!last) {
      Cons<float> f{hi[0] + d[0], hi[1] + d[1], hi[2] + d[2], hi[3], hi[4] + d[4]};
      const float fr = f.rho, fe = f.rE;
      enforce_physical(&f, gf);
      if (f.rho != fr) d[0] = f.rho - hi[0];
      if (f.rE != fe) d[4] = f.rE - hi[4];
      o[0] = f.rho;
      o[1] = f.ru;
      o[2] = f.rv;
      o[3] = f.rw;
      o[4] = f.rE;
    } else {
      float h[5], l[5];
      for (int k = 0; k < 5; ++k) ff_add(hi[k], lo[k], d[k], &h[k], &l[k]);
      const Cons<double> f{h[0], h[1], h[2], h[3], h[4]};
      if (!positivity_safe(f, gm1)) {
        Cons<double> s{double(h[0]) + l[0], double(h[1]) + l[1], double(h[2]) + l[2], double(h[3]) + l[3],
                       double(h[4]) + l[4]};
        enforce_physical(&s, gamma);
        ff_split(s.rho, &h[0], &l[0]);
        ff_split(s.ru, &h[1], &l[1]);
        ff_split(s.rv, &h[2], &l[2]);
        ff_split(s.rw, &h[3], &l[3]);
        ff_split(s.rE, &h[4], &l[4]);
      }
      for (int k = 0; k < 5; ++k) {
        hi[k] = h[k];
        lo[k] = l[k];
        o[k] = static_cast<double>(h[k]) + static_cast<double>(l[k]);
      }
    }
    for (int k = 0; k < 5; ++k) (*delta)[5 * c + k] = d[k];
  }
}

template <class R, class A>
class Solver {
  static constexpr bool kMixed = !std::is_same<R, A>::value;

 public:
  Solver(const aero_mesh_desc& md, const aero_case_desc& cd) : cfg_(cd) {
    load_mesh(md, &mr_);
    load_mesh(md, &ma_);
    resolve();
    reset_run();
    const size_t n = static_cast<size_t>(mr_.num_cells);
    U_.resize(n * 5);
    for (size_t c = 0; c < n; ++c) {
      U_[5 * c + 0] = cons_inf_.rho;
      U_[5 * c + 1] = cons_inf_.ru;
      U_[5 * c + 2] = cons_inf_.rv;
      U_[5 * c + 3] = cons_inf_.rw;
      U_[5 * c + 4] = cons_inf_.rE;
    }
    split_state();
    last_res_.assign(n * 5, R(0));
    last_sr_.assign(n, R(0));
  }

  void set_state(const double* u) {
    for (size_t i = 0; i < U_.size(); ++i) U_[i] = static_cast<A>(u[i]);
    split_state();
  }
  void get_state(double* u) const {
    for (size_t i = 0; i < U_.size(); ++i) u[i] = static_cast<double>(U_[i]);
  }
  void last_residual(double* r, double* s) const {
    for (size_t i = 0; i < last_res_.size(); ++i) r[i] = last_res_[i];
    for (size_t i = 0; i < last_sr_.size(); ++i) s[i] = last_sr_[i];
  }

  void reset_run() {
    iter_ = 0;
    cfl_scale_ = A(1);
    prev_l2_ = A(-1);
    mon_ = Monitor<A>();
    mon_.residual_target = A(cfg_.residual_reduction_target);
    mon_.stab_tol = A(cfg_.force_stability_tol);
    mon_.window = cfg_.force_stability_window;
    mon_.min_iterations = cfg_.min_iterations;
    mon_.drift_tol = A(cfg_.force_mean_drift_tol);
    mon_.init();
    stage_ = cfg_.all_speed_staged_controller ? 1 : 0;
    stage_b_fmin_ = st_fmin_high_;
    stage_b_progress_ = 0;
    pjump_below_ = 0;
    freeze_ = 0;
    has_prev_cd_ = false;
    done_ = false;
  }

  // Residual of one stage on a given conserved state (euler_solver.cpp:802-837).
  void residual(const double* u, int second_order, double stab, int as_fix, double as_fmin,
                double as_ramp, double* res, double* sr, double* grad, int* diag,
                double* fscale = nullptr) {
    const int n = mr_.num_cells;
    std::vector<Prim<R>> w(static_cast<size_t>(n));
    for (int c = 0; c < n; ++c) {
      const Cons<R> cs{R(u[5 * c]), R(u[5 * c + 1]), R(u[5 * c + 2]), R(u[5 * c + 3]),
                       R(u[5 * c + 4])};
      w[c] = cons_to_prim(cs, nm_.gamma);
    }
    Numerics<R> nm = nm_;
    nm.second_order = second_order != 0;
    nm.stab_mach_floor = R(stab);
    nm.as_fix = as_fix != 0;
    nm.as_fmin = R(as_fmin);
    nm.as_ramp = R(as_ramp);
    const std::vector<R> g = nm.second_order ? green_gauss(mr_, w)
                                             : std::vector<R>(static_cast<size_t>(n) * 10, R(0));
    std::vector<R> r, s;
    std::vector<double> fs;
    AssemblyDiag dg;
    assemble(mr_, w, g, nm, &r, &s, &dg, fscale ? &fs : nullptr);
    if (fscale)
      for (size_t i = 0; i < fs.size(); ++i) fscale[i] = fs[i];
    for (size_t i = 0; i < r.size(); ++i) res[i] = r[i];
    for (size_t i = 0; i < s.size(); ++i) sr[i] = s[i];
    if (grad)
      for (size_t i = 0; i < g.size(); ++i) grad[i] = g[i];
    if (diag) {
      diag[0] = dg.first_order_fallback;
      diag[1] = dg.diffusive_fallback;
      diag[2] = dg.first_failure_face;
    }
  }

  // Iteration loop body (euler_solver.cpp:771-1208). Returns 0, or AERO_ERR_NONFINITE.
  int run(int count, aero_iter_record* recs, int* n_done) {
    int done = 0;
    int status = AERO_OK;
    const int n = mr_.num_cells;
    for (int k = 0; k < count && !done_; ++k) {
      const int iter = iter_;
      const bool second = iter >= std::max(cfg_.startup_first_order_iters, 0);
      const A cfl = schedule_cfl(cfl_start_, cfl_max_, cfg_.cfl_ramp_iters, iter, cfl_scale_);
      const A stab = schedule_stab_floor(stab_start_, stab_target_, stab_ramp_, iter);
      bool as_fix;
      A as_fmin, as_ramp;
      if (!cfg_.all_speed_staged_controller) {
        as_fix = cfg_.all_speed_flux_fix != 0;
        as_fmin = as_fmin_;
        as_ramp = schedule_all_speed_ramp<A>(as_ramp_start_, as_ramp_iters_, iter);
      } else if (stage_ == 1) {
        as_fix = false;
        as_fmin = st_fmin_high_;
        as_ramp = A(0);
      } else {
        as_fix = cfg_.all_speed_flux_fix != 0;
        as_fmin = std::clamp(stage_b_fmin_, st_fmin_low_, st_fmin_high_);
        if (as_ramp_iters_ <= 0) {
          as_ramp = A(1);
        } else {
          as_ramp = std::clamp(
              static_cast<A>(stage_b_progress_) / static_cast<A>(std::max(as_ramp_iters_, 1)),
              A(0), A(1));
        }
      }
      Numerics<R> nm = nm_;
      nm.second_order = second;
      nm.stab_mach_floor = R(stab);
      nm.as_fix = as_fix;
      nm.as_fmin = R(as_fmin);
      nm.as_ramp = R(as_ramp);

      const std::vector<A> un = U_;
      std::vector<A> us = U_, next;
      std::vector<float> delta(kMixed ? U_.size() : 0, 0.0f);
      std::vector<Prim<R>> w(static_cast<size_t>(n));
      std::vector<R> res, sr;
      AssemblyDiag itd;
      for (int stage = 0; stage < cfg_.rk_stages; ++stage) {
        for (int c = 0; c < n; ++c) {
          const Cons<R> cs{R(us[5 * c]), R(us[5 * c + 1]), R(us[5 * c + 2]), R(us[5 * c + 3]),
                           R(us[5 * c + 4])};
          w[c] = cons_to_prim(cs, nm.gamma);
        }
        const std::vector<R> g = second ? green_gauss(mr_, w)
                                        : std::vector<R>(static_cast<size_t>(n) * 10, R(0));
        AssemblyDiag dg;
        assemble(mr_, w, g, nm, &res, &sr, &dg);
        itd.first_order_fallback += dg.first_order_fallback;
        itd.diffusive_fallback += dg.diffusive_fallback;
        std::vector<A> rp(res.begin(), res.end());
        if constexpr (kMixed) {
          // the FP32 mode's energy row (the case's precond_fp64): 1 all in double; 2, and by
          // default below Mach 0.1, the row in double from a float beta; else float
          const int pm = cfg_.precond_fp64;
          if (pm == 1) {
            precondition_residual<R, A>(w, nm, &rp);
          } else if (pm == 2 || (pm == 0 && cfg_.mach < 0.1)) {
            precondition_residual_row64(w, nm, &rp);
          } else {
            precondition_residual_fma(w, nm, &rp);
          }
        } else {
          precondition_residual<R, A>(w, nm, &rp);
        }
        const std::vector<R> dtr = dt_over_volume(sr, R(cfl), cfg_.local_time_stepping != 0);
        if constexpr (kMixed) {
          rk_stage_delta(stage, stage == cfg_.rk_stages - 1, &uhi_, &ulo_, rp, dtr, static_cast<double>(nm.gamma),
                         &delta, &us);
        } else {
          const std::vector<A> dta(dtr.begin(), dtr.end());
          rk_stage<A>(stage, un, us, rp, dta, A(nm.gamma), &next);
          us.swap(next);
        }
      }
      U_ = us;
      symmetry(iter);
      last_res_ = res;
      last_sr_ = sr;

      aero_iter_record rec{};
      rec.iter = iter;
      rec.first_order_fallback_faces = itd.first_order_fallback;
      rec.diffusive_fallback_faces = itd.diffusive_fallback;
      rec.cfl = cfl;
      rec.stab_mach_floor = stab;
      rec.all_speed_f_min = as_fmin;
      rec.all_speed_ramp_weight = as_ramp;
      if (second) rec.flags |= AERO_REC_SECOND_ORDER;
      if (as_fix) rec.flags |= AERO_REC_ALL_SPEED_FIX;
      if (stage_ == 1) rec.flags |= AERO_REC_STAGE_A;
      if (stage_ == 2) rec.flags |= AERO_REC_STAGE_B;

      // Non-finite trap (euler_solver.cpp:908-946).
      bool bad = false;
      for (A x : U_) {
        if (!std::isfinite(x)) {
          bad = true;
          break;
        }
      }
      std::vector<A> p(static_cast<size_t>(n));
      std::vector<Prim<A>> pe(static_cast<size_t>(n));
      std::vector<Prim<R>> pr(kMixed ? static_cast<size_t>(n) : 0);
      A dp_dom = A(0), dp_wall = A(0);
      if (!bad) {
        for (int c = 0; c < n; ++c) {
          const Cons<A> cs{U_[5 * c], U_[5 * c + 1], U_[5 * c + 2], U_[5 * c + 3], U_[5 * c + 4]};
          const Prim<A> pw = cons_to_prim(cs, A(nm.gamma));
          if (!std::isfinite(pw.rho) || !std::isfinite(pw.u) || !std::isfinite(pw.v) ||
              !std::isfinite(pw.w) || !std::isfinite(pw.p)) {
            bad = true;
            break;
          }
          pe[c] = pw;
          p[c] = pw.p;
          A adp = std::abs(pw.p - p_inf_);
          if constexpr (kMixed) {  // the FP32 mode forms these monitors from the bulk state, in R
            const Prim<R> wr =
                cons_to_prim(Cons<R>{R(cs.rho), R(cs.ru), R(cs.rv), R(cs.rw), R(cs.rE)}, nm.gamma);
            if (!std::isfinite(wr.rho) || !std::isfinite(wr.u) || !std::isfinite(wr.v) ||
                !std::isfinite(wr.p)) {
              bad = true;
              break;
            }
            pr[c] = wr;
            adp = A(std::abs(wr.p - R(p_inf_)));
            // forces and wall monitors from the bulk (float) primitive state as well
            pe[c] = Prim<A>{A(wr.rho), A(wr.u), A(wr.v), A(wr.w), A(wr.p)};
            p[c] = A(wr.p);
          }
          dp_dom = std::max(dp_dom, adp);
          if (wall_adjacent_[c]) dp_wall = std::max(dp_wall, adp);
        }
      }
      if (bad) {
        rec.flags |= AERO_REC_NONFINITE;
        if (recs) recs[done] = rec;
        ++done;
        ++iter_;
        done_ = true;
        status = AERO_ERR_NONFINITE;
        break;
      }
      rec.max_abs_dp_domain = dp_dom;
      rec.max_abs_dp_wall = dp_wall;

      const Norms<A> nr = norms(res);
      const A ratio = mon_.update_residual(nr.l2);
      if (prev_l2_ > A(0)) {
        if (nr.l2 > prev_l2_ * A(1.05)) {
          cfl_scale_ = std::max(cfl_scale_ * A(0.65), A(0.05));
        } else if (nr.l2 < prev_l2_ * A(0.90)) {
          cfl_scale_ = std::min(cfl_scale_ * A(1.03), A(1));
        }
      }
      prev_l2_ = nr.l2;

      const ForceDiag<A> fd = force_diagnostics(ma_, p, ref_);
      const Forces<A> fa = integrate_forces(ma_, p, ref_, false);
      const Forces<A> fg = integrate_forces(ma_, p, ref_, true);
      const V3<A> drift = mon_.update_forces(fg);
      const bool stable = mon_.stable();
      V3<A> mdrift{A(0), A(0), A(0)};
      mon_.drift(&mdrift);
      const bool dstable = mon_.drift_stable();

      // wall and far-field monitors (euler_solver.cpp:976-1026)
      {
        A un_max = A(0), cp_lo = std::numeric_limits<A>::max(), cp_hi = std::numeric_limits<A>::lowest();
        int cp_bad = 0;
        const A q = A(0.5) * ref_.rho_inf * ref_.speed_inf * ref_.speed_inf + A(1.0e-12);
        int nwall = 0;
        for (int f = 0; f < ma_.num_faces; ++f) {
          if (ma_.neighbor[f] >= 0 || ma_.bc[f] != kSlipWall) continue;
          ++nwall;
          const Prim<A>& w = pe[ma_.owner[f]];
          un_max = std::max(un_max, std::abs(w.u * ma_.normal[3 * f] + w.v * ma_.normal[3 * f + 1] +
                                             w.w * ma_.normal[3 * f + 2]));
          const A cp = (w.p - A(cfg_.p_inf)) / q;
          if (std::isfinite(cp)) {
            cp_lo = std::min(cp_lo, cp);
            cp_hi = std::max(cp_hi, cp);
          } else {
            ++cp_bad;
          }
        }
        if (nwall == 0) cp_lo = cp_hi = A(0);
        A ff[4] = {A(0), A(0), A(0), A(0)};
        for (int f = 0; f < ma_.num_faces; ++f) {
          if (ma_.neighbor[f] >= 0 || ma_.bc[f] != kFarfield) continue;
          if constexpr (kMixed) {
            const Prim<R>& w = pr[ma_.owner[f]];
            ff[0] = std::max(ff[0], A(std::abs(w.p - R(cfg_.p_inf))));
            ff[1] = std::max(ff[1], A(std::abs(w.rho - R(ref_.rho_inf))));
            ff[2] = std::max(ff[2], A(std::abs(w.u - R(u_inf_))));
            ff[3] = std::max(ff[3], A(std::abs(w.v - R(v_inf_))));
          } else {
            const Prim<A>& w = pe[ma_.owner[f]];
            ff[0] = std::max(ff[0], std::abs(w.p - A(cfg_.p_inf)));
            ff[1] = std::max(ff[1], std::abs(w.rho - ref_.rho_inf));
            ff[2] = std::max(ff[2], std::abs(w.u - u_inf_));
            ff[3] = std::max(ff[3], std::abs(w.v - v_inf_));
          }
        }
        rec.max_wall_un = un_max;
        rec.max_wall_mass_flux = 0.0;
        rec.wall_cp_min = cp_lo;
        rec.wall_cp_max = cp_hi;
        rec.wall_cp_nonfinite = cp_bad;
        rec.max_farfield_abs_dp = ff[0];
        rec.max_farfield_abs_drho = ff[1];
        rec.max_farfield_abs_du = ff[2];
        rec.max_farfield_abs_dv = ff[3];
      }

      const A pj_all = pjump(false), pj_wall = pjump(true);
      rec.controller_action = controller(iter, stable, pj_wall);

      rec.residual_l1 = nr.l1;
      rec.residual_l2 = nr.l2;
      rec.residual_linf = nr.linf;
      rec.residual_ratio = ratio;
      rec.cl = fg.cl;
      rec.cd = fg.cd;
      rec.cm = fg.cm;
      rec.lift = fg.lift;
      rec.drag = fg.drag;
      rec.moment = fg.moment;
      rec.cl_abs = fa.cl;
      rec.cd_abs = fa.cd;
      rec.cm_abs = fa.cm;
      rec.fx_gauge = fd.fx_gauge;
      rec.fy_gauge = fd.fy_gauge;
      rec.fx_abs = fd.fx_abs;
      rec.fy_abs = fd.fy_abs;
      rec.sum_nax = fd.sum_nax;
      rec.sum_nay = fd.sum_nay;
      rec.dcl = drift[0];
      rec.dcd = drift[1];
      rec.dcm = drift[2];
      rec.mean_dcl = mdrift[0];
      rec.mean_dcd = mdrift[1];
      rec.mean_dcm = mdrift[2];
      rec.cfl_scale = cfl_scale_;
      rec.p_jump_energy_nd = pj_all;
      rec.p_jump_energy_wall_nd = pj_wall;
      if (stable) rec.flags |= AERO_REC_FORCE_WINDOW_STABLE;
      if (dstable) rec.flags |= AERO_REC_FORCE_DRIFT_STABLE;
      const bool conv = mon_.converged(iter, ratio);
      if (conv) rec.flags |= AERO_REC_CONVERGED;
      if (recs) recs[done] = rec;
      ++done;
      ++iter_;
      if (conv) done_ = true;
    }
    if (n_done) *n_done = done;
    return status;
  }

 private:
  template <class T>
  static void load_mesh(const aero_mesh_desc& md, Mesh<T>* m) {
    m->num_cells = md.num_cells;
    m->num_faces = md.num_faces;
    const int F = md.num_faces, N = md.num_cells;
    m->owner.assign(md.face_owner, md.face_owner + F);
    m->neighbor.assign(md.face_neighbor, md.face_neighbor + F);
    m->bc.assign(md.face_bc, md.face_bc + F);
    m->normal.resize(3 * static_cast<size_t>(F));
    m->center.resize(3 * static_cast<size_t>(F));
    m->area.resize(F);
    for (int i = 0; i < 3 * F; ++i) {
      m->normal[i] = static_cast<T>(md.face_normal[i]);
      m->center[i] = static_cast<T>(md.face_center[i]);
    }
    for (int f = 0; f < F; ++f) m->area[f] = static_cast<T>(md.face_area[f]);
    m->volume.resize(N);
    m->cell_center.resize(3 * static_cast<size_t>(N));
    for (int c = 0; c < N; ++c) m->volume[c] = static_cast<T>(md.cell_volume[c]);
    for (int i = 0; i < 3 * N; ++i) m->cell_center[i] = static_cast<T>(md.cell_center[i]);
    m->wall_faces.assign(md.wall_faces, md.wall_faces + md.num_wall_faces);
  }

  // euler_solver.cpp:340-357, 120-140, 493-526, 543-566
  void resolve() {
    const aero_case_desc& c = cfg_;
    const A gamma = A(c.gamma);
    A rho_inf = A(c.rho_inf);
    if (rho_inf <= A(0)) rho_inf = A(c.p_inf) / (A(c.gas_constant) * A(c.t_inf));
    const A alpha = A(c.aoa_deg) * (K<A>::pi / A(180));
    const A a_inf = std::sqrt(gamma * A(c.p_inf) / rho_inf);
    const A v_inf = std::max(A(c.mach), A(0)) * a_inf;
    const Prim<A> pinf{rho_inf, v_inf * std::cos(alpha), v_inf * std::sin(alpha), A(0), A(c.p_inf)};
    cons_inf_ = prim_to_cons(pinf, gamma);
    u_inf_ = pinf.u;
    v_inf_ = pinf.v;
    p_inf_ = A(c.p_inf);
    ref_.rho_inf = rho_inf;
    ref_.p_inf = A(c.p_inf);
    ref_.aoa_deg = A(c.aoa_deg);
    ref_.speed_inf = v_inf;
    ref_.chord = A(c.chord);
    ref_.x_ref = A(c.x_ref);
    ref_.y_ref = A(c.y_ref);
    pressure_ref_ = std::max(rho_inf * a_inf * a_inf, A(1.0e-12));

    nm_.gamma = R(gamma);
    nm_.farfield = Cons<R>{R(cons_inf_.rho), R(cons_inf_.ru), R(cons_inf_.rv), R(cons_inf_.rw),
                           R(cons_inf_.rE)};
    nm_.flux = c.flux;
    nm_.limiter = c.limiter;
    nm_.low_mach_fix = c.low_mach_fix != 0;
    nm_.mach_cutoff = R(c.mach_cutoff);
    nm_.precond_farfield_bc = c.precond_farfield_bc != 0;
    nm_.as_cutoff = R(c.all_speed_mach_cutoff);
    // build_precondition_config (euler_solver.cpp:340-357)
    {
      const A minf = std::max(A(c.mach), A(1.0e-4));
      const A auto_bmin = std::max(A(1.0e-4), std::min(A(1.0e-3), A(0.1) * minf));
      nm_.precond = c.precond_on != 0;
      const A mref = std::max(A(c.precond_mach_ref) > A(0) ? A(c.precond_mach_ref) : minf, A(1.0e-4));
      const A mmin =
          std::max(A(c.precond_mach_min) > A(0) ? A(c.precond_mach_min) : A(1.0e-6), A(1.0e-6));
      const A bmin =
          std::max(A(c.precond_beta_min) > A(0) ? A(c.precond_beta_min) : auto_bmin, A(1.0e-4));
      const A bmax = std::max(A(c.precond_beta_max), bmin);
      nm_.pc_mach_ref = R(mref);
      nm_.pc_mach_min = R(mmin);
      nm_.pc_beta_min = R(bmin);
      nm_.pc_beta_max = R(bmax);
    }
    // resolve_stabilization_floor_schedule (euler_solver.cpp:120-140)
    {
      const A minf = std::max(A(c.mach), A(1.0e-4));
      const A ks = c.stab_floor_k_start >= 0.0 ? A(c.stab_floor_k_start) : A(c.stab_floor_start) / minf;
      const A kt =
          c.stab_floor_k_target >= 0.0 ? A(c.stab_floor_k_target) : A(c.stab_floor_target) / minf;
      stab_start_ = std::clamp(std::max(ks, A(0)) * minf, A(0), A(1));
      stab_target_ = std::clamp(std::max(kt, A(0)) * minf, A(0), A(1));
      stab_ramp_ = std::max(c.stab_ramp_iters, 0);
    }
    cfl_start_ = A(c.cfl_start);
    cfl_max_ = A(c.cfl_max);
    as_fmin_ = std::clamp(A(c.all_speed_f_min), A(1.0e-6), A(1));
    as_ramp_start_ = std::max(c.all_speed_ramp_start_iter, 0);
    as_ramp_iters_ = std::max(c.all_speed_ramp_iters, 0);
    st_a_min_ = std::max(c.all_speed_stage_a_min_iters, 0);
    st_a_max_ = std::max(c.all_speed_stage_a_max_iters, 0);
    st_fmin_high_ = std::clamp(A(c.all_speed_stage_f_min_high), A(1.0e-6), A(1));
    st_fmin_mid_ = std::clamp(std::min(A(c.all_speed_stage_f_min_mid), st_fmin_high_), A(1.0e-6), A(1));
    st_fmin_low_ = std::clamp(std::min(A(c.all_speed_stage_f_min_low), st_fmin_mid_), A(1.0e-6), A(1));
    {
      const A minf = std::max(A(c.mach), A(1.0e-4));
      const A autopj =
          std::clamp(A(1.6e-2) * minf * minf * minf * minf, A(1.0e-9), A(2.0e-6));
      pj_target_ = A(c.all_speed_pjump_wall_target) <= A(0) ? autopj : A(c.all_speed_pjump_wall_target);
    }
    pj_spike_ = std::max(A(c.all_speed_pjump_spike_factor), A(1));
    pj_hold_ = std::max(c.all_speed_pjump_hold_iters, 1);
    freeze_iters_ = std::max(c.all_speed_freeze_iters, 0);
    cfl_drop_ = std::clamp(A(c.all_speed_cfl_drop_factor), A(0.05), A(1));
    cfl_restore_ = std::clamp(A(c.all_speed_cfl_restore_factor), A(1), A(1.2));
    cfl_min_scale_ = std::clamp(A(c.all_speed_cfl_min_scale), A(0.01), A(1));

    wall_adjacent_.assign(static_cast<size_t>(mr_.num_cells), 0);
    for (int f = 0; f < mr_.num_faces; ++f) {
      if (mr_.neighbor[f] < 0 && mr_.bc[f] == kSlipWall) wall_adjacent_[mr_.owner[f]] = 1;
    }
  }

  // euler_solver.cpp:309-339 with the value formed in A
  Norms<A> norms(const std::vector<R>& res) const {
    double l1 = 0.0, l2s = 0.0, linf = 0.0;
    if constexpr (kMixed) {  // per-cell terms in float, accumulated in double
      for (int c = 0; c < mr_.num_cells; ++c) {
        const R inv = R(1) / std::max(mr_.volume[c], K<R>::vol_floor);
        const R v0 = res[5 * c] * inv, v1 = res[5 * c + 1] * inv, v2 = res[5 * c + 2] * inv,
                v3 = res[5 * c + 4] * inv;
        const R a0 = std::abs(v0), a1 = std::abs(v1), a2 = std::abs(v2), a3 = std::abs(v3);
        l1 += static_cast<double>(((a0 + a1) + a2) + a3);
        l2s += static_cast<double>(((v0 * v0 + v1 * v1) + v2 * v2) + v3 * v3);
        linf = std::max(linf, static_cast<double>(std::max(std::max(std::max(a0, a1), a2), a3)));
      }
      Norms<A> out;
      out.l1 = static_cast<A>(l1);
      out.l2 = static_cast<A>(std::sqrt(l2s / std::max(1, mr_.num_cells * 5)));
      out.linf = static_cast<A>(linf);
      return out;
    }
    for (int c = 0; c < ma_.num_cells; ++c) {
      const A inv = A(1) / std::max(ma_.volume[c], K<A>::vol_floor);
      for (int k = 0; k < 5; ++k) {
        const A val = A(res[5 * c + k]) * inv;
        const double a = std::abs(static_cast<double>(val));
        l1 += a;
        l2s += a * a;
        linf = std::max(linf, a);
      }
    }
    Norms<A> out;
    out.l1 = static_cast<A>(l1);
    out.l2 = static_cast<A>(std::sqrt(l2s / std::max(1, ma_.num_cells * 5)));
    out.linf = static_cast<A>(linf);
    return out;
  }

  // euler_solver.cpp:418-450
  void symmetry(int iter) {
    if (!cfg_.aoa0_symmetry_enforce || cfg_.aoa0_symmetry_enforce_interval <= 0) return;
    if (std::abs(A(cfg_.aoa_deg)) > A(1.0e-12)) return;
    if (((iter + 1) % cfg_.aoa0_symmetry_enforce_interval) != 0) return;
    const A gamma = A(nm_.gamma);
    for (int c = 0; c < mr_.num_cells; ++c) {
      const Cons<A> s{U_[5 * c], U_[5 * c + 1], U_[5 * c + 2], U_[5 * c + 3], U_[5 * c + 4]};
      Prim<A> w = cons_to_prim(s, gamma);
      w.v = A(0);
      w.w = A(0);
      const Cons<A> o = prim_to_cons(w, gamma);
      U_[5 * c] = o.rho;
      U_[5 * c + 1] = o.ru;
      U_[5 * c + 2] = o.rv;
      U_[5 * c + 3] = o.rw;
      U_[5 * c + 4] = o.rE;
    }
    split_state();
  }

  // Pressure-jump energy over interior faces (euler_solver.cpp:1027-1063), using the
  // primitive pressure of the stored state.
  A pjump(bool wall_only) const {
    double sum = 0.0;
    int count = 0;
    const A gamma = A(nm_.gamma);
    for (int f = 0; f < ma_.num_faces; ++f) {
      const int o = ma_.owner[f], nb = ma_.neighbor[f];
      if (nb < 0) continue;
      if (wall_only && !wall_adjacent_[o] && !wall_adjacent_[nb]) continue;
      const Cons<A> so{U_[5 * o], U_[5 * o + 1], U_[5 * o + 2], U_[5 * o + 3], U_[5 * o + 4]};
      const Cons<A> sn{U_[5 * nb], U_[5 * nb + 1], U_[5 * nb + 2], U_[5 * nb + 3], U_[5 * nb + 4]};
      const A dp = cons_to_prim(so, gamma).p - cons_to_prim(sn, gamma).p;
      sum += static_cast<double>(dp) * static_cast<double>(dp);
      ++count;
    }
    const double pr2 = static_cast<double>(pressure_ref_) * static_cast<double>(pressure_ref_) + 1.0e-24;
    return count > 0 ? static_cast<A>((sum / static_cast<double>(count)) / pr2) : A(0);
  }

  // All-speed staged controller (euler_solver.cpp:1068-1139).
  // Returns the controller action code of the reference's diagnostics CSV.
  int controller(int iter, bool stable, A pj_wall) {
    if (!cfg_.all_speed_staged_controller) return 0;
    if (stage_ == 1) {
      const bool ready = (iter + 1 >= st_a_min_) && stable;
      const bool timeout = (st_a_max_ > 0) && (iter + 1 >= st_a_max_);
      if ((ready || timeout) && cfg_.all_speed_flux_fix) {
        stage_ = 2;
        stage_b_fmin_ = st_fmin_high_;
        stage_b_progress_ = 0;
        pjump_below_ = 0;
        freeze_ = 0;
        return ready ? 10 : 11;
      }
      return 0;
    }
    int action = 0;
    const A spike_thr = (pj_target_ > A(0)) ? pj_target_ * pj_spike_ : std::numeric_limits<A>::max();
    const bool spike = pj_wall > spike_thr;
    const bool good = (pj_target_ <= A(0)) || (pj_wall <= pj_target_);
    if (spike) {
      freeze_ = freeze_iters_;
      pjump_below_ = 0;
      stage_b_fmin_ = std::min(st_fmin_high_, stage_b_fmin_ + A(0.05));
      cfl_scale_ = std::max(cfl_scale_ * cfl_drop_, cfl_min_scale_);
      return 20;
    }
    if (freeze_ > 0) --freeze_;
    if (good) {
      ++pjump_below_;
    } else {
      pjump_below_ = 0;
    }
    if (freeze_ == 0) {
      if (stage_b_fmin_ > st_fmin_mid_ + A(1.0e-6) && pjump_below_ >= pj_hold_) {
        stage_b_fmin_ = st_fmin_mid_;
        pjump_below_ = 0;
        action = 31;
      } else if (stage_b_fmin_ > st_fmin_low_ + A(1.0e-6) && pjump_below_ >= pj_hold_) {
        stage_b_fmin_ = st_fmin_low_;
        pjump_below_ = 0;
        action = 32;
      } else if (stage_b_fmin_ <= st_fmin_low_ + A(1.0e-6) && good) {
        ++stage_b_progress_;
        if (action == 0) action = 33;
      }
      if (good) {
        cfl_scale_ = std::min(cfl_scale_ * cfl_restore_, A(1));
      } else if (pj_target_ > A(0) && pj_wall > pj_target_) {
        cfl_scale_ = std::max(cfl_scale_ * cfl_drop_, cfl_min_scale_);
        if (action == 0) action = 21;
      }
    }
    return action;
  }

  aero_case_desc cfg_;
  Mesh<R> mr_;
  Mesh<A> ma_;
  Numerics<R> nm_;
  Cons<A> cons_inf_;
  A p_inf_ = A(0), pressure_ref_ = A(1), u_inf_ = A(0), v_inf_ = A(0);
  Reference<A> ref_;
  A cfl_start_ = A(0), cfl_max_ = A(0);
  A stab_start_ = A(0), stab_target_ = A(0);
  int stab_ramp_ = 0;
  A as_fmin_ = A(0.05);
  int as_ramp_start_ = 0, as_ramp_iters_ = 0;
  int st_a_min_ = 0, st_a_max_ = 0;
  A st_fmin_high_ = A(0.2), st_fmin_mid_ = A(0.1), st_fmin_low_ = A(0.05);
  A pj_target_ = A(0), pj_spike_ = A(1.5);
  int pj_hold_ = 1, freeze_iters_ = 0;
  A cfl_drop_ = A(0.8), cfl_restore_ = A(1.02), cfl_min_scale_ = A(0.1);
  std::vector<unsigned char> wall_adjacent_;

  std::vector<A> U_;
  std::vector<float> uhi_, ulo_;  // mixed mode: float-float pairs of U_ (U_ == hi + lo)

  // mixed mode: split U_ into float-float pairs and set U_ to their sum
  void split_state() {
    if constexpr (kMixed) {
      uhi_.resize(U_.size());
      ulo_.resize(U_.size());
      for (size_t i = 0; i < U_.size(); ++i) {
        ff_split(static_cast<double>(U_[i]), &uhi_[i], &ulo_[i]);
        U_[i] = static_cast<A>(static_cast<double>(uhi_[i]) + static_cast<double>(ulo_[i]));
      }
    }
  }
  std::vector<R> last_res_, last_sr_;
  Monitor<A> mon_;
  int iter_ = 0;
  A cfl_scale_ = A(1), prev_l2_ = A(-1);
  int stage_ = 0;  // 0 single, 1 A, 2 B
  A stage_b_fmin_ = A(0.2);
  int stage_b_progress_ = 0, pjump_below_ = 0, freeze_ = 0;
  bool has_prev_cd_ = false;
  bool done_ = false;
};

}  // namespace aero_oracle
