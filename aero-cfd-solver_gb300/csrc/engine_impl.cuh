// engine_impl.cuh -- device solver for one bulk precision T (float or double). Included by
// engine_f32.cu and engine_f64.cu, which instantiate it.
#pragma once

#include "aero_face_kernels.cuh"
#include "engine.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace aero {

#define AERO_CK(expr)                       \
  do {                                      \
    cudaError_t e_ = (expr);                \
    if (e_ != cudaSuccess && err_ == cudaSuccess) err_ = e_; \
  } while (0)

template <class T>
class EngineT final : public Engine {
  using V4 = typename Vec<T>::v4;
  using V2 = typename Vec<T>::v2;

 public:
  EngineT(const HostSlots& hs, const aero_case_desc& cfg, const Resolved& rs, cudaStream_t st)
      : hs_(hs), cfg_(cfg), rs_(rs), st_(st) {}

  ~EngineT() override {
    for (auto& g : graph_) {
      if (g) cudaGraphExecDestroy(g);
    }
    if (ev_fork_) cudaEventDestroy(ev_fork_);
    if (ev_join_) cudaEventDestroy(ev_join_);
    if (side_) cudaStreamDestroy(side_);
    for (void* p : allocs_) cudaFree(p);
    if (flush_) cudaFree(flush_);
    if (pin_state_) cudaFreeHost(pin_state_);
  }

  bool init(std::string* err) override {
    n_ = hs_.n;
    d_ = hs_.d;
    block_ = cfg_.block_size > 0 ? cfg_.block_size : 128;
    if (block_ != 64 && block_ != 128 && block_ != 256) {
      *err = "block_size must be 64, 128 or 256";
      return false;
    }
    nblocks_ = (n_ + block_ - 1) / block_;
    const size_t ns = static_cast<size_t>(n_) * d_;

    // slot table; normals and areas in T (exact conversions of the double geometry)
    link_ = upload(hs_.link);
    std::vector<V2> nrm(ns);
    std::vector<T> area(ns);
    for (size_t i = 0; i < ns; ++i) {
      nrm[i].x = T(hs_.nx[i]);
      nrm[i].y = T(hs_.ny[i]);
      area[i] = T(hs_.area[i]);
    }
    nrm_ = upload(nrm);
    area_ = upload(area);
    std::vector<T> inv_vol(static_cast<size_t>(n_));
    for (int c = 0; c < n_; ++c) inv_vol[c] = T(1) / std::max(T(hs_.vol[c]), T(1.0e-12));
    inv_vol_ = upload(inv_vol);
    // face table in T (exact conversions; MUSCL offsets formed in T from T coordinates)
    {
      const size_t nf = hs_.f_orig.size();
      std::vector<int2> fc(nf);
      std::vector<V2> fn(nf), doff(nf), noff(nf);
      std::vector<T> fa(nf);
      for (size_t i = 0; i < nf; ++i) {
        fc[i] = make_int2(hs_.f_own[i], hs_.f_nb[i]);
        fn[i].x = T(hs_.f_nx[i]);
        fn[i].y = T(hs_.f_ny[i]);
        fa[i] = T(hs_.f_area[i]);
        const int o = hs_.f_own_old[i], b = hs_.f_nb_old[i];
        doff[i].x = T(hs_.f_cx[i]) - T(hs_.ccx[o]);
        doff[i].y = T(hs_.f_cy[i]) - T(hs_.ccy[o]);
        if (hs_.f_nb[i] >= 0) {
          noff[i].x = T(hs_.f_cx[i]) - T(hs_.ccx[b]);
          noff[i].y = T(hs_.f_cy[i]) - T(hs_.ccy[b]);
        } else {
          noff[i].x = noff[i].y = T(0);
        }
      }
      df_.nf = static_cast<int>(nf);
      df_.cells = upload(fc);
      df_.nrm = upload(fn);
      df_.area = upload(fa);
      df_.doff = upload(doff);
      df_.noff = upload(noff);
      dg_.n = n_;
      dg_.d = d_;
      dg_.slot = upload(hs_.gslot);
      F_ = alloc<V4>(nf);
      FS_ = alloc<T>(nf);
    }
    perm_dev_ = upload(hs_.perm);
    // monitor tables: per-cell flags, owner-sorted wall entries, and a partials slot for each
    // update block that holds wall entries
    std::vector<int> block_slot(static_cast<size_t>(nblocks_), -1);
    int n_wall_blocks = 0;
    for (int b = 0; b < nblocks_; ++b) {
      const int c0 = b * block_, c1 = std::min(n_, c0 + block_);
      for (int c = c0; c < c1; ++c) {
        if (hs_.flags[c] >= 4) {
          block_slot[b] = n_wall_blocks++;
          break;
        }
      }
    }
    flags_ = upload(hs_.flags);
    ms_.flags = flags_;
    ms_.wall_first = upload(hs_.wall_first);
    ms_.wkind = upload(hs_.wkind.empty() ? std::vector<unsigned char>{0} : hs_.wkind);
    ms_.wnx = upload(nonempty(hs_.wnx));
    ms_.wny = upload(nonempty(hs_.wny));
    ms_.warea = upload(nonempty(hs_.warea));
    ms_.wx = upload(nonempty(hs_.wx));
    ms_.wy = upload(nonempty(hs_.wy));
    {
      auto to_f = [](const std::vector<double>& v) {
        std::vector<float> f(v.empty() ? 1 : v.size(), 0.0f);
        for (size_t i = 0; i < v.size(); ++i) f[i] = float(v[i]);
        return f;
      };
      ms_.wnx_f = upload(to_f(hs_.wnx));
      ms_.wny_f = upload(to_f(hs_.wny));
      ms_.warea_f = upload(to_f(hs_.warea));
      ms_.wx_f = upload(to_f(hs_.wx));
      ms_.wy_f = upload(to_f(hs_.wy));
    }
    ms_.block_slot = upload(block_slot);
    ms_.p_inf = rs_.p_inf;
    ms_.rho_inf = rs_.rho_inf;
    ms_.u_inf = rs_.v_inf * rs_.cos_a;
    ms_.v_inf = rs_.v_inf * rs_.sin_a;
    ms_.q_inf = rs_.q_inf;
    ms_.x_ref = cfg_.x_ref;
    ms_.y_ref = cfg_.y_ref;
    ms_.gamma = rs_.gamma;
    ms_.p_inf_f = float(ms_.p_inf);
    ms_.rho_inf_f = float(ms_.rho_inf);
    ms_.u_inf_f = float(ms_.u_inf);
    ms_.v_inf_f = float(ms_.v_inf);
    ms_.q_inf_f = float(ms_.q_inf);
    ms_.x_ref_f = float(ms_.x_ref);
    ms_.y_ref_f = float(ms_.y_ref);

    // state
    W_ = alloc<V4>(n_);
    gx_ = alloc<V4>(n_);
    gy_ = alloc<V4>(n_);
    R_ = alloc<V4>(n_);
    SR_ = alloc<T>(n_);
    if (cfg_.rk_stages > 1) {  // the first stage's residual, kept apart from the last stage's
      R0_ = alloc<V4>(n_);
      SR0_ = alloc<T>(n_);
    } else {
      R0_ = R_;
      SR0_ = SR_;
    }
    fb_ = alloc<int>(4);
    Un_ = alloc<d4>(n_);
    Us_ = alloc<V4>(n_);
    sref_.un = Un_;
    if (sizeof(T) == 4) {
      sref_.hi = alloc<float4>(n_);
      sref_.lo = alloc<float4>(n_);
    }
    Ueval_ = alloc<d4>(n_);
    if (sizeof(T) == 4) {
      part_.norms_f = alloc<float>(3 * nblocks_);
    } else {
      part_.norms = alloc<double>(3 * nblocks_);
    }
    part_.mon = alloc<long long>(kMon * nblocks_);
    if (sizeof(T) == 4) {
      part_.wall_f = alloc<float>(kWall * std::max(n_wall_blocks, 1));
    } else {
      part_.wall = alloc<double>(kWall * std::max(n_wall_blocks, 1));
    }
    part_.nb = nblocks_;
    part_.nwb = n_wall_blocks;
    part_.pjump = alloc<double>(4 * nblocks_);
    part_.srmax = alloc<double>(nblocks_ * (block_ / 32));
    ctrl_ = alloc<Ctrl>(1);
    ctrl_eval_ = alloc<Ctrl>(1);
    rec_cap_ = 1024;
    recs_ = alloc<Record>(rec_cap_);
    if (err_ != cudaSuccess) {
      *err = std::string("device allocation/upload failed: ") + cudaGetErrorString(err_);
      return false;
    }

    dm_.n = n_;
    dm_.d = d_;
    dm_.link = link_;
    dm_.nrm = nrm_;
    dm_.area = area_;
    dm_.inv_vol = inv_vol_;
    dg_.inv_vol = inv_vol_;

    fp_.gamma = T(rs_.gamma);
    fp_.farfield = Cons<T>{T(rs_.cons_inf[0]), T(rs_.cons_inf[1]), T(rs_.cons_inf[2]), T(rs_.cons_inf[3])};
    fp_.limiter = cfg_.limiter;
    fp_.precond = cfg_.precond_on;
    fp_.low_mach_fix = cfg_.low_mach_fix;
    fp_.precond_farfield_bc = cfg_.precond_farfield_bc;
    fp_.as_fix = 0;
    fp_.mach_cutoff = T(cfg_.mach_cutoff);
    fp_.pc_mach_ref = T(rs_.pc_mach_ref);
    fp_.pc_mach_min = T(rs_.pc_mach_min);
    fp_.pc_beta_min = T(rs_.pc_beta_min);
    fp_.pc_beta_max = T(rs_.pc_beta_max);
    fp_.stab_floor = T(0);
    fp_.as_cutoff = T(cfg_.all_speed_mach_cutoff);
    fp_.as_fmin = T(rs_.as_fmin);
    fp_.as_ramp = T(1);

    pc_.enabled = cfg_.precond_on;
    pc_.gamma = rs_.gamma;
    pc_.mach_ref = double(fp_.pc_mach_ref);
    pc_.mach_min = double(fp_.pc_mach_min);
    pc_.beta_min = double(fp_.pc_beta_min);
    pc_.beta_max = double(fp_.pc_beta_max);
    pc_.gamma_f = float(rs_.gamma);
    pc_.gm1_f = float(rs_.gamma - 1.0);

    CtrlConfig& c = cc_;
    std::memset(&c, 0, sizeof(c));
    c.n_cells = n_;
    c.n_wall = hs_.n_slip;
    c.n_wall_blocks = n_wall_blocks;
    c.bulk_f32 = sizeof(T) == 4 ? 1 : 0;
    c.rk_stages = cfg_.rk_stages;
    c.local_dt = cfg_.local_time_stepping;
    c.cfl_ramp = cfg_.cfl_ramp_iters;
    c.stab_ramp = std::max(cfg_.stab_ramp_iters, 0);
    c.as_ramp_start = std::max(cfg_.all_speed_ramp_start_iter, 0);
    c.as_ramp_iters = std::max(cfg_.all_speed_ramp_iters, 0);
    c.startup_first_order = cfg_.startup_first_order_iters;
    c.min_iterations = cfg_.min_iterations;
    c.window = std::min(std::max(cfg_.force_stability_window, 1), kMaxForceWindow);
    c.staged = cfg_.all_speed_staged_controller;
    c.st_a_min = std::max(cfg_.all_speed_stage_a_min_iters, 0);
    c.st_a_max = std::max(cfg_.all_speed_stage_a_max_iters, 0);
    c.pj_hold = std::max(cfg_.all_speed_pjump_hold_iters, 1);
    c.freeze_iters = std::max(cfg_.all_speed_freeze_iters, 0);
    c.as_fix_cfg = cfg_.all_speed_flux_fix;
    c.n_blocks = nblocks_;
    pjump_on_ = cfg_.all_speed_staged_controller || cfg_.diagnostics;
    sym_on_ = cfg_.aoa0_symmetry_enforce && cfg_.aoa0_symmetry_enforce_interval > 0 &&
              !(std::fabs(cfg_.aoa_deg) > 1.0e-12);
    c.pjump_blocks = pjump_on_ ? nblocks_ : 0;
    c.cfl_start = cfg_.cfl_start;
    c.cfl_max = cfg_.cfl_max;
    c.stab_start = rs_.stab_start;
    c.stab_target = rs_.stab_target;
    c.as_fmin = rs_.as_fmin;
    c.residual_target = cfg_.residual_reduction_target;
    c.stab_tol = cfg_.force_stability_tol;
    c.drift_tol = cfg_.force_mean_drift_tol > 0.0 ? cfg_.force_mean_drift_tol : cfg_.force_stability_tol;
    c.st_fmin_high = rs_.st_fmin_high;
    c.st_fmin_mid = rs_.st_fmin_mid;
    c.st_fmin_low = rs_.st_fmin_low;
    c.pj_target = rs_.pj_target;
    c.pj_spike = rs_.pj_spike;
    c.cfl_drop = rs_.cfl_drop;
    c.cfl_restore = rs_.cfl_restore;
    c.cfl_min_scale = rs_.cfl_min_scale;
    c.p_inf = rs_.p_inf;
    c.q_inf = rs_.q_inf;
    c.chord = std::max(cfg_.chord, 1.0e-8);
    c.s_ref = c.chord * 1.0;
    c.cos_a = rs_.cos_a;
    c.sin_a = rs_.sin_a;
    c.x_ref = cfg_.x_ref;
    c.y_ref = cfg_.y_ref;
    c.pressure_ref = rs_.pressure_ref;
    c.gamma = rs_.gamma;
    c.rho_inf = rs_.rho_inf;
    c.u_inf = rs_.v_inf * rs_.cos_a;
    c.v_inf = rs_.v_inf * rs_.sin_a;

    AERO_CK(cudaMemsetAsync(fb_, 0, 4 * sizeof(int), st_));
    // the controller of iteration i runs beside the gradient and first residual of iteration
    // i+1 (which need none of its outputs) when the first residual has a buffer of its own
    // and the residual reads no controller-scheduled low-Mach weights
    defer_control_ = cfg_.rk_stages > 1 && !rs_.lm;
    if (defer_control_) {
      AERO_CK(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
      AERO_CK(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
      AERO_CK(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming));
    }
    // freestream initial state
    std::vector<d4> u0(static_cast<size_t>(n_), d4{rs_.cons_inf[0], rs_.cons_inf[1], rs_.cons_inf[2], rs_.cons_inf[3]});
    AERO_CK(cudaMemcpyAsync(Un_, u0.data(), sizeof(d4) * n_, cudaMemcpyHostToDevice, st_));
    state_from_staging();
    w_valid_ = false;
    reset_run();
    AERO_CK(cudaStreamSynchronize(st_));
    if (err_ != cudaSuccess) {
      *err = std::string("initialisation failed: ") + cudaGetErrorString(err_);
      return false;
    }
    return true;
  }

  EngineView view() const override {
    EngineView v{};
    v.n = n_;
    v.precision = sizeof(T) == 4 ? AERO_PRECISION_FP32 : AERO_PRECISION_FP64;
    v.flux = cfg_.flux;
    v.lm = rs_.lm;
    v.block = block_;
    cudaGetDevice(&v.device);
    v.dm = &dm_;
    v.df = &df_;
    v.dg = &dg_;
    v.nf = df_.nf;
    v.fp = &fp_;
    v.perm_dev = perm_dev_;
    v.stream = st_;
    return v;
  }

  cudaError_t last_cuda_error() override {
    const cudaError_t e = err_;
    err_ = cudaSuccess;
    return e;
  }

  void reset_run() override {
    Ctrl h;
    std::memset(&h, 0, sizeof(h));
    h.iter = 0;
    h.cfl_scale = 1.0;
    h.prev_l2 = -1.0;
    h.initial_l2 = -1.0;
    h.stage = cfg_.all_speed_staged_controller ? 1 : 0;
    h.stage_b_fmin = rs_.st_fmin_high;
    apply_schedule(cc_, &h);
    host_ctrl_ = h;
    AERO_CK(cudaMemcpyAsync(ctrl_, &host_ctrl_, sizeof(Ctrl), cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaMemsetAsync(fb_, 0, 4 * sizeof(int), st_));
    AERO_CK(cudaStreamSynchronize(st_));
  }

  // State transfers go through a page-locked staging buffer in the device order.
  void set_state(const double* u) override {
    d4* h = pinned_state();
    for (int cn = 0; cn < n_; ++cn) {
      const double* s = u + 5 * static_cast<size_t>(hs_.perm[cn]);
      h[cn] = d4{s[0], s[1], s[2], s[4]};
    }
    AERO_CK(cudaMemcpyAsync(Un_, h, sizeof(d4) * n_, cudaMemcpyHostToDevice, st_));
    state_from_staging();
    AERO_CK(cudaStreamSynchronize(st_));
    w_valid_ = false;
  }

  void get_state(double* u) override {
    d4* h = pinned_state();
    state_to_staging();
    AERO_CK(cudaMemcpyAsync(h, Un_, sizeof(d4) * n_, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    for (int cn = 0; cn < n_; ++cn) {
      double* s = u + 5 * static_cast<size_t>(hs_.perm[cn]);
      s[0] = h[cn].x;
      s[1] = h[cn].y;
      s[2] = h[cn].z;
      s[3] = 0.0;
      s[4] = h[cn].w;
    }
  }

  void get_primitive(double* rho, double* u, double* v, double* p) override {
    std::vector<d4> h(static_cast<size_t>(n_));
    state_to_staging();
    AERO_CK(cudaMemcpyAsync(h.data(), Un_, sizeof(d4) * n_, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    for (int cn = 0; cn < n_; ++cn) {
      const int co = hs_.perm[cn];
      // host restatement of cons_to_prim (euler_flux.cpp:115-127) in double
      const double r = std::max(h[cn].x, 1.0e-8);
      const double inv = 1.0 / r;
      const double uu = h[cn].y * inv, vv = h[cn].z * inv;
      const double ke = 0.5 * r * (uu * uu + vv * vv);
      rho[co] = r;
      u[co] = uu;
      v[co] = vv;
      p[co] = std::max((rs_.gamma - 1.0) * (h[cn].w - ke), 1.0e-8);
    }
  }

  void residual(const double* u, int second, double stab, int as_fix, double as_fmin, double as_ramp,
                double* res, double* sr, double* grad) override {
    std::vector<d4> h(static_cast<size_t>(n_));
    for (int cn = 0; cn < n_; ++cn) {
      const double* s = u + 5 * static_cast<size_t>(hs_.perm[cn]);
      h[cn] = d4{s[0], s[1], s[2], s[4]};
    }
    AERO_CK(cudaMemcpyAsync(Ueval_, h.data(), sizeof(d4) * n_, cudaMemcpyHostToDevice, st_));
    Ctrl ce;
    std::memset(&ce, 0, sizeof(ce));
    set_eval_schedule(&ce, stab, as_fix, as_fmin, as_ramp);
    AERO_CK(cudaMemcpyAsync(ctrl_eval_, &ce, sizeof(Ctrl), cudaMemcpyHostToDevice, st_));
    k_refresh_prim<T><<<nblocks_, block_, 0, st_>>>(n_, Ueval_, W_, rs_.gamma);
    if (second) k_gradient<T><<<nblocks_, block_, 0, st_>>>(dm_, W_, gx_, gy_, ctrl_eval_);
    launch_residual(second != 0, false, ctrl_eval_, &ctrl_eval_->fo_fallback, R_, SR_, 0);
    AERO_CK(cudaGetLastError());
    w_valid_ = false;
    download_residual(res, sr);
    if (grad) {
      std::vector<V4> hx(static_cast<size_t>(n_)), hy(static_cast<size_t>(n_));
      if (second) {
        AERO_CK(cudaMemcpyAsync(hx.data(), gx_, sizeof(V4) * n_, cudaMemcpyDeviceToHost, st_));
        AERO_CK(cudaMemcpyAsync(hy.data(), gy_, sizeof(V4) * n_, cudaMemcpyDeviceToHost, st_));
      }
      AERO_CK(cudaStreamSynchronize(st_));
      for (int cn = 0; cn < n_; ++cn) {
        double* g = grad + 10 * static_cast<size_t>(hs_.perm[cn]);
        if (!second) {
          for (int k = 0; k < 10; ++k) g[k] = 0.0;
          continue;
        }
        const V4 a = hx[cn], b = hy[cn];
        g[0] = a.x; g[1] = b.x;  // rho
        g[2] = a.y; g[3] = b.y;  // u
        g[4] = a.z; g[5] = b.z;  // v
        g[6] = 0.0; g[7] = 0.0;  // w
        g[8] = a.w; g[9] = b.w;  // p
      }
    }
  }

  void last_residual(double* res, double* sr) override { download_residual(res, sr); }

  int run(int n, aero_iter_record* recs, int* n_done) override {
    static_assert(sizeof(Record) == sizeof(aero_iter_record), "record layout");
    int executed = 0;
    if (!w_valid_) refresh();
    AERO_CK(cudaMemcpyAsync(&host_ctrl_, ctrl_, sizeof(Ctrl), cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    int status = AERO_OK;
    while (executed < n && !host_ctrl_.done && err_ == cudaSuccess) {
      const int chunk = std::min(n - executed, rec_cap_);
      const int it0 = host_ctrl_.iter;
      host_rec_base_ = it0;
      AERO_CK(cudaMemcpyAsync(&ctrl_->rec_base, &host_rec_base_, sizeof(int), cudaMemcpyHostToDevice, st_));
      launch_iterations(it0, chunk, [](int) {}, [](int) {});
      AERO_CK(cudaMemcpyAsync(&host_ctrl_, ctrl_, sizeof(Ctrl), cudaMemcpyDeviceToHost, st_));
      AERO_CK(cudaStreamSynchronize(st_));
      const int k = host_ctrl_.iter - it0;
      if (recs && k > 0) {
        AERO_CK(cudaMemcpyAsync(recs + executed, recs_, sizeof(Record) * k, cudaMemcpyDeviceToHost, st_));
        AERO_CK(cudaStreamSynchronize(st_));
      }
      executed += k;
      if (k < chunk && !host_ctrl_.done) break;  // should not happen
    }
    if (host_ctrl_.nonfinite) status = AERO_ERR_NONFINITE;
    if (err_ != cudaSuccess) status = AERO_ERR_CUDA;
    if (n_done) *n_done = executed;
    return status;
  }

  // Device time of n iterations between CUDA events on the context's stream. With
  // flush_l2, a buffer larger than L2 is overwritten before every iteration and only the
  // iterations themselves are timed (one event pair per iteration, times summed).
  int time_iterations(int n, int use_graph, int flush_l2, double* ms) override {
    const int it0 = begin_untracked();
    if (use_graph) {  // instantiate every graph the loop uses before timing
      for (int j = 0; j < std::min(n, 2); ++j) {
        for (const int it : {it0 + j, it0 + n - 1 - j}) {
          ensure_graph(second_at(it), it & 1, defer_control_, defer_control_ && it > it0);
        }
      }
    }
    if (flush_l2 && !ensure_flush_buffer()) return AERO_ERR_NOMEM;
    const int npairs = flush_l2 ? n : 1;
    std::vector<cudaEvent_t> ev(2 * static_cast<size_t>(npairs));
    for (auto& e : ev) AERO_CK(cudaEventCreate(&e));
    auto before = [&](int j) {
      if (flush_l2) {
        AERO_CK(cudaMemsetAsync(flush_, j & 0xff, flush_bytes_, st_));
        AERO_CK(cudaEventRecord(ev[2 * j], st_));
      } else if (j == 0) {
        AERO_CK(cudaEventRecord(ev[0], st_));
      }
    };
    auto after = [&](int j) {
      if (flush_l2) {
        AERO_CK(cudaEventRecord(ev[2 * j + 1], st_));
      } else if (j == n - 1) {
        AERO_CK(cudaEventRecord(ev[1], st_));
      }
    };
    if (use_graph) {
      launch_iterations(it0, n, before, after);
    } else {
      for (int j = 0; j < n; ++j) {
        before(j);
        launch_iteration(second_at(it0 + j), (it0 + j) & 1, false, false, Direct{});
        after(j);
      }
    }
    AERO_CK(cudaStreamSynchronize(st_));
    double total = 0.0;
    for (int k = 0; k < npairs; ++k) {
      float f = 0.0f;
      AERO_CK(cudaEventElapsedTime(&f, ev[2 * k], ev[2 * k + 1]));
      total += f;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    *ms = total;
    return end_untracked();
  }

  // Per kernel class: summed device time (ms) and launches over n iterations, each kernel
  // bracketed by its own events. Classes: 0 gradient, 1 residual face pass (+ cell pass under
  // global time stepping), 2 update (+ cell gather under local time stepping), 3 global-dt
  // reduction, 4 symmetry + pressure-jump, 5 controller.
  int profile_kernels(int n, int flush_l2, double* ms, int* launches) override {
    const int it0 = begin_untracked();
    if (flush_l2 && !ensure_flush_buffer()) return AERO_ERR_NOMEM;
    for (int k = 0; k < 6; ++k) {
      ms[k] = 0.0;
      launches[k] = 0;
    }
    // every launch between its own event pair; all queued back to back, read after one sync
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    for (int j = 0; j < n; ++j) {
      if (flush_l2) AERO_CK(cudaMemsetAsync(flush_, j & 0xff, flush_bytes_, st_));
      launch_iteration(second_at(it0 + j), (it0 + j) & 1, false, false, [&](int cls, auto&& launch) {
        cudaEvent_t a = nullptr, b = nullptr;
        AERO_CK(cudaEventCreate(&a));
        AERO_CK(cudaEventCreate(&b));
        AERO_CK(cudaEventRecord(a, st_));
        launch();
        AERO_CK(cudaEventRecord(b, st_));
        marks.push_back({cls, {a, b}});
      });
    }
    AERO_CK(cudaStreamSynchronize(st_));
    for (auto& mk : marks) {
      float f = 0.0f;
      AERO_CK(cudaEventElapsedTime(&f, mk.second.first, mk.second.second));
      ms[mk.first] += f;
      ++launches[mk.first];
      cudaEventDestroy(mk.second.first);
      cudaEventDestroy(mk.second.second);
    }
    return end_untracked();
  }

  void info(long long* out, int n) override {
    long long v[8] = {n_, hs_.nf, d_, launches_per_iteration(true), static_cast<long long>(bytes_),
                      sizeof(T) == 4 ? AERO_PRECISION_FP32 : AERO_PRECISION_FP64, block_, nblocks_};
    for (int i = 0; i < n && i < 8; ++i) out[i] = v[i];
  }

 private:
  template <class U>
  static std::vector<U> nonempty(const std::vector<U>& v) {
    return v.empty() ? std::vector<U>(1, U()) : v;
  }
  template <class U>
  U* alloc(size_t count) {
    void* p = nullptr;
    const size_t b = std::max<size_t>(count, 1) * sizeof(U);
    const cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      if (err_ == cudaSuccess) err_ = e;
      return nullptr;
    }
    AERO_CK(cudaMemsetAsync(p, 0, b, st_));
    allocs_.push_back(p);
    bytes_ += b;
    return static_cast<U*>(p);
  }
  template <class U>
  U* upload(const std::vector<U>& v) {
    U* p = alloc<U>(v.size());
    if (p) AERO_CK(cudaMemcpyAsync(p, v.data(), sizeof(U) * v.size(), cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    return p;
  }

  bool second_at(int it) const { return it >= std::max(cfg_.startup_first_order_iters, 0); }

  long long launches_per_iteration(bool second) const {
    // gradient, face pass, update (+ cell pass and time-step reduction with a global step)
    const int per_stage = (second ? 1 : 0) + 2 + (cfg_.local_time_stepping ? 0 : 2);
    return static_cast<long long>(per_stage) * cfg_.rk_stages + (pjump_on_ ? 1 : 0) + (sym_on_ ? 1 : 0) + 1;
  }

  void refresh() {
    if constexpr (sizeof(T) == 4) {
      k_prim_from_image<<<nblocks_, block_, 0, st_>>>(n_, sref_.hi, W_, pc_.gamma_f);
    } else {
      k_refresh_prim<T><<<nblocks_, block_, 0, st_>>>(n_, Un_, W_, rs_.gamma);
    }
    AERO_CK(cudaGetLastError());
    w_valid_ = true;
  }

  // FP32 keeps the state as float-float pairs and uses Un_ as the double staging array.
  void state_from_staging() {
    if (sizeof(T) == 4) k_split_state<<<nblocks_, block_, 0, st_>>>(n_, Un_, sref_.hi, sref_.lo);
    AERO_CK(cudaGetLastError());
  }
  void state_to_staging() {
    if (sizeof(T) == 4) k_combine_state<<<nblocks_, block_, 0, st_>>>(n_, sref_.hi, sref_.lo, Un_);
    AERO_CK(cudaGetLastError());
  }

  void download_residual(double* res, double* sr) {
    std::vector<V4> hr(static_cast<size_t>(n_));
    std::vector<T> hs(static_cast<size_t>(n_));
    AERO_CK(cudaMemcpyAsync(hr.data(), R_, sizeof(V4) * n_, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaMemcpyAsync(hs.data(), SR_, sizeof(T) * n_, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    for (int cn = 0; cn < n_; ++cn) {
      const int co = hs_.perm[cn];
      double* r = res + 5 * static_cast<size_t>(co);
      r[0] = hr[cn].x;
      r[1] = hr[cn].y;
      r[2] = hr[cn].z;
      r[3] = 0.0;
      r[4] = hr[cn].w;
      if (sr) sr[co] = hs[cn];
    }
  }

  ResidualLaunch<T> residual_args(Ctrl* ctrl, int* fb, V4* R, T* SR, int global_dt) {
    ResidualLaunch<T> a;
    a.block = block_;
    a.st = st_;
    a.faces = df_;
    a.gather = dg_;
    a.fp = fp_;
    a.W = W_;
    a.gx = gx_;
    a.gy = gy_;
    a.F = F_;
    a.FS = FS_;
    a.R = R;
    a.SR = SR;
    a.part = part_;
    a.ctrl = ctrl;
    a.fb = fb;
    a.global_dt = global_dt;
    return a;
  }
  void launch_residual(bool second, bool norms, Ctrl* ctrl, int* fb, V4* R, T* SR, int global_dt) {
    launch_residual_passes(residual_args(ctrl, fb, R, SR, global_dt), cfg_.flux, second, rs_.lm != 0, norms);
  }

  template <bool PRECOND, bool LAST, bool GATHER>
  void update_t(int stage, int global_dt, V4* R, T* SR) {
    k_update<T, PRECOND, LAST, GATHER><<<nblocks_, block_, 0, st_>>>(n_, stage, pc_, R, SR, dg_, F_, FS_, W_, sref_,
                                                                     Us_, ms_, part_, ctrl_, global_dt);
  }
  template <bool PRECOND>
  void update_p(int stage, bool last, int global_dt, V4* R, T* SR) {
    if (global_dt) {  // residual already gathered (the global time step needs all of SR first)
      if (last) update_t<PRECOND, true, false>(stage, global_dt, R, SR);
      else update_t<PRECOND, false, false>(stage, global_dt, R, SR);
    } else {
      if (last) update_t<PRECOND, true, true>(stage, global_dt, R, SR);
      else update_t<PRECOND, false, true>(stage, global_dt, R, SR);
    }
  }

  struct Direct {
    template <class L>
    void operator()(int, L&& launch) const {
      launch();
    }
  };

  // The launches of one iteration; `wrap(kernel_class, launch)` issues each one. `parity`
  // (iteration & 1) selects the fallback counters. With `defer`, the controller of this
  // iteration is left to the next one (or to launch_control); with `pending`, the previous
  // iteration's controller (parity ^ 1) is forked onto the side stream beside this
  // iteration's gradient and first residual and joined before the first update, the first
  // kernel that reads its outputs.
  template <class Wrap>
  void launch_iteration(bool second, int parity, bool defer, bool pending, Wrap&& wrap) {
    const int global_dt = cfg_.local_time_stepping ? 0 : 1;
    const int ns = cfg_.rk_stages;
    int* fb = fb_ + 2 * parity;
    for (int stage = 0; stage < ns; ++stage) {
      const bool last = stage == ns - 1;
      V4* R = stage == 0 ? R0_ : R_;
      T* SR = stage == 0 ? SR0_ : SR_;
      if (stage == 0 && pending) {
        AERO_CK(cudaEventRecord(ev_fork_, st_));
        AERO_CK(cudaStreamWaitEvent(side_, ev_fork_, 0));
        wrap(5, [&] {
          k_control<<<1, kCtlThreads, 0, side_>>>(cc_, part_, ctrl_, recs_, rec_cap_, fb_ + 2 * (parity ^ 1));
        });
        AERO_CK(cudaEventRecord(ev_join_, side_));
      }
      if (second) wrap(0, [&] { k_gradient<T><<<nblocks_, block_, 0, st_>>>(dm_, W_, gx_, gy_, ctrl_); });
      const ResidualLaunch<T> ra = residual_args(ctrl_, fb, R, SR, global_dt);
      wrap(1, [&] { launch_face_pass(ra, cfg_.flux, second, rs_.lm != 0); });
      if (global_dt) wrap(1, [&] { launch_gather_pass(ra, last); });
      if (stage == 0 && pending) AERO_CK(cudaStreamWaitEvent(st_, ev_join_, 0));
      if (global_dt) {
        wrap(3, [&] { k_srmax<<<1, 1024, 0, st_>>>(part_.srmax, nblocks_ * (block_ / 32), ctrl_); });
      }
      wrap(2, [&] {
        if (cfg_.precond_on) {
          update_p<true>(stage, last, global_dt, R, SR);
        } else {
          update_p<false>(stage, last, global_dt, R, SR);
        }
      });
    }
    if (sym_on_) {
      wrap(4, [&] {
        k_symmetry<T><<<nblocks_, block_, 0, st_>>>(n_, cfg_.aoa0_symmetry_enforce_interval, rs_.gamma, sref_,
                                                     W_, ms_, part_, ctrl_);
      });
    }
    if (pjump_on_) {
      wrap(4, [&] { k_pjump<T><<<nblocks_, block_, 0, st_>>>(dm_, sref_, flags_, rs_.gamma, part_, ctrl_); });
    }
    if (!defer) launch_control(parity, wrap);
    AERO_CK(cudaGetLastError());
  }
  template <class Wrap>
  void launch_control(int parity, Wrap&& wrap) {
    wrap(5, [&] { k_control<<<1, kCtlThreads, 0, st_>>>(cc_, part_, ctrl_, recs_, rec_cap_, fb_ + 2 * parity); });
  }

  // Iterations it0 .. it0+n-1 back to back, through the per-iteration CUDA graphs; with the
  // deferred controller, each iteration's controller overlaps the next iteration's start and
  // the last one runs after the loop. `between(j)` runs on the stream before iteration j and
  // `after(j)` after it (timing marks, L2 flushes).
  template <class Before, class After>
  void launch_iterations(int it0, int n, Before&& between, After&& after) {
    for (int j = 0; j < n; ++j) {
      const int it = it0 + j;
      between(j);
      launch_iteration_graph(second_at(it), it & 1, defer_control_, defer_control_ && j > 0);
      if (defer_control_ && j == n - 1) launch_control(it & 1, Direct{});
      after(j);
    }
  }

  // Start/end of a run whose records are not kept (timing, profiling).
  int begin_untracked() {
    if (!w_valid_) refresh();
    AERO_CK(cudaMemcpyAsync(&host_ctrl_, ctrl_, sizeof(Ctrl), cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    host_rec_base_ = -(1 << 30);
    AERO_CK(cudaMemcpyAsync(&ctrl_->rec_base, &host_rec_base_, sizeof(int), cudaMemcpyHostToDevice, st_));
    return host_ctrl_.iter;
  }
  int end_untracked() {
    AERO_CK(cudaMemcpyAsync(&host_ctrl_, ctrl_, sizeof(Ctrl), cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    if (err_ != cudaSuccess) return AERO_ERR_CUDA;
    return host_ctrl_.nonfinite ? AERO_ERR_NONFINITE : AERO_OK;
  }

  d4* pinned_state() {
    if (pin_state_ == nullptr) {
      if (cudaMallocHost(reinterpret_cast<void**>(&pin_state_), sizeof(d4) * static_cast<size_t>(n_)) !=
          cudaSuccess) {
        cudaGetLastError();
        pin_state_ = nullptr;
        pin_fallback_.resize(static_cast<size_t>(n_));
        return pin_fallback_.data();
      }
    }
    return pin_state_;
  }

  bool ensure_flush_buffer() {
    if (flush_) return true;
    flush_bytes_ = size_t(256) << 20;  // twice the 129 MB L2
    if (cudaMalloc(&flush_, flush_bytes_) != cudaSuccess) {
      cudaGetLastError();
      flush_ = nullptr;
      return false;
    }
    return true;
  }

  static int graph_index(bool second, int parity, bool defer, bool pending) {
    return (second ? 1 : 0) | (parity << 1) | ((defer ? 1 : 0) << 2) | ((pending ? 1 : 0) << 3);
  }
  void ensure_graph(bool second, int parity, bool defer, bool pending) {
    const int i = graph_index(second, parity, defer, pending);
    if (graph_[i]) return;
    cudaGraph_t g = nullptr;
    AERO_CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
    launch_iteration(second, parity, defer, pending, Direct{});
    AERO_CK(cudaStreamEndCapture(st_, &g));
    if (g) {
      AERO_CK(cudaGraphInstantiate(&graph_[i], g, 0));
      cudaGraphDestroy(g);
    }
  }

  void launch_iteration_graph(bool second, int parity, bool defer, bool pending) {
    ensure_graph(second, parity, defer, pending);
    const int i = graph_index(second, parity, defer, pending);
    if (graph_[i]) {
      AERO_CK(cudaGraphLaunch(graph_[i], st_));
    } else {
      launch_iteration(second, parity, defer, pending, Direct{});
    }
  }

  HostSlots hs_;
  aero_case_desc cfg_;
  Resolved rs_;
  cudaStream_t st_;
  cudaError_t err_ = cudaSuccess;
  std::vector<void*> allocs_;
  size_t bytes_ = 0;
  int n_ = 0, d_ = 0, block_ = 128, nblocks_ = 0, rec_cap_ = 0;
  bool pjump_on_ = false, sym_on_ = false, w_valid_ = false;
  int* link_ = nullptr;
  V2* nrm_ = nullptr;
  T* area_ = nullptr;
  DevFaces<T> df_{};
  DevGather<T> dg_{};
  V4* F_ = nullptr;   // per face: F*A
  T* FS_ = nullptr;   // per face: wave-speed term
  T* inv_vol_ = nullptr;
  unsigned char* flags_ = nullptr;
  int* perm_dev_ = nullptr;
  MonitorSet ms_{};
  V4 *W_ = nullptr, *gx_ = nullptr, *gy_ = nullptr, *R_ = nullptr;
  T* SR_ = nullptr;
  d4* Un_ = nullptr;     // FP64: the conserved state; FP32: double staging for transfers
  StateRef sref_{};
  V4* Us_ = nullptr;    // FP64: stage state; FP32: stage increment (delta form)
  d4* Ueval_ = nullptr;  // conserved state given to aero_residual
  Partials part_{};
  Ctrl* ctrl_ = nullptr;
  Ctrl* ctrl_eval_ = nullptr;
  Record* recs_ = nullptr;
  Ctrl host_ctrl_{};
  int host_rec_base_ = 0;
  DevMesh<T> dm_{};
  FaceParams<T> fp_{};
  PrecondD pc_{};
  CtrlConfig cc_{};
  cudaGraphExec_t graph_[16] = {};
  bool defer_control_ = false;
  cudaStream_t side_ = nullptr;
  cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
  V4* R0_ = nullptr;
  T* SR0_ = nullptr;
  int* fb_ = nullptr;  // [2 parities][first-order, diffusive] fallback counters
  void* flush_ = nullptr;
  size_t flush_bytes_ = 0;
  d4* pin_state_ = nullptr;
  std::vector<d4> pin_fallback_;
};

#undef AERO_CK

}  // namespace aero
