// engine_impl.cuh -- device solver for one bulk precision T (float or double), for one case or
// a batch of cases packed into one set of arrays. Included by engine_f32.cu and
// engine_f64.cu, which instantiate it.
//
// Packing: case k's cells occupy [c0_k, c0_k + n_k) of the per-cell arrays and its faces
// [f0_k, f0_k + nf_k) of the per-face arrays; both ranges start on a block boundary, so every
// block of the cell and face kernels belongs to exactly one case (tables cblk / fblk give its
// case and the end of that case's range). Neighbour ids, face ids and wall entries are
// offset by the case's bases, so the kernels see one mesh of disjoint components; per-case
// constants (free stream, schedule, controller) are arrays indexed by the case. A case's
// cells keep the block layout of a single-case run, so a batch reproduces single runs.
#pragma once

#include "aero_adjoint.cuh"
#include "aero_tma.cuh"
#include "aero_face_kernels.cuh"
#include "engine.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
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

  // Where case k lives in the packed arrays.
  struct Pack {
    int n, nf, d;    // cells, faces, faces per cell
    int c0, f0;      // first cell, first face
    int cb0, ncb;    // first cell block, cell blocks
    int fb0, nfb;    // first face block, face blocks
    int w0;          // first wall entry
    int ws0, nws;    // first wall-partial slot, slots
  };

 public:
  EngineT(const std::vector<HostSlots>& hs, const std::vector<aero_case_desc>& cfg, const std::vector<Resolved>& rs,
          cudaStream_t st)
      : hs_(hs), cfg_(cfg), rs_(rs), st_(st) {}

  ~EngineT() override {
    for (auto& g : graph_) {
      if (g) cudaGraphExecDestroy(g);
    }
    if (adj_graph_) cudaGraphExecDestroy(adj_graph_);
    if (kr_graph_) cudaGraphExecDestroy(kr_graph_);
    if (ev_fork_) cudaEventDestroy(ev_fork_);
    if (ev_join_) cudaEventDestroy(ev_join_);
    if (side_) cudaStreamDestroy(side_);
    for (void* p : allocs_) cudaFree(p);
    if (flush_) cudaFree(flush_);
    if (pin_state_) cudaFreeHost(pin_state_);
  }

  bool init(std::string* err) override {
    K_ = static_cast<int>(hs_.size());
    if (K_ < 1 || cfg_.size() != hs_.size() || rs_.size() != hs_.size()) {
      *err = "no cases";
      return false;
    }
    const aero_case_desc& c0 = cfg_[0];
    block_ = c0.block_size > 0 ? c0.block_size : 128;
    if (block_ != 64 && block_ != 128 && block_ != 256) {
      *err = "block_size must be 64, 128 or 256";
      return false;
    }
    cpt_ = c0.cells_per_thread > 0 ? c0.cells_per_thread : 1;
    if (cpt_ != 1 && cpt_ != 2) {
      *err = "cells_per_thread must be 1 or 2";
      return false;
    }
    lm_ = rs_[0].lm;
    for (int k = 1; k < K_; ++k) {  // settings that select kernel variants are shared
      const aero_case_desc& c = cfg_[k];
      if (c.flux != c0.flux || c.limiter != c0.limiter || c.precision != c0.precision ||
          c.rk_stages != c0.rk_stages || c.local_time_stepping != c0.local_time_stepping ||
          c.startup_first_order_iters != c0.startup_first_order_iters || c.precond_on != c0.precond_on ||
          rs_[k].lm != lm_ || (c.block_size > 0 ? c.block_size : 128) != block_ ||
          (c.cells_per_thread > 0 ? c.cells_per_thread : 1) != cpt_) {
        *err = "cases of one batch must share flux, limiter, precision, RK stages, time-step mode, "
               "start-up length, low-Mach switches, block size and cells per thread";
        return false;
      }
    }

    // ---- packed layout
    pk_.resize(K_);
    int ntot = 0, ftot = 0, cb = 0, fbk = 0, wtot = 0, wslots = 0;
    d_ = 0;
    std::vector<std::vector<int>> case_block_slot(K_);
    for (int k = 0; k < K_; ++k) {
      const HostSlots& h = hs_[k];
      Pack& p = pk_[k];
      p.n = h.n;
      p.nf = static_cast<int>(h.f_orig.size());
      p.d = h.d;
      p.c0 = ntot;
      p.f0 = ftot;
      p.ncb = (p.n + block_ - 1) / block_;
      p.nfb = (p.nf + block_ - 1) / block_;
      p.cb0 = cb;
      p.fb0 = fbk;
      p.w0 = wtot;
      ntot += p.ncb * block_;
      ftot += p.nfb * block_;
      cb += p.ncb;
      fbk += p.nfb;
      wtot += static_cast<int>(h.wkind.size());
      d_ = std::max(d_, h.d);
      // a wall-partial slot for each cell block of the case that holds wall entries
      std::vector<int>& bs = case_block_slot[k];
      bs.assign(p.ncb, -1);
      p.ws0 = wslots;
      p.nws = 0;
      for (int b = 0; b < p.ncb; ++b) {
        const int e = std::min(p.n, (b + 1) * block_);
        for (int c = b * block_; c < e; ++c) {
          if (h.flags[c] >= 4) {
            bs[b] = wslots + p.nws++;
            break;
          }
        }
      }
      wslots += p.nws;
    }
    ntot_ = ntot;
    ftot_ = ftot;
    ncb_ = cb;
    nfb_ = fbk;
    ncells_ = 0;
    nfaces_ = 0;
    for (const Pack& p : pk_) {
      ncells_ += p.n;
      nfaces_ += p.nf;
    }

    // ---- slot table (gradient, pressure jump) and gather slots, stride ntot
    {
      const size_t ns = static_cast<size_t>(ntot_) * d_;
      std::vector<int> link(ns, kPad), gslot(ns, kPad);
      std::vector<V2> nrm(ns), gvec(ns);
      std::vector<T> area(ns, T(0));
      std::vector<T> inv_vol(static_cast<size_t>(ntot_), T(1));
      std::vector<unsigned char> flags(static_cast<size_t>(ntot_), 0);
      std::vector<int> wall_first(static_cast<size_t>(ntot_), 0);
      for (auto& v : nrm) v.x = v.y = T(0);
      for (auto& v : gvec) v.x = v.y = T(0);
      for (int k = 0; k < K_; ++k) {
        const HostSlots& h = hs_[k];
        const Pack& p = pk_[k];
        for (int j = 0; j < h.d; ++j) {
          for (int c = 0; c < h.n; ++c) {
            const size_t src = static_cast<size_t>(j) * h.n + c;
            const size_t dst = static_cast<size_t>(j) * ntot_ + p.c0 + c;
            const int l = h.link[src];
            link[dst] = l >= 0 ? ((((l >> 1) + p.c0) << 1) | (l & 1)) : l;
            const int g = h.gslot[src];
            gslot[dst] = g >= 0 ? ((((g >> 1) + p.f0) << 1) | (g & 1)) : g;
            nrm[dst].x = T(h.nx[src]);
            nrm[dst].y = T(h.ny[src]);
            area[dst] = T(h.area[src]);
            if (l != kPad) {  // the face vector in T as the gradient formed it, halved with a neighbour
              const T h2 = l >= 0 ? T(0.5) : T(1);
              gvec[dst].x = h2 * (nrm[dst].x * area[dst]);
              gvec[dst].y = h2 * (nrm[dst].y * area[dst]);
            }
          }
        }
        for (int c = 0; c < h.n; ++c) {
          inv_vol[p.c0 + c] = T(1) / std::max(T(h.vol[c]), T(1.0e-12));
          flags[p.c0 + c] = h.flags[c];
          wall_first[p.c0 + c] = h.wall_first[c] + p.w0;
        }
      }
      link_ = upload(link);
      nrm_ = upload(nrm);
      area_ = upload(area);
      gvec_ = upload(gvec);
      inv_vol_ = upload(inv_vol);
      flags_ = upload(flags);
      dg_.slot = upload(gslot);
      ms_.flags = flags_;
      ms_.wall_first = upload(wall_first);
    }
    // ---- face table in T (exact conversions; MUSCL offsets formed in T from T coordinates)
    {
      std::vector<int2> fc(static_cast<size_t>(ftot_), make_int2(0, -1));
      std::vector<V2> fn(static_cast<size_t>(ftot_)), doff(static_cast<size_t>(ftot_)),
          noff(static_cast<size_t>(ftot_));
      std::vector<T> fa(static_cast<size_t>(ftot_), T(0));
      for (auto* v : {&fn, &doff, &noff}) {
        for (auto& x : *v) x.x = x.y = T(0);
      }
      for (int k = 0; k < K_; ++k) {
        const HostSlots& h = hs_[k];
        const Pack& p = pk_[k];
        for (int i = 0; i < p.nf; ++i) {
          const size_t q = static_cast<size_t>(p.f0) + i;
          fc[q] = make_int2(h.f_own[i] + p.c0, h.f_nb[i] >= 0 ? h.f_nb[i] + p.c0 : h.f_nb[i]);
          fn[q].x = T(h.f_nx[i]);
          fn[q].y = T(h.f_ny[i]);
          fa[q] = T(h.f_area[i]);
          const int o = h.f_own_old[i], b = h.f_nb_old[i];
          doff[q].x = T(h.f_cx[i]) - T(h.ccx[o]);
          doff[q].y = T(h.f_cy[i]) - T(h.ccy[o]);
          if (h.f_nb[i] >= 0) {
            noff[q].x = T(h.f_cx[i]) - T(h.ccx[b]);
            noff[q].y = T(h.f_cy[i]) - T(h.ccy[b]);
          }
        }
      }
      df_.nf = ftot_;
      df_.cells = upload(fc);
      df_.nrm = upload(fn);
      df_.area = upload(fa);
      df_.doff = upload(doff);
      df_.noff = upload(noff);
      F_ = alloc<V4>(ftot_);
      FS_ = alloc<T>(ftot_);
    }
    // ---- wall entries, block tables
    {
      std::vector<unsigned char> wkind;
      std::vector<double> wnx, wny, warea, wx, wy;
      for (const HostSlots& h : hs_) {
        wkind.insert(wkind.end(), h.wkind.begin(), h.wkind.end());
        wnx.insert(wnx.end(), h.wnx.begin(), h.wnx.end());
        wny.insert(wny.end(), h.wny.begin(), h.wny.end());
        warea.insert(warea.end(), h.warea.begin(), h.warea.end());
        wx.insert(wx.end(), h.wx.begin(), h.wx.end());
        wy.insert(wy.end(), h.wy.begin(), h.wy.end());
      }
      ms_.wkind = upload(nonempty(wkind));
      ms_.wnx = upload(nonempty(wnx));
      ms_.wny = upload(nonempty(wny));
      ms_.warea = upload(nonempty(warea));
      ms_.wx = upload(nonempty(wx));
      ms_.wy = upload(nonempty(wy));
      auto to_f = [](const std::vector<double>& v) {
        std::vector<float> f(v.empty() ? 1 : v.size(), 0.0f);
        for (size_t i = 0; i < v.size(); ++i) f[i] = float(v[i]);
        return f;
      };
      ms_.wnx_f = upload(to_f(wnx));
      ms_.wny_f = upload(to_f(wny));
      ms_.warea_f = upload(to_f(warea));
      ms_.wx_f = upload(to_f(wx));
      ms_.wy_f = upload(to_f(wy));
      std::vector<int> block_slot;
      std::vector<int2> cblk, fblk;
      std::vector<int> srfirst;
      for (int k = 0; k < K_; ++k) {
        const Pack& p = pk_[k];
        block_slot.insert(block_slot.end(), case_block_slot[k].begin(), case_block_slot[k].end());
        for (int b = 0; b < p.ncb; ++b) cblk.push_back(make_int2(k, p.c0 + p.n));
        for (int b = 0; b < p.nfb; ++b) fblk.push_back(make_int2(k, p.f0 + p.nf));
        srfirst.push_back(p.cb0 * (block_ / 32));
      }
      srfirst.push_back(ncb_ * (block_ / 32));
      ms_.block_slot = upload(block_slot);
      cblk_ = upload(cblk);
      fblk_ = upload(fblk);
      srfirst_ = upload(srfirst);
      nwslots_ = wslots;
    }
    std::vector<int> perm0(hs_[0].perm);
    perm_dev_ = upload(perm0);
    {
      std::vector<int> iperm_all(static_cast<size_t>(ntot_), 0);  // original -> device cell within the case
      for (int k = 0; k < K_; ++k) {
        const std::vector<int>& pm = hs_[k].perm;
        for (int cn = 0; cn < static_cast<int>(pm.size()); ++cn) iperm_all[pk_[k].c0 + pm[cn]] = cn;
      }
      iperm_all_dev_ = upload(iperm_all);
    }
    // direct state exchange with host arrays where the GPU walks the host's page tables
    {
      int dev = 0, pageable = 0, host_tables = 0;
      cudaGetDevice(&dev);
      if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) !=
              cudaSuccess) {
        cudaGetLastError();
        pageable = host_tables = 0;
      }
      const char* off = std::getenv("AERO_HOST_STAGING");
      host_direct_ = pageable == 1 && host_tables == 1 && !(off && off[0] == '1');
    }

    // ---- state and work arrays
    W_ = alloc<V4>(ntot_);
    gx_ = alloc<V4>(ntot_);
    gy_ = alloc<V4>(ntot_);
    R_ = alloc<V4>(ntot_);
    SR_ = alloc<T>(ntot_);
    const bool global_dt = !c0.local_time_stepping;
    if (c0.rk_stages > 1 && global_dt) {  // the first stage's residual, kept apart from the last stage's
      R0_ = alloc<V4>(ntot_);
      SR0_ = alloc<T>(ntot_);
    } else {
      R0_ = R_;
      SR0_ = SR_;
    }
    fb_ = alloc<int>(4 * static_cast<size_t>(K_));
    Un_ = alloc<d4>(ntot_);
    Us_ = alloc<V4>(ntot_);
    sref_.un = Un_;
    if (sizeof(T) == 4) {
      sref_.hi = alloc<float4>(ntot_);
      sref_.lo = alloc<float4>(ntot_);
    }
    Ueval_ = alloc<d4>(ntot_);
    if (sizeof(T) == 4) {
      part_.norms_f = alloc<float>(kNorm * static_cast<size_t>(ncb_));
    } else {
      part_.norms = alloc<double>(kNorm * static_cast<size_t>(ncb_));
    }
    part_.mon = alloc<long long>(kMon * static_cast<size_t>(ncb_));
    if (sizeof(T) == 4) {
      part_.wall_f = alloc<float>(kWall * static_cast<size_t>(std::max(nwslots_, 1)));
    } else {
      part_.wall = alloc<double>(kWall * static_cast<size_t>(std::max(nwslots_, 1)));
    }
    part_.nb = ncb_;
    part_.nwb = nwslots_;
    part_.pjump = alloc<double>(4 * static_cast<size_t>(ncb_));
    part_.srmax = alloc<double>(static_cast<size_t>(ncb_) * (block_ / 32));
    ctrls_ = alloc<Ctrl>(K_);
    ctrl_eval_ = alloc<Ctrl>(1);
    rec_cap_ = 1024;
    recs_ = alloc<Record>(static_cast<size_t>(K_) * rec_cap_);
    ccs_dev_ = alloc<CtrlConfig>(K_);
    fps_dev_ = alloc<FaceParams<T>>(K_);
    pcs_dev_ = alloc<PrecondD>(K_);
    mcs_dev_ = alloc<MonitorConsts>(K_);
    if (err_ != cudaSuccess) {
      *err = std::string("device allocation/upload failed: ") + cudaGetErrorString(err_);
      return false;
    }

    dm_.n = ntot_;
    dm_.d = d_;
    dm_.link = link_;
    dm_.nrm = nrm_;
    dm_.area = area_;
    dm_.gvec = gvec_;
    dm_.inv_vol = inv_vol_;
    dg_.n = ntot_;
    dg_.d = d_;
    dg_.inv_vol = inv_vol_;
    {
      // programmatic dependent launch of the iteration's kernels (AERO_PDL=1; off by
      // default: 1.7% off the 131k-cell step, 0.5% onto the 524k-cell one, and each kernel's
      // recorded span then includes its wait for the predecessor)
      const char* env = std::getenv("AERO_PDL");
      pdl_ = env && env[0] == '1';
    }
    // the gradient pass of the iterations: persistent CTAs streaming their tiles through
    // shared memory with bulk copies, where each CTA gets three or more tiles
    // (AERO_BULK_COPY=0 never, =1 always)
    {
      const char* env = std::getenv("AERO_BULK_COPY");
      const int mode = (env && env[0] == '0') ? 0 : ((env && env[0] == '1') ? 1 : -1);
      grad_smem_ = grad_tma_smem<T>(block_, d_);
      int dev = 0, sms = 0, smem_optin = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      // two tile buffers of B cells x D slots: cells with many faces (up to 32 per cell) at
      // block 256 need more shared memory than a CTA can have, and then the plain gather
      // kernel runs; forcing the bulk-copy pass (AERO_BULK_COPY=1) there is an error
      const bool fits = grad_smem_ <= static_cast<size_t>(smem_optin);
      if (mode == 1 && !fits) {
        *err = "the bulk-copy gradient pass needs " + std::to_string(grad_smem_) +
               " bytes of shared memory per block, more than the device's " + std::to_string(smem_optin) +
               " (AERO_BULK_COPY=1 with this block size and faces per cell)";
        return false;
      }
      if (mode != 0 && fits) {
        int per_sm = 0;
        if (grad_smem_ > 48 * 1024) {
          AERO_CK(cudaFuncSetAttribute(k_gradient_tma<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(grad_smem_)));
        }
        AERO_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gradient_tma<T>, block_, grad_smem_));
        grad_grid_ = std::min(ncb_, std::max(1, per_sm) * std::max(1, sms));
        // the copies of a CTA's next tile overlap its current one only with several tiles
        // per CTA. Measured against the gather pass: 2.2 tiles per CTA (524k cells) 13.5 us
        // against 12.9 us; 20 tiles (the 4.8 M-cell sweep) 88.6 us against 110.6 us
        grad_tma_ = mode == 1 || ncb_ >= 3 * grad_grid_;
      }
      // [0] wait-expired word, [1] poll limit of the bulk-copy waits (-1: the default)
      tma_err_ = alloc<int>(2);
      const int init_words[2] = {0, -1};
      AERO_CK(cudaMemcpyAsync(tma_err_, init_words, sizeof(init_words), cudaMemcpyHostToDevice, st_));
      AERO_CK(cudaStreamSynchronize(st_));
    }

    // ---- per-case constants
    ccs_.resize(K_);
    fps_.resize(K_);
    pcs_.resize(K_);
    mcs_.resize(K_);
    pjump_on_ = false;
    sym_on_ = false;
    for (int k = 0; k < K_; ++k) {
      setup_case(k);
      pjump_on_ = pjump_on_ || ccs_[k].pjump_blocks > 0;
      sym_on_ = sym_on_ || mcs_[k].sym_interval > 0;
    }
    AERO_CK(cudaMemcpyAsync(ccs_dev_, ccs_.data(), sizeof(CtrlConfig) * K_, cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaMemcpyAsync(fps_dev_, fps_.data(), sizeof(FaceParams<T>) * K_, cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaMemcpyAsync(pcs_dev_, pcs_.data(), sizeof(PrecondD) * K_, cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaMemcpyAsync(mcs_dev_, mcs_.data(), sizeof(MonitorConsts) * K_, cudaMemcpyHostToDevice, st_));
    cell_cases_ = Cases<T>{cblk_, ctrls_, fps_dev_, pcs_dev_, mcs_dev_, tma_err_};
    face_cases_ = Cases<T>{fblk_, ctrls_, fps_dev_, pcs_dev_, mcs_dev_, tma_err_};

    // the controller of iteration i runs beside the gradient and first face pass of
    // iteration i+1 (which need none of its outputs) for RK3 runs; with low-Mach weights in
    // the residual only when no case runs the staged all-speed controller, whose weights
    // depend on the previous iteration: the others depend on the iteration index alone and
    // reach the face passes through two parity slots that the controller fills two
    // iterations ahead
    bool staged_any = false;
    for (int k = 0; k < K_; ++k) staged_any = staged_any || ccs_[k].staged != 0;
    defer_control_ = c0.rk_stages > 1 && (!lm_ || !staged_any);
    lm_defer_ = defer_control_ && lm_;
    if (lm_defer_) lms_ = alloc<LmSched>(2 * static_cast<size_t>(K_));
    if (defer_control_) {
      AERO_CK(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
      AERO_CK(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
      AERO_CK(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming));
    }
    // freestream initial state
    {
      std::vector<d4> u0(static_cast<size_t>(ntot_));
      for (int k = 0; k < K_; ++k) {
        const Pack& p = pk_[k];
        const d4 fs{rs_[k].cons_inf[0], rs_[k].cons_inf[1], rs_[k].cons_inf[2], rs_[k].cons_inf[3]};
        for (int c = 0; c < p.ncb * block_; ++c) u0[p.c0 + c] = fs;
      }
      AERO_CK(cudaMemcpyAsync(Un_, u0.data(), sizeof(d4) * ntot_, cudaMemcpyHostToDevice, st_));
      AERO_CK(cudaStreamSynchronize(st_));
    }
    state_from_staging(0, ntot_);
    w_valid_ = false;
    reset_run();
    AERO_CK(cudaStreamSynchronize(st_));
    if (err_ != cudaSuccess) {
      *err = std::string("initialisation failed: ") + cudaGetErrorString(err_);
      return false;
    }
    return true;
  }

  int n_cases() const override { return K_; }

  EngineView view() const override {
    EngineView v{};
    v.n = pk_[0].n;
    v.ntot = ntot_;
    v.nf = ftot_;
    v.cblocks = ncb_;
    v.fblocks = nfb_;
    v.precision = sizeof(T) == 4 ? AERO_PRECISION_FP32 : AERO_PRECISION_FP64;
    v.flux = cfg_[0].flux;
    v.lm = lm_;
    v.block = block_;
    cudaGetDevice(&v.device);
    v.gamma = rs_[0].gamma;
    v.dm = &dm_;
    v.df = &df_;
    v.dg = &dg_;
    v.fps = fps_dev_;
    v.pcs = pcs_dev_;
    v.mcs = mcs_dev_;
    v.cblk = cblk_;
    v.fblk = fblk_;
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
    host_ctrls_.assign(K_, Ctrl{});
    for (int k = 0; k < K_; ++k) {
      Ctrl& h = host_ctrls_[k];
      std::memset(&h, 0, sizeof(h));
      h.iter = 0;
      h.cfl_scale = 1.0;
      h.prev_l2 = -1.0;
      h.initial_l2 = -1.0;
      h.initial_l2rho = -1.0;
      h.stage = cfg_[k].all_speed_staged_controller ? 1 : 0;
      h.stage_b_fmin = rs_[k].st_fmin_high;
      apply_schedule(ccs_[k], &h);
    }
    AERO_CK(cudaMemcpyAsync(ctrls_, host_ctrls_.data(), sizeof(Ctrl) * K_, cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaMemsetAsync(fb_, 0, 4 * sizeof(int) * K_, st_));
    AERO_CK(cudaStreamSynchronize(st_));
  }

  // fn(begin, end) over [0, n) on up to 8 host threads (one for small n)
  template <class Fn>
  static void host_parallel(int n, Fn&& fn) {
    const int hw = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    const int nt = std::min({8, hw, std::max(1, n / 16384)});
    if (nt <= 1) {
      fn(0, n);
      return;
    }
    std::vector<std::thread> pool;
    const int chunk = (n + nt - 1) / nt;
    for (int t = 1; t < nt; ++t) {
      const int b = t * chunk, e = std::min(n, b + chunk);
      if (b < e) pool.emplace_back([&fn, b, e] { fn(b, e); });
    }
    fn(0, std::min(n, chunk));
    for (auto& th : pool) th.join();
  }

  // State transfers go through a page-locked staging buffer in the device order; the
  // renumbering copies run on several host threads.
  void set_state(int k, const double* u) override {
    const Pack& p = pk_[k];
    if (host_direct_) {
      k_state_from_host<<<(p.n + kXferCells - 1) / kXferCells, kXferCells, 0, st_>>>(p.n, u, iperm_all_dev_ + p.c0,
                                                                                         Un_ + p.c0);
      AERO_CK(cudaGetLastError());
      state_from_staging(p.c0, p.n);
      AERO_CK(cudaStreamSynchronize(st_));
      w_valid_ = false;
      return;
    }
    d4* h = pinned_state();
    const int* perm = hs_[k].perm.data();
    host_parallel(p.n, [&](int b, int e) {
      for (int cn = b; cn < e; ++cn) {
        const double* s = u + 5 * static_cast<size_t>(perm[cn]);
        h[cn] = d4{s[0], s[1], s[2], s[4]};
      }
    });
    AERO_CK(cudaMemcpyAsync(Un_ + p.c0, h, sizeof(d4) * p.n, cudaMemcpyHostToDevice, st_));
    state_from_staging(p.c0, p.n);
    AERO_CK(cudaStreamSynchronize(st_));
    w_valid_ = false;
  }

  void get_state(int k, double* u) override {
    const Pack& p = pk_[k];
    if (host_direct_) {
      state_to_staging(p.c0, p.n);
      k_state_to_host<<<(p.n + kXferCells - 1) / kXferCells, kXferCells, 0, st_>>>(p.n, Un_ + p.c0,
                                                                                       iperm_all_dev_ + p.c0, u);
      AERO_CK(cudaGetLastError());
      AERO_CK(cudaStreamSynchronize(st_));
      return;
    }
    d4* h = pinned_state();
    state_to_staging(p.c0, p.n);
    AERO_CK(cudaMemcpyAsync(h, Un_ + p.c0, sizeof(d4) * p.n, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    const int* perm = hs_[k].perm.data();
    host_parallel(p.n, [&](int b, int e) {
      for (int cn = b; cn < e; ++cn) {
        double* s = u + 5 * static_cast<size_t>(perm[cn]);
        s[0] = h[cn].x;
        s[1] = h[cn].y;
        s[2] = h[cn].z;
        s[3] = 0.0;
        s[4] = h[cn].w;
      }
    });
  }

  void get_primitive(int k, double* rho, double* u, double* v, double* p) override {
    const Pack& pc = pk_[k];
    std::vector<d4> h(static_cast<size_t>(pc.n));
    state_to_staging(pc.c0, pc.n);
    AERO_CK(cudaMemcpyAsync(h.data(), Un_ + pc.c0, sizeof(d4) * pc.n, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    for (int cn = 0; cn < pc.n; ++cn) {
      const int co = hs_[k].perm[cn];
      // host restatement of cons_to_prim (euler_flux.cpp:115-127) in double
      const double r = std::max(h[cn].x, 1.0e-8);
      const double inv = 1.0 / r;
      const double uu = h[cn].y * inv, vv = h[cn].z * inv;
      const double ke = 0.5 * r * (uu * uu + vv * vv);
      rho[co] = r;
      u[co] = uu;
      v[co] = vv;
      p[co] = std::max((rs_[k].gamma - 1.0) * (h[cn].w - ke), 1.0e-8);
    }
  }

  // One residual evaluation of case 0 (single-case engines).
  void residual(const double* u, int second, double stab, int as_fix, double as_fmin, double as_ramp,
                double* res, double* sr, double* grad) override {
    const Pack& p = pk_[0];
    std::vector<d4> h(static_cast<size_t>(p.n));
    for (int cn = 0; cn < p.n; ++cn) {
      const double* s = u + 5 * static_cast<size_t>(hs_[0].perm[cn]);
      h[cn] = d4{s[0], s[1], s[2], s[4]};
    }
    AERO_CK(cudaMemcpyAsync(Ueval_, h.data(), sizeof(d4) * p.n, cudaMemcpyHostToDevice, st_));
    Ctrl ce;
    std::memset(&ce, 0, sizeof(ce));
    set_eval_schedule(&ce, stab, as_fix, as_fmin, as_ramp);
    AERO_CK(cudaMemcpyAsync(ctrl_eval_, &ce, sizeof(Ctrl), cudaMemcpyHostToDevice, st_));
    const Cases<T> ccs{cblk_, ctrl_eval_, fps_dev_, pcs_dev_, mcs_dev_};
    const Cases<T> fcs{fblk_, ctrl_eval_, fps_dev_, pcs_dev_, mcs_dev_};
    k_refresh_prim<T><<<ncb_, block_, 0, st_>>>(p.n, Ueval_, W_, rs_[0].gamma);
    if (second) k_gradient<T><<<ncb_, block_, 0, st_>>>(dm_, W_, gx_, gy_, ccs);
    ResidualLaunch<T> a = residual_args(&ctrl_eval_->fo_fallback, R_, SR_, 0);
    a.cell_cases = ccs;
    a.face_cases = fcs;
    launch_residual_passes(a, cfg_[0].flux, second != 0, lm_ != 0, false);
    AERO_CK(cudaGetLastError());
    w_valid_ = false;
    download_residual(0, res, sr);
    if (grad) {
      std::vector<V4> hx(static_cast<size_t>(p.n)), hy(static_cast<size_t>(p.n));
      if (second) {
        AERO_CK(cudaMemcpyAsync(hx.data(), gx_, sizeof(V4) * p.n, cudaMemcpyDeviceToHost, st_));
        AERO_CK(cudaMemcpyAsync(hy.data(), gy_, sizeof(V4) * p.n, cudaMemcpyDeviceToHost, st_));
      }
      AERO_CK(cudaStreamSynchronize(st_));
      for (int cn = 0; cn < p.n; ++cn) {
        double* g = grad + 10 * static_cast<size_t>(hs_[0].perm[cn]);
        if (!second) {
          for (int k = 0; k < 10; ++k) g[k] = 0.0;
          continue;
        }
        const V4 a4 = hx[cn], b4 = hy[cn];
        g[0] = a4.x; g[1] = b4.x;  // rho
        g[2] = a4.y; g[3] = b4.y;  // u
        g[4] = a4.z; g[5] = b4.z;  // v
        g[6] = 0.0; g[7] = 0.0;    // w
        g[8] = a4.w; g[9] = b4.w;  // p
      }
    }
  }

  void last_residual(int k, double* res, double* sr) override { download_residual(k, res, sr); }

  int run(int n, aero_iter_record* recs, int* n_done) override {
    static_assert(sizeof(Record) == sizeof(aero_iter_record), "record layout");
    std::vector<int> executed(K_, 0);
    if (!w_valid_) refresh();
    download_ctrls();
    int status = AERO_OK;
    int e = 0;  // iterations launched in this call (every running case runs all of them)
    auto running = [&] {
      for (const Ctrl& c : host_ctrls_) {
        if (!c.done) return true;
      }
      return false;
    };
    while (e < n && running() && err_ == cudaSuccess) {
      const int chunk = std::min(n - e, rec_cap_);
      int it0 = 0;
      for (const Ctrl& c : host_ctrls_) {
        if (!c.done) {
          it0 = c.iter;
          break;
        }
      }
      std::vector<int> base(K_, it0);
      AERO_CK(cudaMemcpy2DAsync(&ctrls_->rec_base, sizeof(Ctrl), base.data(), sizeof(int), sizeof(int), K_,
                                cudaMemcpyHostToDevice, st_));
      std::vector<char> was_running(K_);
      for (int k = 0; k < K_; ++k) was_running[k] = host_ctrls_[k].done ? 0 : 1;
      launch_iterations(it0, chunk, [](int) {}, [](int) {});
      download_ctrls();
      for (int k = 0; k < K_; ++k) {
        if (!was_running[k]) continue;
        const int got = host_ctrls_[k].iter - it0;
        if (recs && got > 0) {
          AERO_CK(cudaMemcpyAsync(recs + static_cast<size_t>(k) * n + executed[k],
                                  recs_ + static_cast<size_t>(k) * rec_cap_, sizeof(Record) * got,
                                  cudaMemcpyDeviceToHost, st_));
        }
        executed[k] += got;
      }
      AERO_CK(cudaStreamSynchronize(st_));
      e += chunk;
    }
    for (const Ctrl& c : host_ctrls_) {
      if (c.nonfinite) status = AERO_ERR_NONFINITE;
    }
    if (recover_from_expired_wait()) status = AERO_ERR_TIMEOUT;
    if (err_ != cudaSuccess) status = AERO_ERR_CUDA;
    if (n_done) {
      for (int k = 0; k < K_; ++k) n_done[k] = executed[k];
    }
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

  // ---- discrete adjoint (FP64, one case) -------------------------------------------------
  int adjoint_linearize(double w_cd, double w_cl, int second_order) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (K_ != 1 || !std::isfinite(w_cd) || !std::isfinite(w_cl)) return AERO_ERR_INVALID;
      if (!adj_alloc_) {
        Ulin_ = alloc<d4>(ntot_);
        Wlin_ = alloc<d4>(ntot_);
        SRlin_ = alloc<double>(ntot_);
        gxlin_ = alloc<d4>(ntot_);
        gylin_ = alloc<d4>(ntot_);
        Jf_ = alloc<double>(static_cast<size_t>(ftot_) * 4 * kJac);
        adj_face_ = alloc<double>(static_cast<size_t>(ftot_) * kJac);
        mw_ = alloc<d4>(ntot_);
        mgx_ = alloc<d4>(ntot_);
        mgy_ = alloc<d4>(ntot_);
        adj_r_ = alloc<d4>(ntot_);
        adj_g_ = alloc<d4>(ntot_);
        lam_ = alloc<d4>(ntot_);
        lam_n_ = alloc<d4>(ntot_);
        adj_v_ = alloc<d4>(ntot_);
        adj_rn_ = alloc<double>(ncb_);
        adj_hist_ = alloc<double>(kAdjHist);
        adj_counter_ = alloc<int>(1);
        adj_face_out_ = alloc<double>(ftot_);
        ctrl_lin_ = alloc<Ctrl>(1);
        adj_alloc_ = true;
        if (err_ != cudaSuccess) return AERO_ERR_NOMEM;
      }
      // the linearisation point: the current state, its primitives, gradients and residual
      download_ctrls();
      Ctrl lin = host_ctrls_[0];
      lin.done = 0;
      lin.nonfinite = 0;
      AERO_CK(cudaMemcpyAsync(ctrl_lin_, &lin, sizeof(Ctrl), cudaMemcpyHostToDevice, st_));
      adj_second_ = second_order < 0 ? second_at(lin.iter) : second_order != 0;
      adj_wcd_ = w_cd;
      adj_wcl_ = w_cl;
      if (adj_graph_) {  // the transpose product's launches depend on the order
        cudaGraphExecDestroy(adj_graph_);
        adj_graph_ = nullptr;
      }
      if (kr_graph_) {
        cudaGraphExecDestroy(kr_graph_);
        kr_graph_ = nullptr;
      }
      const Cases<T> ccs{cblk_, ctrl_lin_, fps_dev_, pcs_dev_, mcs_dev_};
      const Cases<T> fcs{fblk_, ctrl_lin_, fps_dev_, pcs_dev_, mcs_dev_};
      refresh();
      if (adj_second_) k_gradient<T><<<ncb_, block_, 0, st_>>>(dm_, W_, gx_, gy_, ccs);
      ResidualLaunch<T> a = residual_args(&ctrl_eval_->fo_fallback, R_, SR_, 0);
      a.cell_cases = ccs;
      a.face_cases = fcs;
      launch_residual_passes(a, cfg_[0].flux, adj_second_, lm_ != 0, false);
      AERO_CK(cudaMemcpyAsync(Ulin_, Un_, sizeof(d4) * ntot_, cudaMemcpyDeviceToDevice, st_));
      AERO_CK(cudaMemcpyAsync(Wlin_, W_, sizeof(d4) * ntot_, cudaMemcpyDeviceToDevice, st_));
      AERO_CK(cudaMemcpyAsync(SRlin_, SR_, sizeof(double) * ntot_, cudaMemcpyDeviceToDevice, st_));
      if (adj_second_) {
        AERO_CK(cudaMemcpyAsync(gxlin_, gx_, sizeof(d4) * ntot_, cudaMemcpyDeviceToDevice, st_));
        AERO_CK(cudaMemcpyAsync(gylin_, gy_, sizeof(d4) * ntot_, cudaMemcpyDeviceToDevice, st_));
      }
      launch_face_jac();
      w_valid_ = false;
      // objective gradient dJ/dU: J is linear in the gauge force, J = (ex Fx + ey Fy) / (q S)
      const CtrlConfig& cc = ccs_[0];
      const double ex = w_cd * cc.cos_a - w_cl * cc.sin_a;
      const double ey = w_cd * cc.sin_a + w_cl * cc.cos_a;
      adj_ex_ = ex;
      adj_ey_ = ey;
      k_adj_objective<<<ncb_, block_, 0, st_>>>(cblk_, Ulin_, rs_[0].gamma, ms_, ex, ey,
                                                1.0 / (cc.q_inf * cc.s_ref), adj_g_);
      AERO_CK(cudaMemsetAsync(lam_, 0, sizeof(d4) * ntot_, st_));
      AERO_CK(cudaGetLastError());
      AERO_CK(cudaStreamSynchronize(st_));
      adj_ready_ = err_ == cudaSuccess;
      return adj_ready_ ? AERO_OK : AERO_ERR_CUDA;
    }
  }

  int adjoint_vjp(const double* v, double* out) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (!adj_ready_) return AERO_ERR_INVALID;
      upload_cells(v, adj_v_);
      apply_vjp(adj_v_, adj_r_);
      download_cells(adj_r_, out);
      return err_ == cudaSuccess ? AERO_OK : AERO_ERR_CUDA;
    }
  }

  int adjoint_objective_gradient(double* g) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (!adj_ready_) return AERO_ERR_INVALID;
      download_cells(adj_g_, g);
      return err_ == cudaSuccess ? AERO_OK : AERO_ERR_CUDA;
    }
  }

  // Pseudo-time solve of (dR/dU)^T lam = -dJ/dU with the primal's SSP-RK3 and local steps,
  // continuing from the current lam: one captured graph per iteration (copy of lam, three
  // transpose products and stages, the residual norm into a device history), launched in
  // chunks with one host synchronisation per chunk. history[k]: RMS over cells of
  // (dR/dU)^T lam + dJ/dU at the start of iteration k.
  int adjoint_solve(int iters, double cfl, double* history) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (!adj_ready_ || iters < 0 || !(cfl > 0.0)) return AERO_ERR_INVALID;
      if (adj_graph_ && adj_graph_cfl_ != cfl) {
        cudaGraphExecDestroy(adj_graph_);
        adj_graph_ = nullptr;
      }
      if (!adj_graph_) {
        cudaGraph_t g = nullptr;
        AERO_CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        adjoint_iteration(cfl);
        AERO_CK(cudaStreamEndCapture(st_, &g));
        if (g) {
          AERO_CK(cudaGraphInstantiate(&adj_graph_, g, 0));
          cudaGraphDestroy(g);
        }
        if (!adj_graph_) return AERO_ERR_CUDA;
        adj_graph_cfl_ = cfl;
      }
      std::vector<double> h(static_cast<size_t>(kAdjHist));
      for (int done = 0; done < iters;) {
        const int n = std::min(kAdjHist, iters - done);
        AERO_CK(cudaMemsetAsync(adj_counter_, 0, sizeof(int), st_));
        for (int i = 0; i < n; ++i) AERO_CK(cudaGraphLaunch(adj_graph_, st_));
        AERO_CK(cudaMemcpyAsync(h.data(), adj_hist_, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
        AERO_CK(cudaStreamSynchronize(st_));
        if (err_ != cudaSuccess) break;
        if (history) std::copy(h.begin(), h.begin() + n, history + done);
        done += n;
      }
      return err_ == cudaSuccess ? AERO_OK : AERO_ERR_CUDA;
    }
  }

  int adjoint_lambda(double* lam) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (!adj_ready_) return AERO_ERR_INVALID;
      download_cells(lam_, lam);
      return err_ == cudaSuccess ? AERO_OK : AERO_ERR_CUDA;
    }
  }

  // dJ/d(alpha) per degree at the linearisation point: the explicit term of the force
  // rotation plus lam^T dR/d(alpha) through the far-field state.
  int adjoint_dalpha(double* out) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (!adj_ready_ || out == nullptr) return AERO_ERR_INVALID;
      const CtrlConfig& cc = ccs_[0];
      const Resolved& rs = rs_[0];
      const double rad = 3.14159265358979323846 / 180.0;
      const double rho = rs.cons_inf[0], vmag = rs.v_inf;
      const d4 dfar{0.0, -rho * vmag * cc.sin_a * rad, rho * vmag * cc.cos_a * rad, 0.0};
      const int grid = nfb_;
      if (cfg_[0].flux == AERO_FLUX_HLLC) {
        if (lm_) {
          k_adj_dalpha<1, true><<<grid, block_, 0, st_>>>(df_, fblk_, fps_dev_, ctrl_lin_, W_lin(), dfar, lam_, adj_face_out_);
        } else {
          k_adj_dalpha<1, false><<<grid, block_, 0, st_>>>(df_, fblk_, fps_dev_, ctrl_lin_, W_lin(), dfar, lam_, adj_face_out_);
        }
      } else {
        if (lm_) {
          k_adj_dalpha<0, true><<<grid, block_, 0, st_>>>(df_, fblk_, fps_dev_, ctrl_lin_, W_lin(), dfar, lam_, adj_face_out_);
        } else {
          k_adj_dalpha<0, false><<<grid, block_, 0, st_>>>(df_, fblk_, fps_dev_, ctrl_lin_, W_lin(), dfar, lam_, adj_face_out_);
        }
      }
      std::vector<double> per_face(static_cast<size_t>(ftot_));
      AERO_CK(cudaMemcpyAsync(per_face.data(), adj_face_out_, sizeof(double) * ftot_, cudaMemcpyDeviceToHost, st_));
      AERO_CK(cudaStreamSynchronize(st_));
      double lam_dr = 0.0;
      for (int i = 0; i < pk_[0].nf; ++i) lam_dr += per_face[i];
      // explicit term from the gauge force at the state
      double fx = 0.0, fy = 0.0;
      const std::vector<double> pw = wall_pressures();
      const HostSlots& hs = hs_[0];
      for (int c = 0; c < pk_[0].n; ++c) {
        const int cnt = hs.flags[c] >> 2;
        for (int j = hs.wall_first[c]; j < hs.wall_first[c] + cnt; ++j) {
          if (!(hs.wkind[j] & 1)) continue;
          fx += (pw[c] - rs.p_inf) * hs.wnx[j] * hs.warea[j];
          fy += (pw[c] - rs.p_inf) * hs.wny[j] * hs.warea[j];
        }
      }
      const double qs = cc.q_inf * cc.s_ref;
      // dCD/d(alpha) = CL and dCL/d(alpha) = -CD per radian at a fixed force
      const double explicit_term = (adj_wcd_ * (-fx * cc.sin_a + fy * cc.cos_a) +
                                    adj_wcl_ * (-fx * cc.cos_a - fy * cc.sin_a)) / qs;
      *out = explicit_term * rad + lam_dr;
      return err_ == cudaSuccess ? AERO_OK : AERO_ERR_CUDA;
    }
  }

  // dJ/dX . dX for a geometry tangent (same connectivity as the mesh): the force term at
  // fixed state plus lam^T (dR/dX . dX) through the gradients, MUSCL offsets, normals and
  // lengths.
  int adjoint_geometry(const aero_mesh_desc& t, double* dj) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (!adj_ready_ || dj == nullptr) return AERO_ERR_INVALID;
      const HostSlots& hs = hs_[0];
      const Pack& pk = pk_[0];
      if (t.num_cells != hs.n || t.num_faces != hs.nf || !t.face_normal || !t.face_center || !t.face_area ||
          !t.cell_volume || !t.cell_center)
        return AERO_ERR_INVALID;
      HostSlots g;
      map_geometry(t, hs, &g);
      const size_t ns = static_cast<size_t>(ntot_) * d_;
      std::vector<double2> dnrm(ns, make_double2(0.0, 0.0));
      std::vector<double> darea(ns, 0.0), dinv(static_cast<size_t>(ntot_), 0.0);
      for (int j = 0; j < hs.d; ++j) {
        for (int c = 0; c < hs.n; ++c) {
          const size_t src = static_cast<size_t>(j) * hs.n + c, dst = static_cast<size_t>(j) * ntot_ + c;
          dnrm[dst] = make_double2(g.nx[src], g.ny[src]);
          darea[dst] = g.area[src];
        }
      }
      for (int c = 0; c < hs.n; ++c) {
        const double v = hs.vol[c];
        dinv[c] = v > 1.0e-12 ? -g.vol[c] / (v * v) : 0.0;  // inv_vol = 1 / max(V, 1e-12)
      }
      std::vector<double2> dfn(static_cast<size_t>(ftot_), make_double2(0.0, 0.0)), ddoff(dfn), dnoff(dfn);
      std::vector<double> dfa(static_cast<size_t>(ftot_), 0.0);
      for (int i = 0; i < pk.nf; ++i) {
        const int o = hs.f_own_old[i], b = hs.f_nb_old[i];
        dfn[i] = make_double2(g.f_nx[i], g.f_ny[i]);
        dfa[i] = g.f_area[i];
        ddoff[i] = make_double2(g.f_cx[i] - g.ccx[o], g.f_cy[i] - g.ccy[o]);
        if (hs.f_nb[i] >= 0) dnoff[i] = make_double2(g.f_cx[i] - g.ccx[b], g.f_cy[i] - g.ccy[b]);
      }
      if (!geo_alloc_) {
        geo_nrm_ = alloc<double2>(ns);
        geo_area_ = alloc<double>(ns);
        geo_inv_ = alloc<double>(ntot_);
        geo_fn_ = alloc<double2>(ftot_);
        geo_fa_ = alloc<double>(ftot_);
        geo_doff_ = alloc<double2>(ftot_);
        geo_noff_ = alloc<double2>(ftot_);
        geo_gx_ = alloc<d4>(ntot_);
        geo_gy_ = alloc<d4>(ntot_);
        geo_alloc_ = true;
        if (err_ != cudaSuccess) return AERO_ERR_NOMEM;
      }
      AERO_CK(cudaMemcpyAsync(geo_nrm_, dnrm.data(), sizeof(double2) * ns, cudaMemcpyHostToDevice, st_));
      AERO_CK(cudaMemcpyAsync(geo_area_, darea.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, st_));
      AERO_CK(cudaMemcpyAsync(geo_inv_, dinv.data(), sizeof(double) * ntot_, cudaMemcpyHostToDevice, st_));
      AERO_CK(cudaMemcpyAsync(geo_fn_, dfn.data(), sizeof(double2) * ftot_, cudaMemcpyHostToDevice, st_));
      AERO_CK(cudaMemcpyAsync(geo_fa_, dfa.data(), sizeof(double) * ftot_, cudaMemcpyHostToDevice, st_));
      AERO_CK(cudaMemcpyAsync(geo_doff_, ddoff.data(), sizeof(double2) * ftot_, cudaMemcpyHostToDevice, st_));
      AERO_CK(cudaMemcpyAsync(geo_noff_, dnoff.data(), sizeof(double2) * ftot_, cudaMemcpyHostToDevice, st_));
      if (adj_second_) {
        k_adj_geo_grad<<<ncb_, block_, 0, st_>>>(dm_, geo_nrm_, geo_area_, geo_inv_, cblk_, Wlin_, geo_gx_, geo_gy_);
      }
      auto go = [&](auto kern) {
        kern<<<nfb_, block_, 0, st_>>>(df_, geo_fn_, geo_fa_, geo_doff_, geo_noff_, fblk_, fps_dev_, ctrl_lin_, Wlin_,
                                       gxlin_, gylin_, geo_gx_, geo_gy_, lam_, adj_face_out_);
      };
      const bool hllc = cfg_[0].flux == AERO_FLUX_HLLC, lm = lm_ != 0, sec = adj_second_;
      if (hllc) {
        if (sec) {
          if (lm) go(k_adj_geo_face<1, true, true>);
          else go(k_adj_geo_face<1, true, false>);
        } else {
          if (lm) go(k_adj_geo_face<1, false, true>);
          else go(k_adj_geo_face<1, false, false>);
        }
      } else {
        if (sec) {
          if (lm) go(k_adj_geo_face<0, true, true>);
          else go(k_adj_geo_face<0, true, false>);
        } else {
          if (lm) go(k_adj_geo_face<0, false, true>);
          else go(k_adj_geo_face<0, false, false>);
        }
      }
      AERO_CK(cudaGetLastError());
      std::vector<double> per_face(static_cast<size_t>(pk.nf));
      AERO_CK(cudaMemcpyAsync(per_face.data(), adj_face_out_, sizeof(double) * pk.nf, cudaMemcpyDeviceToHost, st_));
      AERO_CK(cudaStreamSynchronize(st_));
      double lam_dr = 0.0;
      for (double v : per_face) lam_dr += v;
      // the objective's own dependence: the force patch's normals and lengths
      const std::vector<double> pw = wall_pressures();
      const double pinf = rs_[0].p_inf;
      double s = 0.0;
      for (int c = 0; c < pk.n; ++c) {
        const int cnt = hs.flags[c] >> 2;
        for (int j = hs.wall_first[c]; j < hs.wall_first[c] + cnt; ++j) {
          if (!(hs.wkind[j] & 1)) continue;
          const double dnax = g.wnx[j] * hs.warea[j] + hs.wnx[j] * g.warea[j];
          const double dnay = g.wny[j] * hs.warea[j] + hs.wny[j] * g.warea[j];
          s += (pw[c] - pinf) * (adj_ex_ * dnax + adj_ey_ * dnay);
        }
      }
      const CtrlConfig& cc = ccs_[0];
      *dj = s / (cc.q_inf * cc.s_ref) + lam_dr;
      return err_ == cudaSuccess ? AERO_OK : AERO_ERR_CUDA;
    }
  }

  // Transpose of adjoint_geometry with the current lam: dJ/d(geometry) for every face normal
  // [3F], face centre [3F], face length [F], cell volume [N] and cell centre [3N] of the
  // original numbering (z components 0), so that for every geometry tangent t,
  // adjoint_geometry(t) = sum of these times t.
  int adjoint_geometry_vjp(double* bn, double* bc, double* ba, double* bv, double* bcc) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (!adj_ready_ || !bn || !bc || !ba || !bv || !bcc) return AERO_ERR_INVALID;
      const HostSlots& hs = hs_[0];
      const Pack& pk = pk_[0];
      std::fill(bn, bn + 3 * static_cast<size_t>(hs.nf), 0.0);
      std::fill(bc, bc + 3 * static_cast<size_t>(hs.nf), 0.0);
      std::fill(ba, ba + hs.nf, 0.0);
      std::fill(bv, bv + hs.n, 0.0);
      std::fill(bcc, bcc + 3 * static_cast<size_t>(hs.n), 0.0);
      const size_t ns = static_cast<size_t>(ntot_) * d_;
      if (!geo_vjp_alloc_) {
        geo_face_vjp_ = alloc<double>(7 * static_cast<size_t>(ftot_));
        geo_slot_vjp_ = alloc<double>(3 * ns);
        geo_inv_vjp_ = alloc<double>(ntot_);
        geo_vjp_alloc_ = true;
        if (err_ != cudaSuccess) return AERO_ERR_NOMEM;
      }
      const bool sec = adj_second_;
      if (sec) {  // the gradients' adjoint under lam, then its geometric part
        k_adj_face_vjp<kJac><<<nfb_, block_, 0, st_>>>(df_, fblk_, Jf_, lam_, adj_face_);
        k_adj_gather<kJac><<<ncb_, block_, 0, st_>>>(dg_, cblk_, adj_face_, mw_, mgx_, mgy_);
        AERO_CK(cudaMemsetAsync(geo_slot_vjp_, 0, sizeof(double) * 3 * ns, st_));
        k_adj_geo_grad_vjp<<<ncb_, block_, 0, st_>>>(dm_, cblk_, Wlin_, mgx_, mgy_, geo_slot_vjp_, geo_inv_vjp_);
      }
      auto go = [&](auto kern) {
        kern<<<nfb_, block_, 0, st_>>>(df_, fblk_, fps_dev_, ctrl_lin_, Wlin_, gxlin_, gylin_, lam_, geo_face_vjp_);
      };
      const bool hllc = cfg_[0].flux == AERO_FLUX_HLLC, lm = lm_ != 0;
      if (hllc) {
        if (sec) {
          if (lm) go(k_adj_geo_face_vjp<1, true, true>);
          else go(k_adj_geo_face_vjp<1, true, false>);
        } else {
          if (lm) go(k_adj_geo_face_vjp<1, false, true>);
          else go(k_adj_geo_face_vjp<1, false, false>);
        }
      } else {
        if (sec) {
          if (lm) go(k_adj_geo_face_vjp<0, true, true>);
          else go(k_adj_geo_face_vjp<0, true, false>);
        } else {
          if (lm) go(k_adj_geo_face_vjp<0, false, true>);
          else go(k_adj_geo_face_vjp<0, false, false>);
        }
      }
      AERO_CK(cudaGetLastError());
      std::vector<double> fv(7 * static_cast<size_t>(pk.nf)), sv, iv;
      AERO_CK(cudaMemcpyAsync(fv.data(), geo_face_vjp_, sizeof(double) * fv.size(), cudaMemcpyDeviceToHost, st_));
      if (sec) {
        sv.resize(3 * ns);
        iv.resize(static_cast<size_t>(ntot_));
        AERO_CK(cudaMemcpyAsync(sv.data(), geo_slot_vjp_, sizeof(double) * sv.size(), cudaMemcpyDeviceToHost, st_));
        AERO_CK(cudaMemcpyAsync(iv.data(), geo_inv_vjp_, sizeof(double) * iv.size(), cudaMemcpyDeviceToHost, st_));
      }
      AERO_CK(cudaStreamSynchronize(st_));
      if (err_ != cudaSuccess) return AERO_ERR_CUDA;
      // face pass: normal, length, and the MUSCL offsets dO = c_f - c_owner, dN = c_f - c_nb
      for (int i = 0; i < pk.nf; ++i) {
        const double* r = fv.data() + 7 * static_cast<size_t>(i);
        const int f = hs.f_orig[i];
        bn[3 * f] += r[0];
        bn[3 * f + 1] += r[1];
        ba[f] += r[2];
        if (sec && hs.f_nb[i] >= 0) {
          const int o = hs.f_own_old[i], b = hs.f_nb_old[i];
          bc[3 * f] += r[3] + r[5];
          bc[3 * f + 1] += r[4] + r[6];
          bcc[3 * o] -= r[3];
          bcc[3 * o + 1] -= r[4];
          bcc[3 * b] -= r[5];
          bcc[3 * b + 1] -= r[6];
        }
      }
      if (sec) {  // gradient pass: slot normals and lengths are the faces'; 1/V = 1/max(V, 1e-12)
        for (int j = 0; j < hs.d; ++j) {
          for (int c = 0; c < hs.n; ++c) {
            const int f = hs.slot_face[static_cast<size_t>(j) * hs.n + c];
            if (f < 0) continue;
            const double* r = sv.data() + 3 * (static_cast<size_t>(j) * ntot_ + c);
            bn[3 * f] += r[0];
            bn[3 * f + 1] += r[1];
            ba[f] += r[2];
          }
        }
        for (int c = 0; c < hs.n; ++c) {
          const double v = hs.vol[c];
          if (v > 1.0e-12) bv[hs.perm[c]] += -iv[c] / (v * v);
        }
      }
      // the objective's own dependence on the force patch's normals and lengths
      const std::vector<double> pw = wall_pressures();
      const double pinf = rs_[0].p_inf;
      const CtrlConfig& cc = ccs_[0];
      const double scale = 1.0 / (cc.q_inf * cc.s_ref);
      for (int c = 0; c < pk.n; ++c) {
        const int cnt = hs.flags[c] >> 2;
        for (int j = hs.wall_first[c]; j < hs.wall_first[c] + cnt; ++j) {
          if (!(hs.wkind[j] & 1)) continue;
          const int f = hs.w_face[j];
          const double coef = (pw[c] - pinf) * scale;
          bn[3 * f] += coef * adj_ex_ * hs.warea[j];
          bn[3 * f + 1] += coef * adj_ey_ * hs.warea[j];
          ba[f] += coef * (adj_ex_ * hs.wnx[j] + adj_ey_ * hs.wny[j]);
        }
      }
      return AERO_OK;
    }
  }

  // info[0] cells, [1] faces, [2] slots per cell, [3] launches per iteration, [4] device
  // bytes, [5] precision, [6] block size, [7] cell blocks, [8] cases
  void info(long long* out, int n) override {
    long long v[10] = {ncells_, nfaces_, d_, launches_per_iteration(true), static_cast<long long>(bytes_),
                       sizeof(T) == 4 ? AERO_PRECISION_FP32 : AERO_PRECISION_FP64, block_, ncb_, K_,
                       grad_tma_ ? 1 : 0};
    for (int i = 0; i < n && i < 10; ++i) out[i] = v[i];
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
    if (p && !v.empty()) AERO_CK(cudaMemcpyAsync(p, v.data(), sizeof(U) * v.size(), cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    return p;
  }

  // Per-case constants: face parameters, preconditioner, monitors, controller.
  void setup_case(int k) {
    const aero_case_desc& cfg = cfg_[k];
    const Resolved& rs = rs_[k];
    const Pack& p = pk_[k];
    FaceParams<T>& fp = fps_[k];
    fp.gamma = T(rs.gamma);
    fp.inv_gm1 = T(1.0 / (rs.gamma - 1.0));
    fp.farfield = Cons<T>{T(rs.cons_inf[0]), T(rs.cons_inf[1]), T(rs.cons_inf[2]), T(rs.cons_inf[3])};
    fp.limiter = cfg.limiter;
    fp.precond = cfg.precond_on;
    fp.low_mach_fix = cfg.low_mach_fix;
    fp.precond_farfield_bc = cfg.precond_farfield_bc;
    fp.as_fix = 0;
    fp.mach_cutoff = T(cfg.mach_cutoff);
    fp.pc_mach_ref = T(rs.pc_mach_ref);
    fp.pc_mach_min = T(rs.pc_mach_min);
    fp.pc_beta_min = T(rs.pc_beta_min);
    fp.pc_beta_max = T(rs.pc_beta_max);
    fp.stab_floor = T(0);
    fp.as_cutoff = T(cfg.all_speed_mach_cutoff);
    fp.as_fmin = T(rs.as_fmin);
    fp.as_ramp = T(1);

    PrecondD& pc = pcs_[k];
    pc.enabled = cfg.precond_on;
    // energy row of FP32 contexts: -1 float, 1 IEEE double, 2 double-float, 0 double-float
    // below Mach 0.1 and float above
    pc.fp64 = cfg.precond_fp64 == 1 ? 1
              : (cfg.precond_fp64 == 2 || (cfg.precond_fp64 == 0 && cfg.mach < 0.1)) ? 2 : 0;
    pc.gamma = rs.gamma;
    pc.mach_ref = double(fp.pc_mach_ref);
    pc.mach_min = double(fp.pc_mach_min);
    pc.beta_min = double(fp.pc_beta_min);
    pc.beta_max = double(fp.pc_beta_max);
    pc.gamma_f = float(rs.gamma);
    pc.gm1_f = float(rs.gamma - 1.0);
    pc.pfe = Kn<double>::p_floor / (rs.gamma - 1.0);
    pc.mach_ref_f = float(pc.mach_ref);
    pc.mach_min_f = float(pc.mach_min);
    pc.beta_min_f = float(pc.beta_min);
    pc.beta_max_f = float(pc.beta_max);

    MonitorConsts& mc = mcs_[k];
    mc.p_inf = rs.p_inf;
    mc.rho_inf = rs.rho_inf;
    mc.u_inf = rs.v_inf * rs.cos_a;
    mc.v_inf = rs.v_inf * rs.sin_a;
    mc.q_inf = rs.q_inf;
    mc.x_ref = cfg.x_ref;
    mc.y_ref = cfg.y_ref;
    mc.gamma = rs.gamma;
    mc.p_inf_f = float(mc.p_inf);
    mc.rho_inf_f = float(mc.rho_inf);
    mc.u_inf_f = float(mc.u_inf);
    mc.v_inf_f = float(mc.v_inf);
    mc.q_inf_f = float(mc.q_inf);
    mc.x_ref_f = float(mc.x_ref);
    mc.y_ref_f = float(mc.y_ref);
    const bool sym = cfg.aoa0_symmetry_enforce && cfg.aoa0_symmetry_enforce_interval > 0 &&
                     !(std::fabs(cfg.aoa_deg) > 1.0e-12);
    mc.sym_interval = sym ? cfg.aoa0_symmetry_enforce_interval : 0;

    CtrlConfig& c = ccs_[k];
    std::memset(&c, 0, sizeof(c));
    c.n_cells = p.n;
    c.n_wall = hs_[k].n_slip;
    c.n_wall_blocks = p.nws;
    c.wall_base = p.ws0;
    c.block_base = p.cb0;
    c.n_blocks = p.ncb;
    c.bulk_f32 = sizeof(T) == 4 ? 1 : 0;
    c.rk_stages = cfg.rk_stages;
    c.local_dt = cfg.local_time_stepping;
    c.cfl_ramp = cfg.cfl_ramp_iters;
    c.stab_ramp = std::max(cfg.stab_ramp_iters, 0);
    c.as_ramp_start = std::max(cfg.all_speed_ramp_start_iter, 0);
    c.as_ramp_iters = std::max(cfg.all_speed_ramp_iters, 0);
    c.startup_first_order = cfg.startup_first_order_iters;
    c.min_iterations = cfg.min_iterations;
    c.window = std::min(std::max(cfg.force_stability_window, 1), kMaxForceWindow);
    c.staged = cfg.all_speed_staged_controller;
    c.st_a_min = std::max(cfg.all_speed_stage_a_min_iters, 0);
    c.st_a_max = std::max(cfg.all_speed_stage_a_max_iters, 0);
    c.pj_hold = std::max(cfg.all_speed_pjump_hold_iters, 1);
    c.freeze_iters = std::max(cfg.all_speed_freeze_iters, 0);
    c.as_fix_cfg = cfg.all_speed_flux_fix;
    c.pjump_blocks = (cfg.all_speed_staged_controller || cfg.diagnostics) ? p.ncb : 0;
    c.cfl_start = cfg.cfl_start;
    c.cfl_max = cfg.cfl_max;
    c.stab_start = rs.stab_start;
    c.stab_target = rs.stab_target;
    c.as_fmin = rs.as_fmin;
    c.residual_target = cfg.residual_reduction_target;
    c.stab_tol = cfg.force_stability_tol;
    c.drift_tol = cfg.force_mean_drift_tol > 0.0 ? cfg.force_mean_drift_tol : cfg.force_stability_tol;
    c.st_fmin_high = rs.st_fmin_high;
    c.st_fmin_mid = rs.st_fmin_mid;
    c.st_fmin_low = rs.st_fmin_low;
    c.pj_target = rs.pj_target;
    c.pj_spike = rs.pj_spike;
    c.cfl_drop = rs.cfl_drop;
    c.cfl_restore = rs.cfl_restore;
    c.cfl_min_scale = rs.cfl_min_scale;
    c.p_inf = rs.p_inf;
    c.q_inf = rs.q_inf;
    c.chord = std::max(cfg.chord, 1.0e-8);
    c.s_ref = c.chord * 1.0;
    c.cos_a = rs.cos_a;
    c.sin_a = rs.sin_a;
    c.x_ref = cfg.x_ref;
    c.y_ref = cfg.y_ref;
    c.pressure_ref = rs.pressure_ref;
    c.gamma = rs.gamma;
    c.rho_inf = rs.rho_inf;
    c.u_inf = rs.v_inf * rs.cos_a;
    c.v_inf = rs.v_inf * rs.sin_a;
    c.rho_l2_target = cfg.density_l2_target;
  }

  // ---- adjoint helpers (FP64)
  const d4* W_lin() const { return Wlin_; }

  void launch_face_jac() {
    if constexpr (sizeof(T) == 8) {
      const int grid = nfb_;
      auto go = [&](auto kern) {
        kern<<<grid, block_, 0, st_>>>(df_, fblk_, fps_dev_, ctrl_lin_, W_lin(),
                                                    reinterpret_cast<const d4*>(gx_), reinterpret_cast<const d4*>(gy_), Jf_);
      };
      const bool hllc = cfg_[0].flux == AERO_FLUX_HLLC, lm = lm_ != 0, sec = adj_second_;
      if (hllc) {
        if (sec) {
          if (lm) go(k_adj_face_jac<1, true, true>);
          else go(k_adj_face_jac<1, true, false>);
        } else {
          if (lm) go(k_adj_face_jac<1, false, true>);
          else go(k_adj_face_jac<1, false, false>);
        }
      } else {
        if (sec) {
          if (lm) go(k_adj_face_jac<0, true, true>);
          else go(k_adj_face_jac<0, true, false>);
        } else {
          if (lm) go(k_adj_face_jac<0, false, true>);
          else go(k_adj_face_jac<0, false, false>);
        }
      }
      AERO_CK(cudaGetLastError());
    }
  }

  static constexpr int kAdjHist = 4096;  // iterations per host synchronisation

  // One RK3 iteration of z toward (dR/dU)^T z + src = 0 (zn: the iteration's start copy);
  // with_norm: the RMS of (dR/dU)^T z + src at its start into the device history.
  void adjoint_iteration(double cfl, d4* z, d4* zn, const d4* src, bool with_norm) {
    if constexpr (sizeof(T) == 8) {
      AERO_CK(cudaMemcpyAsync(zn, z, sizeof(d4) * ntot_, cudaMemcpyDeviceToDevice, st_));
      for (int stage = 0; stage < 3; ++stage) {
        apply_vjp(z, adj_r_);
        const bool nrm = with_norm && stage == 0;
        k_adj_stage<<<ncb_, block_, 0, st_>>>(cblk_, stage, cfl, SRlin_, adj_r_, src, zn, z, nrm ? adj_rn_ : nullptr);
        if (nrm) k_adj_norm<<<1, 256, 0, st_>>>(adj_rn_, ncb_, pk_[0].n, adj_hist_, adj_counter_, kAdjHist);
      }
    }
  }
  void adjoint_iteration(double cfl) { adjoint_iteration(cfl, lam_, lam_n_, adj_g_, true); }

  // ---- restarted GMRES on (dR/dU)^T lam = -dJ/dU, right-preconditioned by `smooth`
  // iterations of the RK3 smoother from zero (a fixed linear operator P). The smoother alone
  // diverges where the primal's own iteration has not settled (limit cycles of the limiters
  // leave a few growing modes); the Krylov outer iteration removes them.
  int vlen() const { return pk_[0].n; }
  int vgrid() const { return (vlen() + 255) / 256; }

  // host copies of V_r . w for r < rows (two-stage deterministic reduction)
  void vdots(const d4* V, int rows, const d4* w, double* out) {
    const int nb = vgrid();
    k_vdot_rows<<<dim3(nb, rows), 256, 0, st_>>>(V, static_cast<size_t>(ntot_), w, vlen(), kr_part_);
    k_rows_sum<<<rows, 256, 0, st_>>>(kr_part_, nb, kr_out_);
    AERO_CK(cudaMemcpyAsync(out, kr_out_, sizeof(double) * rows, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
  }
  double vnorm(const d4* w) {
    double s = 0.0;
    vdots(w, 1, w, &s);
    return std::sqrt(s);
  }
  // w = alpha w + sum coef[r] V_r
  void vcombine(d4* w, double alpha, const d4* V, const double* coef, int rows) {
    AERO_CK(cudaMemcpyAsync(kr_coef_, coef, sizeof(double) * rows, cudaMemcpyHostToDevice, st_));
    k_vcombine<<<vgrid(), 256, 0, st_>>>(w, alpha, V, static_cast<size_t>(ntot_), kr_coef_, rows, vlen());
  }
  // z = P x: `smooth` smoother iterations on (dR/dU)^T z = x from z = 0, as one graph
  // (smooth = 0: P = identity)
  void precondition(const d4* x, double cfl, int smooth) {
    if (smooth == 0) {
      k_vaxpby<<<vgrid(), 256, 0, st_>>>(1.0, x, 0.0, kr_z_, vlen());
      return;
    }
    if (kr_graph_ && (kr_graph_cfl_ != cfl || kr_graph_smooth_ != smooth)) {
      cudaGraphExecDestroy(kr_graph_);
      kr_graph_ = nullptr;
    }
    k_vaxpby<<<vgrid(), 256, 0, st_>>>(-1.0, x, 0.0, kr_src_, vlen());
    if (!kr_graph_) {
      cudaGraph_t g = nullptr;
      AERO_CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
      AERO_CK(cudaMemsetAsync(kr_z_, 0, sizeof(d4) * ntot_, st_));
      for (int i = 0; i < smooth; ++i) adjoint_iteration(cfl, kr_z_, kr_zn_, kr_src_, false);
      AERO_CK(cudaStreamEndCapture(st_, &g));
      if (g) {
        AERO_CK(cudaGraphInstantiate(&kr_graph_, g, 0));
        cudaGraphDestroy(g);
      }
      kr_graph_cfl_ = cfl;
      kr_graph_smooth_ = smooth;
    }
    if (kr_graph_) AERO_CK(cudaGraphLaunch(kr_graph_, st_));
  }

 public:
  int adjoint_set_lambda(const double* lam) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (!adj_ready_) return AERO_ERR_INVALID;
      upload_cells(lam, lam_);
      return err_ == cudaSuccess ? AERO_OK : AERO_ERR_CUDA;
    }
  }

  int adjoint_solve_krylov(int max_iters, int restart, int smooth, double cfl, double rtol, double* history,
                           int* done_out) override {
    if constexpr (sizeof(T) != 8) {
      return AERO_ERR_INVALID;
    } else {
      if (!adj_ready_ || max_iters < 0 || restart < 1 || restart > 512 || smooth < 0 || !(cfl > 0.0) ||
          !(rtol >= 0.0))
        return AERO_ERR_INVALID;
      const int m = restart;
      if (kr_m_ < m) {  // Krylov basis and work vectors (kept for later solves)
        kr_V_ = alloc<d4>(static_cast<size_t>(m + 1) * ntot_);
        kr_m_ = m;
        if (!kr_w_) {
          kr_w_ = alloc<d4>(ntot_);
          kr_z_ = alloc<d4>(ntot_);
          kr_zn_ = alloc<d4>(ntot_);
          kr_src_ = alloc<d4>(ntot_);
        }
        kr_part_ = alloc<double>(static_cast<size_t>(m + 1) * vgrid());
        kr_out_ = alloc<double>(m + 1);
        kr_coef_ = alloc<double>(m + 1);
        if (kr_graph_) {
          cudaGraphExecDestroy(kr_graph_);
          kr_graph_ = nullptr;
        }
        if (err_ != cudaSuccess) return AERO_ERR_NOMEM;
      }
      auto Vr = [&](int r) { return kr_V_ + static_cast<size_t>(r) * ntot_; };
      // b = -g
      k_vaxpby<<<vgrid(), 256, 0, st_>>>(-1.0, adj_g_, 0.0, kr_w_, vlen());
      const double bnorm = vnorm(kr_w_);
      int done = 0;
      std::vector<double> H(static_cast<size_t>(m + 1) * m), cs(m), sn(m), gv(m + 1), h(m + 1), h2(m + 1), y(m);
      while (err_ == cudaSuccess) {
        // r = b - A^T lam
        apply_vjp(lam_, kr_w_);
        k_vaxpby<<<vgrid(), 256, 0, st_>>>(-1.0, adj_g_, -1.0, kr_w_, vlen());
        const double beta = vnorm(kr_w_);
        if (!(beta > rtol * bnorm) || done >= max_iters || !std::isfinite(beta)) {
          if (history && done < max_iters && done == 0) history[0] = bnorm > 0.0 ? beta / bnorm : 0.0;
          break;
        }
        k_vaxpby<<<vgrid(), 256, 0, st_>>>(1.0 / beta, kr_w_, 0.0, Vr(0), vlen());
        std::fill(gv.begin(), gv.end(), 0.0);
        gv[0] = beta;
        int j = 0;
        bool stop = false;
        for (; j < m && done < max_iters; ++j) {
          precondition(Vr(j), cfl, smooth);
          apply_vjp(kr_z_, kr_w_);
          // classical Gram-Schmidt, twice
          vdots(Vr(0), j + 1, kr_w_, h.data());
          for (int i = 0; i <= j; ++i) h2[i] = -h[i];
          vcombine(kr_w_, 1.0, Vr(0), h2.data(), j + 1);
          vdots(Vr(0), j + 1, kr_w_, h2.data());
          for (int i = 0; i <= j; ++i) {
            h[i] += h2[i];
            h2[i] = -h2[i];
          }
          vcombine(kr_w_, 1.0, Vr(0), h2.data(), j + 1);
          const double hn = vnorm(kr_w_);
          if (hn > 0.0) k_vaxpby<<<vgrid(), 256, 0, st_>>>(1.0 / hn, kr_w_, 0.0, Vr(j + 1), vlen());
          // Givens rotations on column j
          for (int i = 0; i < j; ++i) {
            const double t = cs[i] * h[i] + sn[i] * h[i + 1];
            h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
            h[i] = t;
          }
          const double den = std::hypot(h[j], hn);
          cs[j] = den > 0.0 ? h[j] / den : 1.0;
          sn[j] = den > 0.0 ? hn / den : 0.0;
          h[j] = den;
          gv[j + 1] = -sn[j] * gv[j];
          gv[j] = cs[j] * gv[j];
          for (int i = 0; i <= j; ++i) H[static_cast<size_t>(i) * m + j] = h[i];
          const double res = std::fabs(gv[j + 1]);
          if (history) history[done] = bnorm > 0.0 ? res / bnorm : 0.0;
          ++done;
          if (!(res > rtol * bnorm) || !(hn > 0.0) || !std::isfinite(res)) {
            ++j;
            stop = true;
            break;
          }
        }
        // lam += P (V y), y = R^-1 g
        for (int i = j - 1; i >= 0; --i) {
          double s = gv[i];
          for (int k = i + 1; k < j; ++k) s -= H[static_cast<size_t>(i) * m + k] * y[k];
          y[i] = s / H[static_cast<size_t>(i) * m + i];
        }
        if (j > 0) {
          AERO_CK(cudaMemsetAsync(kr_w_, 0, sizeof(d4) * ntot_, st_));
          vcombine(kr_w_, 1.0, Vr(0), y.data(), j);
          precondition(kr_w_, cfl, smooth);
          k_vaxpby<<<vgrid(), 256, 0, st_>>>(1.0, kr_z_, 1.0, lam_, vlen());
        }
        AERO_CK(cudaGetLastError());
        if (stop && done >= max_iters) break;
        if (done >= max_iters) break;
      }
      AERO_CK(cudaStreamSynchronize(st_));
      if (done_out) *done_out = done;
      return err_ == cudaSuccess ? AERO_OK : AERO_ERR_CUDA;
    }
  }

 private:

  // out = (dR/dU)^T v on device arrays
  void apply_vjp(const d4* v, d4* out) {
    if constexpr (sizeof(T) == 8) {
      if (adj_second_) {
        k_adj_face_vjp<kJac><<<nfb_, block_, 0, st_>>>(df_, fblk_, Jf_, v, adj_face_);
        k_adj_gather<kJac><<<ncb_, block_, 0, st_>>>(dg_, cblk_, adj_face_, mw_, mgx_, mgy_);
        k_adj_green_gauss<<<ncb_, block_, 0, st_>>>(dm_, cblk_, mgx_, mgy_, mw_);
      } else {
        k_adj_face_vjp<8><<<nfb_, block_, 0, st_>>>(df_, fblk_, Jf_, v, adj_face_);
        k_adj_gather<8><<<ncb_, block_, 0, st_>>>(dg_, cblk_, adj_face_, mw_, mgx_, mgy_);
      }
      k_adj_prim<<<ncb_, block_, 0, st_>>>(cblk_, Ulin_, rs_[0].gamma, mw_, out);
    }
  }

  void upload_cells(const double* u, d4* dst) {
    const Pack& p = pk_[0];
    std::vector<d4> h(static_cast<size_t>(ntot_), d4{0.0, 0.0, 0.0, 0.0});
    for (int cn = 0; cn < p.n; ++cn) {
      const double* s = u + 5 * static_cast<size_t>(hs_[0].perm[cn]);
      h[cn] = d4{s[0], s[1], s[2], s[4]};
    }
    AERO_CK(cudaMemcpyAsync(dst, h.data(), sizeof(d4) * ntot_, cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaStreamSynchronize(st_));
  }
  void download_cells(const d4* src, double* u) {
    const Pack& p = pk_[0];
    std::vector<d4> h(static_cast<size_t>(p.n));
    AERO_CK(cudaMemcpyAsync(h.data(), src, sizeof(d4) * p.n, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    for (int cn = 0; cn < p.n; ++cn) {
      double* s = u + 5 * static_cast<size_t>(hs_[0].perm[cn]);
      s[0] = h[cn].x;
      s[1] = h[cn].y;
      s[2] = h[cn].z;
      s[3] = 0.0;
      s[4] = h[cn].w;
    }
  }

  // Pressure of the cells that own wall entries at the linearisation point (the gauge
  // pressure force, post/forces.cpp:208-294, integrates p_owner - p_inf); 0 elsewhere.
  std::vector<double> wall_pressures() {
    const Pack& pk = pk_[0];
    std::vector<d4> h(static_cast<size_t>(pk.n));
    AERO_CK(cudaMemcpyAsync(h.data(), Ulin_, sizeof(d4) * pk.n, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    const HostSlots& hs = hs_[0];
    const double g = rs_[0].gamma;
    std::vector<double> p(static_cast<size_t>(pk.n), 0.0);
    for (int c = 0; c < pk.n; ++c) {
      if (!(hs.flags[c] >> 2)) continue;
      const double r = std::max(h[c].x, 1.0e-8), inv = 1.0 / r, u = h[c].y * inv, v = h[c].z * inv;
      p[c] = std::max((g - 1.0) * (h[c].w - 0.5 * r * (u * u + v * v)), 1.0e-8);
    }
    return p;
  }

  // After a kernel gave up a bounded wait: the iteration it belonged to was not applied
  // (the updates skipped it and its controller stopped the run without a record). Clear the
  // word, let the stopped cases run again from their last applied iteration, and rebuild
  // the primitive state from the conserved state, which that iteration did not touch.
  // Returns whether a wait had expired.
  bool recover_from_expired_wait() {
    int expired = 0;
    AERO_CK(cudaMemcpy(&expired, tma_err_, sizeof(int), cudaMemcpyDeviceToHost));
    if (!expired || err_ != cudaSuccess) return expired != 0;
    download_ctrls();
    for (Ctrl& c : host_ctrls_) {
      if (c.wait_stop) {
        c.wait_stop = 0;
        c.done = 0;
      }
    }
    AERO_CK(cudaMemcpyAsync(ctrls_, host_ctrls_.data(), sizeof(Ctrl) * K_, cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaMemsetAsync(tma_err_, 0, sizeof(int), st_));
    AERO_CK(cudaStreamSynchronize(st_));
    w_valid_ = false;
    return true;
  }

 public:
  // Poll limit of the bounded waits on bulk copies (< 0: the default, about a second).
  int set_wait_limit(int polls) override {
    const int v = polls < 0 ? -1 : polls;
    AERO_CK(cudaMemcpyAsync(tma_err_ + 1, &v, sizeof(int), cudaMemcpyHostToDevice, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    return err_ == cudaSuccess ? AERO_OK : AERO_ERR_CUDA;
  }
  bool uses_bulk_copy_gradient() const override { return grad_tma_; }

 private:
  void download_ctrls() {
    host_ctrls_.resize(K_);
    AERO_CK(cudaMemcpyAsync(host_ctrls_.data(), ctrls_, sizeof(Ctrl) * K_, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
  }

  // Start/end of a run whose records are not kept (timing, profiling).
  int begin_untracked() {
    if (!w_valid_) refresh();
    download_ctrls();
    std::vector<int> base(K_, -(1 << 30));
    AERO_CK(cudaMemcpy2DAsync(&ctrls_->rec_base, sizeof(Ctrl), base.data(), sizeof(int), sizeof(int), K_,
                              cudaMemcpyHostToDevice, st_));
    int it0 = 0;
    for (const Ctrl& c : host_ctrls_) it0 = std::max(it0, c.iter);
    return it0;
  }
  int end_untracked() {
    const bool expired = recover_from_expired_wait();
    download_ctrls();
    if (err_ != cudaSuccess) return AERO_ERR_CUDA;
    if (expired) return AERO_ERR_TIMEOUT;
    for (const Ctrl& c : host_ctrls_) {
      if (c.nonfinite) return AERO_ERR_NONFINITE;
    }
    return AERO_OK;
  }

  d4* pinned_state() {
    if (pin_state_ == nullptr) {
      int nmax = 0;
      for (const Pack& p : pk_) nmax = std::max(nmax, p.n);
      if (cudaMallocHost(reinterpret_cast<void**>(&pin_state_), sizeof(d4) * static_cast<size_t>(nmax)) !=
          cudaSuccess) {
        cudaGetLastError();
        pin_state_ = nullptr;
        pin_fallback_.resize(static_cast<size_t>(nmax));
        return pin_fallback_.data();
      }
    }
    return pin_state_;
  }

  bool second_at(int it) const { return it >= std::max(cfg_[0].startup_first_order_iters, 0); }

  long long launches_per_iteration(bool second) const {
    // gradient, face pass, update (+ cell pass and time-step reduction with a global step)
    const int per_stage = (second ? 1 : 0) + 2 + (cfg_[0].local_time_stepping ? 0 : 2);
    return static_cast<long long>(per_stage) * cfg_[0].rk_stages + (pjump_on_ ? 1 : 0) + (sym_on_ ? 1 : 0) + 1;
  }

  void refresh() {
    if constexpr (sizeof(T) == 4) {
      k_prim_from_image<<<ncb_, block_, 0, st_>>>(ntot_, sref_.hi, W_, pcs_[0].gamma_f);
    } else {
      k_refresh_prim<T><<<ncb_, block_, 0, st_>>>(ntot_, Un_, W_, rs_[0].gamma);
    }
    AERO_CK(cudaGetLastError());
    w_valid_ = true;
  }

  // FP32 keeps the state as float-float pairs and uses Un_ as the double staging array.
  void state_from_staging(int c0, int n) {
    const int grid = (n + block_ - 1) / block_;
    if (sizeof(T) == 4) k_split_state<<<grid, block_, 0, st_>>>(n, Un_ + c0, sref_.hi + c0, sref_.lo + c0);
    AERO_CK(cudaGetLastError());
  }
  void state_to_staging(int c0, int n) {
    const int grid = (n + block_ - 1) / block_;
    if (sizeof(T) == 4) k_combine_state<<<grid, block_, 0, st_>>>(n, sref_.hi + c0, sref_.lo + c0, Un_ + c0);
    AERO_CK(cudaGetLastError());
  }

  void download_residual(int k, double* res, double* sr) {
    const Pack& p = pk_[k];
    std::vector<V4> hr(static_cast<size_t>(p.n));
    std::vector<T> hs(static_cast<size_t>(p.n));
    AERO_CK(cudaMemcpyAsync(hr.data(), R_ + p.c0, sizeof(V4) * p.n, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaMemcpyAsync(hs.data(), SR_ + p.c0, sizeof(T) * p.n, cudaMemcpyDeviceToHost, st_));
    AERO_CK(cudaStreamSynchronize(st_));
    for (int cn = 0; cn < p.n; ++cn) {
      const int co = hs_[k].perm[cn];
      double* r = res + 5 * static_cast<size_t>(co);
      r[0] = hr[cn].x;
      r[1] = hr[cn].y;
      r[2] = hr[cn].z;
      r[3] = 0.0;
      r[4] = hr[cn].w;
      if (sr) sr[co] = hs[cn];
    }
  }

  ResidualLaunch<T> residual_args(int* fb, V4* R, T* SR, int global_dt) {
    ResidualLaunch<T> a;
    a.block = block_;
    a.st = st_;
    a.faces = df_;
    a.gather = dg_;
    a.face_cases = face_cases_;
    a.cell_cases = cell_cases_;
    a.W = W_;
    a.gx = gx_;
    a.gy = gy_;
    a.F = F_;
    a.FS = FS_;
    a.R = R;
    a.SR = SR;
    a.part = part_;
    a.fb = fb;
    a.global_dt = global_dt;
    return a;
  }

  template <bool PRECOND, bool LAST, bool GATHER>
  void update_t(int stage, int global_dt, V4* R, T* SR, bool pdl) {
    auto kern = k_update<T, PRECOND, LAST, GATHER>;
    const int pf = resident_blocks(kern, block_);
    AERO_CK(launch_kernel(kern, ncb_, block_, 0, st_, pdl, stage, cell_cases_, R, SR, dg_, F_, FS_, W_, sref_, Us_,
                          ms_, part_, global_dt, pf));
  }
  template <bool PRECOND>
  void update_p(int stage, bool last, int global_dt, V4* R, T* SR, bool pdl = false) {
    if (global_dt) {  // residual already gathered (the global time step needs all of SR first)
      if (last) update_t<PRECOND, true, false>(stage, global_dt, R, SR, pdl);
      else update_t<PRECOND, false, false>(stage, global_dt, R, SR, pdl);
    } else {
      if (last) update_t<PRECOND, true, true>(stage, global_dt, R, SR, pdl);
      else update_t<PRECOND, false, true>(stage, global_dt, R, SR, pdl);
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
  // iteration's gradient and first face pass and joined before the first update, the first
  // kernel that reads its outputs.
  template <class Wrap>
  void launch_iteration(bool second, int parity, bool defer, bool pending, Wrap&& wrap) {
    const int global_dt = cfg_[0].local_time_stepping ? 0 : 1;
    const int ns = cfg_[0].rk_stages;
    int* fb = fb_ + 2 * parity;
    for (int stage = 0; stage < ns; ++stage) {
      const bool last = stage == ns - 1;
      V4* R = stage == 0 ? R0_ : R_;
      T* SR = stage == 0 ? SR0_ : SR_;
      if (stage == 0 && pending) {
        AERO_CK(cudaEventRecord(ev_fork_, st_));
        AERO_CK(cudaStreamWaitEvent(side_, ev_fork_, 0));
        wrap(5, [&] {
          k_control<<<K_, kCtlThreads, 0, side_>>>(ccs_dev_, part_, ctrls_, recs_, rec_cap_, fb_ + 2 * (parity ^ 1),
                                                   lm_defer_ ? lms_ : nullptr);
        });
        AERO_CK(cudaEventRecord(ev_join_, side_));
      }
      // programmatic dependent launch of the gradient, face and update kernels (not of the
      // update that also waits for the controller on the side stream)
      const bool pdl = pdl_ && !global_dt;
      if (second) {
        wrap(0, [&] {
          if (grad_tma_) {
            AERO_CK(launch_kernel(k_gradient_tma<T>, grad_grid_, block_, grad_smem_, st_, pdl, dm_, W_, gx_, gy_,
                                  cell_cases_, ncb_, tma_err_));
          } else if (cpt_ == 2) {
            AERO_CK(launch_kernel(k_gradient<T, 2>, (ncb_ + 1) / 2, block_, 0, st_, pdl, dm_, W_, gx_, gy_, cell_cases_,
                                  ncb_));
          } else {
            AERO_CK(launch_kernel(k_gradient<T, 1>, ncb_, block_, 0, st_, pdl, dm_, W_, gx_, gy_, cell_cases_, 0));
          }
        });
      }
      ResidualLaunch<T> ra = residual_args(fb, R, SR, global_dt);
      ra.pdl = pdl;
      if (defer && lm_defer_) {
        ra.lms = lms_;
        ra.parity = parity;
      }
      wrap(1, [&] { launch_face_pass(ra, cfg_[0].flux, second, lm_ != 0); });
      if (global_dt) wrap(1, [&] { launch_gather_pass(ra, last); });
      if (stage == 0 && pending) AERO_CK(cudaStreamWaitEvent(st_, ev_join_, 0));
      if (global_dt) {
        wrap(3, [&] { k_srmax<<<K_, 1024, 0, st_>>>(part_.srmax, srfirst_, ctrls_); });
      }
      const bool pdl_update = pdl && !(stage == 0 && pending);
      wrap(2, [&] {
        if (cfg_[0].precond_on) {
          update_p<true>(stage, last, global_dt, R, SR, pdl_update);
        } else {
          update_p<false>(stage, last, global_dt, R, SR, pdl_update);
        }
      });
    }
    if (sym_on_) {
      wrap(4, [&] { k_symmetry<T><<<ncb_, block_, 0, st_>>>(cell_cases_, sref_, W_, ms_, part_); });
    }
    if (pjump_on_) {
      wrap(4, [&] { k_pjump<T><<<ncb_, block_, 0, st_>>>(dm_, sref_, flags_, cell_cases_, part_); });
    }
    if (!defer) launch_control(parity, wrap);
    AERO_CK(cudaGetLastError());
  }
  template <class Wrap>
  void launch_control(int parity, Wrap&& wrap) {
    wrap(5, [&] {
      k_control<<<K_, kCtlThreads, 0, st_>>>(ccs_dev_, part_, ctrls_, recs_, rec_cap_, fb_ + 2 * parity,
                                             lm_defer_ ? lms_ : nullptr);
    });
  }

  // Iterations it0 .. it0+n-1 back to back, through the per-iteration CUDA graphs; with the
  // deferred controller, each iteration's controller overlaps the next iteration's start and
  // the last one runs after the loop. `between(j)` runs on the stream before iteration j and
  // `after(j)` after it (timing marks, L2 flushes).
  template <class Before, class After>
  void launch_iterations(int it0, int n, Before&& between, After&& after) {
    if (lm_defer_ && n > 0) {  // the low-Mach weights of the first two iterations
      std::vector<LmSched> q(2 * static_cast<size_t>(K_));
      for (int k = 0; k < K_; ++k) {
        for (int it = it0; it < it0 + 2; ++it) q[2 * k + (it & 1)] = lm_sched_of(ccs_[k], it);
      }
      AERO_CK(cudaMemcpyAsync(lms_, q.data(), sizeof(LmSched) * q.size(), cudaMemcpyHostToDevice, st_));
    }
    for (int j = 0; j < n; ++j) {
      const int it = it0 + j;
      between(j);
      launch_iteration_graph(second_at(it), it & 1, defer_control_, defer_control_ && j > 0);
      if (defer_control_ && j == n - 1) launch_control(it & 1, Direct{});
      after(j);
    }
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

  std::vector<HostSlots> hs_;
  std::vector<aero_case_desc> cfg_;
  std::vector<Resolved> rs_;
  cudaStream_t st_;
  cudaError_t err_ = cudaSuccess;
  std::vector<void*> allocs_;
  size_t bytes_ = 0;
  int K_ = 0, lm_ = 0;
  std::vector<Pack> pk_;
  int ntot_ = 0, ftot_ = 0, ncb_ = 0, nfb_ = 0, nwslots_ = 0, d_ = 0;
  long long ncells_ = 0, nfaces_ = 0;
  int block_ = 128, rec_cap_ = 0;
  bool pjump_on_ = false, sym_on_ = false, w_valid_ = false;
  int* link_ = nullptr;
  V2* nrm_ = nullptr;
  T* area_ = nullptr;
  V2* gvec_ = nullptr;
  DevFaces<T> df_{};
  DevGather<T> dg_{};
  V4* F_ = nullptr;   // per face: F*A
  T* FS_ = nullptr;   // per face: wave-speed term
  T* inv_vol_ = nullptr;
  unsigned char* flags_ = nullptr;
  int* perm_dev_ = nullptr;  // case 0: new -> original cell
  int* iperm_all_dev_ = nullptr;  // every case's original -> new cell, at the case's cell offset
  bool host_direct_ = false;     // the GPU reads and writes host state arrays in place
  bool grad_tma_ = false;        // gradient pass through bulk copies into shared memory
  bool pdl_ = false;             // programmatic dependent launch of the iteration's kernels
  int cpt_ = 1;                  // cells per thread of the gather gradient pass (1 or 2)
  size_t grad_smem_ = 0;
  int grad_grid_ = 0;
  int* tma_err_ = nullptr;       // set by a kernel whose bounded wait on a copy expired
  int2* cblk_ = nullptr;     // per cell block: (case, end of the case's cells)
  int2* fblk_ = nullptr;     // per face block: (case, end of the case's faces)
  int* srfirst_ = nullptr;   // per case: first per-warp time-step partial, [K + 1]
  MonitorSet ms_{};
  V4 *W_ = nullptr, *gx_ = nullptr, *gy_ = nullptr, *R_ = nullptr;
  T* SR_ = nullptr;
  d4* Un_ = nullptr;     // FP64: the conserved state; FP32: double staging for transfers
  StateRef sref_{};
  V4* Us_ = nullptr;     // FP64: stage state; FP32: stage increment (delta form)
  d4* Ueval_ = nullptr;  // conserved state given to aero_residual
  Partials part_{};
  Ctrl* ctrls_ = nullptr;      // [K]
  Ctrl* ctrl_eval_ = nullptr;  // aero_residual
  Record* recs_ = nullptr;     // [K][rec_cap]
  CtrlConfig* ccs_dev_ = nullptr;
  FaceParams<T>* fps_dev_ = nullptr;
  PrecondD* pcs_dev_ = nullptr;
  MonitorConsts* mcs_dev_ = nullptr;
  std::vector<CtrlConfig> ccs_;
  std::vector<FaceParams<T>> fps_;
  std::vector<PrecondD> pcs_;
  std::vector<MonitorConsts> mcs_;
  std::vector<Ctrl> host_ctrls_;
  Cases<T> cell_cases_{}, face_cases_{};
  DevMesh<T> dm_{};
  cudaGraphExec_t graph_[16] = {};
  bool defer_control_ = false;
  bool lm_defer_ = false;      // deferred controller with low-Mach weights from parity slots
  LmSched* lms_ = nullptr;     // [case][2] low-Mach weights by iteration parity
  // discrete adjoint (FP64)
  bool adj_alloc_ = false, adj_ready_ = false, adj_second_ = false;
  double adj_wcd_ = 0.0, adj_wcl_ = 0.0, adj_ex_ = 0.0, adj_ey_ = 0.0;
  d4 *gxlin_ = nullptr, *gylin_ = nullptr;
  // geometry tangent scratch
  bool geo_alloc_ = false;
  double2 *geo_nrm_ = nullptr, *geo_fn_ = nullptr, *geo_doff_ = nullptr, *geo_noff_ = nullptr;
  double *geo_area_ = nullptr, *geo_inv_ = nullptr, *geo_fa_ = nullptr;
  d4 *geo_gx_ = nullptr, *geo_gy_ = nullptr;
  double* Jf_ = nullptr;        // per face: 4 x kJac local Jacobian
  double* adj_face_ = nullptr;  // per face: kJac transpose-product contributions
  double* adj_face_out_ = nullptr;
  bool geo_vjp_alloc_ = false;
  double *geo_face_vjp_ = nullptr, *geo_slot_vjp_ = nullptr, *geo_inv_vjp_ = nullptr;
  d4 *mw_ = nullptr, *mgx_ = nullptr, *mgy_ = nullptr, *adj_r_ = nullptr, *adj_g_ = nullptr;
  d4 *lam_ = nullptr, *lam_n_ = nullptr, *adj_v_ = nullptr;
  double* adj_rn_ = nullptr;     // per cell block: sum of the squared adjoint residual
  double* adj_hist_ = nullptr;   // per iteration of a chunk: RMS adjoint residual
  int* adj_counter_ = nullptr;
  cudaGraphExec_t adj_graph_ = nullptr;
  double adj_graph_cfl_ = 0.0;
  // Krylov solve: basis (kr_m_ + 1 vectors of ntot cells), work vectors, reductions
  int kr_m_ = 0;
  d4 *kr_V_ = nullptr, *kr_w_ = nullptr, *kr_z_ = nullptr, *kr_zn_ = nullptr, *kr_src_ = nullptr;
  double *kr_part_ = nullptr, *kr_out_ = nullptr, *kr_coef_ = nullptr;
  cudaGraphExec_t kr_graph_ = nullptr;
  double kr_graph_cfl_ = 0.0;
  int kr_graph_smooth_ = -1;
  Ctrl* ctrl_lin_ = nullptr;
  d4 *Ulin_ = nullptr, *Wlin_ = nullptr;  // state and primitives at the linearisation point
  double* SRlin_ = nullptr;               // its spectral radii (the adjoint's local steps)
  cudaStream_t side_ = nullptr;
  cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
  V4* R0_ = nullptr;
  T* SR0_ = nullptr;
  int* fb_ = nullptr;  // [case][2 parities][first-order, diffusive] fallback counters
  void* flush_ = nullptr;
  size_t flush_bytes_ = 0;
  d4* pin_state_ = nullptr;
  std::vector<d4> pin_fallback_;
};

#undef AERO_CK

}  // namespace aero
