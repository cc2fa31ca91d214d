// aero_tma.cuh -- bulk asynchronous copies (cp.async.bulk, completed on an mbarrier) into
// shared memory, and the Green-Gauss gradient pass built on them.
//
// The gradient reads, per cell block, streams that are contiguous in the cell-major layouts
// (the slot table's links, normals and lengths for every slot, the block's own primitive
// states and inverse volumes). A persistent CTA walks its tiles (cell blocks) with two
// shared-memory buffers: one elected thread issues the bulk copies of tile i+1 while the
// block computes tile i from shared memory, so the streamed loads are in flight during the
// arithmetic and the dependent neighbour gathers. Neighbours inside the tile are read from
// the staged states; the others from global memory.
//
// Every wait on an mbarrier is bounded: on expiry the kernel records an error word for the
// host, waits (again bounded) for its copies still in flight, and returns.
#pragma once

#include <cstdint>

#include "aero_kernels.cuh"

namespace aero {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
// global -> shared, 16-byte aligned addresses, size a multiple of 16 bytes
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// true when the phase with the given parity completed; false after `limit` polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit) {
  const uint32_t a = smem_addr(bar);
  for (int i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

constexpr int kTmaPolls = 1 << 20;  // ~1 s of polling before a wait is given up

// Shared-memory layout of one tile buffer for B cells and D slots.
struct GradTile {
  uint32_t link, gvec, w, inv, bytes;  // byte offsets; bytes: size of one buffer
  uint32_t tx;                              // bytes the copies of one tile deliver
};
template <class T>
__host__ __device__ inline GradTile grad_tile(int B, int D) {
  using V2 = typename Vec<T>::v2;
  using V4 = typename Vec<T>::v4;
  GradTile g;
  uint32_t off = 0;
  auto take = [&](uint32_t b) {
    const uint32_t o = off;
    off += (b + 15u) & ~15u;
    return o;
  };
  g.link = take(uint32_t(D) * B * 4u);
  g.gvec = take(uint32_t(D) * B * uint32_t(sizeof(V2)));
  g.w = take(uint32_t(B) * uint32_t(sizeof(V4)));
  g.inv = take(uint32_t(B) * uint32_t(sizeof(T)));
  g.bytes = off;
  g.tx = uint32_t(D) * B * (4u + uint32_t(sizeof(V2))) + uint32_t(B) * uint32_t(sizeof(V4) + sizeof(T));
  return g;
}
// dynamic shared memory of the kernel: two buffers and two mbarriers
template <class T>
inline size_t grad_tma_smem(int B, int D) {
  return 2 * size_t(grad_tile<T>(B, D).bytes) + 16;
}

// Green-Gauss gradients (cell_gradient's arithmetic, same order) over ntiles cell blocks of
// blockDim.x cells; blockDim.x must be the engine's block size (64, 128 or 256) so that every
// copied segment is 16-byte aligned and a multiple of 16 bytes.
//
// Bounded waits: wait[1] is the poll limit of the wait on each tile's copies (negative: the
// default kTmaPolls). A CTA whose wait runs out records wait[0] = 1, then waits (bounded by
// kTmaPolls, whatever the limit) for its copies still in flight into either buffer, so that
// none lands after it has exited, and returns without computing its remaining tiles. The
// gradients of those tiles are then missing, so the update kernels discard the iteration
// (Cases::wait) and the host reports AERO_ERR_TIMEOUT.
template <class T>
__global__ void __launch_bounds__(256) k_gradient_tma(DevMesh<T> m, const typename Vec<T>::v4* __restrict__ W,
                                                      typename Vec<T>::v4* __restrict__ gx,
                                                      typename Vec<T>::v4* __restrict__ gy, Cases<T> cs,
                                                      int ntiles, int* __restrict__ wait) {
  using V2 = typename Vec<T>::v2;
  using V4 = typename Vec<T>::v4;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int s_ok;
  const int B = blockDim.x, D = m.d;
  const GradTile L = grad_tile<T>(B, D);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * size_t(L.bytes));
  int tile = blockIdx.x;
  if (tile >= ntiles) return;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  auto issue = [&](int t, int buf) {  // one thread
    unsigned char* base = smem + size_t(buf) * L.bytes;
    const size_t c0 = size_t(t) * B;
    mbar_expect_tx(&bar[buf], L.tx);
    for (int k = 0; k < D; ++k) {
      const size_t s0 = size_t(k) * m.n + c0;
      bulk_copy_g2s(base + L.link + size_t(k) * B * 4, m.link + s0, uint32_t(B) * 4u, &bar[buf]);
      bulk_copy_g2s(base + L.gvec + size_t(k) * B * sizeof(V2), m.gvec + s0, uint32_t(B * sizeof(V2)), &bar[buf]);
    }
    bulk_copy_g2s(base + L.w, W + c0, uint32_t(B * sizeof(V4)), &bar[buf]);
    bulk_copy_g2s(base + L.inv, m.inv_vol + c0, uint32_t(B * sizeof(T)), &bar[buf]);
  };
  pdl_trigger();
  pdl_wait();  // the copies read W
  const int limit = wait[1] < 0 ? kTmaPolls : wait[1];
  if (threadIdx.x == 0) issue(tile, 0);
  uint32_t phase0 = 0, phase1 = 0;
  for (int i = 0; tile < ntiles; ++i, tile += gridDim.x) {
    const int buf = i & 1;
    const int next = tile + gridDim.x;
    if (threadIdx.x == 0) {
      if (next < ntiles) {
        fence_proxy_async_smem();  // the block's reads of that buffer come before the copies
        issue(next, buf ^ 1);
      }
      s_ok = mbar_wait(&bar[buf], buf ? phase1 : phase0, limit) ? 1 : 0;
    }
    __syncthreads();
    if (!s_ok) {  // uniform: record the failure, let the copies in flight land, return
      if (threadIdx.x == 0) {
        atomicExch(&wait[0], 1);
        mbar_wait(&bar[buf], buf ? phase1 : phase0, kTmaPolls);
        if (next < ntiles) mbar_wait(&bar[buf ^ 1], buf ? phase0 : phase1, kTmaPolls);
      }
      __syncthreads();
      return;
    }
    if (buf) {
      phase1 ^= 1u;
    } else {
      phase0 ^= 1u;
    }
    const unsigned char* base = smem + size_t(buf) * L.bytes;
    const int* sl = reinterpret_cast<const int*>(base + L.link);
    const V2* sg = reinterpret_cast<const V2*>(base + L.gvec);
    const V4* sw = reinterpret_cast<const V4*>(base + L.w);
    const T* si = reinterpret_cast<const T*>(base + L.inv);
    const int2 bd = cs.blk[tile];
    const int c0 = tile * B, c = c0 + threadIdx.x;
    if (c < bd.y && !cs.ctrl[bd.x].done) {
      const int j = threadIdx.x;
      const V4 wc = sw[j];
      T ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0};
      for (int k = 0; k < D; ++k) {
        const int link = sl[k * B + j];
        if (link == kPad) break;
        const V2 g = sg[k * B + j];
        V4 wo = wc;
        if (link >= 0) {
          const int o = link >> 1;
          const unsigned off = static_cast<unsigned>(o - c0);
          wo = off < static_cast<unsigned>(B) ? sw[off] : W[o];
        }
        grad_slot_terms<T>(link, wc, wo, g, ax, ay);
      }
      const T inv = si[j];
      V4 ox, oy;
      ox.x = ax[0] * inv; ox.y = ax[1] * inv; ox.z = ax[2] * inv; ox.w = ax[3] * inv;
      oy.x = ay[0] * inv; oy.y = ay[1] * inv; oy.z = ay[2] * inv; oy.w = ay[3] * inv;
      gx[c] = ox;
      gy[c] = oy;
    }
    __syncthreads();  // the buffer is free for the copies issued in the next iteration
  }
}

}  // namespace aero
