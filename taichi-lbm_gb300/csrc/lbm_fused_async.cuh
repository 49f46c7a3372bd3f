// Persistent variants of the fused step: same arithmetic as k_fused (they
// share fused_tail), different ways of keeping DRAM requests in flight.
//
// k_fused_async<.., NW, NS>: each warp owns a ring of NS shared-memory
// stages.  A stage holds, for one row segment of 128 nodes, the nine source
// rows (row y - cy_k of population k) over columns [x0 - PADE, x0 + 128 +
// PADE): 16 bytes of halo on each side, so the +-1 x shift of the pull is a
// shifted shared-memory read.  One lane issues the nine cp.async.bulk copies
// of a stage and an mbarrier counts their bytes; the warp runs NS - 1
// segments ahead, independently of the registers the collision needs.
//
// k_fused_prefetch: each warp loops over its segments and issues the next
// segment's vector loads into registers before colliding the current one.
//
// Every wait on an mbarrier is bounded by a clock64 budget (the plan's
// wait_cycles, default WAIT_CYCLES); on expiry the warp records
// LBM_STATUS_TIMEOUT in *status, waits (bounded by WAIT_CYCLES) for the
// copies it still has in flight, the expired one included, and returns.
#pragma once

#include "lbm_fused.cuh"

namespace lbm {

constexpr int AV = 4;            // nodes per lane in the persistent variants
constexpr int AITEM = 32 * AV;   // nodes per row segment
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz

template <int ST, int NW, int NS>
struct AsyncGeom {
  using T = typename Storage<ST>::T;
  static constexpr int PADE = 16 / (int)sizeof(T);
  static constexpr int ROW = AITEM + 2 * PADE;
  static constexpr int STAGE_ELEMS = 9 * ROW;
  static constexpr int WARP_BYTES = NS * STAGE_ELEMS * (int)sizeof(T);
  static constexpr int SMEM = NW * WARP_BYTES + NW * NS * 8;
  static_assert((ROW * sizeof(T)) % 16 == 0, "staged rows must stay 16-byte aligned");
  static_assert(WARP_BYTES % 16 == 0, "warp rings must stay 16-byte aligned");
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; false when the budget (clock cycles) ran out.  The first
// test does not block, so a budget shorter than a copy's flight time runs
// out before the copy lands (the short-budget test of the timeout path).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long budget) {
  const long long t0 = clock64();
  if (mbar_test_wait(bar, parity)) return true;
  while (clock64() - t0 <= budget) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  return false;
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_mbarrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}


// Fix-ups of the gather at the lattice's x edges: node 0 pulls column nx-1
// on links with cx = +1, node nx-1 pulls column 0 on links with cx = -1.
template <int ST>
__device__ __forceinline__ void edge_fixups(const FusedParams& p, float (&f)[AV][9], int y, int x0, bool live) {
  using S = Storage<ST>;
  using T = typename S::T;
  if (!live) return;
  const int ilast = p.nx - 1 - x0;
  const bool first = x0 == 0, last = ilast >= 0 && ilast < AV;
  if (!first && !last) return;
  const T* src = reinterpret_cast<const T*>(p.src);
#pragma unroll
  for (int k = 1; k < 9; ++k) {
    const T* grow = src + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch;
    if (CX(k) == 1 && first) f[0][k] = S::dec(load1(grow + (p.nx - 1)), p.wsh[k], p.fq);
    if (CX(k) == -1 && last) {
      const float v0 = S::dec(load1(grow), p.wsh[k], p.fq);
#pragma unroll
      for (int i = 0; i < AV; ++i)
        if (i == ilast) f[i][k] = v0;
    }
  }
}

template <int MODEL, bool PL, int ST, int NW, int NS>
__global__ void __launch_bounds__(NW * 32) k_fused_async(const FusedParams p, int32_t* status) {
  using S = Storage<ST>;
  using T = typename S::T;
  using G = AsyncGeom<ST, NW, NS>;
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* ring = reinterpret_cast<T*>(smem + warp * G::WARP_BYTES);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + NW * G::WARP_BYTES) + warp * NS;
  if (lane == 0) {
    for (int s = 0; s < NS; ++s) mbar_init(&bars[s], 1);
    fence_mbarrier_init();
  }
  __syncwarp();

  const T* src = reinterpret_cast<const T*>(p.src);
  const long long nitems = (long long)p.ny * p.nseg;
  const long long gw = (long long)blockIdx.x * NW + warp;
  const long long GW = (long long)gridDim.x * NW;

  // stage the nine source rows of the warp's n-th segment into slot n % NS
  auto issue = [&](long long n) {
    const long long it = gw + n * GW;
    if (it >= nitems || lane != 0) return;
    const int y = (int)(it / p.nseg), seg = (int)(it - (long long)y * p.nseg);
    const int x0 = seg * AITEM;
    int start = x0 - G::PADE, soff = 0;
    if (start < 0) {  // the lattice's first segment: no left halo in memory
      soff = -start;
      start = 0;
    }
    const int end = min(x0 + AITEM + G::PADE, p.pitch);  // never past the row's storage
    const uint32_t bytes = (uint32_t)(end - start) * (uint32_t)sizeof(T);
    T* stage = ring + (int)(n % NS) * G::STAGE_ELEMS;
    uint64_t* bar = &bars[n % NS];
    fence_proxy_async_smem();  // earlier generic reads of this slot before the async writes
    mbar_arrive_expect_tx(bar, 9 * bytes);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const T* row = src + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch;
      bulk_copy_g2s(stage + k * G::ROW + soff, row + start, bytes, bar);
    }
  };

  for (int n = 0; n < NS - 1; ++n) issue(n);
  for (long long n = 0;; ++n) {
    const long long it = gw + n * GW;
    if (it >= nitems) break;
    issue(n + NS - 1);
    const int slot = (int)(n % NS);
    const bool ok = mbar_wait_bounded(&bars[slot], (uint32_t)((n / NS) & 1), p.wait_cycles);
    if (!__all_sync(0xffffffffu, ok)) {
      if (lane == 0) atomicOr(status, LBM_STATUS_TIMEOUT);
      // drain, with the long budget: the copies still in flight, issued for
      // segments n .. n + NS - 1, land before the warp leaves its ring
      for (long long m = n; m < n + NS; ++m)
        if (gw + m * GW < nitems) mbar_wait_bounded(&bars[m % NS], (uint32_t)((m / NS) & 1), WAIT_CYCLES);
      return;
    }
    const int y = (int)(it / p.nseg), seg = (int)(it - (long long)y * p.nseg);
    const int x0 = seg * AITEM + lane * AV;
    const bool live = x0 < p.nx;
    const T* stage = ring + slot * G::STAGE_ELEMS;
    float f[AV][9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const T* r = stage + k * G::ROW + G::PADE + lane * AV - CX(k);
#pragma unroll
      for (int i = 0; i < AV; ++i) f[i][k] = S::dec(r[i], p.wsh[k], p.fq);
    }
    __syncwarp();
    edge_fixups<ST>(p, f, y, x0, live);
    fused_tail<MODEL, PL, ST, AV>(p, f, y, seg, x0, live);
  }
}

// One segment's raw source values: the nine aligned vectors, plus the two
// elements that cross the segment edges (lane 0's left, lane 31's right).
template <typename T>
struct RawSeg {
  T v[9][AV];
  T left[3], right[3];  // links with cx = +1 (1, 5, 8) and cx = -1 (3, 6, 7)
};

template <int ST>
__device__ __forceinline__ void load_segment(const FusedParams& p, long long it, int lane,
                                             RawSeg<typename Storage<ST>::T>& r) {
  using T = typename Storage<ST>::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  const int y = (int)(it / p.nseg), seg = (int)(it - (long long)y * p.nseg);
  const int x0 = seg * AITEM + lane * AV;
  if (x0 >= p.nx) return;
  int li = 0, ri = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const T* row = src + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch;
    load_vec<T, AV>(row + x0, r.v[k]);
    if (CX(k) == 1) r.left[li++] = load1(row + wrap(x0 - 1, p.nx));
    if (CX(k) == -1) r.right[ri++] = load1(row + wrap(x0 + AV, p.nx));
  }
}

template <int MODEL, bool PL, int ST>
__global__ void __launch_bounds__(256) k_fused_prefetch(const FusedParams p) {
  using S = Storage<ST>;
  using T = typename S::T;
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long nitems = (long long)p.ny * p.nseg;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long GW = ((long long)gridDim.x * blockDim.x) >> 5;
  RawSeg<T> cur, nxt;
  if (gw < nitems) load_segment<ST>(p, gw, lane, cur);
  for (long long it = gw; it < nitems; it += GW) {
    if (it + GW < nitems) load_segment<ST>(p, it + GW, lane, nxt);
    const int y = (int)(it / p.nseg), seg = (int)(it - (long long)y * p.nseg);
    const int x0 = seg * AITEM + lane * AV;
    const bool live = x0 < p.nx;
    float f[AV][9];
    int li = 0, ri = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float c[AV];
#pragma unroll
      for (int i = 0; i < AV; ++i) c[i] = live ? S::dec(cur.v[k][i], p.wsh[k], p.fq) : 0.0f;
      if (CX(k) == 0) {
#pragma unroll
        for (int i = 0; i < AV; ++i) f[i][k] = c[i];
      } else if (CX(k) == 1) {
        float left = __shfl_up_sync(FULL, c[AV - 1], 1);
        if (lane == 0 && live) left = S::dec(cur.left[li], p.wsh[k], p.fq);
        ++li;
        f[0][k] = left;
#pragma unroll
        for (int i = 1; i < AV; ++i) f[i][k] = c[i - 1];
      } else {
        float right = __shfl_down_sync(FULL, c[0], 1);
        if (lane == 31 && live) right = S::dec(cur.right[ri], p.wsh[k], p.fq);
        ++ri;
#pragma unroll
        for (int i = 0; i < AV - 1; ++i) f[i][k] = c[i + 1];
        f[AV - 1][k] = right;
      }
    }
    // node nx-1 pulls column 0 on cx = -1 links (the lane-31 element covers
    // only a segment that ends exactly at nx)
    const int ilast = p.nx - 1 - x0;
    if (live && ilast >= 0 && ilast < AV) {
      const T* src = reinterpret_cast<const T*>(p.src);
#pragma unroll
      for (int k = 1; k < 9; ++k)
        if (CX(k) == -1) {
          const float v0 = S::dec(load1(src + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch), p.wsh[k], p.fq);
#pragma unroll
          for (int i = 0; i < AV; ++i)
            if (i == ilast) f[i][k] = v0;
        }
    }
    fused_tail<MODEL, PL, ST, AV>(p, f, y, seg, x0, live);
    cur = nxt;
  }
}

}  // namespace lbm
