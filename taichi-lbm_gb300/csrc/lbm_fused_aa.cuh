// In-place (AA-pattern) form of the fused step: one population buffer.
//
// The ping-pong step reads the post-collision state from one buffer and
// writes the next into the other.  The in-place step keeps one buffer and
// alternates two phases whose every node reads and writes the same nine
// locations, so no node overwrites what another still has to read:
//
//  * phase A (the buffer in pull layout: slot k of node x holds the
//    post-collision f*_k(x)) gathers f_k(x) as the pull step does, from slot k
//    of x - c_k, or from slot opp(k) of x itself across a bounce-back link,
//    and after the collision writes f*_opp(k)(x) back where it read f_k.
//    The buffer is then in the swapped layout: slot opp(k) of x holds the
//    streamed f_k(x).
//  * phase B reads f_k(x) from slot opp(k) of x and writes f*_k(x) to slot k
//    of x: the pull layout again, with no neighbour access at all.
//
// A run of an odd number of steps ends after phase A; k_aa_swap then moves
// every streamed pair back to the pull layout, so between runs the buffer
// always holds the state the ping-pong step would hold.  The same values are
// read, rounded and stored as in the ping-pong step, only at other
// addresses, so both give the same bits.
//
// The pairing needs every cut link to be cut on both sides: a node that
// bounces back the population coming from a colliding neighbour must be
// bounced back by that neighbour too, and no colliding node may stream from
// a node outside the collision group (whose frozen populations an in-place
// buffer would not keep).  The plan compiler checks both.  Boundary programs
// that read a neighbour's post-stream populations (NEEM, ABC neighbours,
// open boundaries) read them from p.aa_vals, which k_aa_sites fills before
// the step's other kernels start.
#pragma once

#include "lbm_fused.cuh"
#include "lbm_fused_lean.cuh"

namespace lbm {

// stored values as 32-bit words for warp shuffles
__device__ __forceinline__ unsigned to_word(float v) { return __float_as_uint(v); }
__device__ __forceinline__ unsigned to_word(__half v) { return __half_as_ushort(v); }
__device__ __forceinline__ unsigned to_word(__nv_bfloat16 v) { return __bfloat16_as_ushort(v); }
__device__ __forceinline__ unsigned to_word(short v) { return (unsigned short)v; }
template <typename T>
__device__ __forceinline__ T from_word(unsigned w);
template <>
__device__ __forceinline__ float from_word<float>(unsigned w) { return __uint_as_float(w); }
template <>
__device__ __forceinline__ __half from_word<__half>(unsigned w) { return __ushort_as_half((unsigned short)w); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_word<__nv_bfloat16>(unsigned w) {
  return __ushort_as_bfloat16((unsigned short)w);
}
template <>
__device__ __forceinline__ short from_word<short>(unsigned w) { return (short)(unsigned short)w; }

// one stored value from a lean (unshifted-arithmetic) value, as store_raw
// rounds it; the fixed-point storage goes through the conserving store
template <int ST>
__device__ __forceinline__ typename Storage<ST>::T enc_raw(float v) {
  if constexpr (ST == LBM_STORE_F32) return v;
  else if constexpr (ST == LBM_STORE_F16S) return __float2half_rn(v);
  else return __float2bfloat16_rn(v);
}

// Moments, collision and encoding of one lane's V nodes of a plain segment
// (lean_collide_store without its stores): raw[i][k] is node i's stored
// post-collision population k.  mine: this lane's nodes are stored by the
// caller (not by the marked-lane kernel).
template <int MODEL, bool PL, int ST, int V, int FORCE>
__device__ __forceinline__ void aa_collide_encode(const FusedParams& p, float (&h)[V][9], int y, int x0, bool mine,
                                                  typename Storage<ST>::T (&raw)[V][9]) {
  const bool live = x0 < p.nx && mine;
  const size_t rowoff = (size_t)y * p.pitch;
  float tau[V];
  if (PL) {
    if (live) {
      load_vec<float, V>(p.tau + rowoff + x0, tau);
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) tau[i] = 1.0f;
    }
  }
  float mass[V];
  if constexpr (ST == LBM_STORE_I16S) {
#pragma unroll
    for (int i = 0; i < V; ++i) mass[i] = node_sum(h[i]);
  }
#pragma unroll
  for (int i = 0; i < V; ++i) {
    const float st = collide_lean<FusedParams, MODEL, PL, FORCE>(p, h[i], PL ? tau[i] : 0.0f);
    if (PL) tau[i] = st;
  }
  if (PL && live) store_vec<float, V>(p.tau + rowoff + x0, tau);
  if constexpr (ST == LBM_STORE_I16S) {
    int bad = 0;
#pragma unroll
    for (int i = 0; i < V; ++i) {
      unsigned b[9];
      const int out = i16_conserve_bits(h[i], mass[i], b, p.fiq);
      if (live && x0 + i < p.nx) bad |= out;
#pragma unroll
      for (int k = 0; k < 9; ++k) raw[i][k] = (short)(unsigned short)(b[k] & 0xffffu);
    }
    report_bits(p.status, bad);
  } else {
    bool bad = false;
#pragma unroll
    for (int i = 0; i < V; ++i) {
      bad = bad || (live && x0 + i < p.nx && not_finite(h[i][0]));
#pragma unroll
      for (int k = 0; k < 9; ++k) raw[i][k] = enc_raw<ST>(h[i][k]);
    }
    report_status(p.status, LBM_STATUS_NONFINITE, bad);
  }
}

// Elements [A, B) of v stored at p + A in aligned pieces of at most 16 B
// (A, B known at compile time, p aligned to V elements).
template <typename T, int A, int B>
__host__ __device__ constexpr int store_piece() {
  int n = 16 / (int)sizeof(T);
  while (n > 1 && (A % n != 0 || A + n > B)) n /= 2;
  return n;
}
template <typename T, int V, int A, int B>
__device__ __forceinline__ void store_part(T* p, const T (&v)[V]) {
  if constexpr (A < B) {
    constexpr int n = store_piece<T, A, B>();
    using R = typename Raw<n * (int)sizeof(T)>::type;
    R r;
    memcpy(&r, &v[A], sizeof(R));
    *reinterpret_cast<R*>(p + A) = r;
    store_part<T, V, A + n, B>(p, v);
  }
}

// Phase A stores of one lane: node x writes population opp(k) to slot k of
// x - c_k.  Along x that is a shift by one element, so the lane assembles the
// aligned V elements [x0, x0 + V) of each row from its own nodes and one
// neighbour lane's node (a warp shuffle) and stores them as one vector when
// all V producers are stored here; the element whose producer is in the next
// or previous segment is that segment's to write (one scalar store by its
// lane 0 or lane 31), the wrap-around of x by the lanes holding nodes 0 and
// nx-1, and a marked lane's nodes by the marked-lane kernel.
template <int ST, int V>
__device__ __forceinline__ void aa_scatter(const FusedParams& p, const typename Storage<ST>::T (&raw)[V][9], int y,
                                           int x0, int lane, uint32_t mask) {
  using T = typename Storage<ST>::T;
  constexpr unsigned FULL = 0xffffffffu;
  T* dst = reinterpret_cast<T*>(p.dst);
  const bool mine = !((mask >> lane) & 1u);
  const bool live = x0 < p.nx;
  const bool next_mine = lane < 31 && !((mask >> (lane + 1)) & 1u);
  const bool prev_mine = lane > 0 && !((mask >> (lane - 1)) & 1u);
  const int ilast = p.nx - 1 - x0;  // node nx-1's index in this lane, if in [0, V)
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int o = OPP(k);
    T* row = dst + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch;
    T v[V];
    bool ok[V];
    if (CX(k) == 0) {  // element i <- node i
#pragma unroll
      for (int i = 0; i < V; ++i) {
        v[i] = raw[i][o];
        ok[i] = mine && x0 + i < p.nx;
      }
    } else if (CX(k) == 1) {  // element i <- node i + 1; the last from the next lane's node 0
      const T nxt = from_word<T>(__shfl_down_sync(FULL, to_word(raw[0][o]), 1));
#pragma unroll
      for (int i = 0; i < V; ++i) {
        v[i] = i < V - 1 ? raw[i + 1 < V ? i + 1 : 0][o] : nxt;
        ok[i] = (i < V - 1 ? mine : next_mine) && x0 + i + 1 < p.nx;
      }
    } else {  // element i <- node i - 1; the first from the previous lane's node V-1
      const T prv = from_word<T>(__shfl_up_sync(FULL, to_word(raw[V - 1][o]), 1));
#pragma unroll
      for (int i = 0; i < V; ++i) {
        v[i] = i > 0 ? raw[i > 0 ? i - 1 : 0][o] : prv;
        ok[i] = (i > 0 ? mine : prev_mine) && x0 + i < p.nx;
      }
    }
    bool all = live;
#pragma unroll
    for (int i = 0; i < V; ++i) all = all && ok[i];
    if (all) {
      store_vec<T, V>(row + x0, v);
    } else if (live) {
#pragma unroll
      for (int i = 0; i < V; ++i)
        if (ok[i]) row[x0 + i] = v[i];
    }
    if (CX(k) == 1 && lane == 0 && mine && live) row[wrap(x0 - 1, p.nx)] = raw[0][o];  // node x0 -> x0 - 1
    if (CX(k) == -1 && mine) {
      if (lane == 31 && x0 + V < p.nx) row[x0 + V] = raw[V - 1][o];  // the last node -> next segment
#pragma unroll
      for (int i = 0; i < V; ++i)
        if (i == ilast) row[0] = raw[i][o];  // node nx-1 -> column 0
    }
  }
}

// aa_scatter for an interior segment with no marked lane (x0s > 0,
// x0s + 32 V < nx, mask 0): every producer is stored here, so only the
// segment edges differ from a vector store per lane (16-bit storages: 7 %
// faster in place than the general scatter)
template <int ST, int V>
__device__ __forceinline__ void aa_scatter_interior(const FusedParams& p, const typename Storage<ST>::T (&raw)[V][9],
                                                    int y, int x0, int lane) {
  using T = typename Storage<ST>::T;
  constexpr unsigned FULL = 0xffffffffu;
  T* dst = reinterpret_cast<T*>(p.dst);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int o = OPP(k);
    T* row = dst + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch + x0;
    T v[V];
    if (CX(k) == 0) {
#pragma unroll
      for (int i = 0; i < V; ++i) v[i] = raw[i][o];
      store_vec<T, V>(row, v);
    } else if (CX(k) == 1) {  // element i <- node i + 1; node 0 -> x0 - 1
      const T nxt = from_word<T>(__shfl_down_sync(FULL, to_word(raw[0][o]), 1));
#pragma unroll
      for (int i = 0; i < V; ++i) v[i] = i < V - 1 ? raw[i + 1 < V ? i + 1 : 0][o] : nxt;
      if (lane < 31) store_vec<T, V>(row, v);
      else store_part<T, V, 0, V - 1>(row, v);
      if (lane == 0) row[-1] = raw[0][o];
    } else {  // element i <- node i - 1; node V-1 -> x0 + V
      const T prv = from_word<T>(__shfl_up_sync(FULL, to_word(raw[V - 1][o]), 1));
#pragma unroll
      for (int i = 0; i < V; ++i) v[i] = i > 0 ? raw[i > 0 ? i - 1 : 0][o] : prv;
      if (lane > 0) store_vec<T, V>(row, v);
      else store_part<T, V, 1, V>(row, v);
      if (lane == 31) row[V] = raw[V - 1][o];
    }
  }
}

// The plain segments of one in-place step (every segment; marked lanes are
// gathered but stored by k_aa_lanes).  Grid as k_fused_bulk.
template <int MODEL, bool PL, int ST, int V, int FORCE, int PHASE>
__global__ void __launch_bounds__(256) k_aa_bulk(const FusedParams p) {
  using T = typename Storage<ST>::T;
  const int lane = threadIdx.x & 31;
  const int y = blockIdx.y + gridDim.y * blockIdx.z;
  const int seg = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (seg >= p.nseg || y >= p.ny) return;  // whole warps
  uint32_t mask;
  ldg_early(p.lane_mask + (size_t)y * p.nseg + seg, mask);
  const int x0s = seg * 32 * V, x0 = x0s + lane * V;
  float h[V][9];
  if constexpr (PHASE == AA_PHASE_A) {
    if (x0s > 0 && x0s + 32 * V < p.nx) gather_interior<FusedParams, ST, V>(p, y, x0, lane, h);
    else gather_edge<FusedParams, ST, V>(p, y, x0, lane, h);
    if (mask == 0xffffffffu) return;  // uniform over the warp
    T raw[V][9];
    aa_collide_encode<MODEL, PL, ST, V, FORCE>(p, h, y, x0, !((mask >> lane) & 1u), raw);
    // (fp32 takes the general scatter only: both forms inlined cost it 5 registers and more time)
    if (ST != LBM_STORE_F32 && mask == 0u && x0s > 0 && x0s + 32 * V < p.nx)
      aa_scatter_interior<ST, V>(p, raw, y, x0, lane);
    else aa_scatter<ST, V>(p, raw, y, x0, lane, mask);
  } else {
    // f_k(x) is in slot opp(k) of x itself
    const T* src = reinterpret_cast<const T*>(p.src) + (size_t)y * p.pitch + x0;
    const bool live = x0 < p.nx;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float c[V];
      if (live) {
        load_raw<ST, V>(src + (size_t)OPP(k) * p.plane, c, fix_of(p));
      } else {
#pragma unroll
        for (int i = 0; i < V; ++i) c[i] = 0.0f;
      }
#pragma unroll
      for (int i = 0; i < V; ++i) h[i][k] = c[i];
    }
    if (mask == 0xffffffffu) return;
    lean_collide_store<FusedParams, MODEL, PL, ST, V, FORCE>(p, h, y, x0, (mask >> lane) & 1u);
  }
}

// One node of a marked lane in an in-place step: lane_node's general path
// (bounce-back links, boundary programs, saved moments) with the phase's
// reads and writes.  A node outside the collision group is left as it is:
// nothing streams from it and its locations are never written.
template <int MODEL, bool PL, int ST, int PHASE>
__device__ __forceinline__ void aa_lane_node(const FusedParams& p, int y, int x) {
  using S = Storage<ST>;
  using T = typename S::T;
  T* buf = reinterpret_cast<T*>(p.dst);
  const T* src = reinterpret_cast<const T*>(p.src);
  const float Fx = p.has_force ? p.gx : 0.0f, Fy = p.has_force ? p.gy : 0.0f;
  if (x >= p.nx) return;
  const size_t q = (size_t)y * p.pitch + x;
  const unsigned code = p.code[q];
  if (!(code & LBM_CODE_ACTIVE)) return;
  float f[9];
  if constexpr (PHASE == AA_PHASE_A) {
    gather_node<ST>(p, x, y, f);
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) f[k] = S::dec(load1(src + (size_t)OPP(k) * p.plane + q), p.wsh[k], p.fq);
  }
  const unsigned prog = code >> LBM_CODE_PROG_SHIFT;
  for (int s = 0; prog && s < LBM_PROG_LEN; ++s) {
    const int bi = p.prog[prog][s];
    if (bi < 0) break;
    apply_bc<ST>(p, bi, x, y, f);
  }
  float mass = 0.0f;
  if constexpr (ST == LBM_STORE_I16S)
    mass = prog ? i16_mass_rounded(f, p.wsh, p.fiq, p.fq) : i16_mass(f, p.wsh, p.fiq, p.fq);
  const float rho = ((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])) + f[8];
  const float jx = (f[1] - f[3]) + (f[5] - f[6]) + (f[8] - f[7]);
  const float jy = (f[2] - f[4]) + (f[5] + f[6]) - (f[7] + f[8]);
  const float ux = (jx + 0.5f * Fx) / rho, uy = (jy + 0.5f * Fy) / rho;
  if (code & LBM_CODE_SAVE) {
    p.mom_out[q] = rho;
    p.mom_out[p.plane + q] = ux;
    p.mom_out[2 * p.plane + q] = uy;
  }
  const float st = relax_collide<MODEL, PL>(p, f, rho, ux, uy, Fx, Fy, PL ? p.tau[q] : 0.0f);
  if (PL) p.tau[q] = st;
  T v[9];
  if constexpr (ST == LBM_STORE_I16S) {
    short n[9];
    report_bits(p.status, i16_store_node(f, p.wsh, mass, n, p.fiq));
#pragma unroll
    for (int k = 0; k < 9; ++k) v[k] = n[k];
  } else {
    report_status(p.status, LBM_STATUS_NONFINITE, not_finite(f[0]));
#pragma unroll
    for (int k = 0; k < 9; ++k) v[k] = S::enc(f[k], p.wsh[k], p.fiq);
  }
  if constexpr (PHASE == AA_PHASE_A) {
    buf[q] = v[0];
#pragma unroll
    for (int k = 1; k < 9; ++k) {
      if (code & (1u << (k - 1))) {
        buf[(size_t)OPP(k) * p.plane + q] = v[OPP(k)];
      } else {
        const int xs = wrap(x - CX(k), p.nx), ys = wrap(y - CY(k), p.ny);
        buf[(size_t)k * p.plane + (size_t)ys * p.pitch + xs] = v[OPP(k)];
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) buf[(size_t)k * p.plane + q] = v[k];
  }
}

// V threads per listed lane, one per node (as k_fused_lanes)
template <int MODEL, bool PL, int ST, int V, int PHASE>
__global__ void __launch_bounds__(128) k_aa_lanes(const FusedParams p) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)p.nlanes * V) return;
  const int e = p.lanes[t / V];
  const int item = e >> 5, lane = e & 31;
  const int y = item / p.nseg;
  aa_lane_node<MODEL, PL, ST, PHASE>(p, y, (item - y * p.nseg) * 32 * V + lane * V + (int)(t % V));
}

// The post-stream populations of the nodes boundary programs read, before
// the step overwrites them (one thread per listed node).
template <int ST, int PHASE>
__global__ void k_aa_sites(const FusedParams p) {
  using S = Storage<ST>;
  using T = typename S::T;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.aa_nsites) return;
  const int q = p.aa_sites[t];
  const int y = q / p.pitch, x = q - y * p.pitch;
  float g[9];
  if constexpr (PHASE == AA_PHASE_A) {
    gather_node<ST>(p, x, y, g);
  } else {
    const T* src = reinterpret_cast<const T*>(p.src);
#pragma unroll
    for (int k = 0; k < 9; ++k) g[k] = S::dec(load1(src + (size_t)OPP(k) * p.plane + q), p.wsh[k], p.fq);
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) p.aa_vals[(size_t)t * 9 + k] = g[k];
}

// After a phase A: every pair of slots that a streaming link joins, slot k of
// x and slot opp(k) of x + c_k, swaps its two values (one thread per node,
// for k = 1, 2, 5, 6, so each pair has one owner); bounce-back slots are
// already in place.  The buffer is in pull layout afterwards.
template <int ST>
__global__ void k_aa_swap(const FusedParams p) {
  using T = typename Storage<ST>::T;
  T* buf = reinterpret_cast<T*>(p.dst);
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= p.nx) return;
  for (int y = blockIdx.y; y < p.ny; y += gridDim.y) {
    if (!(p.code[(size_t)y * p.pitch + x] & LBM_CODE_ACTIVE)) continue;
#pragma unroll
    for (int k = 1; k < 9; ++k) {
      if (k != 1 && k != 2 && k != 5 && k != 6) continue;
      const int tx = wrap(x + CX(k), p.nx), ty = wrap(y + CY(k), p.ny);
      const unsigned ct = p.code[(size_t)ty * p.pitch + tx];
      if (!(ct & LBM_CODE_ACTIVE) || (ct & (1u << (k - 1)))) continue;  // no stream from x to x + c_k
      T* a = buf + (size_t)k * p.plane + (size_t)y * p.pitch + x;
      T* b = buf + (size_t)OPP(k) * p.plane + (size_t)ty * p.pitch + tx;
      const T va = *a;
      *a = *b;
      *b = va;
    }
  }
}

// ------------------------------------------------------------ launchers
template <int MODEL, bool PL, int ST, int V, int PHASE>
int launch_aa_mp(const FusedParams& p, cudaStream_t s, cudaStream_t s2) {
  if (p.nlanes > 0) {
    k_aa_lanes<MODEL, PL, ST, V, PHASE><<<(unsigned)(((long long)p.nlanes * V + 127) / 128), 128, 0, s2>>>(p);
    int rc = lbm_err::launch("in-place step (marked lanes)");
    if (rc) return rc;
  }
  const int wpb = p.nseg < 8 ? p.nseg : 8;
  const unsigned gy = p.ny < 65535 ? (unsigned)p.ny : 65535u;
  const dim3 grid((unsigned)((p.nseg + wpb - 1) / wpb), gy, (unsigned)((p.ny + gy - 1) / gy));
  if (p.has_force) k_aa_bulk<MODEL, PL, ST, V, 1, PHASE><<<grid, 32 * wpb, 0, s>>>(p);
  else k_aa_bulk<MODEL, PL, ST, V, 0, PHASE><<<grid, 32 * wpb, 0, s>>>(p);
  return lbm_err::launch("in-place step (plain segments)");
}

template <int ST, int V, int PHASE>
int launch_aa_v(const FusedParams& p, cudaStream_t s, cudaStream_t s2) {
  const bool pl = p.fluid_model == LBM_POWERLAW;
  switch (p.model * 2 + (pl ? 1 : 0)) {
    case 0: return launch_aa_mp<LBM_BGK, false, ST, V, PHASE>(p, s, s2);
    case 1: return launch_aa_mp<LBM_BGK, true, ST, V, PHASE>(p, s, s2);
    case 2: return launch_aa_mp<LBM_TRT, false, ST, V, PHASE>(p, s, s2);
    case 3: return launch_aa_mp<LBM_TRT, true, ST, V, PHASE>(p, s, s2);
    case 4: return launch_aa_mp<LBM_MRT, false, ST, V, PHASE>(p, s, s2);
    case 5: return launch_aa_mp<LBM_MRT, true, ST, V, PHASE>(p, s, s2);
    default: return lbm_err::set(LBM_ERR_ARG, "unknown collision model %d", p.model);
  }
}

// one in-place step (p.aa = its phase): the marked lanes on s2, the plain
// segments on s; the sites of boundary reads must already be gathered
template <int ST>
int launch_aa(const FusedParams& p, int V, cudaStream_t s, cudaStream_t s2);

template <int ST>
int launch_aa_sites(const FusedParams& p, cudaStream_t s) {
  if (p.aa_nsites <= 0) return LBM_OK;
  const unsigned blocks = (unsigned)((p.aa_nsites + 127) / 128);
  if (p.aa == AA_PHASE_A) k_aa_sites<ST, AA_PHASE_A><<<blocks, 128, 0, s>>>(p);
  else k_aa_sites<ST, AA_PHASE_B><<<blocks, 128, 0, s>>>(p);
  return lbm_err::launch("in-place step (boundary read sites)");
}

template <int ST>
int launch_aa_swap(const FusedParams& p, cudaStream_t s) {
  const unsigned gy = p.ny < 4096 ? (unsigned)p.ny : 4096u;
  k_aa_swap<ST><<<dim3((unsigned)((p.nx + 127) / 128), gy), 128, 0, s>>>(p);
  return lbm_err::launch("in-place step (layout swap)");
}

}  // namespace lbm

#define LBM_AA_EXTERN(ST)                                                              \
  namespace lbm {                                                                      \
  extern template int launch_aa<ST>(const FusedParams&, int, cudaStream_t, cudaStream_t); \
  extern template int launch_aa_sites<ST>(const FusedParams&, cudaStream_t);           \
  extern template int launch_aa_swap<ST>(const FusedParams&, cudaStream_t);            \
  }

#define LBM_AA_INSTANTIATE(ST, VA, VB)                                                          \
  namespace lbm {                                                                               \
  template <>                                                                                   \
  int launch_aa<ST>(const FusedParams& p, int V, cudaStream_t s, cudaStream_t s2) {             \
    if (p.aa != AA_PHASE_A && p.aa != AA_PHASE_B)                                               \
      return lbm_err::set(LBM_ERR_ARG, "in-place step phase %d", p.aa);                         \
    if (V == VA)                                                                                \
      return p.aa == AA_PHASE_A ? launch_aa_v<ST, VA, AA_PHASE_A>(p, s, s2)                     \
                                : launch_aa_v<ST, VA, AA_PHASE_B>(p, s, s2);                    \
    if (V == VB)                                                                                \
      return p.aa == AA_PHASE_A ? launch_aa_v<ST, VB, AA_PHASE_A>(p, s, s2)                     \
                                : launch_aa_v<ST, VB, AA_PHASE_B>(p, s, s2);                    \
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "nodes_per_thread %d not built for this storage", V); \
  }                                                                                             \
  template int launch_aa_sites<ST>(const FusedParams&, cudaStream_t);                           \
  template int launch_aa_swap<ST>(const FusedParams&, cudaStream_t);                            \
  }
