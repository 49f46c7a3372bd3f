// Fused pull-scheme D2Q9 step for sm_103a.
//
// One launch = the boundary pass of step n-1 (stream carriers compiled into
// per-node bounce bits, then the rewrite boundaries in insertion order) and
// the moments + collision of step n, for the whole lattice.  State between
// launches is the post-collision population set; see lbm_gb300.h.
//
// Work decomposition: one warp owns one row segment of 32*V x-consecutive
// nodes; each lane owns V nodes.  Population k of the V nodes is fetched with
// one aligned V-wide load from row (y - cy_k); the x shift by cx_k = +-1 is
// done with one warp shuffle, lane 0 / lane 31 fetching the single element
// that crosses the segment edge.  Every population element of the source is
// therefore read from DRAM once and every output element written once
// (72 B per fp32 lattice update), with 128-bit loads and stores.
//
// Segments whose nodes are all plain (collide, stream all links, no boundary
// program, no saved moments) skip the per-node code load entirely; the others
// take the per-node path (bounce-back links, boundary programs, saved moments).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "lbm_common.cuh"

namespace lbm {

struct FusedParams {
  int nx, ny, pitch, nseg;
  size_t plane;
  const void* src;
  void* dst;
  const float* mom_in;
  float* mom_out;
  const uint16_t* code;
  const uint8_t* seg_flags;
  float* tau;
  int model, fluid_model, has_force;
  float omega, omega_a, magic, tau_min, tau_max, pl_m, pl_n;
  float s[9];
  float gx, gy;
  int nbc;
  LbmBoundary bc[LBM_MAX_BC];
  int8_t prog[LBM_MAX_PROG][LBM_PROG_LEN];
  // single-component Shan-Chen (k_fused_sc): interaction strength, the
  // lattice's uniform temperature and the pseudopotential
  int sc;
  float g_coh, sc_T;
  LbmEos eos;
  // two-pass direct step: segments with a nonzero flag, in (y * nseg + seg)
  // order, handled by k_fused_special; k_fused_bulk skips them
  const int32_t* special;
  int nspecial;
  // prefetching two-pass step: the plain segments, same order
  const int32_t* plain;
  int nplain;
  int tune;  // LBM_PIPE_ASYNC / LBM_PIPE_PREFETCH tuning index
  // lane-granular two-pass step: bit l of lane_mask[y * nseg + seg] marks a
  // lane with a node that is not plain; lanes lists those lanes
  // ((y * nseg + seg) * 32 + lane), handled by k_fused_lanes
  const uint32_t* lane_mask;
  const int32_t* lanes;
  int nlanes;
  // 16-bit storage holds f_k - wsh[k], wsh[k] = w_k * rho_ref (the plan's
  // reference density); fp32 storage ignores it
  float wsh[9];
  float rho_shift;  // sum_k wsh[k]
  float mwsh[9];    // MRT moments of the shift, M wsh
  // fixed-point storage (LBM_STORE_I16S): step fq = 2^-e, its inverse fiq,
  // and foff = (2^23 + 2^15) fq (the pair decode's offset)
  float fq, fiq, foff;
  // sticky device status word (LBM_STATUS_* bits), or null: stores that
  // leave the fixed-point range or hold a non-finite value set a bit
  int32_t* status;
  // LBM_PIPE_ASYNC: clock-cycle budget of each wait on a staged copy
  long long wait_cycles;
  // in-place AA-pattern step (lbm_fused_aa.cuh): the phase of the running
  // launch (0 outside an AA step, AA_PHASE_A / AA_PHASE_B), and the
  // post-stream populations of the nodes boundary programs read
  // (aa_vals[s * 9 + k] for the node at plane offset aa_sites[s], ascending),
  // gathered before the step overwrites them
  int aa;
  const int32_t* aa_sites;
  int aa_nsites;
  float* aa_vals;
};
constexpr int AA_PHASE_A = 1, AA_PHASE_B = 2;

// The fields the lean (plain-segment) kernels read: a compact copy of
// FusedParams that a batched kernel can stage per warp in shared memory.
struct LeanParams {
  int nx, ny, pitch, nseg;
  size_t plane;
  const void* src;
  void* dst;
  float* tau;
  float omega, omega_a, magic, tau_min, tau_max, pl_m, pl_n;
  float gx, gy;
  float rho_shift;
  uint32_t nseg_mul;  // item / nseg = (umulhi(item, nseg_mul) + item) >> nseg_shift
  int nseg_shift;
  float s[9];
  float wsh[9];
  float mwsh[9];
  // single-component Shan-Chen
  float g_coh, sc_T;
  LbmEos eos;
  int sc_rows;  // rows of a strip item
  int model;    // collision model (batched kernels branch on it per lattice)
  const uint32_t* lane_mask;  // lanes not to store (FusedParams::lane_mask), or null
  float fq, fiq, foff;        // fixed-point step (FusedParams::fq)
  int32_t* status;            // FusedParams::status
};

// Division by an invariant divisor d (1 <= d < 2^31) as a multiply-high and
// shift (Granlund and Montgomery, "Division by invariant integers using
// multiplication", 1994, round-up variant): l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (mulhi(m, n) + n) >> l.
inline void fast_div_setup(uint32_t d, uint32_t* mul, int* shift) {
  int l = 0;
  while ((1ull << l) < d) ++l;
  *mul = (uint32_t)((((1ull << 32) * ((1ull << l) - d)) / d) + 1);
  *shift = l;
}
__device__ __forceinline__ int fast_div(int n, uint32_t mul, int shift) {
  const unsigned long long t = __umulhi((uint32_t)n, mul);
  return (int)((t + (uint32_t)n) >> shift);
}

inline LeanParams lean_of(const FusedParams& f) {
  LeanParams l;
  l.nx = f.nx;
  l.ny = f.ny;
  l.pitch = f.pitch;
  l.nseg = f.nseg;
  l.plane = f.plane;
  l.src = f.src;
  l.dst = f.dst;
  l.tau = f.tau;
  l.omega = f.omega;
  l.omega_a = f.omega_a;
  l.magic = f.magic;
  l.tau_min = f.tau_min;
  l.tau_max = f.tau_max;
  l.pl_m = f.pl_m;
  l.pl_n = f.pl_n;
  l.gx = f.gx;
  l.gy = f.gy;
  l.rho_shift = f.rho_shift;
  fast_div_setup((uint32_t)f.nseg, &l.nseg_mul, &l.nseg_shift);
  for (int a = 0; a < 9; ++a) {
    l.s[a] = f.s[a];
    l.wsh[a] = f.wsh[a];
    l.mwsh[a] = f.mwsh[a];
  }
  l.g_coh = f.g_coh;
  l.sc_T = f.sc_T;
  l.eos = f.eos;
  l.sc_rows = 16;
  l.model = f.model;
  l.lane_mask = f.lane_mask;
  l.fq = f.fq;
  l.fiq = f.fiq;
  l.foff = f.foff;
  l.status = f.status;
  return l;
}

// word-wise copy of a trivially copyable struct by `n` cooperating threads
template <typename T>
__device__ __forceinline__ void copy_words(T* dst, const T* src, int tid, int n) {
  static_assert(sizeof(T) % 4 == 0, "struct size must be a multiple of 4 bytes");
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
  for (int i = tid; i < (int)(sizeof(T) / 4); i += n) d[i] = s[i];
}

// ------------------------------------------------------------ storage
template <int ST>
struct Storage;
// Every storage decodes with (stored value, shift w, fixed-point step q) and
// encodes with (value, shift w, inverse step iq); only the fixed-point
// storage reads q and iq.
template <>
struct Storage<LBM_STORE_F32> {
  using T = float;
  static __device__ __forceinline__ float dec(T v, float, float) { return v; }
  static __device__ __forceinline__ double dec64(T v, float, float) { return (double)v; }
  static __device__ __forceinline__ T enc(float v, float, float) { return v; }
};
template <>
struct Storage<LBM_STORE_F16S> {
  using T = __half;
  static __device__ __forceinline__ float dec(T v, float w, float) { return __half2float(v) + w; }
  static __device__ __forceinline__ double dec64(T v, float w, float) { return (double)__half2float(v) + (double)w; }
  static __device__ __forceinline__ T enc(float v, float w, float) { return __float2half_rn(v - w); }
};
template <>
struct Storage<LBM_STORE_BF16S> {
  using T = __nv_bfloat16;
  static __device__ __forceinline__ float dec(T v, float w, float) { return __bfloat162float(v) + w; }
  static __device__ __forceinline__ double dec64(T v, float w, float) {
    return (double)__bfloat162float(v) + (double)w;
  }
  static __device__ __forceinline__ T enc(float v, float w, float) { return __float2bfloat16_rn(v - w); }
};

// 16-bit fixed point, shifted (LBM_STORE_I16S): the state holds the integer
// n = round((f_k - w_k rho_ref) / Q) as int16, with the plan's step
// Q = 2^-e (LbmPlanDesc.fixed_exp, default e = 19), so |f_k - w_k rho_ref| <
// 2^15 Q (1/16 at the default).  Every stored value is a multiple of Q below
// 2^15 Q, so a sum of a node's nine values is exact in FP32 (9 * 2^15 <
// 2^24): a collision can store its populations with their sum, the node's
// mass, unchanged to the bit (i16_conserve_bits), which floating-point storage
// cannot.  Rounding is to nearest even through the 1.5 * 2^23 magic
// constant (x + 1.5 * 2^23 rounds x to an integer for |x| < 2^22); values
// outside the range saturate, and the store reports them.
constexpr float I16_MAGIC = 12582912.0f;  // 1.5 * 2^23
constexpr float I16_LO = I16_MAGIC - 32768.0f, I16_HI = I16_MAGIC + 32767.0f;

// the nearest step count of a shifted value, saturated, as an integer float
__device__ __forceinline__ float i16_steps(float h, float iq) {
  const float n = fmaf(h, iq, I16_MAGIC) - I16_MAGIC;
  return fminf(fmaxf(n, -32768.0f), 32767.0f);
}
// an integer float in [-32768, 32767] -> its int16 bits (in the low half)
__device__ __forceinline__ unsigned i16_bits(float n) { return __float_as_uint(n + I16_MAGIC) & 0xffffu; }

template <>
struct Storage<LBM_STORE_I16S> {
  using T = short;
  static __device__ __forceinline__ float dec(T v, float w, float q) { return fmaf((float)v, q, w); }
  static __device__ __forceinline__ double dec64(T v, float w, float q) {
    return (double)v * (double)q + (double)w;
  }
  static __device__ __forceinline__ T enc(float v, float w, float iq) { return (short)i16_bits(i16_steps(v - w, iq)); }
};

// Mass-conserving quantisation of one node's post-collision populations
// for the fixed-point storage: populations 1..8 round to their nearest
// step, and population 0 takes the rest of the node's pre-collision mass
// d (a sum of stored values, exact), so the stored sum equals d exactly.
// Colliding nodes without a boundary program conserve so, and a closed
// lattice keeps its mass to the bit.  A node whose populations a boundary
// program rewrote holds values that are not multiples of Q; its d is the
// node's post-boundary mass rounded once to the nearest step
// (i16_mass_rounded), not the sum of its nine values each rounded: that sum
// carries up to 4.5 steps of rounding per node and step, which an open
// channel whose outlet does not pin the density (PressureNEEM writes
// rho_value to total_rho only) accumulates as a drift of its mass.
// h: shifted post-collision values; iq = 1 / Q.  b[k]: the int16 bits of the
// stored step counts in the low half of each word.  The rounding yields
// t = n + 1.5 * 2^23 as a float, whose bit pattern is that of 1.5 * 2^23
// plus n, so the step counts add up as integers without a conversion.
// Returns LBM_STATUS_SATURATED when a value left the range (or was NaN),
// plus LBM_STATUS_NONFINITE when the node's values are NaN (a NaN in a
// node's moments reaches all nine populations, so population 1 tells).
// The range test is on the largest |h_k| (one max per value): below 32767.5
// steps every value rounds into the int16 range, and only then are the
// values stored unclamped; a value within half a step of -32768 steps also
// takes the clamping path (and is reported), which stores the same bits.
__device__ __forceinline__ int i16_conserve_bits(const float (&h)[9], float d, unsigned (&b)[9], float iq) {
  const unsigned mb = __float_as_uint(I16_MAGIC);
  unsigned s = 0u;  // sum of the rounded bit patterns of populations 1..8
  float m = 0.0f;   // largest |h_k| of populations 1..8
#pragma unroll
  for (int k = 1; k < 9; ++k) {
    b[k] = __float_as_uint(fmaf(h[k], iq, I16_MAGIC));
    s += b[k];
    m = fmaxf(m, fabsf(h[k]));
  }
  const bool out = !(m * iq < 32767.5f) || h[1] != h[1];
  if (out) {  // saturated or not finite: clamp (a NaN clamps to -32768)
    s = 0u;
#pragma unroll
    for (int k = 1; k < 9; ++k) {
      b[k] = __float_as_uint(fminf(fmaxf(fmaf(h[k], iq, I16_MAGIC), I16_LO), I16_HI));
      s += b[k];
    }
  }
  // d / Q is an integer of magnitude below 9 * 2^15, so d / Q + 1.5 * 2^23 is
  // exact; the steps of populations 1..8 sum to s - 8 * bits(1.5 * 2^23)
  const int n0 = (int)(__float_as_uint(fmaf(d, iq, I16_MAGIC)) - mb) - (int)(s - 8u * mb);
  b[0] = (unsigned)min(max(n0, -32768), 32767);
  const bool sat = out || n0 < -32768 || n0 > 32767;
  return (sat ? LBM_STATUS_SATURATED : 0) | (h[1] != h[1] ? LBM_STATUS_NONFINITE : 0);
}

// The general (unshifted) path holds f = n Q + w rounded to FP32; the nearest
// step of f - w recovers n exactly (the FP32 rounding is far below Q / 2).
// i16_mass: a node's stored sum from its unshifted values (exact), and
// i16_store_node: the conserving quantisation of a node's post-collision f
// as int16 step counts (the LBM_STATUS_* bits of i16_conserve_bits).
__device__ __forceinline__ float i16_mass(const float (&f)[9], const float (&w)[9], float iq, float q) {
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 9; ++k) s += i16_steps(f[k] - w[k], iq);
  return s * q;
}
// a boundary node's post-boundary mass, summed in float and rounded once
// to the nearest step
__device__ __forceinline__ float i16_mass_rounded(const float (&f)[9], const float (&w)[9], float iq, float q) {
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 9; ++k) s += f[k] - w[k];
  return (fmaf(s, iq, I16_MAGIC) - I16_MAGIC) * q;
}
__device__ __forceinline__ int i16_store_node(const float (&f)[9], const float (&w)[9], float mass,
                                              short (&out)[9], float iq) {
  float h[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) h[k] = f[k] - w[k];
  unsigned b[9];
  const int bad = i16_conserve_bits(h, mass, b, iq);
#pragma unroll
  for (int k = 0; k < 9; ++k) out[k] = (short)(b[k] & 0xffffu);
  return bad;
}

// a post-collision value that is not finite (NaN or infinite)
__device__ __forceinline__ bool not_finite(float v) { return !(fabsf(v) <= 3.402823466e38f); }

// Record a status bit in the sticky status word, if the plan has one, for
// the lanes of the calling warp that pass bad.  One lane of the warp does
// the atomic, and only when the bit is not yet set: a diverged lattice has
// every node bad on every step, and an atomic per node and step on one word
// would serialise the whole launch.
__device__ __forceinline__ void report_status(int32_t* status, int bit, bool bad = true) {
  const unsigned am = __activemask();
  const unsigned any = __ballot_sync(am, bad);
  if (!any || !status) return;
  if ((int)(threadIdx.x & 31) == __ffs(any) - 1) {
    if (!(*(volatile const int32_t*)status & bit)) atomicOr(status, bit);
  }
}
// the same for a set of LBM_STATUS_* bits per lane (OR over the warp)
__device__ __forceinline__ void report_bits(int32_t* status, int bits) {
  const unsigned am = __activemask();
  const int all = __reduce_or_sync(am, (unsigned)bits);
  if (!all || !status) return;
  if ((int)(threadIdx.x & 31) == __ffs(am) - 1) {
    if ((*(volatile const int32_t*)status & all) != all) atomicOr(status, all);
  }
}

template <int BYTES>
struct Raw;
template <>
struct Raw<16> { using type = uint4; };
template <>
struct Raw<8> { using type = uint2; };
template <>
struct Raw<4> { using type = unsigned int; };
template <>
struct Raw<2> { using type = unsigned short; };

// Aligned loads/stores of V consecutive elements in pieces of at most 16 B.
template <typename T, int V>
__device__ __forceinline__ void load_vec(const T* p, T (&out)[V]) {
  constexpr int B = sizeof(T) * V > 16 ? 16 : sizeof(T) * V;
  constexpr int E = B / sizeof(T);
  using R = typename Raw<B>::type;
#pragma unroll
  for (int c = 0; c < V / E; ++c) {
    R r = __ldg(reinterpret_cast<const R*>(p + c * E));
    memcpy(&out[c * E], &r, B);
  }
}
template <typename T, int V>
__device__ __forceinline__ void store_vec(T* p, const T (&in)[V]) {
  constexpr int B = sizeof(T) * V > 16 ? 16 : sizeof(T) * V;
  constexpr int E = B / sizeof(T);
  using R = typename Raw<B>::type;
#pragma unroll
  for (int c = 0; c < V / E; ++c) {
    R r;
    memcpy(&r, &in[c * E], B);
    __stcs(reinterpret_cast<R*>(p + c * E), r);
  }
}
template <typename T>
__device__ __forceinline__ T load1(const T* p) {
  using R = typename Raw<sizeof(T)>::type;
  R r = __ldg(reinterpret_cast<const R*>(p));
  T out;
  memcpy(&out, &r, sizeof(T));
  return out;
}

__device__ __forceinline__ int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// population k is unknown for a plane boundary of direction dir
// (BoundaryCondition.py:63-72): exactly the links with c_k . c_dir = -1
__host__ __device__ constexpr bool is_unknown(int dir, int k) {
  return CX(k) * CX(dir) + CY(k) * CY(dir) == -1;
}

// Post-stream populations of node (x, y): the stream carriers' result, read
// from the post-collision source with the node's bounce bits.
template <int ST>
__device__ __forceinline__ void gather_node(const FusedParams& p, int x, int y, float g[9]) {
  using S = Storage<ST>;
  using T = typename S::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  const unsigned code = p.code[(size_t)y * p.pitch + x];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    if (k > 0 && (code & (1u << (k - 1)))) {
      g[k] = S::dec(load1(src + OPP(k) * p.plane + (size_t)y * p.pitch + x), p.wsh[OPP(k)], p.fq);
    } else {
      const int xs = wrap(x - CX(k), p.nx), ys = wrap(y - CY(k), p.ny);
      g[k] = S::dec(load1(src + k * p.plane + (size_t)ys * p.pitch + xs), p.wsh[k], p.fq);
    }
  }
}

// Post-stream populations of node (x, y) that a boundary program reads.  An
// in-place AA step overwrites them while it runs, so it gathers them into
// p.aa_vals first and a program looks them up there (binary search of the
// node's plane offset); every other step pulls them from its source.
template <int ST>
__device__ __forceinline__ void read_site(const FusedParams& p, int x, int y, float g[9]) {
  if (!p.aa) {
    gather_node<ST>(p, x, y, g);
    return;
  }
  const int q = y * p.pitch + x;
  int lo = 0, hi = p.aa_nsites - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (p.aa_sites[mid] < q) lo = mid + 1;
    else hi = mid;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) g[k] = p.aa_nsites > 0 ? p.aa_vals[(size_t)lo * 9 + k] : 0.0f;
}

__device__ __forceinline__ float bc_rhow(int dir, float vx, float vy, const float f[9]) {
  // BoundaryCondition.py:119-129
  if (dir == 2) return 1.0f / (1.0f + vy) * (f[0] + f[1] + f[3] + 2.0f * (f[2] + f[5] + f[6]));
  if (dir == 4) return 1.0f / (1.0f - vy) * (f[0] + f[1] + f[3] + 2.0f * (f[4] + f[7] + f[8]));
  if (dir == 1) return 1.0f / (1.0f + vx) * (f[0] + f[2] + f[4] + 2.0f * (f[1] + f[5] + f[8]));
  return 1.0f / (1.0f - vx) * (f[0] + f[2] + f[4] + 2.0f * (f[3] + f[6] + f[7]));
}

__device__ __forceinline__ bool is_unknown_dyn(int dir, int k) {
  return CX(k) * cx_dyn(dir) + CY(k) * cy_dyn(dir) == -1;
}

// One rewrite boundary on node (x, y) whose post-stream populations are f.
// Moments read from mom_in are the start-of-step values the reference reads
// (its rho/vel fields still hold them when the boundary pass runs).
template <int ST>
__device__ __noinline__ void apply_bc(const FusedParams& p, int bci, int x, int y, float f[9]) {
  const LbmBoundary& b = p.bc[bci];
  const int dir = b.direction;
  const int x2 = x - cx_dyn(dir), y2 = y - cy_dyn(dir);
  const size_t q = (size_t)y * p.pitch + x, q2 = (size_t)y2 * p.pitch + x2;
  float Ux = b.velocity[0], Uy = b.velocity[1];
  if (b.velocity_per_node) {
    Ux = b.velocity_per_node[q];
    Uy = b.velocity_per_node[p.plane + q];
  }
  switch (b.kind) {
    case LBM_BC_VELOCITY_EQ: {  // BoundaryCondition.py:137-147
      const float r = bc_rhow(dir, Ux, Uy, f), uu = Ux * Ux + Uy * Uy;
#pragma unroll
      for (int k = 0; k < 9; ++k) f[k] = feq_k(k, r, Ux, Uy, uu);
      break;
    }
    case LBM_BC_VELOCITY_NEEM: {  // BoundaryCondition.py:154-166
      const float r = bc_rhow(dir, Ux, Uy, f), uu = Ux * Ux + Uy * Uy;
      float g[9];
      read_site<ST>(p, x2, y2, g);
      const float r2 = p.mom_in[q2], u2x = p.mom_in[p.plane + q2], u2y = p.mom_in[2 * p.plane + q2];
      const float uu2 = u2x * u2x + u2y * u2y;
#pragma unroll
      for (int k = 0; k < 9; ++k) f[k] = feq_k(k, r, Ux, Uy, uu) + g[k] - feq_k(k, r2, u2x, u2y, uu2);
      break;
    }
    case LBM_BC_VELOCITY_BB: {  // BoundaryCondition.py:85-102
      const float rw = p.mom_in[q];
#pragma unroll
      for (int k = 1; k < 9; ++k)
        if (is_unknown_dyn(dir, k)) f[k] += 6.0f * W(k) * rw * ((float)CX(k) * Ux + (float)CY(k) * Uy);
      break;
    }
    case LBM_BC_PRESSURE_ABC: {  // BoundaryCondition.py:182-205
      const float ux = 1.5f * p.mom_in[p.plane + q] - 0.5f * p.mom_in[p.plane + q2];
      const float uy = 1.5f * p.mom_in[2 * p.plane + q] - 0.5f * p.mom_in[2 * p.plane + q2];
      const float uw2 = ux * ux + uy * uy;
#pragma unroll
      for (int k = 1; k < 9; ++k)
        if (is_unknown_dyn(dir, k)) {
          const float cu = (float)CX(k) * ux + (float)CY(k) * uy;
          f[k] = -f[k] + 2.0f * W(k) * b.rho_value * (1.0f + 4.5f * cu * cu - 1.5f * uw2);
        }
      break;
    }
    case LBM_BC_PRESSURE_NEEM: {  // BoundaryCondition.py:215-226
      float g[9];
      read_site<ST>(p, x2, y2, g);
      const float r = p.mom_in[q], r2 = p.mom_in[q2];
      const float ux = p.mom_in[p.plane + q2], uy = p.mom_in[2 * p.plane + q2];
      const float uu = ux * ux + uy * uy;
#pragma unroll
      for (int k = 1; k < 9; ++k)
        if (is_unknown_dyn(dir, k)) f[k] = feq_k(k, r, ux, uy, uu) + g[k] - feq_k(k, r2, ux, uy, uu);
      break;
    }
    case LBM_BC_OPEN_NEUMANN:  // BoundaryCondition.py:321-334
    case LBM_BC_OPEN_CONV1: {  // BoundaryCondition.py:342-359
      float g[9];
      read_site<ST>(p, x2, y2, g);
      float lam = 0.0f;
      if (b.kind == LBM_BC_OPEN_CONV1) {
        const float ux = p.mom_in[p.plane + q2], uy = p.mom_in[2 * p.plane + q2];
        lam = sqrtf(ux * ux + uy * uy);
      }
#pragma unroll
      for (int k = 1; k < 9; ++k)
        if (is_unknown_dyn(dir, k)) f[k] = b.kind == LBM_BC_OPEN_CONV1 ? (f[k] + lam * g[k]) / (1.0f + lam) : g[k];
      break;
    }
    case LBM_BC_OPEN_EXTRAP: {  // BoundaryCondition.py:400-411
      float g2[9], g3[9];
      read_site<ST>(p, x2, y2, g2);
      read_site<ST>(p, x2 - cx_dyn(dir), y2 - cy_dyn(dir), g3);
#pragma unroll
      for (int k = 1; k < 9; ++k)
        if (is_unknown_dyn(dir, k)) f[k] = 2.0f * g2[k] - g3[k];
      break;
    }
    default:
      break;
  }
}

}  // namespace lbm

namespace lbm {

// Relaxation + collision of one node in place; returns the new relaxation
// state (power law) or the old one.
// FORCE: 1 / 0 = body force on / off at compile time, -1 = read p.has_force
template <int MODEL, bool PL, int FORCE = -1>
__device__ __forceinline__ float relax_collide(const FusedParams& p, float f[9], float rho, float ux, float uy,
                                               float Fx, float Fy, float state) {
  const bool force = FORCE < 0 ? p.has_force != 0 : FORCE == 1;
  if (MODEL == LBM_MRT) {
    float s[9];
#pragma unroll
    for (int a = 0; a < 9; ++a) s[a] = p.s[a];
    if (PL) {
      // CollisionEngine.py:332-377 with the previous step's s7 = s8 = state,
      // then :322-329 for the new rate
      const float uu = ux * ux + uy * uy;
      float fn[9], mn[9], mneq[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) fn[k] = f[k] - feq_k(k, rho, ux, uy, uu);
      mrt_forward(fn, mn);
      s[7] = s[8] = state;
#pragma unroll
      for (int a = 0; a < 9; ++a) mn[a] *= s[a];
      mrt_backward(mn, mneq);
      const float gamma = shear_from_neq(mneq, -1.5f / rho);
      const float t = powerlaw_tau(p.pl_m, p.pl_n, gamma, p.tau_min, p.tau_max);
      state = 1.0f / t;
      s[7] = s[8] = state;
    }
    collide_mrt(f, rho, ux, uy, Fx, Fy, s, force);
    return state;
  }
  float om = p.omega, oa = p.omega_a;
  if (PL) {
    // CollisionEngine.py:80-92 / 166-178 (previous tau), then :72-78 / 157-164
    const float uu = ux * ux + uy * uy;
    float fn[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) fn[k] = f[k] - feq_k(k, rho, ux, uy, uu);
    const float gamma = shear_from_neq(fn, -1.5f / rho / state);
    const float t = powerlaw_tau(p.pl_m, p.pl_n, gamma, p.tau_min, p.tau_max);
    state = t;
    om = 1.0f / t;
    if (MODEL == LBM_TRT) oa = 1.0f / (p.magic / (t - 0.5f) + 0.5f);
  }
  if (MODEL == LBM_BGK) collide_bgk(f, rho, ux, uy, Fx, Fy, om, force);
  else collide_trt(f, rho, ux, uy, Fx, Fy, om, oa, force);
  return state;
}

// GENERAL = false: the segment is known to be plain (no per-node codes);
// FORCE as in relax_collide
template <int MODEL, bool PL, int ST, int V, bool GENERAL = true, int FORCE = -1>
__device__ __forceinline__ void fused_tail(const FusedParams& p, float (&f)[V][9], int y, int seg, int x0,
                                           bool live);

template <int ST, int V>
__device__ __forceinline__ void gather_direct(const FusedParams& p, int y, int seg, int lane, float (&f)[V][9]);

template <int MODEL, bool PL, int ST, int V>
__global__ void __launch_bounds__(256) k_fused(const FusedParams p) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= (long long)p.ny * p.nseg) return;  // whole warps only
  const int y = (int)(warp / p.nseg);
  const int seg = (int)(warp - (long long)y * p.nseg);
  const int x0 = seg * 32 * V + lane * V;
  float f[V][9];
  gather_direct<ST, V>(p, y, seg, lane, f);
  fused_tail<MODEL, PL, ST, V>(p, f, y, seg, x0, x0 < p.nx);
}

// General kernel of the two-pass direct step (the lean one is k_fused_bulk,
// lbm_fused_lean.cuh): the flagged segments listed in p.special.
template <int MODEL, bool PL, int ST, int V>
__global__ void __launch_bounds__(256) k_fused_special(const FusedParams p) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= p.nspecial) return;
  const int item = p.special[warp];
  const int y = item / p.nseg;
  const int seg = item - y * p.nseg;
  const int x0 = seg * 32 * V + lane * V;
  float f[V][9];
  gather_direct<ST, V>(p, y, seg, lane, f);
  fused_tail<MODEL, PL, ST, V>(p, f, y, seg, x0, x0 < p.nx);
}

// Pull-stream gather of one row segment (32*V nodes, V per lane): one aligned
// V-wide load per population, +-1 x shifts by warp shuffles, the segment-edge
// elements by lane 0 / lane 31, and node nx-1's wrap-around fix-up.
template <int ST, int V>
__device__ __forceinline__ void gather_direct(const FusedParams& p, int y, int seg, int lane, float (&f)[V][9]) {
  using S = Storage<ST>;
  using T = typename S::T;
  constexpr unsigned FULL = 0xffffffffu;
  const int x0 = seg * 32 * V + lane * V;
  const bool live = x0 < p.nx;
  const int ilast = p.nx - 1 - x0;  // index of node nx-1 in this chunk, if in [0, V)
  const T* src = reinterpret_cast<const T*>(p.src);
  // ---- pull-stream gather: one aligned V-wide load per population
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const T* row = src + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch;
    float c[V];
    if (live) {
      T raw[V];
      load_vec<T, V>(row + x0, raw);
#pragma unroll
      for (int i = 0; i < V; ++i) c[i] = S::dec(raw[i], p.wsh[k], p.fq);
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) c[i] = 0.0f;
    }
    if (CX(k) == 0) {
#pragma unroll
      for (int i = 0; i < V; ++i) f[i][k] = c[i];
    } else if (CX(k) == 1) {
      float left = __shfl_up_sync(FULL, c[V - 1], 1);
      if (lane == 0 && live) left = S::dec(load1(row + wrap(x0 - 1, p.nx)), p.wsh[k], p.fq);
      f[0][k] = left;
#pragma unroll
      for (int i = 1; i < V; ++i) f[i][k] = c[i - 1];
    } else {
      float right = __shfl_down_sync(FULL, c[0], 1);
      if (lane == 31 && live) right = S::dec(load1(row + wrap(x0 + V, p.nx)), p.wsh[k], p.fq);
#pragma unroll
      for (int i = 0; i < V - 1; ++i) f[i][k] = c[i + 1];
      f[V - 1][k] = right;
      if (live && ilast < V) {  // node nx-1 pulls from column 0
        const float v0 = S::dec(load1(row), p.wsh[k], p.fq);
#pragma unroll
        for (int i = 0; i < V; ++i)
          if (i == ilast) f[i][k] = v0;
      }
    }
  }
}

// After the gather: the per-node path (bounce-back links, boundary
// programs), moments, relaxation, collision and the stores of one lane's V
// x-consecutive nodes starting at x0 in row y.
template <int MODEL, bool PL, int ST, int V, bool GENERAL, int FORCE>
__device__ __forceinline__ void fused_tail(const FusedParams& p, float (&f)[V][9], int y, int seg, int x0,
                                           bool live) {
  using S = Storage<ST>;
  using T = typename S::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  const size_t rowoff = (size_t)y * p.pitch;
  // ---- per-node path: bounce-back links, boundary programs
  const unsigned flag = GENERAL ? p.seg_flags[(size_t)y * p.nseg + seg] : 0u;
  unsigned code[V];
#pragma unroll
  for (int i = 0; i < V; ++i) code[i] = LBM_CODE_ACTIVE;
  if (flag) {
    if (live) {
      uint16_t raw[V];
      load_vec<uint16_t, V>(p.code + rowoff + x0, raw);
#pragma unroll
      for (int i = 0; i < V; ++i) code[i] = (x0 + i < p.nx) ? raw[i] : 0u;
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) code[i] = 0u;
    }
#pragma unroll
    for (int i = 0; i < V; ++i) {
      if (code[i] & 0xffu) {
#pragma unroll
        for (int k = 1; k < 9; ++k)
          if (code[i] & (1u << (k - 1)))
            f[i][k] = S::dec(load1(src + (size_t)OPP(k) * p.plane + rowoff + x0 + i), p.wsh[OPP(k)], p.fq);
      }
      const unsigned prog = code[i] >> LBM_CODE_PROG_SHIFT;
      if (prog) {
        float t[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) t[k] = f[i][k];
        for (int s = 0; s < LBM_PROG_LEN; ++s) {
          const int bi = p.prog[prog][s];
          if (bi < 0) break;
          apply_bc<ST>(p, bi, x0 + i, y, t);
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) f[i][k] = t[k];
      }
    }
  }

  // ---- moments, relaxation, collision
  float tau[V];
  if (PL) {
    if (live) {
      load_vec<float, V>(p.tau + rowoff + x0, tau);
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) tau[i] = 1.0f;
    }
  }
  const bool force = FORCE < 0 ? p.has_force != 0 : FORCE == 1;
  const float Fx = force ? p.gx : 0.0f, Fy = force ? p.gy : 0.0f;
  float mass[V];  // fixed-point storage: each node's stored sum before the collision
#pragma unroll
  for (int i = 0; i < V; ++i) {
    float* fi = f[i];
    if constexpr (ST == LBM_STORE_I16S)
      mass[i] = (code[i] >> LBM_CODE_PROG_SHIFT) ? i16_mass_rounded(f[i], p.wsh, p.fiq, p.fq)
                                                 : i16_mass(f[i], p.wsh, p.fiq, p.fq);
    const float rho = ((fi[0] + fi[1]) + (fi[2] + fi[3])) + ((fi[4] + fi[5]) + (fi[6] + fi[7])) + fi[8];
    const float jx = (fi[1] - fi[3]) + (fi[5] - fi[6]) + (fi[8] - fi[7]);
    const float jy = (fi[2] - fi[4]) + (fi[5] + fi[6]) - (fi[7] + fi[8]);
    const float ux = (jx + 0.5f * Fx) / rho, uy = (jy + 0.5f * Fy) / rho;
    if (flag && (code[i] & LBM_CODE_SAVE)) {
      const size_t q = rowoff + x0 + i;
      p.mom_out[q] = rho;
      p.mom_out[p.plane + q] = ux;
      p.mom_out[2 * p.plane + q] = uy;
    }
    const float st = relax_collide<MODEL, PL, FORCE>(p, fi, rho, ux, uy, Fx, Fy, PL ? tau[i] : 0.0f);
    if (!(code[i] & LBM_CODE_ACTIVE)) {
      // not in the collision group: its post-collision populations never
      // change (the reference never writes f2 there), so carry them over
      if (live) {
#pragma unroll
        for (int k = 0; k < 9; ++k) fi[k] = S::dec(load1(src + (size_t)k * p.plane + rowoff + x0 + i), p.wsh[k], p.fq);
        if constexpr (ST == LBM_STORE_I16S) mass[i] = i16_mass(f[i], p.wsh, p.fiq, p.fq);
      }
    } else if (PL) {
      tau[i] = st;
    }
  }
  if (!live) return;
  if (PL) store_vec<float, V>(p.tau + rowoff + x0, tau);
  T* dst = reinterpret_cast<T*>(p.dst);
  if constexpr (ST == LBM_STORE_I16S) {
    short q[V][9];
    int bits = 0;
#pragma unroll
    for (int i = 0; i < V; ++i) {
      const int b = i16_store_node(f[i], p.wsh, mass[i], q[i], p.fiq);
      if ((code[i] & LBM_CODE_ACTIVE) && x0 + i < p.nx) bits |= b;
    }
    report_bits(p.status, bits);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      T raw[V];
#pragma unroll
      for (int i = 0; i < V; ++i) raw[i] = q[i][k];
      store_vec<T, V>(dst + (size_t)k * p.plane + rowoff + x0, raw);
    }
    return;
  }
  bool bad = false;  // a colliding node inside the lattice holds NaN or infinity
#pragma unroll
  for (int i = 0; i < V; ++i) bad = bad || ((code[i] & LBM_CODE_ACTIVE) && x0 + i < p.nx && not_finite(f[i][0]));
  report_status(p.status, LBM_STATUS_NONFINITE, bad);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    T raw[V];
#pragma unroll
    for (int i = 0; i < V; ++i) raw[i] = S::enc(f[i][k], p.wsh[k], p.fiq);
    store_vec<T, V>(dst + (size_t)k * p.plane + rowoff + x0, raw);
  }
}

// The general step of one node (x, row y) of a lane the lane mask marks,
// from per-node gathers: what fused_tail does for a whole segment.  A node
// outside the collision group is not written: its populations never change,
// and the plan's two buffers hold the same values there (lbm_plan_import
// writes both).
// One thread per node: the path is a chain of dependent loads (node code,
// gathers, boundary reads), so nodes of a lane run side by side, not in turn.
template <int MODEL, bool PL, int ST>
__device__ __forceinline__ void lane_node(const FusedParams& __restrict__ p, int y, int x) {
  using S = Storage<ST>;
  using T = typename S::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  T* dst = reinterpret_cast<T*>(p.dst);
  const float Fx = p.has_force ? p.gx : 0.0f, Fy = p.has_force ? p.gy : 0.0f;
  if (x >= p.nx) return;
  {
    const size_t q = (size_t)y * p.pitch + x;
    const unsigned code = p.code[q];
    if (!(code & LBM_CODE_ACTIVE)) return;
    float f[9];
    gather_node<ST>(p, x, y, f);
    const unsigned prog = code >> LBM_CODE_PROG_SHIFT;
    for (int s = 0; prog && s < LBM_PROG_LEN; ++s) {
      const int bi = p.prog[prog][s];
      if (bi < 0) break;
      apply_bc<ST>(p, bi, x, y, f);
    }
    float mass = 0.0f;  // fixed-point storage: the node's stored sum before the collision
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

    if constexpr (ST == LBM_STORE_I16S) {
      short n[9];
      report_bits(p.status, i16_store_node(f, p.wsh, mass, n, p.fiq));
#pragma unroll
      for (int k = 0; k < 9; ++k) dst[(size_t)k * p.plane + q] = n[k];
    } else {
      report_status(p.status, LBM_STATUS_NONFINITE, not_finite(f[0]));
#pragma unroll
      for (int k = 0; k < 9; ++k) dst[(size_t)k * p.plane + q] = S::enc(f[k], p.wsh[k], p.fiq);
    }
  }
}

// V threads per listed lane, one per node.
template <int MODEL, bool PL, int ST, int V>
__global__ void __launch_bounds__(128) k_fused_lanes(const FusedParams p) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)p.nlanes * V) return;
  const int e = p.lanes[t / V];
  const int item = e >> 5, lane = e & 31;
  const int y = item / p.nseg;
  lane_node<MODEL, PL, ST>(p, y, (item - y * p.nseg) * 32 * V + lane * V + (int)(t % V));
}

// Stream + boundary pass only (the last half step of a fused run): writes the
// post-stream populations of every colliding node as fp32.
template <int ST>
__global__ void k_stream_only(const FusedParams p, float* fout) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= p.nx) return;
  const size_t q = (size_t)y * p.pitch + x;
  const unsigned code = p.code[q];
  if (!(code & LBM_CODE_ACTIVE)) return;
  float g[9];
  gather_node<ST>(p, x, y, g);
  const unsigned prog = code >> LBM_CODE_PROG_SHIFT;
  for (int s = 0; prog && s < LBM_PROG_LEN; ++s) {
    const int bi = p.prog[prog][s];
    if (bi < 0) break;
    apply_bc<ST>(p, bi, x, y, g);
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) fout[(size_t)k * p.plane + q] = g[k];
}

template <int ST>
__global__ void k_convert(const FusedParams p, const float* in, void* out, int to_storage) {
  using S = Storage<ST>;
  using T = typename S::T;
  const size_t n = 9 * p.plane;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / p.plane);
    const float w = p.wsh[k];
    if (to_storage) reinterpret_cast<T*>(out)[t] = S::enc(in[t], w, p.fiq);
    else reinterpret_cast<float*>(out)[t] = S::dec(reinterpret_cast<const T*>(p.src)[t], w, p.fq);
  }
}

// Momentum exchange on links into a solid (Ladd): a post-collision
// population f_k(x) heading into a solid neighbour x + c_k returns as
// f_opp(k)(x) = f_k(x) (half-way bounce-back), handing the body 2 c_k f_k(x).
// links: (plane-offset q, k) pairs; one block, FP64 accumulation; writes
// (Fx, Fy) to out.
constexpr int MEX_TPB = 256;

template <int ST>
__global__ void __launch_bounds__(MEX_TPB) k_momentum_exchange(const FusedParams p, const int32_t* links,
                                                               int64_t n, double* out) {
  using S = Storage<ST>;
  using T = typename S::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  double fx = 0.0, fy = 0.0;
  for (int64_t m = threadIdx.x; m < n; m += blockDim.x) {
    const int64_t q = links[2 * m];
    const int k = links[2 * m + 1];
    const double v = S::dec64(src[(size_t)k * p.plane + q], p.wsh[k], p.fq);
    fx += 2.0 * cx_dyn(k) * v;
    fy += 2.0 * cy_dyn(k) * v;
  }
  __shared__ double sh[2][MEX_TPB / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fx += __shfl_down_sync(0xffffffffu, fx, o);
    fy += __shfl_down_sync(0xffffffffu, fy, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = fx;
    sh[1][threadIdx.x >> 5] = fy;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double s = 0.0;
    for (int i = 0; i < MEX_TPB / 32; ++i) s += sh[threadIdx.x][i];
    out[threadIdx.x] = s;
    report_status(p.status, LBM_STATUS_NONFINITE, !(fabs(s) <= 1.7976931348623157e308));
  }
}

// FP64 sums of f, f c_x, f c_y over colliding nodes of the state p.src.
constexpr int REDUCE_BLOCKS = 152 * 4;
constexpr int REDUCE_TPB = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <int ST>
__global__ void __launch_bounds__(REDUCE_TPB) k_reduce_partial(const FusedParams p, double* partials) {
  using S = Storage<ST>;
  using T = typename S::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  const size_t n = (size_t)p.ny * p.pitch;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(q % p.pitch);
    if (x >= p.nx || !(p.code[q] & LBM_CODE_ACTIVE)) continue;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double v = S::dec64(src[(size_t)k * p.plane + q], p.wsh[k], p.fq);
      a0 += v;
      if (CX(k)) a1 += CX(k) * v;
      if (CY(k)) a2 += CY(k) * v;
    }
  }
  __shared__ double sh[3][REDUCE_TPB / 32];
  a0 = warp_sum(a0);
  a1 = warp_sum(a1);
  a2 = warp_sum(a2);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = a0;
    sh[1][w] = a1;
    sh[2][w] = a2;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int i = 0; i < REDUCE_TPB / 32; ++i) s += sh[threadIdx.x][i];
    partials[(size_t)blockIdx.x * 3 + threadIdx.x] = s;
  }
}

template <int ST>
__global__ void k_reduce_final(const double* partials, int nblocks, double* out) {
  // one warp per component, fixed order: deterministic
  const int c = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (c >= 3) return;
  double s = 0.0;
  for (int b = l; b < nblocks; b += 32) s += partials[(size_t)b * 3 + c];
  s = warp_sum(s);
  if (l == 0) out[c] = s;
}

}  // namespace lbm
