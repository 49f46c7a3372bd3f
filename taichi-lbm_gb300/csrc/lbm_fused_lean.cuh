// Lean kernel of the two-pass direct step: plain row segments only.
//
// A plain segment has every node colliding and streaming all nine links,
// with no boundary program and no saved moments, so the step is the pull
// gather, the moments and the collision.  This kernel works on the stored
// values themselves: for 16-bit storage h_k = f_k - wsh_k is the deviation
// from rest at the plan's reference density, and the collision is written in
// terms of h (the shift cancels in every difference f - feq and in the
// moments), so neither a decode nor an encode offset is spent per population.
// The equilibrium of an opposite pair (k, opp k) is built from its symmetric
// and antisymmetric parts, and the velocity from one reciprocal of rho.
// The results agree with the general path (lbm_fused.cuh) to fp32 rounding.
#pragma once

#include "lbm_fused.cuh"

namespace lbm {

// ------------------------------------------------------------ raw conversion
// The fixed-point step of a plan, as the raw conversions use it: q = 2^-e,
// off = (2^23 + 2^15) q, iq = 1 / q (other storages ignore it).
struct Fix {
  float q, off, iq;
};
template <class P>
__device__ __forceinline__ Fix fix_of(const P& p) {
  return Fix{p.fq, p.foff, p.fiq};
}

template <int ST>
__device__ __forceinline__ float raw_to_float(typename Storage<ST>::T v, const Fix& fx);
template <>
__device__ __forceinline__ float raw_to_float<LBM_STORE_F32>(float v, const Fix&) { return v; }
template <>
__device__ __forceinline__ float raw_to_float<LBM_STORE_F16S>(__half v, const Fix&) { return __half2float(v); }
template <>
__device__ __forceinline__ float raw_to_float<LBM_STORE_BF16S>(__nv_bfloat16 v, const Fix&) {
  return __bfloat162float(v);
}
template <>
__device__ __forceinline__ float raw_to_float<LBM_STORE_I16S>(short v, const Fix& fx) { return (float)v * fx.q; }

// two int16 step counts packed in a word -> their shifted values, without
// an integer conversion: 0x4B00xxxx with xxxx = n + 2^15 is the float
// 2^23 + 2^15 + n, and (that - 2^23 - 2^15) * Q is n * Q, exact in one fma
// (Q is a power of two)
__device__ __forceinline__ float2 i16_pair_to_floats(unsigned w, const Fix& fx) {
  const unsigned u = w ^ 0x80008000u;
  const float lo = __uint_as_float(__byte_perm(u, 0x4B000000u, 0x7610));
  const float hi = __uint_as_float(__byte_perm(u, 0x4B000000u, 0x7632));
  return make_float2(fmaf(lo, fx.q, -fx.off), fmaf(hi, fx.q, -fx.off));
}

// V stored values -> floats (no shift)
template <int ST, int V>
__device__ __forceinline__ void raw_to_floats(const typename Storage<ST>::T (&raw)[V], float (&c)[V],
                                              const Fix& fx) {
  if constexpr (ST == LBM_STORE_F32) {
#pragma unroll
    for (int i = 0; i < V; ++i) c[i] = raw[i];
  } else if constexpr (ST == LBM_STORE_F16S) {
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      __half2 t;
      memcpy(&t, &raw[i], sizeof(t));
      const float2 u = __half22float2(t);
      c[i] = u.x;
      c[i + 1] = u.y;
    }
  } else if constexpr (ST == LBM_STORE_BF16S) {
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      __nv_bfloat162 t;
      memcpy(&t, &raw[i], sizeof(t));
      const float2 u = __bfloat1622float2(t);
      c[i] = u.x;
      c[i + 1] = u.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      unsigned w;
      memcpy(&w, &raw[i], sizeof(w));
      const float2 u = i16_pair_to_floats(w, fx);
      c[i] = u.x;
      c[i + 1] = u.y;
    }
  }
}

// Read-only global loads as volatile asm: the compiler may neither drop nor
// sink them below a later branch, so a warp's population loads are in
// flight before it learns (from the segment flag loaded beside them)
// whether it keeps the segment.
__device__ __forceinline__ void ldg_early(const void* p, uint4& r) {
  asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
}
__device__ __forceinline__ void ldg_early(const void* p, uint2& r) {
  asm volatile("ld.global.nc.v2.u32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "l"(p));
}
__device__ __forceinline__ void ldg_early(const void* p, unsigned int& r) {
  asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(r) : "l"(p));
}
__device__ __forceinline__ void ldg_early(const void* p, unsigned short& r) {
  asm volatile("ld.global.nc.u16 %0, [%1];" : "=h"(r) : "l"(p));
}
__device__ __forceinline__ void ldg_early(const void* p, unsigned char& r) {
  unsigned short t;
  asm volatile("ld.global.nc.u8 %0, [%1];" : "=h"(t) : "l"(p));
  r = (unsigned char)t;
}

// V consecutive elements (aligned), pieces of at most 16 B
template <typename T, int V>
__device__ __forceinline__ void load_vec_early(const T* p, T (&out)[V]) {
  constexpr int B = sizeof(T) * V > 16 ? 16 : sizeof(T) * V;
  constexpr int E = B / sizeof(T);
  using R = typename Raw<B>::type;
#pragma unroll
  for (int c = 0; c < V / E; ++c) {
    R r;
    ldg_early(p + c * E, r);
    memcpy(&out[c * E], &r, B);
  }
}
template <typename T>
__device__ __forceinline__ T load1_early(const T* p) {
  typename Raw<sizeof(T)>::type r;
  ldg_early(p, r);
  T out;
  memcpy(&out, &r, sizeof(T));
  return out;
}

// V consecutive stored values -> floats (no shift)
template <int ST, int V>
__device__ __forceinline__ void load_raw(const typename Storage<ST>::T* p, float (&c)[V], const Fix& fx) {
  using T = typename Storage<ST>::T;
  T raw[V];
  load_vec_early<T, V>(p, raw);
  raw_to_floats<ST, V>(raw, c, fx);
}

// V floats -> V consecutive stored values (round to nearest, no shift)
template <int ST, int V>
__device__ __forceinline__ void store_raw(typename Storage<ST>::T* p, const float (&c)[V], const Fix& fx) {
  using T = typename Storage<ST>::T;
  T raw[V];
  if constexpr (ST == LBM_STORE_F32) {
#pragma unroll
    for (int i = 0; i < V; ++i) raw[i] = c[i];
  } else if constexpr (ST == LBM_STORE_F16S) {
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      const __half2 t = __floats2half2_rn(c[i], c[i + 1]);
      memcpy(&raw[i], &t, sizeof(t));
    }
  } else if constexpr (ST == LBM_STORE_BF16S) {
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      const __nv_bfloat162 t = __floats2bfloat162_rn(c[i], c[i + 1]);
      memcpy(&raw[i], &t, sizeof(t));
    }
  } else {
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      const unsigned w = __byte_perm(i16_bits(i16_steps(c[i], fx.iq)), i16_bits(i16_steps(c[i + 1], fx.iq)), 0x5410);
      memcpy(&raw[i], &w, sizeof(w));
    }
  }
  store_vec<T, V>(p, raw);
}

// Pull gather of an interior segment (x0s > 0 and x0s + 32 V < nx): every
// lane is inside the lattice, the elements across the segment's edges exist
// without wrapping, and node nx-1 is not in the segment.
template <class P, int ST, int V>
__device__ __forceinline__ void gather_interior(const P& p, int y, int x0, int lane, float (&h)[V][9]) {
  using T = typename Storage<ST>::T;
  constexpr unsigned FULL = 0xffffffffu;
  const T* src = reinterpret_cast<const T*>(p.src);
  const int ym = wrap(y - 1, p.ny), yp = wrap(y + 1, p.ny);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int ys = CY(k) == 0 ? y : (CY(k) == 1 ? ym : yp);
    const T* row = src + (size_t)k * p.plane + (size_t)ys * p.pitch + x0;
    float c[V];
    load_raw<ST, V>(row, c, fix_of(p));
    if (CX(k) == 0) {
#pragma unroll
      for (int i = 0; i < V; ++i) h[i][k] = c[i];
    } else if (CX(k) == 1) {
      float left = __shfl_up_sync(FULL, c[V - 1], 1);
      if (lane == 0) left = raw_to_float<ST>(load1_early(row - 1), fix_of(p));
      h[0][k] = left;
#pragma unroll
      for (int i = 1; i < V; ++i) h[i][k] = c[i - 1];
    } else {
      float right = __shfl_down_sync(FULL, c[0], 1);
      if (lane == 31) right = raw_to_float<ST>(load1_early(row + V), fix_of(p));
#pragma unroll
      for (int i = 0; i < V - 1; ++i) h[i][k] = c[i + 1];
      h[V - 1][k] = right;
    }
  }
}

// Pull gather of any segment (x edges wrap, lanes past nx read nothing),
// stored values without the shift.
template <class P, int ST, int V>
__device__ __forceinline__ void gather_edge(const P& p, int y, int x0, int lane, float (&h)[V][9]) {
  using T = typename Storage<ST>::T;
  constexpr unsigned FULL = 0xffffffffu;
  const bool live = x0 < p.nx;
  const int ilast = p.nx - 1 - x0;
  const T* src = reinterpret_cast<const T*>(p.src);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const T* row = src + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch;
    float c[V];
    if (live) {
      load_raw<ST, V>(row + x0, c, fix_of(p));
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) c[i] = 0.0f;
    }
    if (CX(k) == 0) {
#pragma unroll
      for (int i = 0; i < V; ++i) h[i][k] = c[i];
    } else if (CX(k) == 1) {
      float left = __shfl_up_sync(FULL, c[V - 1], 1);
      if (lane == 0 && live) left = raw_to_float<ST>(load1_early(row + wrap(x0 - 1, p.nx)), fix_of(p));
      h[0][k] = left;
#pragma unroll
      for (int i = 1; i < V; ++i) h[i][k] = c[i - 1];
    } else {
      float right = __shfl_down_sync(FULL, c[0], 1);
      if (lane == 31 && live) right = raw_to_float<ST>(load1_early(row + wrap(x0 + V, p.nx)), fix_of(p));
#pragma unroll
      for (int i = 0; i < V - 1; ++i) h[i][k] = c[i + 1];
      h[V - 1][k] = right;
      if (live && ilast < V) {  // node nx-1 pulls from column 0
        const float v0 = raw_to_float<ST>(load1_early(row), fix_of(p));
#pragma unroll
        for (int i = 0; i < V; ++i)
          if (i == ilast) h[i][k] = v0;
      }
    }
  }
}

// ------------------------------------------------------------ collision
// Shifted equilibria e_k = feq_k(rho, u) - wsh_k of all nine populations from
// the pair decomposition feq_{k / opp k} = w_k rho (1 - 1.5 u.u + 4.5 (c_k.u)^2)
// +- 3 w_k rho (c_k.u).
// SCALED: every e_k is multiplied by sc (BGK passes omega, so that the
// relaxation h + omega (e - h) becomes one fma, (1 - omega) h + omega e).
template <bool SCALED = false, class P>
__device__ __forceinline__ void shifted_feq(const P& p, float rho, float ux, float uy, float e[9],
                                            float sc = 1.0f) {
  const float base = fmaf(-1.5f, fmaf(ux, ux, uy * uy), 1.0f);
  const float rs = SCALED ? rho * sc : rho;
  const float r0 = rs * W(0), r1 = rs * W(1), r2 = rs * W(5);
  const float a1 = 3.0f * r1, a2 = 3.0f * r2;
  // the shift has three distinct weights (rest, axis, diagonal)
  const float w0 = SCALED ? p.wsh[0] * sc : p.wsh[0];
  const float w1 = SCALED ? p.wsh[1] * sc : p.wsh[1];
  const float w2 = SCALED ? p.wsh[5] * sc : p.wsh[5];
  e[0] = fmaf(r0, base, -w0);
  const float eu[4] = {ux, uy, ux + uy, uy - ux};  // c.u of k = 1, 2, 5, 6
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = q < 2 ? q + 1 : q + 3;
    const float r = q < 2 ? r1 : r2, a = q < 2 ? a1 : a2;
    const float t = fmaf(4.5f * eu[q], eu[q], base);
    const float sym = fmaf(r, t, -(q < 2 ? w1 : w2));
    const float anti = a * eu[q];
    e[k] = sym + anti;
    e[OPP(k)] = sym - anti;
  }
}

// Guo forcing populations F_k (CollisionEngine.py:21-25), by pairs
__device__ __forceinline__ void pair_force(float Fx, float Fy, float ux, float uy, float F[9]) {
  const float uF = fmaf(ux, Fx, uy * Fy);
  F[0] = W(0) * (-3.0f * uF);
  const float eu[4] = {ux, uy, ux + uy, uy - ux};
  const float eF[4] = {Fx, Fy, Fx + Fy, Fy - Fx};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = q < 2 ? q + 1 : q + 3;
    const float w = W(k);
    const float sym = w * fmaf(9.0f * eF[q], eu[q], -3.0f * uF);
    const float anti = (3.0f * w) * eF[q];
    F[k] = sym + anti;
    F[OPP(k)] = sym - anti;
  }
}

// The library is built without implicit fma contraction, so every kernel
// form (single lattice, batched, prefetching) computes a node bit for bit
// alike; the fused multiply-adds below are written out.
__device__ __forceinline__ float shear_lean(const float n[9], float cof) {  // CollisionEngine.py:86-92
  const float Sxx = (n[1] + n[3] + n[5] + n[6] + n[7] + n[8]) * cof;
  const float Syy = (n[2] + n[4] + n[5] + n[6] + n[7] + n[8]) * cof;
  const float Sxy = (n[5] - n[6] + n[7] - n[8]) * cof;
  return sqrtf(2.0f * fmaf(Sxx, Sxx, fmaf(Syy, Syy, 2.0f * (Sxy * Sxy))));
}
__device__ __forceinline__ float powerlaw_tau_lean(float m, float n, float gamma, float lo, float hi) {
  return clamp_tau(fmaf(m * powf(gamma, n - 1.0f), 3.0f, 0.5f), lo, hi);  // FluidModels.py:20-29
}
// MRT transforms (CollisionEngine.py:273-282): forward coefficients are
// 0, +-1, +-2, +-4 (an fma by a power of two rounds as a multiply and add)
__device__ __forceinline__ void mrt_forward_lean(const float f[9], float m[9]) {
#pragma unroll
  for (int a = 0; a < 9; ++a) {
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      constexpr float one = 1.0f;
      const float c = MRT_M(a, k);
      if (c == one) s = s + f[k];
      else if (c == -one) s = s - f[k];
      else if (c != 0.0f) s = fmaf(c, f[k], s);
    }
    m[a] = s;
  }
}
__device__ __forceinline__ void mrt_backward_lean(const float m[9], float f[9]) {
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float s = 0.0f;
#pragma unroll
    for (int a = 0; a < 9; ++a)
      if (MRT_M(a, k) != 0.0f) s = fmaf(MRT_MINV(k, a), m[a], s);
    f[k] = s;
  }
}

// One node: moments, relaxation and collision of the stored values h in
// place; returns the new power-law state (or the old one).  FORCE: 0 none,
// 1 the uniform body force (p.gx, p.gy), 2 the per-node force (Fn_x, Fn_y).
template <class P, int MODEL, bool PL, int FORCE>
__device__ __forceinline__ float collide_lean(const P& p, float h[9], float state, float Fn_x = 0.0f,
                                              float Fn_y = 0.0f) {
  const float dr = ((h[0] + h[1]) + (h[2] + h[3])) + ((h[4] + h[5]) + (h[6] + h[7])) + h[8];
  const float rho = dr + p.rho_shift;
  const float d13 = h[1] - h[3], d24 = h[2] - h[4], d57 = h[5] - h[7], d68 = h[6] - h[8];
  const float jx = d13 + (d57 - d68);
  const float jy = d24 + (d57 + d68);
  const float Fx = FORCE == 1 ? p.gx : (FORCE == 2 ? Fn_x : 0.0f);
  const float Fy = FORCE == 1 ? p.gy : (FORCE == 2 ? Fn_y : 0.0f);
  const float inv = __fdividef(1.0f, rho);  // within 2 ulp; rho is O(1) here
  const float ux = (FORCE ? fmaf(0.5f, Fx, jx) : jx) * inv;
  const float uy = (FORCE ? fmaf(0.5f, Fy, jy) : jy) * inv;
  float F[9];
  if (FORCE) pair_force(Fx, Fy, ux, uy, F);
  if (MODEL == LBM_BGK && !PL) {
    // h' = (1 - omega) h + omega e (+ (1 - omega / 2) F)
    const float om = p.omega, keep = 1.0f - om, cf = 1.0f - 0.5f * om;
    float e[9];
    shifted_feq<true>(p, rho, ux, uy, e, om);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float v = fmaf(keep, h[k], e[k]);
      if (FORCE) v = fmaf(cf, F[k], v);
      h[k] = v;
    }
    return state;
  }
  float e[9];
  shifted_feq(p, rho, ux, uy, e);

  if (MODEL == LBM_MRT) {
    // m = M h; equilibrium moments less the moments of the shift (M wsh)
    float m[9], s[9];
#pragma unroll
    for (int a = 0; a < 9; ++a) s[a] = p.s[a];
    if (PL) {
      // CollisionEngine.py:332-377 with the previous step's s7 = s8 = state
      float n[9], mn[9], mneq[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) n[k] = h[k] - e[k];
      mrt_forward_lean(n, mn);
      s[7] = s[8] = state;
#pragma unroll
      for (int a = 0; a < 9; ++a) mn[a] *= s[a];
      mrt_backward_lean(mn, mneq);
      const float gamma = shear_lean(mneq, -1.5f / rho);
      state = 1.0f / powerlaw_tau_lean(p.pl_m, p.pl_n, gamma, p.tau_min, p.tau_max);
      s[7] = s[8] = state;
    }
    mrt_forward_lean(h, m);
    // equilibrium moments (CollisionEngine.py:388-406)
    const float u2 = fmaf(ux, ux, uy * uy);
    float meq[9];
    meq[0] = rho;
    meq[1] = rho * fmaf(3.0f, u2, -2.0f);
    meq[2] = rho * fmaf(-3.0f, u2, 1.0f);
    meq[3] = rho * ux;
    meq[4] = -meq[3];
    meq[5] = rho * uy;
    meq[6] = -meq[5];
    meq[7] = rho * fmaf(ux, ux, -(uy * uy));
    meq[8] = rho * (ux * uy);
    float mf[9];
    if (FORCE) {  // CollisionEngine.py:408-422
      const float Fu = fmaf(Fx, ux, Fy * uy);
      mf[0] = 0.0f;
      mf[1] = 6.0f * Fu;
      mf[2] = -6.0f * Fu;
      mf[3] = Fx;
      mf[4] = -Fx;
      mf[5] = Fy;
      mf[6] = -Fy;
      mf[7] = 2.0f * fmaf(Fx, ux, -(Fy * uy));
      mf[8] = fmaf(Fy, ux, Fx * uy);
    }
#pragma unroll
    for (int a = 0; a < 9; ++a) {
      // M wsh vanishes beyond the first three moments (the shift is at rest)
      float v = fmaf(-s[a], m[a] - (a < 3 ? meq[a] - p.mwsh[a] : meq[a]), m[a]);
      if (FORCE) v = fmaf(1.0f - 0.5f * s[a], mf[a], v);
      m[a] = v;
    }
    mrt_backward_lean(m, h);
    return state;
  }

  float om = p.omega, oa = p.omega_a;
  if (PL) {
    // CollisionEngine.py:80-92 / 166-178 (previous tau), then :72-78 / 157-164
    float n[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) n[k] = h[k] - e[k];
    const float t = powerlaw_tau_lean(p.pl_m, p.pl_n, shear_lean(n, -1.5f / rho / state), p.tau_min, p.tau_max);
    state = t;
    om = 1.0f / t;
    if (MODEL == LBM_TRT) oa = 1.0f / (p.magic / (t - 0.5f) + 0.5f);
  }
  if (MODEL == LBM_BGK) {
    const float cf = 1.0f - 0.5f * om;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float v = fmaf(om, e[k] - h[k], h[k]);
      if (FORCE) v = fmaf(cf, F[k], v);
      h[k] = v;
    }
    return state;
  }
  // TRT, pairs (1,3), (2,4), (5,7), (6,8): symmetric and antisymmetric parts
  // relax with omega and omega_a (CollisionEngine.py:181-245)
  const float hs = 0.5f * om, ha = 0.5f * oa;
  const float cs = 0.5f * (1.0f - 0.5f * om), ca = 0.5f * (1.0f - 0.5f * oa);
  h[0] = fmaf(om, e[0] - h[0], h[0]);
  if (FORCE) h[0] = fmaf(1.0f - 0.5f * om, F[0], h[0]);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = q < 2 ? q + 1 : q + 3, o = OPP(k);
    float sym = hs * ((e[k] + e[o]) - (h[k] + h[o]));
    float anti = ha * ((e[k] - e[o]) - (h[k] - h[o]));
    if (FORCE) {
      sym = fmaf(cs, F[k] + F[o], sym);
      anti = fmaf(ca, F[k] - F[o], anti);
    }
    h[k] = h[k] + (sym + anti);
    h[o] = h[o] + (sym - anti);
  }
  return state;
}

// sum of a node's nine shifted values (exact for the fixed-point storage)
__device__ __forceinline__ float node_sum(const float (&h)[9]) {
  return ((h[0] + h[1]) + (h[2] + h[3])) + ((h[4] + h[5]) + (h[6] + h[7])) + h[8];
}

// Fixed-point storage: quantise V nodes' post-collision values h with each
// node's pre-collision mass kept (i16_conserve_bits) and store the nine
// planes from p (population k at p + k * plane), two step counts per word.
// Returns the LBM_STATUS_* bits (i16_conserve_bits) of the first nv nodes
// (the ones inside the lattice; the rest is row padding).
template <int V>
__device__ __forceinline__ int store_i16_conserved(short* p, size_t plane, const float (&h)[V][9],
                                                   const float (&mass)[V], float iq, int nv) {
  unsigned b[V][9];
  int bad = 0;
#pragma unroll
  for (int i = 0; i < V; ++i) {
    const int out = i16_conserve_bits(h[i], mass[i], b[i], iq);
    if (i < nv) bad |= out;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    short raw[V];
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      const unsigned w = __byte_perm(b[i][k], b[i + 1][k], 0x5410);
      memcpy(&raw[i], &w, sizeof(w));
    }
    store_vec<short, V>(p + (size_t)k * plane, raw);
  }
  return bad;
}

// Moments, collision and stores of one lane's V nodes (x0.., row y) of a
// plain segment, from the gathered stored values h.
template <class P, int MODEL, bool PL, int ST, int V, int FORCE>
__device__ __forceinline__ void lean_collide_store(const P& p, float (&h)[V][9], int y, int x0, bool skip = false) {
  using T = typename Storage<ST>::T;
  const bool live = x0 < p.nx && !skip;  // skip: another kernel stores this lane
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
  float mass[V];  // fixed-point storage: each node's stored sum before the collision (exact)
  if constexpr (ST == LBM_STORE_I16S) {
#pragma unroll
    for (int i = 0; i < V; ++i) mass[i] = node_sum(h[i]);
  }
#pragma unroll
  for (int i = 0; i < V; ++i) {
    const float st = collide_lean<P, MODEL, PL, FORCE>(p, h[i], PL ? tau[i] : 0.0f);
    if (PL) tau[i] = st;
  }
  if (!live) return;
  if (PL) store_vec<float, V>(p.tau + rowoff + x0, tau);
  T* dst = reinterpret_cast<T*>(p.dst);
  if constexpr (ST == LBM_STORE_I16S) {
    report_bits(p.status, store_i16_conserved<V>(dst + rowoff + x0, p.plane, h, mass, p.fiq, p.nx - x0));
    return;
  }
  bool bad = false;  // a node inside the lattice holds NaN or infinity
#pragma unroll
  for (int i = 0; i < V; ++i) bad = bad || (x0 + i < p.nx && not_finite(h[i][0]));
  report_status(p.status, LBM_STATUS_NONFINITE, bad);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float c[V];
#pragma unroll
    for (int i = 0; i < V; ++i) c[i] = h[i][k];
    store_raw<ST, V>(dst + (size_t)k * p.plane + rowoff + x0, c, fix_of(p));
  }
}

// Two-pass form of the direct step.  k_fused_bulk takes the plain segments
// (seg_flags == 0), with the body force fixed at compile time, and leaves the
// flagged segments to k_fused_special (lbm_fused.cuh), which walks the
// compact list p.special of their indices (y * nseg + seg).  The two write
// disjoint nodes and read only the source state, so they may run in either
// order or concurrently within a step.
// Grid, in dispatch order: blockIdx.x * warps-per-block + warp = segment,
// then row y = blockIdx.y + gridDim.y * blockIdx.z; resident blocks thus
// cover a band of consecutive whole rows (DRAM page locality).
template <int MODEL, bool PL, int ST, int V, int FORCE>
__global__ void __launch_bounds__(256) k_fused_bulk(const FusedParams p) {
  const int lane = threadIdx.x & 31;
  const int y = blockIdx.y + gridDim.y * blockIdx.z;
  const int seg = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (seg >= p.nseg || y >= p.ny) return;
  // with lane masks every segment is gathered here and the marked lanes are
  // stored by k_fused_lanes; else k_fused_special owns a flagged segment
  uint32_t mask;
  if (p.lane_mask) {
    ldg_early(p.lane_mask + (size_t)y * p.nseg + seg, mask);
  } else {
    unsigned char flag;
    ldg_early(p.seg_flags + (size_t)y * p.nseg + seg, flag);
    mask = flag ? 0xffffffffu : 0u;
  }
  const int x0s = seg * 32 * V, x0 = x0s + lane * V;
  float h[V][9];
  if (x0s > 0 && x0s + 32 * V < p.nx) gather_interior<FusedParams, ST, V>(p, y, x0, lane, h);
  else gather_edge<FusedParams, ST, V>(p, y, x0, lane, h);
  if (mask == 0xffffffffu) return;  // uniform over the warp
  lean_collide_store<FusedParams, MODEL, PL, ST, V, FORCE>(p, h, y, x0, (mask >> lane) & 1u);
}

// ------------------------------------------------------------ prefetching form
// k_fused_bulk_pf: persistent warps walk the compact list p.plain of plain
// segments.  Each warp owns a ring of NS shared-memory stages; a stage holds
// what one segment needs from the source: every lane's V elements of the
// nine pulled rows, copied by that lane with cp.async (no registers held
// while in flight), and the 4-byte words that contain the elements across
// the segment's edges.  A warp keeps NS - 1 segments of copies in flight
// while it collides the current one, then reads its own stage back (each
// lane reads only what it copied, so no barrier is needed; cp.async.wait_group
// is the hardware wait for the lane's own copies).
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src) {
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)), "l"(src), "n"(BYTES)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

constexpr __host__ __device__ int edge_slot(int k) {  // the six links with cx = +-1 -> 0..5
  return k == 1 ? 0 : k == 5 ? 1 : k == 8 ? 2 : k == 3 ? 3 : k == 6 ? 4 : 5;
}

template <int ST, int V, int NS>
struct PfGeom {
  using T = typename Storage<ST>::T;
  static constexpr int POP_BYTES = 32 * V * (int)sizeof(T);   // one pulled row chunk of a warp
  static constexpr int EDGE_OFF = 9 * POP_BYTES;               // [6][32] words
  static constexpr int ITEM_OFF = EDGE_OFF + 6 * 32 * 4;       // [32] segment index, per lane
  static constexpr int STAGE_BYTES = ITEM_OFF + 32 * 4;
  static constexpr int WARP_BYTES = NS * STAGE_BYTES;
  static_assert(POP_BYTES % 16 == 0 && STAGE_BYTES % 16 == 0, "stages must stay 16-byte aligned");
};

// element x of a row, as the 4-byte word that holds it (16-bit storage: the
// even/odd pair; the word never passes the row's pitch, which is a multiple
// of 32 elements)
template <int ST>
__device__ __forceinline__ const void* edge_word(const typename Storage<ST>::T* row, int x) {
  return ST == LBM_STORE_F32 ? (const void*)(row + x) : (const void*)(row + (x & ~1));
}
template <int ST>
__device__ __forceinline__ float edge_value(uint32_t w, int x, const Fix& fx) {
  if constexpr (ST == LBM_STORE_F32) {
    return __uint_as_float(w);
  } else {
    const unsigned short b = (unsigned short)((x & 1) ? (w >> 16) : (w & 0xffffu));
    typename Storage<ST>::T t;
    memcpy(&t, &b, 2);
    return raw_to_float<ST>(t, fx);
  }
}

// Issue the cp.async copies of what row y of the segment at x0s needs from
// the source into a stage (no commit): every lane's V elements of the nine
// pulled rows and the 4-byte words holding the elements across the
// segment's edges.
template <class P, int ST, int V, int NS>
__device__ __forceinline__ void stage_issue_row(const P& p, unsigned char* stage, int y, int x0s, int lane) {
  using T = typename Storage<ST>::T;
  using G = PfGeom<ST, V, NS>;
  // the fields are read once, before the copies: each cp.async clobbers
  // memory, and the parameters may live in shared memory (batched kernels)
  const int nx = p.nx;
  const size_t plane = p.plane, pitch = (size_t)p.pitch;
  const T* src = reinterpret_cast<const T*>(p.src);
  const int x0 = x0s + lane * V;
  const bool live = x0 < nx;
  const int ilast = nx - 1 - x0;
  const bool need_right = live && (lane == 31 || (ilast >= 0 && ilast < V));
  const int xl = x0 > 0 ? x0 - 1 : nx - 1;
  const int xr = x0 + V < nx ? x0 + V : 0;
  const T* rows[3] = {src + (size_t)wrap(y + 1, p.ny) * pitch, src + (size_t)y * pitch,
                      src + (size_t)wrap(y - 1, p.ny) * pitch};  // rows y - cy for cy = -1, 0, 1
  uint32_t* edges = reinterpret_cast<uint32_t*>(stage + G::EDGE_OFF);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const T* row = rows[CY(k) + 1] + (size_t)k * plane;
    if (live) cp_async<V * (int)sizeof(T)>(stage + k * G::POP_BYTES + lane * V * (int)sizeof(T), row + x0);
    if (CX(k) == 1 && lane == 0 && live) cp_async<4>(edges + edge_slot(k) * 32 + lane, edge_word<ST>(row, xl));
    if (CX(k) == -1 && need_right) cp_async<4>(edges + edge_slot(k) * 32 + lane, edge_word<ST>(row, xr));
  }
}

// The pull gather of a row from its stage (after its copies have landed;
// each lane reads only what it copied).
template <class P, int ST, int V, int NS>
__device__ __forceinline__ void stage_gather_row(const P& p, const unsigned char* stage, int x0, int lane,
                                                 float (&h)[V][9]) {
  using T = typename Storage<ST>::T;
  using G = PfGeom<ST, V, NS>;
  constexpr unsigned FULL = 0xffffffffu;
  const bool live = x0 < p.nx;
  const int ilast = p.nx - 1 - x0;
  const bool has_last = ilast >= 0 && ilast < V;
  const int xl = x0 > 0 ? x0 - 1 : p.nx - 1;
  const int xr = x0 + V < p.nx ? x0 + V : 0;
  const uint32_t* edges = reinterpret_cast<const uint32_t*>(stage + G::EDGE_OFF);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float c[V];
    if (live) {
      T raw[V];
      memcpy(raw, stage + k * G::POP_BYTES + lane * V * (int)sizeof(T), sizeof(raw));
      raw_to_floats<ST, V>(raw, c, fix_of(p));
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) c[i] = 0.0f;
    }
    if (CX(k) == 0) {
#pragma unroll
      for (int i = 0; i < V; ++i) h[i][k] = c[i];
    } else if (CX(k) == 1) {
      float left = __shfl_up_sync(FULL, c[V - 1], 1);
      if (lane == 0 && live) left = edge_value<ST>(edges[edge_slot(k) * 32 + lane], xl, fix_of(p));
      h[0][k] = left;
#pragma unroll
      for (int i = 1; i < V; ++i) h[i][k] = c[i - 1];
    } else {
      float right = __shfl_down_sync(FULL, c[0], 1);
      float re = 0.0f;
      if ((lane == 31 || has_last) && live) re = edge_value<ST>(edges[edge_slot(k) * 32 + lane], xr, fix_of(p));
      if (lane == 31) right = re;
#pragma unroll
      for (int i = 0; i < V - 1; ++i) h[i][k] = c[i + 1];
      h[V - 1][k] = right;
      if (has_last) {  // node nx-1 pulls from column 0
#pragma unroll
        for (int i = 0; i < V; ++i)
          if (i == ilast) h[i][k] = re;
      }
    }
  }
}

template <int ST, int V, int NS>
__device__ __forceinline__ void pf_issue(const FusedParams& p, unsigned char* stage, int item, int lane) {
  using G = PfGeom<ST, V, NS>;
  if (item >= 0) {
    const int y = item / p.nseg;
    stage_issue_row<FusedParams, ST, V, NS>(p, stage, y, (item - y * p.nseg) * 32 * V, lane);
    reinterpret_cast<int*>(stage + G::ITEM_OFF)[lane] = item;
  }
  cp_async_commit();
}

template <int MODEL, bool PL, int ST, int V, int FORCE, int NS>
__device__ __forceinline__ void pf_consume(const FusedParams& p, const unsigned char* stage, int lane) {
  using G = PfGeom<ST, V, NS>;
  const int item = reinterpret_cast<const int*>(stage + G::ITEM_OFF)[lane];
  const int y = item / p.nseg;
  const int x0 = (item - y * p.nseg) * 32 * V + lane * V;
  float h[V][9];
  stage_gather_row<FusedParams, ST, V, NS>(p, stage, x0, lane, h);
  lean_collide_store<FusedParams, MODEL, PL, ST, V, FORCE>(p, h, y, x0);
}

// blocks per SM the ring's shared memory allows (at most 2048 threads): the
// register budget is set so that many blocks fit
template <int ST, int V, int NW, int NS>
constexpr int pf_min_blocks() {
  constexpr int by_smem = (227 * 1024) / (NW * PfGeom<ST, V, NS>::WARP_BYTES);
  constexpr int by_threads = 2048 / (NW * 32);
  constexpr int b = by_smem < by_threads ? by_smem : by_threads;
  return b < 1 ? 1 : b;
}

template <int MODEL, bool PL, int ST, int V, int FORCE, int NW, int NS>
__global__ void __launch_bounds__(NW * 32, (pf_min_blocks<ST, V, NW, NS>())) k_fused_bulk_pf(const FusedParams p) {
  using G = PfGeom<ST, V, NS>;
  extern __shared__ __align__(16) unsigned char pf_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* ring = pf_smem + warp * G::WARP_BYTES;
  const int gw = blockIdx.x * NW + warp, GW = gridDim.x * NW;
  const int n = p.nplain;
  if (gw >= n) return;
#pragma unroll
  for (int m = 0; m < NS - 1; ++m) {
    const int pos = gw + m * GW;
    pf_issue<ST, V, NS>(p, ring + m * G::STAGE_BYTES, pos < n ? p.plain[pos] : -1, lane);
  }
  int pos_next = gw + (NS - 1) * GW;
  int item_next = pos_next < n ? p.plain[pos_next] : -1;  // read one iteration early
  for (int m = 0;; ++m) {
    if (gw + m * GW >= n) break;
    const int pos_after = pos_next + GW;
    const int item_after = pos_after < n ? p.plain[pos_after] : -1;
    pf_issue<ST, V, NS>(p, ring + ((m + NS - 1) % NS) * G::STAGE_BYTES, item_next, lane);
    cp_async_wait<NS - 1>();  // this lane's copies of segment m have landed
    pf_consume<MODEL, PL, ST, V, FORCE, NS>(p, ring + (m % NS) * G::STAGE_BYTES, lane);
    pos_next = pos_after;
    item_next = item_after;
  }
  cp_async_wait<0>();
}

}  // namespace lbm
