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
template <int ST>
__device__ __forceinline__ float raw_to_float(typename Storage<ST>::T v);
template <>
__device__ __forceinline__ float raw_to_float<LBM_STORE_F32>(float v) { return v; }
template <>
__device__ __forceinline__ float raw_to_float<LBM_STORE_F16S>(__half v) { return __half2float(v); }
template <>
__device__ __forceinline__ float raw_to_float<LBM_STORE_BF16S>(__nv_bfloat16 v) { return __bfloat162float(v); }

// V consecutive stored values -> floats (no shift)
template <int ST, int V>
__device__ __forceinline__ void load_raw(const typename Storage<ST>::T* p, float (&c)[V]) {
  using T = typename Storage<ST>::T;
  T raw[V];
  load_vec<T, V>(p, raw);
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
  } else {
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      __nv_bfloat162 t;
      memcpy(&t, &raw[i], sizeof(t));
      const float2 u = __bfloat1622float2(t);
      c[i] = u.x;
      c[i + 1] = u.y;
    }
  }
}

// V floats -> V consecutive stored values (round to nearest, no shift)
template <int ST, int V>
__device__ __forceinline__ void store_raw(typename Storage<ST>::T* p, const float (&c)[V]) {
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
  } else {
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      const __nv_bfloat162 t = __floats2bfloat162_rn(c[i], c[i + 1]);
      memcpy(&raw[i], &t, sizeof(t));
    }
  }
  store_vec<T, V>(p, raw);
}

// Pull gather of an interior segment (x0s > 0 and x0s + 32 V < nx): every
// lane is inside the lattice, the elements across the segment's edges exist
// without wrapping, and node nx-1 is not in the segment.
template <int ST, int V>
__device__ __forceinline__ void gather_interior(const FusedParams& p, int y, int x0, int lane, float (&h)[V][9]) {
  using T = typename Storage<ST>::T;
  constexpr unsigned FULL = 0xffffffffu;
  const T* src = reinterpret_cast<const T*>(p.src);
  const int ym = wrap(y - 1, p.ny), yp = wrap(y + 1, p.ny);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int ys = CY(k) == 0 ? y : (CY(k) == 1 ? ym : yp);
    const T* row = src + (size_t)k * p.plane + (size_t)ys * p.pitch + x0;
    float c[V];
    load_raw<ST, V>(row, c);
    if (CX(k) == 0) {
#pragma unroll
      for (int i = 0; i < V; ++i) h[i][k] = c[i];
    } else if (CX(k) == 1) {
      float left = __shfl_up_sync(FULL, c[V - 1], 1);
      if (lane == 0) left = raw_to_float<ST>(load1(row - 1));
      h[0][k] = left;
#pragma unroll
      for (int i = 1; i < V; ++i) h[i][k] = c[i - 1];
    } else {
      float right = __shfl_down_sync(FULL, c[0], 1);
      if (lane == 31) right = raw_to_float<ST>(load1(row + V));
#pragma unroll
      for (int i = 0; i < V - 1; ++i) h[i][k] = c[i + 1];
      h[V - 1][k] = right;
    }
  }
}

// Pull gather of any segment (x edges wrap, lanes past nx read nothing),
// stored values without the shift.
template <int ST, int V>
__device__ __forceinline__ void gather_edge(const FusedParams& p, int y, int x0, int lane, float (&h)[V][9]) {
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
      load_raw<ST, V>(row + x0, c);
    } else {
#pragma unroll
      for (int i = 0; i < V; ++i) c[i] = 0.0f;
    }
    if (CX(k) == 0) {
#pragma unroll
      for (int i = 0; i < V; ++i) h[i][k] = c[i];
    } else if (CX(k) == 1) {
      float left = __shfl_up_sync(FULL, c[V - 1], 1);
      if (lane == 0 && live) left = raw_to_float<ST>(load1(row + wrap(x0 - 1, p.nx)));
      h[0][k] = left;
#pragma unroll
      for (int i = 1; i < V; ++i) h[i][k] = c[i - 1];
    } else {
      float right = __shfl_down_sync(FULL, c[0], 1);
      if (lane == 31 && live) right = raw_to_float<ST>(load1(row + wrap(x0 + V, p.nx)));
#pragma unroll
      for (int i = 0; i < V - 1; ++i) h[i][k] = c[i + 1];
      h[V - 1][k] = right;
      if (live && ilast < V) {  // node nx-1 pulls from column 0
        const float v0 = raw_to_float<ST>(load1(row));
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
__device__ __forceinline__ void shifted_feq(const FusedParams& p, float rho, float ux, float uy, float e[9]) {
  const float base = fmaf(-1.5f, fmaf(ux, ux, uy * uy), 1.0f);
  const float r0 = rho * W(0), r1 = rho * W(1), r2 = rho * W(5);
  const float a1 = 3.0f * r1, a2 = 3.0f * r2;
  e[0] = fmaf(r0, base, -p.wsh[0]);
  const float eu[4] = {ux, uy, ux + uy, uy - ux};  // c.u of k = 1, 2, 5, 6
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = q < 2 ? q + 1 : q + 3;
    const float r = q < 2 ? r1 : r2, a = q < 2 ? a1 : a2;
    const float t = fmaf(4.5f * eu[q], eu[q], base);
    const float sym = fmaf(r, t, -p.wsh[k]);
    const float anti = a * eu[q];
    e[k] = sym + anti;
    e[OPP(k)] = sym - anti;
  }
}

// Guo forcing populations F_k (CollisionEngine.py:21-25), by pairs
__device__ __forceinline__ void pair_force(float Fx, float Fy, float ux, float uy, float F[9]) {
  const float uF = ux * Fx + uy * Fy;
  F[0] = W(0) * (-3.0f * uF);
  const float eu[4] = {ux, uy, ux + uy, uy - ux};
  const float eF[4] = {Fx, Fy, Fx + Fy, Fy - Fx};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = q < 2 ? q + 1 : q + 3;
    const float w = W(k);
    const float sym = w * fmaf(9.0f * eF[q], eu[q], -3.0f * uF);
    const float anti = w * 3.0f * eF[q];
    F[k] = sym + anti;
    F[OPP(k)] = sym - anti;
  }
}

// One node: moments, relaxation and collision of the stored values h in
// place; returns the new power-law state (or the old one).
template <int MODEL, bool PL, int FORCE>
__device__ __forceinline__ float collide_lean(const FusedParams& p, float h[9], float state) {
  const float dr = ((h[0] + h[1]) + (h[2] + h[3])) + ((h[4] + h[5]) + (h[6] + h[7])) + h[8];
  const float rho = dr + p.rho_shift;
  const float jx = (h[1] - h[3]) + (h[5] - h[6]) + (h[8] - h[7]);
  const float jy = (h[2] - h[4]) + (h[5] + h[6]) - (h[7] + h[8]);
  const float Fx = FORCE == 1 ? p.gx : 0.0f, Fy = FORCE == 1 ? p.gy : 0.0f;
  const float inv = 1.0f / rho;
  const float ux = (FORCE == 1 ? fmaf(0.5f, Fx, jx) : jx) * inv;
  const float uy = (FORCE == 1 ? fmaf(0.5f, Fy, jy) : jy) * inv;
  float e[9];
  shifted_feq(p, rho, ux, uy, e);
  float F[9];
  if (FORCE == 1) pair_force(Fx, Fy, ux, uy, F);

  if (MODEL == LBM_MRT) {
    // m = M h; equilibrium moments less the moments of the shift (M wsh)
    float n[9], m[9], meq[9], s[9];
#pragma unroll
    for (int a = 0; a < 9; ++a) s[a] = p.s[a];
    if (PL) {
      // CollisionEngine.py:332-377 with the previous step's s7 = s8 = state
#pragma unroll
      for (int k = 0; k < 9; ++k) n[k] = h[k] - e[k];
      float mn[9], mneq[9];
      mrt_forward(n, mn);
      s[7] = s[8] = state;
#pragma unroll
      for (int a = 0; a < 9; ++a) mn[a] *= s[a];
      mrt_backward(mn, mneq);
      const float gamma = shear_from_neq(mneq, -1.5f / rho);
      state = 1.0f / powerlaw_tau(p.pl_m, p.pl_n, gamma, p.tau_min, p.tau_max);
      s[7] = s[8] = state;
    }
    mrt_forward(h, m);
    mrt_meq(rho, ux, uy, meq);
    float mf[9];
    if (FORCE == 1) mrt_mforce(Fx, Fy, ux, uy, mf);
#pragma unroll
    for (int a = 0; a < 9; ++a) {
      float v = m[a] - s[a] * (m[a] - (meq[a] - p.mwsh[a]));
      if (FORCE == 1) v += (1.0f - 0.5f * s[a]) * mf[a];
      m[a] = v;
    }
    mrt_backward(m, h);
    return state;
  }

  float om = p.omega, oa = p.omega_a;
  if (PL) {
    // CollisionEngine.py:80-92 / 166-178 (previous tau), then :72-78 / 157-164
    float n[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) n[k] = h[k] - e[k];
    const float t = powerlaw_tau(p.pl_m, p.pl_n, shear_from_neq(n, -1.5f / rho / state), p.tau_min, p.tau_max);
    state = t;
    om = 1.0f / t;
    if (MODEL == LBM_TRT) oa = 1.0f / (p.magic / (t - 0.5f) + 0.5f);
  }
  if (MODEL == LBM_BGK) {
    const float cf = 1.0f - 0.5f * om;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float v = fmaf(om, e[k] - h[k], h[k]);
      if (FORCE == 1) v = fmaf(cf, F[k], v);
      h[k] = v;
    }
    return state;
  }
  // TRT, pairs (1,3), (2,4), (5,7), (6,8)
  const float cs = 1.0f - 0.5f * om, ca = 1.0f - 0.5f * oa;
  h[0] = fmaf(om, e[0] - h[0], h[0]);
  if (FORCE == 1) h[0] = fmaf(cs, F[0], h[0]);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = q < 2 ? q + 1 : q + 3, o = OPP(k);
    const float hs = 0.5f * (h[k] + h[o]), ha = 0.5f * (h[k] - h[o]);
    const float es = 0.5f * (e[k] + e[o]), ea = 0.5f * (e[k] - e[o]);
    float sym = om * (es - hs), anti = oa * (ea - ha);
    if (FORCE == 1) {
      sym = fmaf(cs, 0.5f * (F[k] + F[o]), sym);
      anti = fmaf(ca, 0.5f * (F[k] - F[o]), anti);
    }
    h[k] = h[k] + sym + anti;
    h[o] = h[o] + sym - anti;
  }
  return state;
}

// Two-pass form of the direct step.  k_fused_bulk takes the plain segments
// (seg_flags == 0), with the body force fixed at compile time, and leaves the
// flagged segments to k_fused_special (lbm_fused.cuh), which walks the
// compact list p.special of their indices (y * nseg + seg).  The two write
// disjoint nodes and read only the source state, so they may run in either
// order or concurrently within a step.
template <int MODEL, bool PL, int ST, int V, int FORCE>
__global__ void __launch_bounds__(256) k_fused_bulk(const FusedParams p) {
  using T = typename Storage<ST>::T;
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= (long long)p.ny * p.nseg) return;
  if (p.seg_flags[warp]) return;  // uniform over the warp
  const int y = (int)(warp / p.nseg);
  const int seg = (int)(warp - (long long)y * p.nseg);
  const int x0s = seg * 32 * V, x0 = x0s + lane * V;
  float h[V][9];
  if (x0s > 0 && x0s + 32 * V < p.nx) gather_interior<ST, V>(p, y, x0, lane, h);
  else gather_edge<ST, V>(p, y, x0, lane, h);
  const bool live = x0 < p.nx;
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
#pragma unroll
  for (int i = 0; i < V; ++i) {
    const float st = collide_lean<MODEL, PL, FORCE>(p, h[i], PL ? tau[i] : 0.0f);
    if (PL) tau[i] = st;
  }
  if (!live) return;
  if (PL) store_vec<float, V>(p.tau + rowoff + x0, tau);
  T* dst = reinterpret_cast<T*>(p.dst);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float c[V];
#pragma unroll
    for (int i = 0; i < V; ++i) c[i] = h[i][k];
    store_raw<ST, V>(dst + (size_t)k * p.plane + rowoff + x0, c);
  }
}

}  // namespace lbm
