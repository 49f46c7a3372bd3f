// Shared device code for the D2Q9 kernels: lattice constants, equilibrium,
// Guo forcing, the three collision operators, rheology, pseudopotentials and
// error reporting.  Formulas follow taichi_lbm/CollisionEngine.py,
// taichi_lbm/FluidModels.py and taichi_lbm/EOS.py (cited per function).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lbm_gb300.h"

namespace lbm {

// D2Q9 set in the reference's order (taichi_lbm/lbm.py:44-45).
__host__ __device__ constexpr int CX(int k) {
  return (k == 1 || k == 5 || k == 8) ? 1 : ((k == 3 || k == 6 || k == 7) ? -1 : 0);
}
__host__ __device__ constexpr int CY(int k) {
  return (k == 2 || k == 5 || k == 6) ? 1 : ((k == 4 || k == 7 || k == 8) ? -1 : 0);
}
// bounce map (taichi_lbm/BoundaryCondition.py:242)
__host__ __device__ constexpr int OPP(int k) {
  return k == 0 ? 0 : (k <= 4 ? ((k + 1) % 4 + 1) : ((k - 3) % 4 + 5));
}
__host__ __device__ constexpr float W(int k) {
  return k == 0 ? 4.0f / 9.0f : (k <= 4 ? 1.0f / 9.0f : 0.25f / 9.0f);
}
// PlaneBoundary unknown populations (taichi_lbm/BoundaryCondition.py:63-72)
__host__ __device__ inline int unknown_pop(int dir, int t) {
  switch (dir) {
    case 1: return t == 0 ? 3 : (t == 1 ? 6 : 7);
    case 3: return t == 0 ? 1 : (t == 1 ? 5 : 8);
    case 4: return t == 0 ? 2 : (t == 1 ? 5 : 6);
    default: return t == 0 ? 4 : (t == 1 ? 7 : 8);
  }
}
__device__ inline int cx_dyn(int k) { return CX(k); }
__device__ inline int cy_dyn(int k) { return CY(k); }
__device__ inline float w_dyn(int k) { return k == 0 ? W(0) : (k <= 4 ? W(1) : W(5)); }

// Equilibrium, CollisionEngine.py:15-18
__device__ __forceinline__ float feq_k(int k, float rho, float ux, float uy, float uu) {
  const float eu = (float)CX(k) * ux + (float)CY(k) * uy;
  return W(k) * rho * (1.0f + 3.0f * eu + 4.5f * eu * eu - 1.5f * uu);
}

// Guo forcing population, CollisionEngine.py:21-25
__device__ __forceinline__ float force_k(int k, float Fx, float Fy, float ux, float uy, float uF) {
  const float cF = (float)CX(k) * Fx + (float)CY(k) * Fy;
  const float cu = (float)CX(k) * ux + (float)CY(k) * uy;
  return W(k) * (3.0f * cF + 9.0f * cF * cu - 3.0f * uF);
}

// Collision.tau_max_min, CollisionEngine.py:29-34
__device__ __forceinline__ float clamp_tau(float t, float lo, float hi) {
  return t < lo ? lo : (t > hi ? hi : t);
}

// PowerLawFluid.apparent_viscosity * 3 + 1/2, clamped (FluidModels.py:20-29,
// CollisionEngine.py:72-78)
__device__ __forceinline__ float powerlaw_tau(float m, float n, float gamma, float lo, float hi) {
  return clamp_tau(m * powf(gamma, n - 1.0f) * 3.0f + 0.5f, lo, hi);
}

// Strain-rate magnitude from non-equilibrium populations, CollisionEngine.py:86-92
__device__ __forceinline__ float shear_from_neq(const float fn[9], float cof) {
  const float Sxx = (fn[1] + fn[3] + fn[5] + fn[6] + fn[7] + fn[8]) * cof;
  const float Syy = (fn[2] + fn[4] + fn[5] + fn[6] + fn[7] + fn[8]) * cof;
  const float Sxy = (fn[5] - fn[6] + fn[7] - fn[8]) * cof;
  return sqrtf(2.0f * (Sxx * Sxx + Syy * Syy + 2.0f * Sxy * Sxy));
}

// MRT transform rows (CollisionEngine.py:273-282); the rows are orthogonal, so
// M^-1 = M^T diag(1/|row|^2) with |row|^2 = 9,36,36,6,12,6,12,4,4.
__host__ __device__ constexpr float MRT_M(int a, int k) {
  // row-major table as a constexpr switch (compile-time folded when unrolled)
  return a == 0 ? 1.0f
       : a == 1 ? (k == 0 ? -4.0f : (k <= 4 ? -1.0f : 2.0f))
       : a == 2 ? (k == 0 ? 4.0f : (k <= 4 ? -2.0f : 1.0f))
       : a == 3 ? (float)CX(k)
       : a == 4 ? (k == 0 ? 0.0f : (k <= 4 ? -2.0f * CX(k) : (float)CX(k)))
       : a == 5 ? (float)CY(k)
       : a == 6 ? (k == 0 ? 0.0f : (k <= 4 ? -2.0f * CY(k) : (float)CY(k)))
       : a == 7 ? (k == 1 || k == 3 ? 1.0f : (k == 2 || k == 4 ? -1.0f : 0.0f))
       : (k == 5 || k == 7 ? 1.0f : (k == 6 || k == 8 ? -1.0f : 0.0f));
}
__host__ __device__ constexpr float MRT_NORM2(int a) {
  return a == 0 ? 9.0f : (a <= 2 ? 36.0f : (a == 3 || a == 5 ? 6.0f : (a == 4 || a == 6 ? 12.0f : 4.0f)));
}
__host__ __device__ constexpr float MRT_MINV(int k, int a) { return MRT_M(a, k) / MRT_NORM2(a); }

__device__ __forceinline__ void mrt_forward(const float f[9], float m[9]) {
#pragma unroll
  for (int a = 0; a < 9; ++a) {
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; ++k)
      if (MRT_M(a, k) != 0.0f) s += MRT_M(a, k) * f[k];
    m[a] = s;
  }
}
__device__ __forceinline__ void mrt_backward(const float m[9], float f[9]) {
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float s = 0.0f;
#pragma unroll
    for (int a = 0; a < 9; ++a)
      if (MRT_M(a, k) != 0.0f) s += MRT_MINV(k, a) * m[a];
    f[k] = s;
  }
}

// Equilibrium moments, CollisionEngine.py:388-406
__device__ __forceinline__ void mrt_meq(float rho, float jx, float jy, float meq[9]) {
  const float u2 = jx * jx + jy * jy;
  meq[0] = rho;
  meq[1] = rho * (-2.0f + 3.0f * u2);
  meq[2] = rho * (1.0f - 3.0f * u2);
  meq[3] = rho * jx;
  meq[4] = -rho * jx;
  meq[5] = rho * jy;
  meq[6] = -rho * jy;
  meq[7] = rho * (jx * jx - jy * jy);
  meq[8] = rho * (jx * jy);
}
// Guo forcing moments, CollisionEngine.py:408-422
__device__ __forceinline__ void mrt_mforce(float Fx, float Fy, float ux, float uy, float mf[9]) {
  const float Fu = Fx * ux + Fy * uy;
  mf[0] = 0.0f;
  mf[1] = 6.0f * Fu;
  mf[2] = -6.0f * Fu;
  mf[3] = Fx;
  mf[4] = -Fx;
  mf[5] = Fy;
  mf[6] = -Fy;
  mf[7] = 2.0f * (Fx * ux - Fy * uy);
  mf[8] = Fy * ux + Fx * uy;
}

// BGK collide in place, CollisionEngine.py:96-110
__device__ __forceinline__ void collide_bgk(float f[9], float rho, float ux, float uy, float Fx, float Fy,
                                            float omega, bool force) {
  const float uu = ux * ux + uy * uy;
  const float uF = ux * Fx + uy * Fy;
  const float cf = 1.0f - 0.5f * omega;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float v = f[k] - omega * (f[k] - feq_k(k, rho, ux, uy, uu));
    if (force) v += cf * force_k(k, Fx, Fy, ux, uy, uF);
    f[k] = v;
  }
}

// TRT collide in place, CollisionEngine.py:181-245 (pairs (1,3),(2,4),(5,7),(6,8))
__device__ __forceinline__ void collide_trt(float f[9], float rho, float ux, float uy, float Fx, float Fy,
                                            float os, float oa, bool force) {
  const float uu = ux * ux + uy * uy;
  const float uF = ux * Fx + uy * Fy;
  float e[9], F[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    e[k] = feq_k(k, rho, ux, uy, uu);
    F[k] = force ? force_k(k, Fx, Fy, ux, uy, uF) : 0.0f;
  }
  const float cs = 1.0f - 0.5f * os, ca = 1.0f - 0.5f * oa;
  f[0] = f[0] - os * (f[0] - e[0]) + cs * F[0];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int k = p < 2 ? p + 1 : p + 3;  // 1, 2, 5, 6
    const int o = OPP(k);                 // 3, 4, 7, 8
    const float fs = 0.5f * (f[k] + f[o]), fa = 0.5f * (f[k] - f[o]);
    const float es = 0.5f * (e[k] + e[o]), ea = 0.5f * (e[k] - e[o]);
    const float Fs = 0.5f * (F[k] + F[o]), Fa = 0.5f * (F[k] - F[o]);
    const float sym = -os * (fs - es) + cs * Fs;
    const float anti = -oa * (fa - ea) + ca * Fa;
    f[k] = f[k] + sym + anti;
    f[o] = f[o] + sym - anti;
  }
}

// MRT collide in place with relaxation rates s[9], CollisionEngine.py:424-451
__device__ __forceinline__ void collide_mrt(float f[9], float rho, float ux, float uy, float Fx, float Fy,
                                            const float s[9], bool force) {
  float m[9], meq[9], mf[9];
  mrt_forward(f, m);
  mrt_meq(rho, ux, uy, meq);
  if (force) mrt_mforce(Fx, Fy, ux, uy, mf);
#pragma unroll
  for (int a = 0; a < 9; ++a) {
    float v = m[a] - s[a] * (m[a] - meq[a]);
    if (force) v += (1.0f - 0.5f * s[a]) * mf[a];
    m[a] = v;
  }
  mrt_backward(m, f);
}

// ---------------------------------------------------------------- EOS
// EOS.py:28-32 (get_psi) over the equations of state EOS.py:40-95
__device__ __forceinline__ float eos_psi(const LbmEos& e, float d, float T) {
  if (e.kind == LBM_EOS_SC) return e.rho0 * (1.0f - expf(-d / e.rho0));
  float p;
  if (e.kind == LBM_EOS_VDW) {
    p = d * e.R * T / (1.0f - e.b * d) - e.a * d * d;
  } else if (e.kind == LBM_EOS_RK) {
    p = d * e.R * T / (1.0f - e.b * d) - e.a * d * d / sqrtf(T) / (1.0f + e.b * d);
  } else if (e.kind == LBM_EOS_PR) {
    const float om = e.omega;
    const float kap = 0.37464f + 1.54226f * om - 0.269922f * om * om;
    const float s = 1.0f + kap * (1.0f - sqrtf(T / e.T_cr));
    const float bd = e.b * d;
    p = d * e.R * T / (1.0f - bd) - e.a * s * s * d * d / (1.0f + 2.0f * bd - bd * bd);
  } else {  // CS
    const float b4 = e.b * d * 0.25f;
    const float one = 1.0f - b4;
    p = d * e.R * T * (1.0f + b4 + b4 * b4 - b4 * b4 * b4) / (one * one * one) - e.a * d * d;
  }
  return sqrtf(fabsf(6.0f / e.G * (p - d / 3.0f)));
}

}  // namespace lbm

// ---------------------------------------------------------------- errors
namespace lbm_err {
int set(int code, const char* fmt, ...);
int cuda(cudaError_t e, const char* what);
int launch(const char* what);
}  // namespace lbm_err
