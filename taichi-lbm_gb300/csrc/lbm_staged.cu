// Per-stage kernels: one launch per reference @ti.kernel method, one thread per
// group node, with exactly that method's effect on the lattice fields.  These
// give the drop-in its unfused call surface (a user's own lbm_solve() keeps
// working) and run the first collision and the last stream of a fused run.
#include "lbm_common.cuh"

namespace {

using namespace lbm;

constexpr int TPB = 256;

struct Idx {
  int nx, ny, pitch;
  size_t plane;
  __device__ size_t at(int i, int j) const { return (size_t)j * pitch + i; }
};
__device__ inline Idx idx_of(const LbmLattice& L) {
  return Idx{L.nx, L.ny, L.pitch, (size_t)L.ny * L.pitch};
}
__device__ inline size_t psi_at(const LbmLattice& L, int i, int j) {
  return (size_t)(j + 1) * L.psi_pitch + (i + 1);
}

inline unsigned blocks_for(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

// ------------------------------------------------------------------ setup
// lbm.py:127-142
__global__ void k_neighbor_classify(LbmLattice L) {
  Idx I = idx_of(L);
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y;
  if (i >= L.nx) return;
  size_t q = I.at(i, j);
  if (L.mask[q] == -1) return;
  unsigned bits = 0x8000u;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    int i2 = i - CX(k), j2 = j - CY(k);
    if (i2 >= 0 && i2 < L.nx && j2 >= 0 && j2 < L.ny && L.mask[I.at(i2, j2)] != -1) bits |= 1u << k;
  }
  L.links[q] = (uint16_t)bits;
}

// lbm.py:119-125
__global__ void k_init_feq(LbmLattice L, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  size_t q = I.at(g[2 * m], g[2 * m + 1]);
  float r = L.rho[q], ux = L.vel[q], uy = L.vel[I.plane + q];
  float uu = ux * ux + uy * uy;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float e = feq_k(k, r, ux, uy, uu);
    L.f[k * I.plane + q] = e;
    L.f2[k * I.plane + q] = e;
  }
}

// ---------------------------------------------------------------- moments
__global__ void k_fill(float* a, size_t n, float v) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; t < n; t += (size_t)gridDim.x * blockDim.x) a[t] = v;
}

void fill(float* a, size_t n, float v, cudaStream_t s) {
  if (!a || n == 0) return;
  unsigned b = (unsigned)((n + TPB - 1) / TPB);
  if (b > 152u * 16u) b = 152u * 16u;
  k_fill<<<b, TPB, 0, s>>>(a, n, v);
}

// lbm.py:153-164 (after the whole-field fills)
__global__ void k_density(LbmLattice L, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  size_t q = I.at(g[2 * m], g[2 * m + 1]);
  float r = 0.0f;
#pragma unroll
  for (int k = 0; k < 9; ++k) r += L.f[k * I.plane + q];
  L.rho[q] = r;
  L.total_rho[q] += r;
}

// lbm.py:166-182
__global__ void k_pressure(LbmLattice L, const int32_t* g, int64_t n, int with_sc, float g_coh) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  int i = g[2 * m], j = g[2 * m + 1];
  size_t q = I.at(i, j);
  float p;
  if (with_sc) {
    float ps = L.psi[psi_at(L, i, j)];
    p = (L.rho[q] + 0.5f * g_coh * ps * ps) / 3.0f;
  } else {
    p = L.rho[q] / 3.0f;
  }
  float v = L.pressure[q] + p;
  L.pressure[q] = v;
  L.total_pressure[q] = v;
}

// lbm.py:215-220
__global__ void k_force_density(LbmLattice L, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  size_t q = I.at(g[2 * m], g[2 * m + 1]);
  float s = L.rho[q] / L.total_rho[q];
  float scx = L.sc_force ? L.sc_force[q] : 0.0f, scy = L.sc_force ? L.sc_force[I.plane + q] : 0.0f;
  L.body_force[q] = scx + s * L.gravity[0];
  L.body_force[I.plane + q] = scy + s * L.gravity[1];
}

// lbm.py:223-237 for one node (also BoundaryCondition.py:287-298)
__device__ inline void velocity_node(const LbmLattice& L, const Idx& I, size_t q) {
  float vx = 0.0f, vy = 0.0f;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float fk = L.f[k * I.plane + q];
    vx += fk * (float)CX(k);
    vy += fk * (float)CY(k);
  }
  vx += 0.5f * L.body_force[q];
  vy += 0.5f * L.body_force[I.plane + q];
  L.vel[q] = vx / L.total_rho[q];
  L.vel[I.plane + q] = vy / L.total_rho[q];
}

__global__ void k_velocity(LbmLattice L, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  velocity_node(L, I, I.at(g[2 * m], g[2 * m + 1]));
}

// BoundaryCondition.py:274-280 for one node
__device__ inline void density_node(const LbmLattice& L, const Idx& I, size_t q) {
  float r = 0.0f;
#pragma unroll
  for (int k = 0; k < 9; ++k) r += L.f[k * I.plane + q];
  L.rho[q] = r;
  L.total_rho[q] = r;
}

// -------------------------------------------------------------- collision
__device__ inline float app_visc(const LbmCollision& c, float gamma) {
  return c.fluid_model == LBM_POWERLAW ? c.pl_m * powf(gamma, c.pl_n - 1.0f) : c.nu;
}

// CollisionEngine.py:65-70, 149-155, 301-318 (diag.fill(1) is done by the host)
__global__ void k_init_tau(LbmLattice L, LbmCollision c, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  size_t q = I.at(g[2 * m], g[2 * m + 1]);
  if (c.model == LBM_BGK) {
    c.tau[q] = c.nu * 3.0f + 0.5f;
  } else if (c.model == LBM_TRT) {
    float ts = c.nu * 3.0f + 0.5f;
    c.tau_sym[q] = ts;
    c.tau_antisym[q] = c.magic / (ts - 0.5f) + 0.5f;
  } else {
    float t = clamp_tau(c.nu * 3.0f + 0.5f, c.tau_min, c.tau_max);
    float tb = clamp_tau(c.nu_bulk * 3.0f + 0.5f, c.tau_min, c.tau_max);
    c.diag[7 * I.plane + q] = 1.0f / t;
    c.diag[8 * I.plane + q] = 1.0f / t;
    c.diag[1 * I.plane + q] = 1.0f / tb;
    c.diag[0 * I.plane + q] = 0.0f;
    c.diag[3 * I.plane + q] = 0.0f;
    c.diag[5 * I.plane + q] = 0.0f;
  }
}

// CollisionEngine.py:80-92, 166-178, 332-377
__global__ void k_shear_rate(LbmLattice L, LbmCollision c, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  size_t q = I.at(g[2 * m], g[2 * m + 1]);
  float r = L.rho[q], ux = L.vel[q], uy = L.vel[I.plane + q];
  float uu = ux * ux + uy * uy;
  float fn[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) fn[k] = L.f[k * I.plane + q] - feq_k(k, r, ux, uy, uu);
  float out;
  if (c.model == LBM_MRT) {
    float mn[9], mneq[9];
    // M^-1 S M fneq with the reference's stored M_inverse
#pragma unroll
    for (int a = 0; a < 9; ++a) {
      float s = 0.0f;
#pragma unroll
      for (int k = 0; k < 9; ++k) s += MRT_M(a, k) * fn[k];
      mn[a] = c.diag[a * I.plane + q] * s;
    }
#pragma unroll
    for (int a = 0; a < 9; ++a) {
      float s = 0.0f;
#pragma unroll
      for (int b = 0; b < 9; ++b) s += c.m_inverse[a * 9 + b] * mn[b];
      mneq[a] = s;
    }
    out = shear_from_neq(mneq, -1.5f / r);
  } else {
    float t = c.model == LBM_BGK ? c.tau[q] : c.tau_sym[q];
    out = shear_from_neq(fn, -1.5f / r / t);
  }
  L.shear_rate[q] = out;
}

// CollisionEngine.py:72-78, 157-164, 322-329
__global__ void k_relaxation_time(LbmLattice L, LbmCollision c, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  size_t q = I.at(g[2 * m], g[2 * m + 1]);
  float t = clamp_tau(app_visc(c, L.shear_rate[q]) * 3.0f + 0.5f, c.tau_min, c.tau_max);
  if (c.model == LBM_BGK) {
    c.tau[q] = t;
  } else if (c.model == LBM_TRT) {
    c.tau_sym[q] = t;
    c.tau_antisym[q] = c.magic / (t - 0.5f) + 0.5f;
  } else {
    c.diag[7 * I.plane + q] = 1.0f / t;
    c.diag[8 * I.plane + q] = 1.0f / t;
  }
}

// CollisionEngine.py:96-110, 223-245, 424-451
__global__ void k_collide(LbmLattice L, LbmCollision c, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  size_t q = I.at(g[2 * m], g[2 * m + 1]);
  float f[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) f[k] = L.f[k * I.plane + q];
  float r = L.rho[q], ux = L.vel[q], uy = L.vel[I.plane + q];
  float Fx = L.body_force[q], Fy = L.body_force[I.plane + q];
  if (c.model == LBM_BGK) {
    collide_bgk(f, r, ux, uy, Fx, Fy, 1.0f / c.tau[q], true);
  } else if (c.model == LBM_TRT) {
    collide_trt(f, r, ux, uy, Fx, Fy, 1.0f / c.tau_sym[q], 1.0f / c.tau_antisym[q], true);
  } else {
    float s[9];
#pragma unroll
    for (int a = 0; a < 9; ++a) s[a] = c.diag[a * I.plane + q];
    collide_mrt(f, r, ux, uy, Fx, Fy, s, true);
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) L.f2[k * I.plane + q] = f[k];
}

// --------------------------------------------------------------- Shan-Chen
// ExternalForce.py:42-47
__global__ void k_update_psi(LbmLattice L, LbmEos e, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  int i = g[2 * m], j = g[2 * m + 1];
  size_t q = I.at(i, j);
  L.psi[psi_at(L, i, j)] = eos_psi(e, L.rho[q], L.temperature[q]);
}

// SC force at one node, ExternalForce.py:50-63 / BoundaryCondition.py:301-312
__device__ inline void sc_force_node(const LbmLattice& L, const Idx& I, int i, int j, float g_coh) {
  float Fx = 0.0f, Fy = 0.0f;
#pragma unroll
  for (int k = 1; k < 9; ++k) {
    float p = L.psi[psi_at(L, i + CX(k), j + CY(k))];
    Fx += W(k) * (float)CX(k) * p;
    Fy += W(k) * (float)CY(k) * p;
  }
  float s = -g_coh * L.psi[psi_at(L, i, j)];
  size_t q = I.at(i, j);
  L.sc_force[q] = Fx * s;
  L.sc_force[I.plane + q] = Fy * s;
}

__global__ void k_sc_force(LbmLattice L, float g_coh, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  sc_force_node(L, I, g[2 * m], g[2 * m + 1], g_coh);
}

// SCBoundaryCondition.py:126-144
__global__ void k_psi_periodic(LbmLattice L, int axis) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (axis == 0) {  // PeriodicPsi_LR: y in [-1, NY]
    int y = t - 1;
    if (y > L.ny) return;
    L.psi[psi_at(L, -1, y)] = L.psi[psi_at(L, L.nx - 1, y)];
    L.psi[psi_at(L, L.nx, y)] = L.psi[psi_at(L, 0, y)];
  } else {  // PeriodicPsi_BT: x in [-1, NX]
    int x = t - 1;
    if (x > L.nx) return;
    L.psi[psi_at(L, x, -1)] = L.psi[psi_at(L, x, L.ny - 1)];
    L.psi[psi_at(L, x, L.ny)] = L.psi[psi_at(L, x, 0)];
  }
}

// SCBoundaryCondition.py:19-110 — open psi boundaries (LBM_PSI_OPEN_*) on
// a group of psi nodes, one thread walking the group in order: the
// convective kinds average the velocity of the neighbours x - c_dir over the
// group first (in group order, as the reference's serial schedule does) and
// relax towards the neighbours with lambda = |U|.  Each node reads only
// psi nodes off the group line, so the order of the updates does not matter.
__global__ void k_psi_open(LbmLattice L, const int32_t* g, int64_t n, int kind, int dir) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  Idx I = idx_of(L);
  const int cx = cx_dyn(dir), cy = cy_dyn(dir);
  float lam = 0.0f;
  if (kind == LBM_PSI_OPEN_CONV1 || kind == LBM_PSI_OPEN_CONV2) {
    float ux = 0.0f, uy = 0.0f;
    for (int64_t m = 0; m < n; ++m) {
      const size_t q2 = I.at(g[2 * m] - cx, g[2 * m + 1] - cy);
      ux = ux + L.vel[q2];
      uy = uy + L.vel[I.plane + q2];
    }
    ux = ux / (float)n;
    uy = uy / (float)n;
    lam = 1.0f * sqrtf(ux * ux + uy * uy);
  }
  for (int64_t m = 0; m < n; ++m) {
    const int i = g[2 * m], j = g[2 * m + 1];
    float* p = L.psi + psi_at(L, i, j);
    const float p2 = L.psi[psi_at(L, i - cx, j - cy)];
    if (kind == LBM_PSI_OPEN_NEUMANN) {
      *p = p2;
    } else if (kind == LBM_PSI_OPEN_CONV1) {
      *p = (*p + lam * p2) / (1.0f + lam);
    } else {
      const float p3 = L.psi[psi_at(L, i - 2 * cx, j - 2 * cy)];
      if (kind == LBM_PSI_OPEN_CONV2) *p = (*p + 2.0f * lam * p2 - 0.5f * lam * p3) / (1.0f + 1.5f * lam);
      else *p = 2.0f * p2 - p3;
    }
  }
}

// SCBoundaryCondition.py:119-123
__global__ void k_psi_fixed(LbmLattice L, const int32_t* g, int64_t n, float v) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  L.psi[psi_at(L, g[2 * m], g[2 * m + 1])] = v;
}

// ------------------------------------------------------- boundary kernels
// BoundaryCondition.py:424-432 (PeriodicAll), 440-449 (Inside), 244-259 (BounceBack)
__global__ void k_stream(LbmLattice L, int kind, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  int i = g[2 * m], j = g[2 * m + 1];
  size_t q = I.at(i, j);
  unsigned links = kind == LBM_BC_PERIODIC ? 0u : L.links[q];
  bool classified = (links & 0x8000u) != 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float v;
    if (kind == LBM_BC_PERIODIC) {
      int x2 = (i - CX(k) + L.nx) % L.nx, y2 = (j - CY(k) + L.ny) % L.ny;
      v = L.f2[k * I.plane + I.at(x2, y2)];
    } else if (!classified) {
      // neighbor entries never written: the reference reads f2[0, 0]
      v = L.f2[k * I.plane + I.at(0, 0)];
    } else if (links & (1u << k)) {
      v = L.f2[k * I.plane + I.at(i - CX(k), j - CY(k))];
    } else if (kind == LBM_BC_BOUNCEBACK) {
      v = L.f2[OPP(k) * I.plane + q];
    } else {
      continue;  // InsideBoundary with no source: an out-of-range read in the reference
    }
    L.f[k * I.plane + q] = v;
  }
}

// BoundaryCondition.py:119-129
__device__ inline float rhow(int dir, float vx, float vy, const float f[9]) {
  if (dir == 2) return 1.0f / (1.0f + vy) * (f[0] + f[1] + f[3] + 2.0f * (f[2] + f[5] + f[6]));
  if (dir == 4) return 1.0f / (1.0f - vy) * (f[0] + f[1] + f[3] + 2.0f * (f[4] + f[7] + f[8]));
  if (dir == 1) return 1.0f / (1.0f + vx) * (f[0] + f[2] + f[4] + 2.0f * (f[1] + f[5] + f[8]));
  return 1.0f / (1.0f - vx) * (f[0] + f[2] + f[4] + 2.0f * (f[3] + f[6] + f[7]));
}

__global__ void k_boundary(LbmLattice L, LbmBoundary b, const int32_t* g, int64_t n) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  Idx I = idx_of(L);
  const int i = g[2 * m], j = g[2 * m + 1];
  const int dir = b.direction;
  const int i2 = i - cx_dyn(dir), j2 = j - cy_dyn(dir);
  const size_t q = I.at(i, j);
  const size_t P = I.plane;
  float Ux = b.velocity[0], Uy = b.velocity[1];
  if (b.velocity_per_node) {
    Ux = b.velocity_per_node[2 * m];
    Uy = b.velocity_per_node[2 * m + 1];
  }
  float f[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) f[k] = L.f[k * P + q];

  switch (b.kind) {
    case LBM_BC_VELOCITY_BB: {  // BoundaryCondition.py:85-102
      float rw = L.rho[q];
      for (int t = 0; t < 3; ++t) {
        int d = unknown_pop(dir, t);
        float cv = (float)cx_dyn(d) * Ux + (float)cy_dyn(d) * Uy;
        L.f[d * P + q] = f[d] + 6.0f * w_dyn(d) * rw * cv;
      }
      break;
    }
    case LBM_BC_VELOCITY_EQ:      // BoundaryCondition.py:137-147
    case LBM_BC_VELOCITY_NEEM: {  // BoundaryCondition.py:154-166
      L.vel[q] = Ux;
      L.vel[P + q] = Uy;
      float r = rhow(dir, Ux, Uy, f);
      L.rho[q] = r;
      float uu = Ux * Ux + Uy * Uy;
      if (b.kind == LBM_BC_VELOCITY_EQ) {
#pragma unroll
        for (int k = 0; k < 9; ++k) L.f[k * P + q] = feq_k(k, r, Ux, Uy, uu);
      } else {
        size_t q2 = I.at(i2, j2);
        float u2x = L.vel[q2], u2y = L.vel[P + q2], r2 = L.rho[q2];
        float uu2 = u2x * u2x + u2y * u2y;
#pragma unroll
        for (int k = 0; k < 9; ++k)
          L.f[k * P + q] = feq_k(k, r, Ux, Uy, uu) + L.f[k * P + q2] - feq_k(k, r2, u2x, u2y, uu2);
      }
      break;
    }
    case LBM_BC_PRESSURE_ABC: {  // BoundaryCondition.py:182-205
      size_t q2 = I.at(i2, j2);
      float ux = 1.5f * L.vel[q] - 0.5f * L.vel[q2];
      float uy = 1.5f * L.vel[P + q] - 0.5f * L.vel[P + q2];
      L.vel[q] = ux;
      L.vel[P + q] = uy;
      L.total_rho[q] = b.rho_value;
      float uw2 = ux * ux + uy * uy;
      for (int t = 0; t < 3; ++t) {
        int d = unknown_pop(dir, t);
        float cu = (float)cx_dyn(d) * ux + (float)cy_dyn(d) * uy;
        float wd = w_dyn(d);
        L.f[d * P + q] = -f[d] + 2.0f * wd * b.rho_value * (1.0f + 4.5f * cu * cu - 1.5f * uw2);
      }
      break;
    }
    case LBM_BC_PRESSURE_NEEM: {  // BoundaryCondition.py:215-226
      size_t q2 = I.at(i2, j2);
      float ux = L.vel[q2], uy = L.vel[P + q2];
      L.vel[q] = ux;
      L.vel[P + q] = uy;
      L.total_rho[q] = b.rho_value;
      float r = L.rho[q], r2 = L.rho[q2];
      float uu = ux * ux + uy * uy;
      for (int t = 0; t < 3; ++t) {
        int d = unknown_pop(dir, t);
        float v = 0.0f;
        // feq(u_nb, rho_self) + f_nb - feq(u_nb, rho_nb), population d
#pragma unroll
        for (int k = 0; k < 9; ++k)
          if (k == d) v = feq_k(k, r, ux, uy, uu) + L.f[k * P + q2] - feq_k(k, r2, ux, uy, uu);
        L.f[d * P + q] = v;
      }
      break;
    }
    case LBM_BC_OPEN_NEUMANN:    // BoundaryCondition.py:321-334
    case LBM_BC_OPEN_CONV1: {    // BoundaryCondition.py:342-359
      size_t q2 = I.at(i2, j2);
      float lam = 0.0f;
      if (b.kind == LBM_BC_OPEN_CONV1) {
        float ux = L.vel[q2], uy = L.vel[P + q2];
        lam = sqrtf(ux * ux + uy * uy);
      }
      for (int t = 0; t < 3; ++t) {
        int d = unknown_pop(dir, t);
        float v = L.f[d * P + q2];
        if (b.kind == LBM_BC_OPEN_CONV1) v = (f[d] + lam * v) / (1.0f + lam);
        L.f[d * P + q] = v;
      }
      density_node(L, I, q);
      velocity_node(L, I, q);
      break;
    }
    case LBM_BC_OPEN_EXTRAP: {  // BoundaryCondition.py:400-411
      size_t q2 = I.at(i2, j2), q3 = I.at(i2 - cx_dyn(dir), j2 - cy_dyn(dir));
      for (int t = 0; t < 3; ++t) {
        int d = unknown_pop(dir, t);
        L.f[d * P + q] = 2.0f * L.f[d * P + q2] - L.f[d * P + q3];
      }
      break;
    }
    default:
      break;
  }
}

// OpenConvective2order, BoundaryCondition.py:369-390: three sweeps over the
// group, in group order, by one thread.  A node's update reads the psi of
// the boundary nodes next to it, which the same sweep rewrites, so the
// result depends on the order the nodes are visited in.  The reference
// makes its sweep loop the kernel's outermost (parallel) loop and visits the
// group inside it, which leaves that order to the scheduler; the order
// here is the serial one, sweep after sweep, node after node.  The group is
// one boundary line, so one thread is enough.
__device__ void open_conv2_node(const LbmLattice& L, const LbmBoundary& b, const int32_t* g, int64_t m);
__global__ void k_open_conv2(LbmLattice L, LbmBoundary b, const int32_t* g, int64_t n) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int it = 0; it < 3; ++it)
    for (int64_t m = 0; m < n; ++m) open_conv2_node(L, b, g, m);
}
__device__ void open_conv2_node(const LbmLattice& L, const LbmBoundary& b, const int32_t* g, int64_t m) {
  Idx I = idx_of(L);
  const size_t P = I.plane;
  const int i = g[2 * m], j = g[2 * m + 1], dir = b.direction;
  const int i2 = i - cx_dyn(dir), j2 = j - cy_dyn(dir);
  const int i3 = i - 2 * cx_dyn(dir), j3 = j - 2 * cy_dyn(dir);
  const size_t q = I.at(i, j), q2 = I.at(i2, j2), q3 = I.at(i3, j3);
  sc_force_node(L, I, i2, j2, b.g_coh);
  float s = L.rho[q2] / L.total_rho[q2];
  L.body_force[q2] = L.sc_force[q2] + s * L.gravity[0];
  L.body_force[P + q2] = L.sc_force[P + q2] + s * L.gravity[1];
  velocity_node(L, I, q2);
  float ux = L.vel[q2], uy = L.vel[P + q2];
  float lam = sqrtf(ux * ux + uy * uy);
  for (int t = 0; t < 3; ++t) {
    int d = unknown_pop(dir, t);
    L.f[d * P + q] = (L.f[d * P + q] + 2.0f * lam * L.f[d * P + q2] - 0.5f * lam * L.f[d * P + q3]) /
                     (1.0f + 1.5f * lam);
  }
  density_node(L, I, q);
  L.psi[psi_at(L, i, j)] = eos_psi(b.eos, L.rho[q], L.temperature[q]);
}

int check_lat(const LbmLattice* L, bool need_f = true);

// ------------------------------------------------------------ immersed boundary
// IBEngine (taichi_lbm/ibm.py:187-246): one thread per IB node.  The stencil
// of a node at (px, py) is the grid nodes floor..ceil in each direction
// (ibm.py:187-194) with weights (1 - |px - i|)(1 - |py - j|) (ibm.py:196-199).
// Stencil nodes outside the lattice are skipped: the reference's insider
// rule keeps nodes strictly inside, and reads there are undefined in it.
__device__ inline float ib_weight(float px, float py, int ix, int iy) {
  return (1.0f - fabsf(px - (float)ix)) * (1.0f - fabsf(py - (float)iy));
}

// InterpolateBodyVelocities (ibm.py:201-223)
__global__ void k_ibm_interpolate(LbmLattice L, LbmIBNodes N) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= N.n) return;
  const Idx I = idx_of(L);
  const float px = N.pos[2 * m], py = N.pos[2 * m + 1];
  const int xb = (int)floorf(px), yb = (int)floorf(py), xt = (int)ceilf(px), yt = (int)ceilf(py);
  float vx = 0.0f, vy = 0.0f;
  for (int ix = xb; ix <= xt; ++ix)
    for (int iy = yb; iy <= yt; ++iy) {
      if (ix < 0 || ix >= L.nx || iy < 0 || iy >= L.ny) continue;
      const float w = ib_weight(px, py, ix, iy);
      const size_t q = I.at(ix, iy);
      vx += L.vel[q] * w;
      vy += L.vel[I.plane + q] * w;
    }
  N.vel[2 * m] = vx;
  N.vel[2 * m + 1] = vy;
  const float fx = 2.0f * (N.vel_desired[2 * m] - vx), fy = 2.0f * (N.vel_desired[2 * m + 1] - vy);
  N.force_temp[2 * m] = fx;
  N.force_temp[2 * m + 1] = fy;
  N.force[2 * m] += fx;
  N.force[2 * m + 1] += fy;
}

// SpreadBodyForces (ibm.py:225-246): several IB nodes add into one grid node,
// so the adds are atomic (the reference's parallel loop adds in an arbitrary
// order as well)
__global__ void k_ibm_spread(LbmLattice L, LbmIBNodes N) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= N.n) return;
  const Idx I = idx_of(L);
  const float px = N.pos[2 * m], py = N.pos[2 * m + 1];
  const int xb = (int)floorf(px), yb = (int)floorf(py), xt = (int)ceilf(px), yt = (int)ceilf(py);
  for (int ix = xb; ix <= xt; ++ix)
    for (int iy = yb; iy <= yt; ++iy) {
      if (ix < 0 || ix >= L.nx || iy < 0 || iy >= L.ny) continue;
      const float w = ib_weight(px, py, ix, iy);
      const size_t q = I.at(ix, iy);
      const float tx = 0.0f + N.force_temp[2 * m] * w, ty = 0.0f + N.force_temp[2 * m + 1] * w;
      const float r2 = L.total_rho[q] * 2.0f;
      atomicAdd(&L.vel[q], tx / r2);
      atomicAdd(&L.vel[I.plane + q], ty / r2);
      atomicAdd(&L.body_force[q], (tx * L.rho[q]) / L.total_rho[q]);
      atomicAdd(&L.body_force[I.plane + q], (ty * L.rho[q]) / L.total_rho[q]);
    }
}

int check_ib(const LbmLattice* L, const LbmIBNodes* N) {
  int rc = check_lat(L, false);
  if (rc) return rc;
  if (!L->vel || !L->rho || !L->total_rho || !L->body_force)
    return lbm_err::set(LBM_ERR_ARG, "immersed boundary needs vel, rho, total_rho and body_force");
  if (!N || N->n < 0) return lbm_err::set(LBM_ERR_ARG, "IB nodes missing or negative count");
  if (N->n > 0 && (!N->pos || !N->vel || !N->vel_desired || !N->force || !N->force_temp))
    return lbm_err::set(LBM_ERR_ARG, "IB node arrays missing");
  return LBM_OK;
}

int check_lat(const LbmLattice* L, bool need_f) {
  if (!L) return lbm_err::set(LBM_ERR_ARG, "lattice is NULL");
  if (L->nx <= 0 || L->ny <= 0 || L->pitch < L->nx)
    return lbm_err::set(LBM_ERR_ARG, "bad lattice shape %d x %d pitch %d", L->nx, L->ny, L->pitch);
  if (need_f && (!L->f || !L->f2)) return lbm_err::set(LBM_ERR_ARG, "population buffers missing");
  return LBM_OK;
}

int check_group(const int32_t* g, int64_t n) {
  if (n < 0) return lbm_err::set(LBM_ERR_ARG, "negative group size");
  if (n > 0 && !g) return lbm_err::set(LBM_ERR_ARG, "group pointer is NULL");
  return LBM_OK;
}

}  // namespace

#define S_ cudaStream_t(stream)
#define CHECK(x)             \
  do {                       \
    int rc__ = (x);          \
    if (rc__) return rc__;   \
  } while (0)

extern "C" {

int lbm_neighbor_classify(const LbmLattice* L, void* stream) {
  CHECK(check_lat(L, false));
  if (!L->mask || !L->links) return lbm_err::set(LBM_ERR_ARG, "mask/links missing");
  dim3 grid((L->nx + TPB - 1) / TPB, L->ny);
  k_neighbor_classify<<<grid, TPB, 0, S_>>>(*L);
  return lbm_err::launch("neighbor_classify");
}

int lbm_init_feq(const LbmLattice* L, const int32_t* g, int64_t n, void* stream) {
  CHECK(check_lat(L));
  CHECK(check_group(g, n));
  if (n) k_init_feq<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n);
  return lbm_err::launch("init_feq");
}

int lbm_density(const LbmLattice* L, const int32_t* g, int64_t n, void* stream) {
  CHECK(check_lat(L));
  CHECK(check_group(g, n));
  size_t N = (size_t)L->ny * L->pitch;
  fill(L->total_rho, N, 0.0f, S_);
  fill(L->rho, N, 0.0f, S_);
  if (n) k_density<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n);
  return lbm_err::launch("density");
}

int lbm_pressure(const LbmLattice* L, const int32_t* g, int64_t n, int32_t with_sc, float g_coh,
                 void* stream) {
  CHECK(check_lat(L, false));
  CHECK(check_group(g, n));
  if (with_sc && !L->psi) return lbm_err::set(LBM_ERR_ARG, "pressure with Shan-Chen needs psi");
  fill(L->pressure, (size_t)L->ny * L->pitch, 0.0f, S_);
  if (n) k_pressure<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n, with_sc, g_coh);
  return lbm_err::launch("pressure");
}

int lbm_ibm_interpolate(const LbmLattice* L, const LbmIBNodes* N, void* stream) {
  CHECK(check_ib(L, N));
  if (N->n) k_ibm_interpolate<<<blocks_for(N->n), TPB, 0, S_>>>(*L, *N);
  return lbm_err::launch("ibm_interpolate");
}

int lbm_ibm_spread(const LbmLattice* L, const LbmIBNodes* N, void* stream) {
  CHECK(check_ib(L, N));
  if (N->n) k_ibm_spread<<<blocks_for(N->n), TPB, 0, S_>>>(*L, *N);
  return lbm_err::launch("ibm_spread");
}

int lbm_force_density(const LbmLattice* L, const int32_t* g, int64_t n, void* stream) {
  CHECK(check_lat(L, false));
  CHECK(check_group(g, n));
  if (n) k_force_density<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n);
  return lbm_err::launch("force_density");
}

int lbm_velocity(const LbmLattice* L, const int32_t* g, int64_t n, void* stream) {
  CHECK(check_lat(L));
  CHECK(check_group(g, n));
  fill(L->vel, (size_t)2 * L->ny * L->pitch, 0.0f, S_);
  if (n) k_velocity<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n);
  return lbm_err::launch("velocity");
}

static int check_coll(const LbmCollision* c) {
  if (!c) return lbm_err::set(LBM_ERR_ARG, "collision is NULL");
  if (c->model == LBM_BGK && !c->tau) return lbm_err::set(LBM_ERR_ARG, "BGK needs tau");
  if (c->model == LBM_TRT && (!c->tau_sym || !c->tau_antisym))
    return lbm_err::set(LBM_ERR_ARG, "TRT needs tau_sym/tau_antisym");
  if (c->model == LBM_MRT && !c->diag) return lbm_err::set(LBM_ERR_ARG, "MRT needs diag");
  if (c->model < 0 || c->model > 2) return lbm_err::set(LBM_ERR_ARG, "unknown collision model");
  return LBM_OK;
}

int lbm_collision_init_tau(const LbmLattice* L, const LbmCollision* c, const int32_t* g, int64_t n,
                           void* stream) {
  CHECK(check_lat(L, false));
  CHECK(check_coll(c));
  CHECK(check_group(g, n));
  if (c->model == LBM_MRT) fill(c->diag, (size_t)9 * L->ny * L->pitch, 1.0f, S_);
  if (n) k_init_tau<<<blocks_for(n), TPB, 0, S_>>>(*L, *c, g, n);
  return lbm_err::launch("init_tau");
}

int lbm_collision_shear_rate(const LbmLattice* L, const LbmCollision* c, const int32_t* g, int64_t n,
                             void* stream) {
  CHECK(check_lat(L));
  CHECK(check_coll(c));
  CHECK(check_group(g, n));
  if (n) k_shear_rate<<<blocks_for(n), TPB, 0, S_>>>(*L, *c, g, n);
  return lbm_err::launch("shear_rate");
}

int lbm_collision_relaxation_time(const LbmLattice* L, const LbmCollision* c, const int32_t* g,
                                  int64_t n, void* stream) {
  CHECK(check_lat(L, false));
  CHECK(check_coll(c));
  CHECK(check_group(g, n));
  if (n) k_relaxation_time<<<blocks_for(n), TPB, 0, S_>>>(*L, *c, g, n);
  return lbm_err::launch("relaxation_time");
}

int lbm_collision_apply(const LbmLattice* L, const LbmCollision* c, const int32_t* g, int64_t n,
                        void* stream) {
  CHECK(check_lat(L));
  CHECK(check_coll(c));
  CHECK(check_group(g, n));
  if (n) k_collide<<<blocks_for(n), TPB, 0, S_>>>(*L, *c, g, n);
  return lbm_err::launch("collision_apply");
}

int lbm_sc_update_psi(const LbmLattice* L, const LbmEos* e, const int32_t* g, int64_t n, void* stream) {
  CHECK(check_lat(L, false));
  CHECK(check_group(g, n));
  if (!e || !L->psi || !L->temperature) return lbm_err::set(LBM_ERR_ARG, "update_psi needs eos/psi/T");
  if (n) k_update_psi<<<blocks_for(n), TPB, 0, S_>>>(*L, *e, g, n);
  return lbm_err::launch("update_psi");
}

int lbm_sc_force(const LbmLattice* L, float g_coh, const int32_t* g, int64_t n, void* stream) {
  CHECK(check_lat(L, false));
  CHECK(check_group(g, n));
  if (!L->psi || !L->sc_force) return lbm_err::set(LBM_ERR_ARG, "sc_force needs psi/SCforce");
  fill(L->sc_force, (size_t)2 * L->ny * L->pitch, 0.0f, S_);
  if (n) k_sc_force<<<blocks_for(n), TPB, 0, S_>>>(*L, g_coh, g, n);
  return lbm_err::launch("sc_force");
}

int lbm_psi_periodic(const LbmLattice* L, int32_t axis, void* stream) {
  CHECK(check_lat(L, false));
  if (!L->psi) return lbm_err::set(LBM_ERR_ARG, "psi missing");
  int n = (axis == 0 ? L->ny : L->nx) + 2;
  k_psi_periodic<<<(n + TPB - 1) / TPB, TPB, 0, S_>>>(*L, axis);
  return lbm_err::launch("psi_periodic");
}

int lbm_psi_open(const LbmLattice* L, const int32_t* g, int64_t n, int32_t kind, int32_t direction,
                 void* stream) {
  int rc = check_lat(L, false);
  if (rc) return rc;
  if (!L->psi) return lbm_err::set(LBM_ERR_ARG, "psi_open: the lattice has no psi field");
  if (kind < LBM_PSI_OPEN_NEUMANN || kind > LBM_PSI_OPEN_EXTRAP) return lbm_err::set(LBM_ERR_ARG, "psi_open: kind %d", kind);
  if (direction < 1 || direction > 4) return lbm_err::set(LBM_ERR_ARG, "psi_open: direction %d", direction);
  if (n < 0 || (n > 0 && !g)) return lbm_err::set(LBM_ERR_ARG, "psi_open: bad group");
  if (n && (kind == LBM_PSI_OPEN_CONV1 || kind == LBM_PSI_OPEN_CONV2) && !L->vel)
    return lbm_err::set(LBM_ERR_ARG, "psi_open: the convective kinds read the velocity field");
  if (n) k_psi_open<<<1, 32, 0, S_>>>(*L, g, n, kind, direction);
  return lbm_err::launch("psi_open");
}

int lbm_psi_fixed(const LbmLattice* L, const int32_t* g, int64_t n, float value, void* stream) {
  CHECK(check_lat(L, false));
  CHECK(check_group(g, n));
  if (!L->psi) return lbm_err::set(LBM_ERR_ARG, "psi missing");
  if (n) k_psi_fixed<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n, value);
  return lbm_err::launch("psi_fixed");
}

int lbm_boundary_apply(const LbmLattice* L, const LbmBoundary* b, const int32_t* g, int64_t n,
                       void* stream) {
  CHECK(check_lat(L));
  CHECK(check_group(g, n));
  if (!b) return lbm_err::set(LBM_ERR_ARG, "boundary is NULL");
  if (n == 0 || b->kind == LBM_BC_FLUID) return LBM_OK;
  switch (b->kind) {
    case LBM_BC_PERIODIC:
    case LBM_BC_INSIDE:
    case LBM_BC_BOUNCEBACK:
      if (b->kind != LBM_BC_PERIODIC && !L->links)
        return lbm_err::set(LBM_ERR_ARG, "stream carrier needs the neighbor table");
      k_stream<<<blocks_for(n), TPB, 0, S_>>>(*L, b->kind, g, n);
      return lbm_err::launch("stream");
    case LBM_BC_OPEN_CONV2:
      if (!L->psi || !L->sc_force || !L->temperature)
        return lbm_err::set(LBM_ERR_ARG, "OpenConvective2order needs the Shan-Chen fields");
      k_open_conv2<<<1, 32, 0, S_>>>(*L, *b, g, n);
      return lbm_err::launch("open_conv2");
    default:
      if (b->kind < LBM_BC_VELOCITY_BB || b->kind > LBM_BC_OPEN_EXTRAP)
        return lbm_err::set(LBM_ERR_ARG, "unknown boundary kind %d", b->kind);
      if (b->direction < 1 || b->direction > 4)
        return lbm_err::set(LBM_ERR_ARG, "boundary direction must be 1..4");
      k_boundary<<<blocks_for(n), TPB, 0, S_>>>(*L, *b, g, n);
      return lbm_err::launch("boundary");
  }
}

}  // extern "C"
