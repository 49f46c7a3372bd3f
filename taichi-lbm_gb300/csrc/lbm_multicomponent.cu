// Multi-component Shan-Chen (taichi_lbm/ExternalForce.py:66-117, lbm.py:145-237
// with num_components > 1): per-stage kernels over a component-major lattice
// (LbmMCLattice), one thread per group node, each with exactly the effect of
// the reference method it replaces.  Components share the mixture velocity,
// total density and total pressure; each has its own populations, density,
// pressure, psi, Shan-Chen force and body force.
#include <cstring>

#include "lbm_common.cuh"

namespace {

using namespace lbm;

constexpr int TPB = 256;
inline unsigned blocks_for(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

struct MI {
  int nx, ny, pitch, psi_pitch, nc;
  size_t plane, psi_plane;
  __device__ size_t at(int i, int j) const { return (size_t)j * pitch + i; }
  __device__ size_t psi(int c, int i, int j) const {
    return (size_t)c * psi_plane + (size_t)(j + 1) * psi_pitch + (i + 1);
  }
};
__device__ inline MI mi_of(const LbmMCLattice& L) {
  return MI{L.nx, L.ny, L.pitch, L.psi_pitch, L.nc, (size_t)L.ny * L.pitch, (size_t)(L.ny + 2) * L.psi_pitch};
}

// lbm.py:119-125: f = f2 = feq(rho_c, vel) for every component
__global__ void k_mc_init_feq(LbmMCLattice L, const int32_t* g, int64_t n) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const MI I = mi_of(L);
  const size_t q = I.at(g[2 * m], g[2 * m + 1]);
  const float ux = L.vel[q], uy = L.vel[I.plane + q];
  const float uu = ux * ux + uy * uy;
  for (int c = 0; c < I.nc; ++c) {
    const float r = L.rho[c * I.plane + q];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const float e = feq_k(k, r, ux, uy, uu);
      L.f[(c * 9 + k) * I.plane + q] = e;
      L.f2[(c * 9 + k) * I.plane + q] = e;
    }
  }
}

// lbm.py:153-164 (after the whole-field fills): rho_c = sum_k f_c, total += rho_c
__global__ void k_mc_density(LbmMCLattice L, const int32_t* g, int64_t n) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const MI I = mi_of(L);
  const size_t q = I.at(g[2 * m], g[2 * m + 1]);
  float tot = L.total_rho[q];
  for (int c = 0; c < I.nc; ++c) {
    float r = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; ++k) r += L.f[(c * 9 + k) * I.plane + q];
    L.rho[c * I.plane + q] = r;
    tot += r;
  }
  L.total_rho[q] = tot;
}

// lbm.py:185-202 (after the fill of pressure): pressure2
__global__ void k_mc_pressure2(LbmMCLattice L, LbmMCShanChen s, const int32_t* g, int64_t n) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const MI I = mi_of(L);
  const int i = g[2 * m], j = g[2 * m + 1];
  const size_t q = I.at(i, j);
  for (int c = 0; c < I.nc; ++c) {
    const float ps = L.psi[I.psi(c, i, j)];
    L.pressure[c * I.plane + q] += (L.rho[c * I.plane + q] + 0.5f * s.g_coh[c][c] * (ps * ps)) / 3.0f;
  }
  float p_ij = 0.0f, p_ii = 0.0f;
  for (int c1 = 0; c1 < I.nc; ++c1) {
    p_ii += L.pressure[c1 * I.plane + q];
    for (int c2 = c1 + 1; c2 < I.nc; ++c2)
      p_ij += s.g_coh[c1][c2] * L.psi[I.psi(c1, i, j)] * L.psi[I.psi(c2, i, j)];
  }
  L.total_pressure[q] = p_ii + p_ij / 6.0f;
}

// ExternalForce.py:86-92: psi of components 0 and 1 from their densities
__global__ void k_mc_update_psi(LbmMCLattice L, LbmMCShanChen s, const int32_t* g, int64_t n) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const MI I = mi_of(L);
  const int i = g[2 * m], j = g[2 * m + 1];
  const size_t q = I.at(i, j);
  for (int c = 0; c < 2; ++c) L.psi[I.psi(c, i, j)] = eos_psi(s.eos[c], L.rho[c * I.plane + q], L.temperature[q]);
}

// SCBoundaryCondition.py:126-144, every component: axis 0 = LR, 1 = BT
__global__ void k_mc_psi_periodic(LbmMCLattice L, int axis) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const MI I = mi_of(L);
  for (int c = 0; c < I.nc; ++c) {
    if (axis == 0) {
      const int y = t - 1;
      if (y > L.ny) return;
      L.psi[I.psi(c, -1, y)] = L.psi[I.psi(c, L.nx - 1, y)];
      L.psi[I.psi(c, L.nx, y)] = L.psi[I.psi(c, 0, y)];
    } else {
      const int x = t - 1;
      if (x > L.nx) return;
      L.psi[I.psi(c, x, -1)] = L.psi[I.psi(c, x, L.ny - 1)];
      L.psi[I.psi(c, x, L.ny)] = L.psi[I.psi(c, x, 0)];
    }
  }
}

// ExternalForce.py:96-117 (after the fill of SCforce): cohesion with the
// other components' psi at fluid neighbours, adhesion g_adh at the others
__global__ void k_mc_sc_force(LbmMCLattice L, LbmMCShanChen s, const int32_t* g, int64_t n) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const MI I = mi_of(L);
  const int i = g[2 * m], j = g[2 * m + 1];
  const size_t q = I.at(i, j);
  for (int c1 = 0; c1 < I.nc; ++c1) {
    float cx = 0.0f, cy = 0.0f, ax = 0.0f, ay = 0.0f;
#pragma unroll
    for (int k = 1; k < 9; ++k) {
      const int x2 = i + CX(k), y2 = j + CY(k);
      const float wcx = W(k) * (float)CX(k), wcy = W(k) * (float)CY(k);
      if (s.fluid[(size_t)(y2 + 1) * L.psi_pitch + (x2 + 1)]) {
        for (int c2 = 0; c2 < I.nc; ++c2) {
          if (c2 == c1) continue;
          const float p = L.psi[I.psi(c2, x2, y2)];
          cx += wcx * p * s.g_coh[c1][c2];
          cy += wcy * p * s.g_coh[c1][c2];
        }
      } else {
        ax += wcx * s.g_adh[c1];
        ay += wcy * s.g_adh[c1];
      }
    }
    const float mp = -L.psi[I.psi(c1, i, j)];
    L.sc_force[(c1 * 2) * I.plane + q] = mp * (cx + ax);
    L.sc_force[(c1 * 2 + 1) * I.plane + q] = mp * (cy + ay);
  }
}

// lbm.py:215-220: body force of every component
__global__ void k_mc_force_density(LbmMCLattice L, const int32_t* g, int64_t n) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const MI I = mi_of(L);
  const size_t q = I.at(g[2 * m], g[2 * m + 1]);
  for (int c = 0; c < I.nc; ++c) {
    const float r = L.rho[c * I.plane + q] / L.total_rho[q];
    L.body_force[(c * 2) * I.plane + q] = L.sc_force[(c * 2) * I.plane + q] + r * L.gravity[0];
    L.body_force[(c * 2 + 1) * I.plane + q] = L.sc_force[(c * 2 + 1) * I.plane + q] + r * L.gravity[1];
  }
}

// lbm.py:223-237: the mixture velocity (sum over components of the momentum
// and half the body force, over the total density)
__global__ void k_mc_velocity(LbmMCLattice L, const int32_t* g, int64_t n) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const MI I = mi_of(L);
  const size_t q = I.at(g[2 * m], g[2 * m + 1]);
  float vx = 0.0f, vy = 0.0f;
  for (int c = 0; c < I.nc; ++c) {
    float tx = 0.0f, ty = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const float fk = L.f[(c * 9 + k) * I.plane + q];
      tx += fk * (float)CX(k);
      ty += fk * (float)CY(k);
    }
    tx += 0.5f * L.body_force[(c * 2) * I.plane + q];
    ty += 0.5f * L.body_force[(c * 2 + 1) * I.plane + q];
    vx += tx;
    vy += ty;
  }
  L.vel[q] = vx / L.total_rho[q];
  L.vel[I.plane + q] = vy / L.total_rho[q];
}

// CollisionEngine.py:96-110 for every component: BGK with the component's
// relaxation time tau[c] ([nc][ny][pitch]), density and body force, and
// the mixture velocity
__global__ void k_mc_bgk(LbmMCLattice L, const float* tau, const int32_t* g, int64_t n) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const MI I = mi_of(L);
  const size_t q = I.at(g[2 * m], g[2 * m + 1]);
  const float ux = L.vel[q], uy = L.vel[I.plane + q];
  for (int c = 0; c < I.nc; ++c) {
    float f[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) f[k] = L.f[(c * 9 + k) * I.plane + q];
    collide_bgk(f, L.rho[c * I.plane + q], ux, uy, L.body_force[(c * 2) * I.plane + q],
                L.body_force[(c * 2 + 1) * I.plane + q], 1.0f / tau[c * I.plane + q], true);
#pragma unroll
    for (int k = 0; k < 9; ++k) L.f2[(c * 9 + k) * I.plane + q] = f[k];
  }
}

// BoundaryCondition.py:419-432 for every component: periodic pull stream
__global__ void k_mc_stream_periodic(LbmMCLattice L, const int32_t* g, int64_t n) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const MI I = mi_of(L);
  const int i = g[2 * m], j = g[2 * m + 1];
  const size_t q = I.at(i, j);
  for (int c = 0; c < I.nc; ++c) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      int xs = i - CX(k), ys = j - CY(k);
      xs = xs < 0 ? xs + L.nx : (xs >= L.nx ? xs - L.nx : xs);
      ys = ys < 0 ? ys + L.ny : (ys >= L.ny ? ys - L.ny : ys);
      L.f[(c * 9 + k) * I.plane + q] = L.f2[(c * 9 + k) * I.plane + I.at(xs, ys)];
    }
  }
}

int check(const LbmMCLattice* L, const int32_t* g, int64_t n) {
  if (!L) return lbm_err::set(LBM_ERR_ARG, "multi-component: NULL lattice");
  if (L->nc < 1 || L->nc > LBM_MC_MAX) return lbm_err::set(LBM_ERR_ARG, "multi-component: nc %d", L->nc);
  if (L->nx <= 0 || L->ny <= 0 || L->pitch < L->nx || L->psi_pitch < L->nx + 2)
    return lbm_err::set(LBM_ERR_ARG, "multi-component: lattice %d x %d pitch %d", L->nx, L->ny, L->pitch);
  if (n < 0 || (n > 0 && !g)) return lbm_err::set(LBM_ERR_ARG, "multi-component: bad group");
  return LBM_OK;
}

void zero(float* a, size_t count, cudaStream_t s) {
  if (a && count) cudaMemsetAsync(a, 0, count * sizeof(float), s);
}

}  // namespace

extern "C" {

#define S_ cudaStream_t(stream)
#define PLANE(L) ((size_t)(L)->ny * (L)->pitch)

int lbm_mc_init_feq(const LbmMCLattice* L, const int32_t* g, int64_t n, void* stream) {
  int rc = check(L, g, n);
  if (rc) return rc;
  if (n) k_mc_init_feq<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n);
  return lbm_err::launch("mc_init_feq");
}

int lbm_mc_density(const LbmMCLattice* L, const int32_t* g, int64_t n, void* stream) {
  int rc = check(L, g, n);
  if (rc) return rc;
  zero(L->rho, (size_t)L->nc * PLANE(L), S_);
  zero(L->total_rho, PLANE(L), S_);
  if (n) k_mc_density<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n);
  return lbm_err::launch("mc_density");
}

int lbm_mc_pressure2(const LbmMCLattice* L, const LbmMCShanChen* s, const int32_t* g, int64_t n, void* stream) {
  int rc = check(L, g, n);
  if (rc) return rc;
  if (!s) return lbm_err::set(LBM_ERR_ARG, "mc_pressure2: NULL Shan-Chen parameters");
  zero(L->pressure, (size_t)L->nc * PLANE(L), S_);
  if (n) k_mc_pressure2<<<blocks_for(n), TPB, 0, S_>>>(*L, *s, g, n);
  return lbm_err::launch("mc_pressure2");
}

int lbm_mc_update_psi(const LbmMCLattice* L, const LbmMCShanChen* s, const int32_t* g, int64_t n, void* stream) {
  int rc = check(L, g, n);
  if (rc) return rc;
  if (!s || L->nc < 2) return lbm_err::set(LBM_ERR_ARG, "mc_update_psi: needs two components and parameters");
  if (n) k_mc_update_psi<<<blocks_for(n), TPB, 0, S_>>>(*L, *s, g, n);
  return lbm_err::launch("mc_update_psi");
}

int lbm_mc_psi_periodic(const LbmMCLattice* L, int32_t axis, void* stream) {
  int rc = check(L, nullptr, 0);
  if (rc) return rc;
  const int n = (axis == 0 ? L->ny : L->nx) + 2;
  k_mc_psi_periodic<<<(n + TPB - 1) / TPB, TPB, 0, S_>>>(*L, axis);
  return lbm_err::launch("mc_psi_periodic");
}

int lbm_mc_sc_force(const LbmMCLattice* L, const LbmMCShanChen* s, const int32_t* g, int64_t n, void* stream) {
  int rc = check(L, g, n);
  if (rc) return rc;
  if (!s || !s->fluid) return lbm_err::set(LBM_ERR_ARG, "mc_sc_force: needs the fluid map");
  zero(L->sc_force, (size_t)L->nc * 2 * PLANE(L), S_);
  if (n) k_mc_sc_force<<<blocks_for(n), TPB, 0, S_>>>(*L, *s, g, n);
  return lbm_err::launch("mc_sc_force");
}

int lbm_mc_force_density(const LbmMCLattice* L, const int32_t* g, int64_t n, void* stream) {
  int rc = check(L, g, n);
  if (rc) return rc;
  if (n) k_mc_force_density<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n);
  return lbm_err::launch("mc_force_density");
}

int lbm_mc_velocity(const LbmMCLattice* L, const int32_t* g, int64_t n, void* stream) {
  int rc = check(L, g, n);
  if (rc) return rc;
  zero(L->vel, 2 * PLANE(L), S_);
  if (n) k_mc_velocity<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n);
  return lbm_err::launch("mc_velocity");
}

int lbm_mc_bgk_apply(const LbmMCLattice* L, const float* tau, const int32_t* g, int64_t n, void* stream) {
  int rc = check(L, g, n);
  if (rc) return rc;
  if (!tau) return lbm_err::set(LBM_ERR_ARG, "mc_bgk_apply: NULL relaxation times");
  if (n) k_mc_bgk<<<blocks_for(n), TPB, 0, S_>>>(*L, tau, g, n);
  return lbm_err::launch("mc_bgk_apply");
}

int lbm_mc_stream_periodic(const LbmMCLattice* L, const int32_t* g, int64_t n, void* stream) {
  int rc = check(L, g, n);
  if (rc) return rc;
  if (n) k_mc_stream_periodic<<<blocks_for(n), TPB, 0, S_>>>(*L, g, n);
  return lbm_err::launch("mc_stream_periodic");
}

}  // extern "C"
