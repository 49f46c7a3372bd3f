// Fused single-component Shan-Chen step on a fully periodic lattice.
//
// The reference's Shan-Chen step (cases/Bubble or two-phase separation.py:
// 197-212) computes, from the post-stream populations of every node,
// rho -> psi(rho, T) (EOS.py:28-47, ExternalForce.py:137-142), wraps psi
// periodically (SCBoundaryCondition.py:365-383), then the force
// F(x) = -g psi(x) sum_k w_k c_k psi(x + c_k) (ExternalForce.py:145-158),
// F_body = F + rho/rho_tot g (lbm.py:215-220), the velocity and the
// collision.  A node's force needs psi of its eight neighbours in the same
// step, so one block owns a tile of SC_ROWS rows x 32*V columns: each warp
// gathers one row (pull stream, as k_fused) and writes psi to shared memory;
// the rows above and below the tile and the column on either side are
// gathered too (they are mostly L2 hits: the neighbouring tiles read the same
// lines), then the force, moments and collision run from registers and the
// shared psi tile.  HBM traffic stays one read and one write of the
// populations per lattice update.
#pragma once

#include "lbm_fused.cuh"

namespace lbm {

constexpr int SC_ROWS = 8;  // rows per block = warps per block

template <int V>
__device__ __forceinline__ float density_of(const float (&f)[V][9], int i) {
  return ((f[i][0] + f[i][1]) + (f[i][2] + f[i][3])) + ((f[i][4] + f[i][5]) + (f[i][6] + f[i][7])) + f[i][8];
}

// rho of one node (scalar periodic pull)
template <int ST>
__device__ __forceinline__ float density_at(const FusedParams& p, int x, int y) {
  using S = Storage<ST>;
  using T = typename S::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  float r = 0.0f;
#pragma unroll
  for (int k = 0; k < 9; ++k)
    r += S::dec(load1(src + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch + wrap(x - CX(k), p.nx)),
                p.wsh[k]);
  return r;
}

template <int MODEL, int ST, int V>
__global__ void __launch_bounds__(SC_ROWS * 32) k_fused_sc(const FusedParams p) {
  using S = Storage<ST>;
  using T = typename S::T;
  constexpr int W_ = 32 * V;       // tile width
  constexpr int PW = W_ + 2;       // psi row: columns x0s-1 .. x0s+W_
  __shared__ float psi[SC_ROWS + 2][PW];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_y = p.ny / SC_ROWS;
  const int ty = blockIdx.x % tiles_y, seg = blockIdx.x / tiles_y;
  const int y0 = ty * SC_ROWS, x0s = seg * W_;
  const int x0 = x0s + lane * V;
  const bool live = x0 < p.nx;
  const int wlast = min(W_, p.nx - x0s);  // nodes of this segment inside the lattice

  // halo rows first (their populations are not kept): warp 0 the row above
  // the tile, the last warp the row below
  if (warp == 0 || warp == SC_ROWS - 1) {
    const int r = warp == 0 ? 0 : SC_ROWS + 1;
    const int yh = wrap(warp == 0 ? y0 - 1 : y0 + SC_ROWS, p.ny);
    float h[V][9];
    gather_direct<ST, V>(p, yh, seg, lane, h);
#pragma unroll
    for (int i = 0; i < V; ++i)
      if (lane * V + i < wlast) psi[r][1 + lane * V + i] = eos_psi(p.eos, density_of<V>(h, i), p.sc_T);
  }
  // column halos of all SC_ROWS + 2 rows: left = column x0s-1, right = the
  // column after the segment's last node (wraps to column 0 at the edge)
  if (lane == 0 || lane == 31) {
    for (int r = warp; r < SC_ROWS + 2; r += SC_ROWS) {
      const int yh = wrap(y0 - 1 + r, p.ny);
      if (lane == 0) psi[r][0] = eos_psi(p.eos, density_at<ST>(p, wrap(x0s - 1, p.nx), yh), p.sc_T);
      else psi[r][1 + wlast] = eos_psi(p.eos, density_at<ST>(p, wrap(x0s + wlast, p.nx), yh), p.sc_T);
    }
  }
  // the warp's own row
  const int y = y0 + warp;
  float f[V][9];
  gather_direct<ST, V>(p, y, seg, lane, f);
  float rho[V];
#pragma unroll
  for (int i = 0; i < V; ++i) {
    rho[i] = density_of<V>(f, i);
    if (lane * V + i < wlast) psi[warp + 1][1 + lane * V + i] = eos_psi(p.eos, rho[i], p.sc_T);
  }
  __syncthreads();

  float s[9];
#pragma unroll
  for (int a = 0; a < 9; ++a) s[a] = p.s[a];
#pragma unroll
  for (int i = 0; i < V; ++i) {
    const int c = 1 + lane * V + i;
    float Fx = 0.0f, Fy = 0.0f;
#pragma unroll
    for (int k = 1; k < 9; ++k) {
      const float ps = psi[warp + 1 + CY(k)][c + CX(k)];
      Fx += W(k) * (float)CX(k) * ps;
      Fy += W(k) * (float)CY(k) * ps;
    }
    const float m = -p.g_coh * psi[warp + 1][c];
    Fx = Fx * m + p.gx;
    Fy = Fy * m + p.gy;
    float* fi = f[i];
    const float r = rho[i];
    const float jx = (fi[1] - fi[3]) + (fi[5] - fi[6]) + (fi[8] - fi[7]);
    const float jy = (fi[2] - fi[4]) + (fi[5] + fi[6]) - (fi[7] + fi[8]);
    const float ux = (jx + 0.5f * Fx) / r, uy = (jy + 0.5f * Fy) / r;
    if (MODEL == LBM_BGK) collide_bgk(fi, r, ux, uy, Fx, Fy, p.omega, true);
    else if (MODEL == LBM_TRT) collide_trt(fi, r, ux, uy, Fx, Fy, p.omega, p.omega_a, true);
    else collide_mrt(fi, r, ux, uy, Fx, Fy, s, true);
  }
  if (!live) return;
  T* dst = reinterpret_cast<T*>(p.dst);
  const size_t rowoff = (size_t)y * p.pitch;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    T raw[V];
#pragma unroll
    for (int i = 0; i < V; ++i) raw[i] = S::enc(f[i][k], p.wsh[k]);
    store_vec<T, V>(dst + (size_t)k * p.plane + rowoff + x0, raw);
  }
}

}  // namespace lbm
