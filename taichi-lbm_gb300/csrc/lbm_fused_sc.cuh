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

#include "lbm_fused_lean.cuh"

namespace lbm {

constexpr int SC_ROWS = 8;  // rows per block = warps per block

// Density of a node from its stored (shifted) values h: the pairwise sum of
// collide_lean, so psi and the collision see the same rho.
__device__ __forceinline__ float density_raw(const float h[9], float rho_shift) {
  return (((h[0] + h[1]) + (h[2] + h[3])) + ((h[4] + h[5]) + (h[6] + h[7])) + h[8]) + rho_shift;
}

// rho of one node (periodic pull of its nine stored values)
template <int ST>
__device__ __forceinline__ float density_at(const FusedParams& p, int x, int y) {
  using T = typename Storage<ST>::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  float h[9];
#pragma unroll
  for (int k = 0; k < 9; ++k)
    h[k] = raw_to_float<ST>(
        load1(src + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch + wrap(x - CX(k), p.nx)));
  return density_raw(h, p.rho_shift);
}

template <int ST, int V>
__device__ __forceinline__ void sc_gather(const FusedParams& p, int y, int x0s, int x0, int lane, float (&h)[V][9]) {
  if (x0s > 0 && x0s + 32 * V < p.nx) gather_interior<FusedParams, ST, V>(p, y, x0, lane, h);
  else gather_edge<FusedParams, ST, V>(p, y, x0, lane, h);
}

// One tile (rows ty*SC_ROWS.., segment seg) by one block of SC_ROWS warps;
// psi is the block's shared tile.  Ends with the block's last read of psi.
template <int MODEL, int ST, int V>
__device__ __forceinline__ void sc_tile(const FusedParams& p, int ty, int seg, float (&psi)[SC_ROWS + 2][32 * V + 2]) {
  using T = typename Storage<ST>::T;
  constexpr int W_ = 32 * V;       // tile width
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int y0 = ty * SC_ROWS, x0s = seg * W_;
  const int x0 = x0s + lane * V;
  const bool live = x0 < p.nx;
  const int wlast = min(W_, p.nx - x0s);  // nodes of this segment inside the lattice

  // halo rows first (their populations are not kept): warp 0 the row above
  // the tile, the last warp the row below
  if (warp == 0 || warp == SC_ROWS - 1) {
    const int r = warp == 0 ? 0 : SC_ROWS + 1;
    const int yh = wrap(warp == 0 ? y0 - 1 : y0 + SC_ROWS, p.ny);
    float hh[V][9];
    sc_gather<ST, V>(p, yh, x0s, x0, lane, hh);
#pragma unroll
    for (int i = 0; i < V; ++i)
      if (lane * V + i < wlast) psi[r][1 + lane * V + i] = eos_psi(p.eos, density_raw(hh[i], p.rho_shift), p.sc_T);
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
  float h[V][9];
  sc_gather<ST, V>(p, y, x0s, x0, lane, h);
#pragma unroll
  for (int i = 0; i < V; ++i)
    if (lane * V + i < wlast) psi[warp + 1][1 + lane * V + i] = eos_psi(p.eos, density_raw(h[i], p.rho_shift), p.sc_T);
  __syncthreads();

#pragma unroll
  for (int i = 0; i < V; ++i) {
    const int c = 1 + lane * V + i;
    float Fx = 0.0f, Fy = 0.0f;  // sum_k w_k c_k psi(x + c_k)
#pragma unroll
    for (int k = 1; k < 9; ++k) {
      const float ps = psi[warp + 1 + CY(k)][c + CX(k)];
      if (CX(k) != 0) Fx = fmaf(W(k) * (float)CX(k), ps, Fx);
      if (CY(k) != 0) Fy = fmaf(W(k) * (float)CY(k), ps, Fy);
    }
    const float m = -p.g_coh * psi[warp + 1][c];
    collide_lean<FusedParams, MODEL, false, 2>(p, h[i], 0.0f, fmaf(Fx, m, p.gx), fmaf(Fy, m, p.gy));
  }
  if (!live) return;
  T* dst = reinterpret_cast<T*>(p.dst);
  const size_t rowoff = (size_t)y * p.pitch;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float v[V];
#pragma unroll
    for (int i = 0; i < V; ++i) v[i] = h[i][k];
    store_raw<ST, V>(dst + (size_t)k * p.plane + rowoff + x0, v);
  }
}

template <int MODEL, int ST, int V>
__global__ void __launch_bounds__(SC_ROWS * 32) k_fused_sc(const FusedParams p) {
  __shared__ float psi[SC_ROWS + 2][32 * V + 2];
  const int tiles_y = p.ny / SC_ROWS;
  sc_tile<MODEL, ST, V>(p, blockIdx.x % tiles_y, blockIdx.x / tiles_y, psi);
}

}  // namespace lbm
