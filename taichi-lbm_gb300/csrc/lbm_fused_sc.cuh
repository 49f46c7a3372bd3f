// Fused single-component Shan-Chen step on a fully periodic lattice.
//
// The reference's Shan-Chen step (cases/Bubble or two-phase separation.py:
// 197-212) computes, from the post-stream populations of every node,
// rho -> psi(rho, T) (EOS.py:28-47, ExternalForce.py:42-47), wraps psi
// periodically (SCBoundaryCondition.py:126-144), then the force
// F(x) = -g psi(x) sum_k w_k c_k psi(x + c_k) (ExternalForce.py:50-63),
// F_body = F + rho/rho_tot g (lbm.py:215-220), the velocity and the
// collision.  A node's force needs psi of its eight neighbours in the same
// step.  Here one warp owns a strip of 32*V columns and SC_CHUNK rows and
// walks down it.  Its lanes copy the rows the strip needs (each lane its own
// V elements of the nine pulled rows, the elements across the strip's edges
// and the populations of the two columns beside it) with cp.async into a
// small ring of shared-memory stages, sc_dist rows ahead of use.  From a
// row's stage the warp computes psi (kept in registers for three rows; the
// x neighbours by warp shuffles) and, one row later, collides the row with
// the force from those three psi rows.  No warp waits for another, and a
// warp's loads run ahead of its arithmetic.  Each strip reads SC_CHUNK + 2
// rows (the extra two are mostly L2 hits: the neighbouring strips read them
// as their own rows), so HBM traffic stays one read and one write of the
// populations per lattice update; psi never leaves the SM.
#pragma once

#include "lbm_fused_lean.cuh"

namespace lbm {

constexpr int SC_CHUNK = 16;  // rows of a strip
constexpr int SC_WARPS = 4;   // warps per block (one strip each)

// Density of a node from its stored (shifted) values h: the pairwise sum of
// collide_lean, so psi and the collision see the same rho.
__device__ __forceinline__ float density_raw(const float h[9], float rho_shift) {
  return (((h[0] + h[1]) + (h[2] + h[3])) + ((h[4] + h[5]) + (h[6] + h[7])) + h[8]) + rho_shift;
}

// psi(rho, T) of EOS.py:28-95 for the fused step: the same equations of
// state, written with fused multiply-adds and one fast reciprocal per
// rational term (__fdividef, within 2 ulp), so psi agrees with the
// per-stage kernels' eos_psi to a few ulp.
__device__ __forceinline__ float eos_psi_lean(const LbmEos& e, float d, float T) {
  if (e.kind == LBM_EOS_SC) return e.rho0 * (1.0f - __expf(-d * __fdividef(1.0f, e.rho0)));
  float p;
  if (e.kind == LBM_EOS_CS) {
    const float b4 = e.b * d * 0.25f;
    const float one = 1.0f - b4;
    const float num = fmaf(b4, fmaf(b4, 1.0f - b4, 1.0f), 1.0f);  // 1 + b4 + b4^2 - b4^3
    p = fmaf(d * e.R * T, __fdividef(num, one * one * one), -(e.a * d * d));
  } else if (e.kind == LBM_EOS_VDW) {
    p = fmaf(d * e.R * T, __fdividef(1.0f, 1.0f - e.b * d), -(e.a * d * d));
  } else if (e.kind == LBM_EOS_RK) {
    const float bd = e.b * d;
    p = fmaf(d * e.R * T, __fdividef(1.0f, 1.0f - bd), -__fdividef(e.a * d * d, sqrtf(T) * (1.0f + bd)));
  } else {  // PR
    const float om = e.omega;
    const float kap = fmaf(om, fmaf(-0.269922f, om, 1.54226f), 0.37464f);
    const float s = fmaf(kap, 1.0f - sqrtf(T / e.T_cr), 1.0f);
    const float bd = e.b * d;
    p = fmaf(d * e.R * T, __fdividef(1.0f, 1.0f - bd), -__fdividef(e.a * s * s * d * d, fmaf(bd, 2.0f - bd, 1.0f)));
  }
  return sqrtf(fabsf(__fdividef(6.0f, e.G) * fmaf(d, -1.0f / 3.0f, p)));
}

// rho of one node (periodic pull of its nine stored values)
template <class P, int ST>
__device__ __forceinline__ float density_at(const P& p, int x, int y) {
  using T = typename Storage<ST>::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  float h[9];
#pragma unroll
  for (int k = 0; k < 9; ++k)
    h[k] = raw_to_float<ST>(load1_early(src + (size_t)k * p.plane + (size_t)wrap(y - CY(k), p.ny) * p.pitch +
                                        wrap(x - CX(k), p.nx)),
                            fix_of(p));
  return density_raw(h, p.rho_shift);
}

// psi of one row of a strip: ps[i] for the lane's V nodes, and, the same in
// every lane, hl = psi of the column left of the strip and hr = psi of the
// column right of its last node (both periodic).
template <int V>
struct ScRow {
  float ps[V];
  float hl, hr;
};

// Rows a warp's copies run ahead of its computation, and its ring of
// stages (PfGeom layout; the 32-word item area holds the halo words).
template <int ST>
__host__ __device__ constexpr int sc_dist() {
  return ST == LBM_STORE_F32 ? 1 : 2;
}
template <int ST>
__host__ __device__ constexpr int sc_slots() {
  return sc_dist<ST>() + 2;
}
template <int ST, int V>
using ScGeom = PfGeom<ST, V, sc_slots<ST>()>;
template <int ST, int V>
__host__ __device__ constexpr int sc_warp_bytes() {
  return sc_slots<ST>() * ScGeom<ST, V>::STAGE_BYTES;
}

// node and link of a halo word: lanes 0..8 hold population `lane` of the
// column left of the strip, lanes 16..24 population `lane - 16` of the
// column right of its last node; returns the source column (or -1)
template <class P, int V>
__device__ __forceinline__ int sc_halo_column(const P& p, int x0s, int lane, int& k) {
  k = lane & 15;
  if (k >= 9) return -1;
  const int wlast = min(32 * V, p.nx - x0s);
  const int xn = lane < 16 ? wrap(x0s - 1, p.nx) : wrap(x0s + wlast, p.nx);
  return wrap(xn - cx_dyn(k), p.nx);
}

// Issue row j of the strip's row sequence (row yb - 1 + j) into its stage,
// then commit (an empty group past the end keeps the group count uniform).
template <class P, int ST, int V>
__device__ __forceinline__ void sc_issue(const P& p, unsigned char* ring, int j, int nrow, int yb, int x0s, int lane) {
  using T = typename Storage<ST>::T;
  using G = ScGeom<ST, V>;
  if (j < nrow) {
    unsigned char* st = ring + (j % sc_slots<ST>()) * G::STAGE_BYTES;
    const int y = wrap(yb - 1 + j, p.ny);
    // the halo word's source first: the copies below clobber memory, and the
    // parameters may live in shared memory (batched strips)
    int k;
    const int xs = sc_halo_column<P, V>(p, x0s, lane, k);
    const T* row = xs >= 0 ? reinterpret_cast<const T*>(p.src) + (size_t)k * p.plane +
                                 (size_t)wrap(y - cy_dyn(k), p.ny) * p.pitch
                           : nullptr;
    stage_issue_row<P, ST, V, sc_slots<ST>()>(p, st, y, x0s, lane);
    if (xs >= 0) cp_async<4>(st + G::ITEM_OFF + lane * 4, edge_word<ST>(row, xs));
  }
  cp_async_commit();
}

// psi of row y from its stage: the lane's V nodes and the two halo columns
// (their nine populations summed by a shuffle tree in the pairwise order of
// density_raw, so a column's psi is the same in every strip that needs it)
// The pulled values replace the copied ones in the stage (each lane its own
// V per population), so the collision reads them back without the gather.
template <class P, int ST, int V>
__device__ __forceinline__ void sc_stage_psi(const P& p, unsigned char* st, int x0s, int lane, ScRow<V>& r) {
  using T = typename Storage<ST>::T;
  using G = ScGeom<ST, V>;
  constexpr unsigned FULL = 0xffffffffu;
  float h[V][9];
  stage_gather_row<P, ST, V, sc_slots<ST>()>(p, st, x0s + lane * V, lane, h);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    T raw[V];
#pragma unroll
    for (int i = 0; i < V; ++i) raw[i] = T(h[i][k]);  // exact: h holds stored values
    memcpy(st + k * G::POP_BYTES + lane * V * (int)sizeof(T), raw, sizeof(raw));
  }
  int k;
  const int xs = sc_halo_column<P, V>(p, x0s, lane, k);
  const float v = xs >= 0 ? edge_value<ST>(reinterpret_cast<const uint32_t*>(st + G::ITEM_OFF)[lane], xs, fix_of(p)) : 0.0f;
  const float a = v + __shfl_down_sync(FULL, v, 1);  // (h0+h1) (h2+h3) (h4+h5) (h6+h7) at k = 0, 2, 4, 6
  const float b = a + __shfl_down_sync(FULL, a, 2);  // at k = 0, 4
  const float c = b + __shfl_down_sync(FULL, b, 4);  // at k = 0
  const float d = c + __shfl_down_sync(FULL, v, 8);  // + h8
  const float rl = __shfl_sync(FULL, d, 0) + p.rho_shift;
  const float rr = __shfl_sync(FULL, d, 16) + p.rho_shift;
#pragma unroll
  for (int i = 0; i < V; ++i) r.ps[i] = eos_psi_lean(p.eos, density_raw(h[i], p.rho_shift), p.sc_T);
  const float e = eos_psi_lean(p.eos, lane == 0 ? rl : rr, p.sc_T);  // lane 0 left, the others right
  r.hl = __shfl_sync(FULL, e, 0);
  r.hr = __shfl_sync(FULL, e, 1);
}

// Force, collision and stores of row y of the strip from the psi of rows
// y-1 (m), y (c), y+1 (n) and the row's stage.
template <class P, int MODEL, int ST, int V>
__device__ __forceinline__ void sc_stage_collide(const P& p, const unsigned char* st, int y, int x0s, int lane,
                                                 const ScRow<V>& m, const ScRow<V>& c, const ScRow<V>& n) {
  using T = typename Storage<ST>::T;
  constexpr unsigned FULL = 0xffffffffu;
  const int x0 = x0s + lane * V;
  const ScRow<V>* rows[3] = {&m, &c, &n};
  float up[3], dn[3];  // psi of the node before the lane's first / after its last
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    up[r] = __shfl_up_sync(FULL, rows[r]->ps[V - 1], 1);
    dn[r] = __shfl_down_sync(FULL, rows[r]->ps[0], 1);
    if (lane == 0) up[r] = rows[r]->hl;
    if (lane == 31) dn[r] = rows[r]->hr;
  }
  // forces first, so that the psi rows are dead while the row is collided
  float Fx[V], Fy[V];
#pragma unroll
  for (int i = 0; i < V; ++i) {
    const bool last = x0 + i == p.nx - 1;  // its right neighbour is column 0: the right halo
    float fx = 0.0f, fy = 0.0f;  // sum_k w_k c_k psi(x + c_k)
#pragma unroll
    for (int k = 1; k < 9; ++k) {
      const ScRow<V>& R = *rows[1 + CY(k)];
      float ps;
      if (CX(k) == 0) ps = R.ps[i];
      else if (CX(k) == -1) ps = i > 0 ? R.ps[i - 1] : up[1 + CY(k)];
      else ps = last ? R.hr : (i < V - 1 ? R.ps[i + 1] : dn[1 + CY(k)]);
      if (CX(k) != 0) fx = fmaf(W(k) * (float)CX(k), ps, fx);
      if (CY(k) != 0) fy = fmaf(W(k) * (float)CY(k), ps, fy);
    }
    const float mm = -p.g_coh * c.ps[i];
    Fx[i] = fmaf(fx, mm, p.gx);
    Fy[i] = fmaf(fy, mm, p.gy);
  }
  float h[V][9];  // the pulled values sc_stage_psi left in the stage
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    T raw[V];
    memcpy(raw, st + k * ScGeom<ST, V>::POP_BYTES + lane * V * (int)sizeof(T), sizeof(raw));
    float c[V];
    raw_to_floats<ST, V>(raw, c, fix_of(p));
#pragma unroll
    for (int i = 0; i < V; ++i) h[i][k] = c[i];
  }
#pragma unroll
  for (int i = 0; i < V; ++i) collide_lean<P, MODEL, false, 2>(p, h[i], 0.0f, Fx[i], Fy[i]);
  if (x0 >= p.nx) return;
  bool bad = false;
#pragma unroll
  for (int i = 0; i < V; ++i) bad = bad || (x0 + i < p.nx && not_finite(h[i][0]));
  report_status(p.status, LBM_STATUS_NONFINITE, bad);
  T* dst = reinterpret_cast<T*>(p.dst);
  const size_t rowoff = (size_t)y * p.pitch;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float v[V];
#pragma unroll
    for (int i = 0; i < V; ++i) v[i] = h[i][k];
    store_raw<ST, V>(dst + (size_t)k * p.plane + rowoff + x0, v, fix_of(p));
  }
}

// One strip item (segment seg, rows chunk * rows ..) by one warp with its
// stage ring: rows yb - 1 .. ye are copied sc_dist rows ahead of use; row j
// of that sequence gives psi at step j and is collided at step j + 1.
template <class P, int MODEL, int ST, int V>
__device__ __forceinline__ void sc_strip(const P& p, int seg, int chunk, int rows, int lane, unsigned char* ring) {
  using G = ScGeom<ST, V>;
  constexpr int D = sc_dist<ST>(), NS = sc_slots<ST>();
  const int x0s = seg * 32 * V;
  const int yb = chunk * rows;
  const int ye = min(yb + rows, p.ny);
  const int nrow = ye - yb + 2;
#pragma unroll
  for (int j = 0; j < D; ++j) sc_issue<P, ST, V>(p, ring, j, nrow, yb, x0s, lane);
  ScRow<V> a, b, c;  // psi of sequence rows j-2, j-1, j
#pragma unroll 1
  for (int j = 0; j < nrow; ++j) {
    sc_issue<P, ST, V>(p, ring, j + D, nrow, yb, x0s, lane);
    cp_async_wait<D>();  // this lane's copies of row j have landed
    sc_stage_psi<P, ST, V>(p, ring + (j % NS) * G::STAGE_BYTES, x0s, lane, c);
    if (j >= 2)
      sc_stage_collide<P, MODEL, ST, V>(p, ring + ((j - 1) % NS) * G::STAGE_BYTES, yb + j - 2, x0s, lane, a, b, c);
    a = b;
    b = c;
  }
  cp_async_wait<0>();
}

// rows per strip item: 2 SC_CHUNK, halved (down to SC_CHUNK / 2) while the
// lattice offers fewer than `want` items (the extra rows per item are two,
// so shorter strips cost more)
inline int sc_rows(int ny, int nseg, int want) {
  int r = 2 * SC_CHUNK;
  while (r > SC_CHUNK / 2 && (long long)nseg * ((ny + r - 1) / r) < want) r /= 2;
  return r;
}

// Strip items of one lattice: item = chunk * nseg + seg, p.sc_rows rows each.
template <int MODEL, int ST, int V>
__global__ void __launch_bounds__(SC_WARPS * 32) k_fused_sc(const LeanParams p, int nitems) {
  extern __shared__ __align__(16) unsigned char sc_ring[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* ring = sc_ring + warp * sc_warp_bytes<ST, V>();
  for (int it = blockIdx.x * SC_WARPS + warp; it < nitems; it += gridDim.x * SC_WARPS) {
    const int chunk = it / p.nseg;
    sc_strip<LeanParams, MODEL, ST, V>(p, it - chunk * p.nseg, chunk, p.sc_rows, lane, ring);
  }
}

}  // namespace lbm
