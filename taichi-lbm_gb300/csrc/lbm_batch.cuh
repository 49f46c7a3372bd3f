// Batched kernels: many independent lattices advance one time step in one
// launch per kernel kind, over a packed tile table.
//
// Every lattice has a device record with two views of its parameters (the
// populations and saved moments read from / written to, for the two
// ping-pong parities).  A tile is (lattice, item): for the plain and flagged
// kind an item is one row segment (y * nseg + seg), for the marked-lane kind
// one lane ((y * nseg + seg) * 32 + lane), for Shan-Chen one
// strip of 32V columns and SC_CHUNK rows (chunk * nseg + seg).  The kernels
// for the segment kinds run one warp per tile; the Shan-Chen strips are
// persistent (a grid sized to the GPU walks the table, a warp per tile).  A
// warp copies its lattice's parameters into its shared memory.  Tables are ordered by lattice,
// then row, so consecutive tiles touch neighbouring memory.
#pragma once

#include "lbm_fused_launch.cuh"

namespace lbm {

struct BatchLattice {
  LeanParams lean[2];   // [parity]
  FusedParams full[2];  // [parity]
  int flip;             // the lattice's parity at batch step parity 0
};

struct BatchTile {
  int lat;
  int item;
};

// the view of lattice `lat` at batch step parity `sp`
__device__ __forceinline__ int view_of(const BatchLattice* lats, int lat, int sp) { return (sp ^ lats[lat].flip) & 1; }

constexpr int BATCH_WARPS = 8;  // warps per block of the segment kinds
// tiles per warp of the lean kind: a block stages its lattice's parameters
// once for BATCH_WARPS * BATCH_TPW tiles, so the two dependent loads in
// front of the first tile (tile -> lattice -> parameters) are paid once
constexpr int BATCH_TPW = 2;

// Plain-path segments of every lattice in the table: BATCH_TPW tiles per
// warp, not persistent (the hardware balances the blocks, so work that runs
// beside this kernel on other streams never leaves a statically assigned
// share behind).  Every
// lattice's tiles are padded to whole blocks (item -1), so a block serves one
// lattice and stages its parameters in shared memory once.  The collision
// model is the lattice's (a branch uniform over the block), so lattices of
// every model share one launch; each branch is the single-lattice kernel's
// own collision and store, so results stay bit-identical to it.
template <bool PL, int ST, int V, int FORCE>
__global__ void __launch_bounds__(BATCH_WARPS * 32) k_batch_lean(const BatchLattice* __restrict__ lats,
                                                                  const BatchTile* __restrict__ tiles, int ntiles,
                                                                  int sp) {
  __shared__ LeanParams p;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t0 = blockIdx.x * (BATCH_WARPS * BATCH_TPW);
  const int lat = tiles[t0].lat;
  copy_words(&p, &lats[lat].lean[view_of(lats, lat, sp)], threadIdx.x, BATCH_WARPS * 32);
  __syncthreads();
#pragma unroll 1
  for (int j = 0; j < BATCH_TPW; ++j) {  // consecutive warps take consecutive tiles
    const BatchTile tile = tiles[t0 + j * BATCH_WARPS + warp];
    if (tile.item < 0) continue;
    const int y = fast_div(tile.item, p.nseg_mul, p.nseg_shift);
    const int seg = tile.item - y * p.nseg;
    const int x0s = seg * 32 * V, x0 = x0s + lane * V;
    uint32_t mask;  // lanes k_batch_lanes stores
    ldg_early(p.lane_mask + tile.item, mask);
    float h[V][9];
    if (x0s > 0 && x0s + 32 * V < p.nx) gather_interior<LeanParams, ST, V>(p, y, x0, lane, h);
    else gather_edge<LeanParams, ST, V>(p, y, x0, lane, h);
    if (mask == 0xffffffffu) continue;
    const bool skip = (mask >> lane) & 1u;
    if (p.model == LBM_BGK) lean_collide_store<LeanParams, LBM_BGK, PL, ST, V, FORCE>(p, h, y, x0, skip);
    else if (p.model == LBM_TRT) lean_collide_store<LeanParams, LBM_TRT, PL, ST, V, FORCE>(p, h, y, x0, skip);
    else lean_collide_store<LeanParams, LBM_MRT, PL, ST, V, FORCE>(p, h, y, x0, skip);
  }
}

// Pipelined form of k_batch_lean (batch lean forms 1 and 2).  A block serves
// BATCH_WARPS * TPW tiles of one lattice; it stages the lattice's parameters
// and its tile list in shared memory once.  Each warp walks its TPW tiles
// (tile j * BATCH_WARPS + warp) through a ring of NS shared-memory stages:
// the stage of a tile holds every lane's V elements of the nine pulled rows,
// the words across the segment's edges (stage_issue_row) and the segment's
// lane mask, all copied by cp.async, so the rows of the next NS - 1 tiles
// are in flight while the warp collides the current one.  Each lane reads
// back only what it copied itself (cp.async.wait_group is the hardware wait
// for the lane's own copies; no barrier).  The gather and the collision are
// the single-lattice kernels' own, so results are bit-identical to them.
template <int ST, int V, int NS>
struct BatchPfGeom {
  using G = PfGeom<ST, V, NS>;
  static constexpr int MASK_OFF = G::STAGE_BYTES;  // [32] copies of the segment's lane mask
  static constexpr int STRIDE = G::STAGE_BYTES + 32 * 4;
  static constexpr int WARP_BYTES = NS * STRIDE;
  static constexpr int BLOCK_BYTES = BATCH_WARPS * WARP_BYTES;
  static_assert(STRIDE % 16 == 0, "stages must stay 16-byte aligned");
};

// (ring stages, tiles per warp) of the pipelined lean forms
template <int FORM>
struct LeanForm;
template <>
struct LeanForm<1> {
  static constexpr int NS = 2, TPW = 4;
};
template <>
struct LeanForm<2> {
  static constexpr int NS = 3, TPW = 8;
};
__host__ __device__ constexpr int lean_block_tiles(int form) {
  return BATCH_WARPS * (form == 1 ? LeanForm<1>::TPW : form == 2 ? LeanForm<2>::TPW : BATCH_TPW);
}

template <bool PL, int ST, int V, int FORCE, int FORM>
__global__ void __launch_bounds__(BATCH_WARPS * 32) k_batch_lean_pf(const BatchLattice* __restrict__ lats,
                                                                     const BatchTile* __restrict__ tiles,
                                                                     int ntiles, int sp) {
  constexpr int NS = LeanForm<FORM>::NS, TPW = LeanForm<FORM>::TPW;
  using B = BatchPfGeom<ST, V, NS>;
  __shared__ LeanParams p;
  __shared__ int items[BATCH_WARPS * TPW];
  extern __shared__ __align__(16) unsigned char lean_ring[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t0 = blockIdx.x * (BATCH_WARPS * TPW);
  const int lat = tiles[t0].lat;
  copy_words(&p, &lats[lat].lean[view_of(lats, lat, sp)], threadIdx.x, BATCH_WARPS * 32);
  for (int i = threadIdx.x; i < BATCH_WARPS * TPW; i += BATCH_WARPS * 32) items[i] = tiles[t0 + i].item;
  __syncthreads();
  unsigned char* ring = lean_ring + warp * B::WARP_BYTES;
  // read once: every cp.async below clobbers memory, which would reload them
  const uint32_t nseg_mul = p.nseg_mul;
  const int nseg_shift = p.nseg_shift, nseg = p.nseg;
  const uint32_t* lane_mask = p.lane_mask;
  // stage the copies of the warp's tile j (none past the last) and commit them as one group
  auto issue = [&](int j) {
    const int item = j < TPW ? items[j * BATCH_WARPS + warp] : -1;
    if (item >= 0) {
      unsigned char* stage = ring + (j % NS) * B::STRIDE;
      const int y = fast_div(item, nseg_mul, nseg_shift);
      stage_issue_row<LeanParams, ST, V, NS>(p, stage, y, (item - y * nseg) * 32 * V, lane);
      cp_async<4>(stage + B::MASK_OFF + lane * 4, lane_mask + item);
    }
    cp_async_commit();
  };
#pragma unroll
  for (int j = 0; j < NS - 1; ++j) issue(j);
#pragma unroll 1
  for (int j = 0; j < TPW; ++j) {
    issue(j + NS - 1);
    cp_async_wait<NS - 1>();  // this lane's copies of tile j have landed
    const int item = items[j * BATCH_WARPS + warp];
    if (item < 0) continue;
    const unsigned char* stage = ring + (j % NS) * B::STRIDE;
    const uint32_t mask = reinterpret_cast<const uint32_t*>(stage + B::MASK_OFF)[lane];
    if (mask == 0xffffffffu) continue;  // uniform over the warp
    const int y = fast_div(item, nseg_mul, nseg_shift);
    const int x0 = (item - y * nseg) * 32 * V + lane * V;
    float h[V][9];
    stage_gather_row<LeanParams, ST, V, NS>(p, stage, x0, lane, h);
    const bool skip = (mask >> lane) & 1u;
    if (p.model == LBM_BGK) lean_collide_store<LeanParams, LBM_BGK, PL, ST, V, FORCE>(p, h, y, x0, skip);
    else if (p.model == LBM_TRT) lean_collide_store<LeanParams, LBM_TRT, PL, ST, V, FORCE>(p, h, y, x0, skip);
    else lean_collide_store<LeanParams, LBM_MRT, PL, ST, V, FORCE>(p, h, y, x0, skip);
  }
  cp_async_wait<0>();
}

// Marked lanes (bounce-back links, boundary programs, saved moments,
// inactive nodes) of every lattice in the table, V threads per lane entry
// ((y * nseg + seg) * 32 + lane), one per node: the general per-node path,
// for the lattice's collision model and fluid model.
template <int ST, int V>
__global__ void __launch_bounds__(128) k_batch_lanes(const BatchLattice* __restrict__ lats,
                                                     const BatchTile* __restrict__ tiles, int ntiles, int sp) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ntiles * V) return;
  const BatchTile tile = tiles[t / V];
  const FusedParams& p = lats[tile.lat].full[view_of(lats, tile.lat, sp)];
  const int item = tile.item >> 5, lane = tile.item & 31;
  const int y = item / p.nseg;
  const int x = (item - y * p.nseg) * 32 * V + lane * V + (int)(t % V);
  switch (p.model * 2 + (p.fluid_model == LBM_POWERLAW ? 1 : 0)) {
    case 0: lane_node<LBM_BGK, false, ST>(p, y, x); break;
    case 1: lane_node<LBM_BGK, true, ST>(p, y, x); break;
    case 2: lane_node<LBM_TRT, false, ST>(p, y, x); break;
    case 3: lane_node<LBM_TRT, true, ST>(p, y, x); break;
    case 4: lane_node<LBM_MRT, false, ST>(p, y, x); break;
    default: lane_node<LBM_MRT, true, ST>(p, y, x); break;
  }
}

// Shan-Chen strips (item = chunk * nseg + seg) of every lattice in the
// table, one warp per strip.
template <int MODEL, int ST, int V>
__global__ void __launch_bounds__(SC_WARPS * 32) k_batch_sc(const BatchLattice* __restrict__ lats,
                                                                const BatchTile* __restrict__ tiles, int ntiles,
                                                                int sp) {
  __shared__ LeanParams lp[SC_WARPS];
  extern __shared__ __align__(16) unsigned char sc_ring[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  LeanParams& p = lp[warp];
  unsigned char* ring = sc_ring + warp * sc_warp_bytes<ST, V>();
  int cur = -1;
  for (int t = blockIdx.x * SC_WARPS + warp; t < ntiles; t += gridDim.x * SC_WARPS) {
    const BatchTile tile = tiles[t];
    if (tile.lat != cur) {
      __syncwarp();
      copy_words(&p, &lats[tile.lat].lean[view_of(lats, tile.lat, sp)], lane, 32);
      __syncwarp();
      cur = tile.lat;
    }
    const int chunk = fast_div(tile.item, p.nseg_mul, p.nseg_shift);
    sc_strip<LeanParams, MODEL, ST, V>(p, tile.item - chunk * p.nseg, chunk, p.sc_rows, lane, ring);
  }
}

// Drag/lift monitors: block b sums the momentum exchanged on monitor b's
// solid links (lattice mon.lat, current post-collision state) and appends
// (Fx, Fy) at series[2 * count], then advances count, so a graph replaying
// the same launch fills consecutive rows.
struct BatchMonitor {
  int lat;
  int64_t nlinks;
  const int32_t* links;  // (site, k) pairs
  double* series;        // [capacity][2]
  int32_t* count;        // device counter
  int32_t capacity;
};

template <int ST>
__global__ void __launch_bounds__(MEX_TPB) k_batch_monitor(const BatchLattice* __restrict__ lats,
                                                           const BatchMonitor* __restrict__ mons, int sp) {
  using S = Storage<ST>;
  using T = typename S::T;
  const BatchMonitor m = mons[blockIdx.x];
  // the post-collision state written by this step is the view's destination
  const FusedParams& p = lats[m.lat].full[view_of(lats, m.lat, sp)];
  const T* src = reinterpret_cast<const T*>(p.dst);
  double fx = 0.0, fy = 0.0;
  for (int64_t i = threadIdx.x; i < m.nlinks; i += blockDim.x) {
    const int64_t q = m.links[2 * i];
    const int k = m.links[2 * i + 1];
    const double v = S::dec64(src[(size_t)k * p.plane + q], p.wsh[k], p.fq);
    fx += 2.0 * cx_dyn(k) * v;
    fy += 2.0 * cy_dyn(k) * v;
  }
  __shared__ double sh[2][MEX_TPB / 32];
  fx = warp_sum(fx);
  fy = warp_sum(fy);
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = fx;
    sh[1][threadIdx.x >> 5] = fy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sx = 0.0, sy = 0.0;
    for (int i = 0; i < MEX_TPB / 32; ++i) {
      sx += sh[0][i];
      sy += sh[1][i];
    }
    const int c = *m.count;
    if (c < m.capacity) {
      m.series[2 * (size_t)c] = sx;
      m.series[2 * (size_t)c + 1] = sy;
    }
    *m.count = c + 1;
    // a diverged member: its force is not finite (any NaN or infinity in
    // the summed links reaches the total)
    report_status(p.status, LBM_STATUS_NONFINITE, !(fabs(sx) <= 1.7976931348623157e308 && fabs(sy) <= 1.7976931348623157e308));
  }
}

// ------------------------------------------------------------ launchers
// kind of a tile group
enum { BATCH_LEAN = 0, BATCH_SC = 1, BATCH_SPECIAL = 2 };  // launch order within a step

struct BatchGroup {
  int kind, model, powerlaw, storage, V, force;
  int form;           // lean kinds: 0 = k_batch_lean, 1 / 2 = k_batch_lean_pf<FORM>
  int offset, count;  // range in the tile table
  int blocks;         // persistent grid (0 until first launch)
};

template <typename K>
int batch_grid(K kern, int threads, int tiles_per_block, int count, int* blocks) {
  if (!*blocks) {
    int per_sm = 0, dev = 0, sms = 0;
    int rc = lbm_err::cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0),
                           "batch: occupancy");
    if (!rc) rc = lbm_err::cuda(cudaGetDevice(&dev), "batch: device");
    if (!rc) rc = lbm_err::cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "batch: SMs");
    if (rc) return rc;
    *blocks = (per_sm > 0 ? per_sm : 1) * sms;
  }
  const int need = (count + tiles_per_block - 1) / tiles_per_block;
  return need < *blocks ? need : *blocks;
}

template <int ST, int V, int FORM>
int launch_batch_lean_pf(BatchGroup& g, const BatchLattice* lats, const BatchTile* t, int sp, cudaStream_t s) {
  constexpr int smem = BatchPfGeom<ST, V, LeanForm<FORM>::NS>::BLOCK_BYTES;
  auto kern = g.powerlaw ? (g.force ? k_batch_lean_pf<true, ST, V, 1, FORM> : k_batch_lean_pf<true, ST, V, 0, FORM>)
                         : (g.force ? k_batch_lean_pf<false, ST, V, 1, FORM> : k_batch_lean_pf<false, ST, V, 0, FORM>);
  if (smem > 48 * 1024) {
    int rc = lbm_err::cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                           "batched step: shared-memory attribute");
    if (rc) return rc;
  }
  constexpr int per = lean_block_tiles(FORM);
  kern<<<(unsigned)((g.count + per - 1) / per), BATCH_WARPS * 32, smem, s>>>(lats, t, g.count, sp);
  return lbm_err::launch("batched step (plain segments, pipelined)");
}

// groups of the segment kinds: lean groups per (power law, force), every
// collision model in one launch; one marked-lane group for every model
template <int ST, int V>
int launch_batch_v(BatchGroup& g, const BatchLattice* lats, const BatchTile* tiles, int sp, cudaStream_t s) {
  if (g.count == 0) return LBM_OK;
  const BatchTile* t = tiles + g.offset;
  if (g.kind == BATCH_SPECIAL) {
    k_batch_lanes<ST, V><<<(unsigned)(((long long)g.count * V + 127) / 128), 128, 0, s>>>(lats, t, g.count, sp);
    return lbm_err::launch("batched step (marked lanes)");
  }
  if (g.form == 1) return launch_batch_lean_pf<ST, V, 1>(g, lats, t, sp, s);
  if (g.form == 2) return launch_batch_lean_pf<ST, V, 2>(g, lats, t, sp, s);
  auto kern = g.powerlaw ? (g.force ? k_batch_lean<true, ST, V, 1> : k_batch_lean<true, ST, V, 0>)
                         : (g.force ? k_batch_lean<false, ST, V, 1> : k_batch_lean<false, ST, V, 0>);
  kern<<<(unsigned)((g.count + BATCH_WARPS * BATCH_TPW - 1) / (BATCH_WARPS * BATCH_TPW)), BATCH_WARPS * 32, 0, s>>>(
      lats, t, g.count, sp);
  return lbm_err::launch("batched step (plain segments)");
}

template <int ST>
int launch_batch_sc(BatchGroup& g, const BatchLattice* lats, const BatchTile* tiles, int sp, cudaStream_t s) {
  if (g.count == 0) return LBM_OK;
  const BatchTile* t = tiles + g.offset;
  auto kern = g.model == LBM_BGK ? k_batch_sc<LBM_BGK, ST, AV>
                                 : (g.model == LBM_TRT ? k_batch_sc<LBM_TRT, ST, AV> : k_batch_sc<LBM_MRT, ST, AV>);
  const int smem = SC_WARPS * sc_warp_bytes<ST, AV>();
  if (!g.blocks) {
    int rc = persistent_blocks(kern, SC_WARPS * 32, smem, &g.blocks);
    if (rc) return rc;
  }
  const int need = (g.count + SC_WARPS - 1) / SC_WARPS;
  kern<<<need < g.blocks ? need : g.blocks, SC_WARPS * 32, smem, s>>>(lats, t, g.count, sp);
  return lbm_err::launch("batched Shan-Chen step");
}

// one group of storage ST for one step
template <int ST>
int launch_batch_group(BatchGroup& g, const BatchLattice* lats, const BatchTile* tiles, int sp, cudaStream_t s);

template <int ST>
int launch_batch_monitors(const BatchLattice* lats, const BatchMonitor* mons, int nmon, int sp, cudaStream_t s) {
  if (nmon == 0) return LBM_OK;
  k_batch_monitor<ST><<<nmon, MEX_TPB, 0, s>>>(lats, mons, sp);
  return lbm_err::launch("batched drag/lift monitors");
}

}  // namespace lbm

#define LBM_BATCH_EXTERN(ST)                                                                                     \
  namespace lbm {                                                                                                \
  extern template int launch_batch_monitors<ST>(const BatchLattice*, const BatchMonitor*, int, int, cudaStream_t); \
  }

#define LBM_BATCH_INSTANTIATE(ST, VA, VB)                                                                       \
  namespace lbm {                                                                                               \
  template <>                                                                                                   \
  int launch_batch_group<ST>(BatchGroup & g, const BatchLattice* lats, const BatchTile* tiles, int sp,          \
                             cudaStream_t s) {                                                                  \
    if (g.kind == BATCH_SC) return launch_batch_sc<ST>(g, lats, tiles, sp, s);                                  \
    if (g.V == VA) return launch_batch_v<ST, VA>(g, lats, tiles, sp, s);                                        \
    if (g.V == VB) return launch_batch_v<ST, VB>(g, lats, tiles, sp, s);                                        \
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "batch: nodes_per_thread %d not built for this storage", g.V);     \
  }                                                                                                             \
  template int launch_batch_monitors<ST>(const BatchLattice*, const BatchMonitor*, int, int, cudaStream_t);     \
  }
