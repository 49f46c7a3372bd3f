// Host-side launchers of the fused kernels, instantiated once per population
// storage type (one translation unit each, so they compile in parallel).
#pragma once

#include "lbm_fused.cuh"
#include "lbm_fused_async.cuh"
#include "lbm_fused_lean.cuh"
#include "lbm_fused_sc.cuh"

namespace lbm {

// Grid of a persistent kernel: as many blocks as fit on every SM.
template <typename K>
int persistent_blocks(K kern, int threads, int smem, int* blocks) {
  if (*blocks) return LBM_OK;
  if (smem > 48 * 1024) {
    int rc = lbm_err::cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                           "persistent step: shared-memory attribute");
    if (rc) return rc;
  }
  int per_sm = 0, dev = 0, sms = 0;
  int rc = lbm_err::cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem),
                         "persistent step: occupancy");
  if (rc) return rc;
  rc = lbm_err::cuda(cudaGetDevice(&dev), "persistent step: device");
  if (rc) return rc;
  rc = lbm_err::cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "persistent step: SMs");
  if (rc) return rc;
  *blocks = (per_sm > 0 ? per_sm : 1) * sms;
  return LBM_OK;
}

// Shan-Chen strips of one lattice: persistent grid of warps, one strip each
template <int MODEL, int ST>
int launch_sc_model(LeanParams p, cudaStream_t s) {
  static int blocks = 0;
  auto kern = k_fused_sc<MODEL, ST, AV>;
  const int smem = SC_WARPS * sc_warp_bytes<ST, AV>();
  int rc = persistent_blocks(kern, SC_WARPS * 32, smem, &blocks);
  if (rc) return rc;
  p.sc_rows = sc_rows(p.ny, p.nseg, 2 * blocks * SC_WARPS);
  const int nitems = p.nseg * ((p.ny + p.sc_rows - 1) / p.sc_rows);
  const int need = (nitems + SC_WARPS - 1) / SC_WARPS;
  kern<<<need < blocks ? need : blocks, SC_WARPS * 32, smem, s>>>(p, nitems);
  return lbm_err::launch("fused Shan-Chen step");
}

template <int ST>
int launch_fused_sc(const FusedParams& fp, cudaStream_t s) {
  const LeanParams p = lean_of(fp);
  switch (fp.model) {
    case LBM_BGK: return launch_sc_model<LBM_BGK, ST>(p, s);
    case LBM_TRT: return launch_sc_model<LBM_TRT, ST>(p, s);
    case LBM_MRT: return launch_sc_model<LBM_MRT, ST>(p, s);
    default: return lbm_err::set(LBM_ERR_ARG, "unknown collision model %d", fp.model);
  }
}

template <int MODEL, bool PL, int ST, int NW, int NS>
int launch_async_mp(const FusedParams& p, int32_t* status, cudaStream_t s) {
  static int blocks = 0;
  auto kern = k_fused_async<MODEL, PL, ST, NW, NS>;
  const int smem = AsyncGeom<ST, NW, NS>::SMEM;
  int rc = persistent_blocks(kern, NW * 32, smem, &blocks);
  if (rc) return rc;
  kern<<<blocks, NW * 32, smem, s>>>(p, status);
  return lbm_err::launch("fused step (async)");
}

template <int MODEL, bool PL, int ST>
int launch_async_tuned(const FusedParams& p, int32_t* status, int tune, cudaStream_t s) {
  switch (tune) {  // (warps per block, stages per warp)
    case 0: return launch_async_mp<MODEL, PL, ST, 8, 2>(p, status, s);
    case 1: return launch_async_mp<MODEL, PL, ST, 6, 3>(p, status, s);
    case 2: return launch_async_mp<MODEL, PL, ST, 4, 4>(p, status, s);
    case 3: return launch_async_mp<MODEL, PL, ST, 16, 2>(p, status, s);
    default: return lbm_err::set(LBM_ERR_ARG, "async tuning %d (0..%d)", tune, LBM_ASYNC_TUNINGS - 1);
  }
}

template <int MODEL, bool PL, int ST>
int launch_prefetch_mp(const FusedParams& p, cudaStream_t s) {
  static int blocks = 0;
  auto kern = k_fused_prefetch<MODEL, PL, ST>;
  int rc = persistent_blocks(kern, 256, 0, &blocks);
  if (rc) return rc;
  kern<<<blocks, 256, 0, s>>>(p);
  return lbm_err::launch("fused step (prefetch)");
}

// pipeline LBM_PIPE_ASYNC (with tune) or LBM_PIPE_PREFETCH
template <int ST>
int launch_fused_persistent(const FusedParams& p, int pipeline, int tune, int32_t* status, cudaStream_t s) {
  const bool pl = p.fluid_model == LBM_POWERLAW;
  const int m = p.model * 2 + (pl ? 1 : 0);
  if (pipeline == LBM_PIPE_PREFETCH) {
    switch (m) {
      case 0: return launch_prefetch_mp<LBM_BGK, false, ST>(p, s);
      case 1: return launch_prefetch_mp<LBM_BGK, true, ST>(p, s);
      case 2: return launch_prefetch_mp<LBM_TRT, false, ST>(p, s);
      case 3: return launch_prefetch_mp<LBM_TRT, true, ST>(p, s);
      case 4: return launch_prefetch_mp<LBM_MRT, false, ST>(p, s);
      case 5: return launch_prefetch_mp<LBM_MRT, true, ST>(p, s);
      default: return lbm_err::set(LBM_ERR_ARG, "unknown collision model %d", p.model);
    }
  }
  switch (m) {
    case 0: return launch_async_tuned<LBM_BGK, false, ST>(p, status, tune, s);
    case 1: return launch_async_tuned<LBM_BGK, true, ST>(p, status, tune, s);
    case 2: return launch_async_tuned<LBM_TRT, false, ST>(p, status, tune, s);
    case 3: return launch_async_tuned<LBM_TRT, true, ST>(p, status, tune, s);
    case 4: return launch_async_tuned<LBM_MRT, false, ST>(p, status, tune, s);
    case 5: return launch_async_tuned<LBM_MRT, true, ST>(p, status, tune, s);
    default: return lbm_err::set(LBM_ERR_ARG, "unknown collision model %d", p.model);
  }
}

template <int MODEL, bool PL, int ST, int V, int FORCE, int NW, int NS>
int launch_pf_mp(const FusedParams& p, cudaStream_t s) {
  static int blocks = 0;
  auto kern = k_fused_bulk_pf<MODEL, PL, ST, V, FORCE, NW, NS>;
  const int smem = NW * PfGeom<ST, V, NS>::WARP_BYTES;
  int rc = persistent_blocks(kern, NW * 32, smem, &blocks);
  if (rc) return rc;
  kern<<<blocks, NW * 32, smem, s>>>(p);
  return lbm_err::launch("fused step (plain segments, prefetching)");
}

template <int MODEL, bool PL, int ST, int V, int FORCE>
int launch_pf_force(const FusedParams& p, cudaStream_t s) {
  switch (p.tune) {  // (warps per block, stages per warp)
    case 0: return launch_pf_mp<MODEL, PL, ST, V, FORCE, 8, 2>(p, s);
    case 1: return launch_pf_mp<MODEL, PL, ST, V, FORCE, 8, 3>(p, s);
    case 2: return launch_pf_mp<MODEL, PL, ST, V, FORCE, 4, 4>(p, s);
    case 3: return launch_pf_mp<MODEL, PL, ST, V, FORCE, 16, 2>(p, s);
    default: return lbm_err::set(LBM_ERR_ARG, "prefetch tuning %d (0..%d)", p.tune, LBM_PREFETCH_TUNINGS - 1);
  }
}

template <int MODEL, bool PL, int ST, int V>
int launch_pf_tuned(const FusedParams& p, cudaStream_t s) {
  if (p.nplain == 0) return LBM_OK;
  return p.has_force ? launch_pf_force<MODEL, PL, ST, V, 1>(p, s) : launch_pf_force<MODEL, PL, ST, V, 0>(p, s);
}

// The listed (flagged) segments on stream s2, then the plain segments, with
// a compile-time force switch, on s.  s2 == s serialises the two; a caller
// passing another stream has forked it from s and joins it back after.
template <int MODEL, bool PL, int ST, int V>
int launch_two_pass(const FusedParams& p, unsigned blocks, cudaStream_t s, cudaStream_t s2) {
  if (p.lane_mask) {  // lane-granular form: the marked lanes, then every segment
    if (p.nlanes > 0) {
      k_fused_lanes<MODEL, PL, ST, V><<<(unsigned)(((long long)p.nlanes * V + 127) / 128), 128, 0, s2>>>(p);
      int rc = lbm_err::launch("fused step (marked lanes)");
      if (rc) return rc;
    }
  } else if (p.nspecial > 0) {
    k_fused_special<MODEL, PL, ST, V><<<(unsigned)((p.nspecial + 7) / 8), 256, 0, s2>>>(p);
    int rc = lbm_err::launch("fused step (flagged segments)");
    if (rc) return rc;
  }
  if constexpr (V >= AV) {
    if (p.plain) return launch_pf_tuned<MODEL, PL, ST, V>(p, s);  // prefetching persistent form
  }
  (void)blocks;
  const int wpb = p.nseg < 8 ? p.nseg : 8;  // warps per block
  const unsigned gy = p.ny < 65535 ? (unsigned)p.ny : 65535u;
  const dim3 grid((unsigned)((p.nseg + wpb - 1) / wpb), gy, (unsigned)((p.ny + gy - 1) / gy));
  if (p.has_force) k_fused_bulk<MODEL, PL, ST, V, 1><<<grid, 32 * wpb, 0, s>>>(p);
  else k_fused_bulk<MODEL, PL, ST, V, 0><<<grid, 32 * wpb, 0, s>>>(p);
  return lbm_err::launch("fused step (plain segments)");
}

template <int ST, int V>
int launch_fused_v(const FusedParams& p, cudaStream_t s, cudaStream_t s2) {
  const long long warps = (long long)p.ny * p.nseg;
  const unsigned blocks = (unsigned)((warps + 7) / 8);
  const bool pl = p.fluid_model == LBM_POWERLAW;
  if (p.special) {
    switch (p.model * 2 + (pl ? 1 : 0)) {
      case 0: return launch_two_pass<LBM_BGK, false, ST, V>(p, blocks, s, s2);
      case 1: return launch_two_pass<LBM_BGK, true, ST, V>(p, blocks, s, s2);
      case 2: return launch_two_pass<LBM_TRT, false, ST, V>(p, blocks, s, s2);
      case 3: return launch_two_pass<LBM_TRT, true, ST, V>(p, blocks, s, s2);
      case 4: return launch_two_pass<LBM_MRT, false, ST, V>(p, blocks, s, s2);
      case 5: return launch_two_pass<LBM_MRT, true, ST, V>(p, blocks, s, s2);
      default: return lbm_err::set(LBM_ERR_ARG, "unknown collision model %d", p.model);
    }
  }
#define LBM_LAUNCH_(M, PL) k_fused<M, PL, ST, V><<<blocks, 256, 0, s>>>(p)
  switch (p.model * 2 + (pl ? 1 : 0)) {
    case 0: LBM_LAUNCH_(LBM_BGK, false); break;
    case 1: LBM_LAUNCH_(LBM_BGK, true); break;
    case 2: LBM_LAUNCH_(LBM_TRT, false); break;
    case 3: LBM_LAUNCH_(LBM_TRT, true); break;
    case 4: LBM_LAUNCH_(LBM_MRT, false); break;
    case 5: LBM_LAUNCH_(LBM_MRT, true); break;
    default: return lbm_err::set(LBM_ERR_ARG, "unknown collision model %d", p.model);
  }
#undef LBM_LAUNCH_
  return lbm_err::launch("fused step");
}

template <int ST>
int launch_fused(const FusedParams& p, int V, cudaStream_t s, cudaStream_t s2);

template <int ST>
int launch_stream_only(const FusedParams& p, float* out, cudaStream_t s) {
  dim3 grid((p.nx + 127) / 128, p.ny);
  k_stream_only<ST><<<grid, 128, 0, s>>>(p, out);
  return lbm_err::launch("fused stream pass");
}

template <int ST>
int launch_convert(const FusedParams& p, const float* in, void* out, int to_storage, cudaStream_t s) {
  k_convert<ST><<<152 * 8, 256, 0, s>>>(p, in, out, to_storage);
  return lbm_err::launch("population convert");
}

template <int ST>
int launch_reduce(const FusedParams& p, double* partials, double* out, cudaStream_t s) {
  k_reduce_partial<ST><<<REDUCE_BLOCKS, REDUCE_TPB, 0, s>>>(p, partials);
  k_reduce_final<ST><<<1, 96, 0, s>>>(partials, REDUCE_BLOCKS, out);
  return lbm_err::launch("moment reduction");
}

template <int ST>
int launch_momentum_exchange(const FusedParams& p, const int32_t* links, int64_t n, double* out,
                             cudaStream_t s) {
  k_momentum_exchange<ST><<<1, MEX_TPB, 0, s>>>(p, links, n, out);
  return lbm_err::launch("momentum exchange");
}

}  // namespace lbm

// Declarations for translation units that call the launchers but must not
// instantiate the kernels themselves (they are built once per storage TU).
#define LBM_EXTERN_STORAGE(ST)                                                                        \
  namespace lbm {                                                                                     \
  extern template int launch_stream_only<ST>(const FusedParams&, float*, cudaStream_t);               \
  extern template int launch_fused_sc<ST>(const FusedParams&, cudaStream_t);                          \
  extern template int launch_fused_persistent<ST>(const FusedParams&, int, int, int32_t*, cudaStream_t);             \
  extern template int launch_convert<ST>(const FusedParams&, const float*, void*, int, cudaStream_t);  \
  extern template int launch_reduce<ST>(const FusedParams&, double*, double*, cudaStream_t);          \
  extern template int launch_momentum_exchange<ST>(const FusedParams&, const int32_t*, int64_t,       \
                                                   double*, cudaStream_t);                            \
  }

#define LBM_INSTANTIATE_STORAGE(ST, VA, VB)                                                    \
  namespace lbm {                                                                               \
  template <>                                                                                   \
  int launch_fused<ST>(const FusedParams& p, int V, cudaStream_t s, cudaStream_t s2) {          \
    if (V == VA) return launch_fused_v<ST, VA>(p, s, s2);                                       \
    if (V == VB) return launch_fused_v<ST, VB>(p, s, s2);                                       \
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "nodes_per_thread %d not built for this storage", V); \
  }                                                                                             \
  template int launch_stream_only<ST>(const FusedParams&, float*, cudaStream_t);                \
  template int launch_fused_sc<ST>(const FusedParams&, cudaStream_t);                            \
  template int launch_fused_persistent<ST>(const FusedParams&, int, int, int32_t*, cudaStream_t);              \
  template int launch_convert<ST>(const FusedParams&, const float*, void*, int, cudaStream_t);  \
  template int launch_reduce<ST>(const FusedParams&, double*, double*, cudaStream_t);           \
  template int launch_momentum_exchange<ST>(const FusedParams&, const int32_t*, int64_t, double*, \
                                            cudaStream_t);                                      \
  }
