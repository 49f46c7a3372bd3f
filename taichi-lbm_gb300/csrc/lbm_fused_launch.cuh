// Host-side launchers of the fused kernels, instantiated once per population
// storage type (one translation unit each, so they compile in parallel).
#pragma once

#include "lbm_fused.cuh"

namespace lbm {

template <int ST, int V>
int launch_fused_v(const FusedParams& p, cudaStream_t s) {
  const long long warps = (long long)p.ny * p.nseg;
  const unsigned blocks = (unsigned)((warps + 7) / 8);
  const bool pl = p.fluid_model == LBM_POWERLAW;
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
int launch_fused(const FusedParams& p, int V, cudaStream_t s);

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

#define LBM_INSTANTIATE_STORAGE(ST, VA, VB)                                                    \
  namespace lbm {                                                                               \
  template <>                                                                                   \
  int launch_fused<ST>(const FusedParams& p, int V, cudaStream_t s) {                           \
    if (V == VA) return launch_fused_v<ST, VA>(p, s);                                           \
    if (V == VB) return launch_fused_v<ST, VB>(p, s);                                           \
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "nodes_per_thread %d not built for this storage", V); \
  }                                                                                             \
  template int launch_stream_only<ST>(const FusedParams&, float*, cudaStream_t);                \
  template int launch_convert<ST>(const FusedParams&, const float*, void*, int, cudaStream_t);  \
  template int launch_reduce<ST>(const FusedParams&, double*, double*, cudaStream_t);           \
  template int launch_momentum_exchange<ST>(const FusedParams&, const int32_t*, int64_t, double*, \
                                            cudaStream_t);                                      \
  }
