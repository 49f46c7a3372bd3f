// Fused-step plans: validation, buffer binding and stream-ordered launches.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>

#include "lbm_fused_aa.cuh"
#include "lbm_fused_launch.cuh"
#include "lbm_plan_internal.h"

LBM_EXTERN_STORAGE(LBM_STORE_F32)
LBM_EXTERN_STORAGE(LBM_STORE_F16S)
LBM_EXTERN_STORAGE(LBM_STORE_BF16S)
LBM_EXTERN_STORAGE(LBM_STORE_I16S)
LBM_AA_EXTERN(LBM_STORE_F32)
LBM_AA_EXTERN(LBM_STORE_F16S)
LBM_AA_EXTERN(LBM_STORE_BF16S)
LBM_AA_EXTERN(LBM_STORE_I16S)

namespace {

using lbm::FusedParams;

int storage_bytes(int st) { return st == LBM_STORE_F32 ? 4 : 2; }

bool aligned(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }

FusedParams params_for(const LbmPlan* pl) {
  FusedParams p = pl->base;
  const int cur = pl->parity;
  p.src = cur ? pl->b.fb : pl->b.fa;
  p.dst = cur ? pl->b.fa : pl->b.fb;
  p.mom_in = cur ? pl->b.mom_b : pl->b.mom_a;
  p.mom_out = cur ? pl->b.mom_a : pl->b.mom_b;
  p.code = pl->b.code;
  p.seg_flags = pl->b.seg_flags;
  p.tau = pl->b.tau;
  p.status = pl->b.status;
  // two-pass forms: direct (special list), prefetch (special and plain lists)
  const bool two = !pl->d.sc && pl->b.special &&
                   (pl->d.pipeline == LBM_PIPE_DIRECT || (pl->d.pipeline == LBM_PIPE_PREFETCH && pl->b.plain));
  p.special = two ? pl->b.special : nullptr;
  p.nspecial = two ? pl->b.nspecial : 0;
  p.plain = two && pl->d.pipeline == LBM_PIPE_PREFETCH ? pl->b.plain : nullptr;
  p.nplain = p.plain ? pl->b.nplain : 0;
  // lane-granular special work (direct pipeline): every segment on the lean
  // kernel, the marked lanes on k_fused_lanes
  const bool lanes = two && pl->d.pipeline == LBM_PIPE_DIRECT && pl->b.lane_mask && pl->b.lanes;
  p.lane_mask = lanes ? pl->b.lane_mask : nullptr;
  p.lanes = lanes ? pl->b.lanes : nullptr;
  p.nlanes = lanes ? pl->b.nlanes : 0;
  return p;
}

int dispatch_fused(const FusedParams& p, int st, int V, cudaStream_t s, cudaStream_t s2,
                   int pipeline = LBM_PIPE_DIRECT, int32_t* status = nullptr, int tune = 0) {
  if (p.sc) {
    switch (st) {
      case LBM_STORE_F32: return lbm::launch_fused_sc<LBM_STORE_F32>(p, s);
      case LBM_STORE_F16S: return lbm::launch_fused_sc<LBM_STORE_F16S>(p, s);
      case LBM_STORE_BF16S: return lbm::launch_fused_sc<LBM_STORE_BF16S>(p, s);
      default: return lbm::launch_fused_sc<LBM_STORE_I16S>(p, s);
    }
  }
  if (pipeline == LBM_PIPE_ASYNC || (pipeline == LBM_PIPE_PREFETCH && !p.plain)) {
    switch (st) {
      case LBM_STORE_F32: return lbm::launch_fused_persistent<LBM_STORE_F32>(p, pipeline, tune, status, s);
      case LBM_STORE_F16S: return lbm::launch_fused_persistent<LBM_STORE_F16S>(p, pipeline, tune, status, s);
      case LBM_STORE_BF16S: return lbm::launch_fused_persistent<LBM_STORE_BF16S>(p, pipeline, tune, status, s);
      default: return lbm::launch_fused_persistent<LBM_STORE_I16S>(p, pipeline, tune, status, s);
    }
  }
  switch (st) {
    case LBM_STORE_F32: return lbm::launch_fused<LBM_STORE_F32>(p, V, s, s2);
    case LBM_STORE_F16S: return lbm::launch_fused<LBM_STORE_F16S>(p, V, s, s2);
    case LBM_STORE_BF16S: return lbm::launch_fused<LBM_STORE_BF16S>(p, V, s, s2);
    default: return lbm::launch_fused<LBM_STORE_I16S>(p, V, s, s2);
  }
}

void release_side(LbmPlan* pl) {
  if (pl->fork) cudaEventDestroy(pl->fork);
  if (pl->join) cudaEventDestroy(pl->join);
  if (pl->side) cudaStreamDestroy(pl->side);
  pl->fork = pl->join = nullptr;
  pl->side = nullptr;
  pl->side_dev = -1;
}

// the side stream and its two events on the current device
int ensure_side(LbmPlan* pl) {
  int dev = 0;
  int rc = lbm_err::cuda(cudaGetDevice(&dev), "plan_run: device");
  if (rc) return rc;
  if (pl->side && pl->side_dev == dev) return LBM_OK;
  release_side(pl);
  int lo = 0, hi = 0;
  rc = lbm_err::cuda(cudaDeviceGetStreamPriorityRange(&lo, &hi), "plan_run: stream priorities");
  if (!rc) rc = lbm_err::cuda(cudaStreamCreateWithPriority(&pl->side, cudaStreamNonBlocking, hi),
                              "plan_run: side stream");
  if (!rc) rc = lbm_err::cuda(cudaEventCreateWithFlags(&pl->fork, cudaEventDisableTiming), "plan_run: event");
  if (!rc) rc = lbm_err::cuda(cudaEventCreateWithFlags(&pl->join, cudaEventDisableTiming), "plan_run: event");
  if (rc) {
    release_side(pl);
    return rc;
  }
  pl->side_dev = dev;
  return LBM_OK;
}

// one fused step on stream s and the parity flip
int step_once(LbmPlan* pl, cudaStream_t s) {
  FusedParams p = params_for(pl);
  const bool fork = p.special && (p.lane_mask ? p.nlanes > 0 : p.nspecial > 0) && pl->b.special_stream;
  cudaStream_t s2 = s;
  if (fork) {
    int rc = ensure_side(pl);
    if (rc) return rc;
    s2 = pl->side;
    rc = lbm_err::cuda(cudaEventRecord(pl->fork, s), "plan_run: fork");
    if (!rc) rc = lbm_err::cuda(cudaStreamWaitEvent(s2, pl->fork, 0), "plan_run: fork");
    if (rc) return rc;
  }
  int rc = dispatch_fused(p, pl->d.storage, pl->d.nodes_per_thread, s, s2, pl->d.pipeline, pl->b.status,
                          pl->d.tune);
  if (fork) {  // join even after a failed launch, so s never runs ahead of s2
    int rj = lbm_err::cuda(cudaEventRecord(pl->join, s2), "plan_run: join");
    if (!rj) rj = lbm_err::cuda(cudaStreamWaitEvent(s, pl->join, 0), "plan_run: join");
    if (!rc) rc = rj;
  }
  if (rc) return rc;
  pl->parity ^= 1;
  return LBM_OK;
}

// one in-place step of the given phase on stream s: the boundary read sites,
// then the marked lanes (side stream) and the plain segments, joined
int aa_step(LbmPlan* pl, int phase, cudaStream_t s) {
  FusedParams p = params_for(pl);
  p.aa = phase;
  p.aa_sites = pl->b.aa_sites;
  p.aa_nsites = pl->b.aa_nsites;
  p.aa_vals = pl->b.aa_vals;
  const int st = pl->d.storage;
  int rc = st == LBM_STORE_F32    ? lbm::launch_aa_sites<LBM_STORE_F32>(p, s)
           : st == LBM_STORE_F16S ? lbm::launch_aa_sites<LBM_STORE_F16S>(p, s)
           : st == LBM_STORE_BF16S ? lbm::launch_aa_sites<LBM_STORE_BF16S>(p, s)
                                   : lbm::launch_aa_sites<LBM_STORE_I16S>(p, s);
  if (rc) return rc;
  const bool fork = p.nlanes > 0 && pl->b.special_stream;
  cudaStream_t s2 = s;
  if (fork) {
    rc = ensure_side(pl);
    if (rc) return rc;
    s2 = pl->side;
    rc = lbm_err::cuda(cudaEventRecord(pl->fork, s), "plan_run: fork");
    if (!rc) rc = lbm_err::cuda(cudaStreamWaitEvent(s2, pl->fork, 0), "plan_run: fork");
    if (rc) return rc;
  }
  const int V = pl->d.nodes_per_thread;
  rc = st == LBM_STORE_F32    ? lbm::launch_aa<LBM_STORE_F32>(p, V, s, s2)
       : st == LBM_STORE_F16S ? lbm::launch_aa<LBM_STORE_F16S>(p, V, s, s2)
       : st == LBM_STORE_BF16S ? lbm::launch_aa<LBM_STORE_BF16S>(p, V, s, s2)
                               : lbm::launch_aa<LBM_STORE_I16S>(p, V, s, s2);
  if (fork) {
    int rj = lbm_err::cuda(cudaEventRecord(pl->join, s2), "plan_run: join");
    if (!rj) rj = lbm_err::cuda(cudaStreamWaitEvent(s, pl->join, 0), "plan_run: join");
    if (!rc) rc = rj;
  }
  if (rc) return rc;
  pl->parity ^= 1;
  return LBM_OK;
}

// back to pull layout after a run that ended on phase A
int aa_swap(LbmPlan* pl, cudaStream_t s) {
  const FusedParams p = params_for(pl);
  switch (pl->d.storage) {
    case LBM_STORE_F32: return lbm::launch_aa_swap<LBM_STORE_F32>(p, s);
    case LBM_STORE_F16S: return lbm::launch_aa_swap<LBM_STORE_F16S>(p, s);
    case LBM_STORE_BF16S: return lbm::launch_aa_swap<LBM_STORE_BF16S>(p, s);
    default: return lbm::launch_aa_swap<LBM_STORE_I16S>(p, s);
  }
}

int mex(LbmPlan* pl, const int32_t* links, int64_t n, double* out, cudaStream_t s) {
  FusedParams p = params_for(pl);
  switch (pl->d.storage) {
    case LBM_STORE_F32: return lbm::launch_momentum_exchange<LBM_STORE_F32>(p, links, n, out, s);
    case LBM_STORE_F16S: return lbm::launch_momentum_exchange<LBM_STORE_F16S>(p, links, n, out, s);
    case LBM_STORE_BF16S: return lbm::launch_momentum_exchange<LBM_STORE_BF16S>(p, links, n, out, s);
    default: return lbm::launch_momentum_exchange<LBM_STORE_I16S>(p, links, n, out, s);
  }
}

// nsteps steps (ping-pong or in place), each followed by the momentum
// exchange into series[2 * step] when series is given.  An in-place run
// alternates phases A and B from A and ends in pull layout.
int run_steps(LbmPlan* pl, int32_t nsteps, const int32_t* links, int64_t n, double* series, cudaStream_t s) {
  for (int32_t st = 0; st < nsteps; ++st) {
    int rc = pl->d.aa ? aa_step(pl, (st & 1) ? lbm::AA_PHASE_B : lbm::AA_PHASE_A, s) : step_once(pl, s);
    if (rc) return rc;
    if (series) {
      rc = mex(pl, links, n, series + 2 * (size_t)st, s);
      if (rc) return rc;
    }
  }
  if (pl->d.aa && (nsteps & 1)) return aa_swap(pl, s);
  return LBM_OK;
}

}  // namespace

lbm::FusedParams lbm_plan_params(const LbmPlan* pl) { return params_for(pl); }

extern "C" {

int lbm_plan_create(const LbmPlanDesc* d, LbmPlan** out) {
  if (!d || !out) return lbm_err::set(LBM_ERR_ARG, "plan_create: NULL argument");
  *out = nullptr;
  if (d->nx <= 0 || d->ny <= 0) return lbm_err::set(LBM_ERR_ARG, "lattice %d x %d", d->nx, d->ny);
  if (d->pitch < d->nx || d->pitch % 32)
    return lbm_err::set(LBM_ERR_ARG, "pitch %d must be >= nx and a multiple of 32", d->pitch);
  if (d->model < LBM_BGK || d->model > LBM_MRT) return lbm_err::set(LBM_ERR_ARG, "model %d", d->model);
  if (d->fluid_model != LBM_NEWTONIAN && d->fluid_model != LBM_POWERLAW)
    return lbm_err::set(LBM_ERR_ARG, "fluid model %d", d->fluid_model);
  if (d->storage < LBM_STORE_F32 || d->storage > LBM_STORE_I16S)
    return lbm_err::set(LBM_ERR_ARG, "storage %d", d->storage);
  const int V = d->nodes_per_thread;
  const bool vok = d->storage == LBM_STORE_F32 ? (V == 2 || V == 4) : (V == 4 || V == 8);
  if (!vok) return lbm_err::set(LBM_ERR_UNSUPPORTED, "nodes_per_thread %d for storage %d", V, d->storage);
  if (d->pipeline < LBM_PIPE_DIRECT || d->pipeline > LBM_PIPE_PREFETCH)
    return lbm_err::set(LBM_ERR_ARG, "pipeline %d", d->pipeline);
  if (d->pipeline != LBM_PIPE_DIRECT && V != lbm::AV && !(d->pipeline == LBM_PIPE_PREFETCH && V == 8))
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "persistent pipelines run %d nodes per thread (prefetch: also 8 "
                        "with 16-bit storage)", lbm::AV);
  if (d->fixed_exp != 0 && (d->fixed_exp < LBM_FIXED_EXP_MIN || d->fixed_exp > LBM_FIXED_EXP_MAX))
    return lbm_err::set(LBM_ERR_ARG, "fixed_exp %d outside [%d, %d]", d->fixed_exp, LBM_FIXED_EXP_MIN,
                        LBM_FIXED_EXP_MAX);
  if (d->wait_cycles < 0) return lbm_err::set(LBM_ERR_ARG, "wait_cycles %lld", (long long)d->wait_cycles);
  if (d->sc && d->storage == LBM_STORE_I16S)  // the strips' stores do not conserve a node's stored sum
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "Shan-Chen plans store fp32, fp16 or bf16 populations");
  if (d->aa != 0 && d->aa != 1) return lbm_err::set(LBM_ERR_ARG, "aa %d (0 or 1)", d->aa);
  if (d->aa && (d->pipeline != LBM_PIPE_DIRECT || d->sc))
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "the in-place step runs the direct pipeline without Shan-Chen");
  if (d->pipeline == LBM_PIPE_ASYNC && d->storage == LBM_STORE_I16S)
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "the fixed-point storage runs the direct or prefetch pipeline");
  if (d->pipeline == LBM_PIPE_ASYNC && (d->tune < 0 || d->tune >= LBM_ASYNC_TUNINGS))
    return lbm_err::set(LBM_ERR_ARG, "async tuning %d", d->tune);
  if (d->pipeline == LBM_PIPE_PREFETCH && (d->tune < 0 || d->tune >= LBM_PREFETCH_TUNINGS))
    return lbm_err::set(LBM_ERR_ARG, "prefetch tuning %d", d->tune);
  if (d->sc) {
    if (d->pipeline != LBM_PIPE_DIRECT || V != lbm::AV)
      return lbm_err::set(LBM_ERR_UNSUPPORTED, "Shan-Chen plans run the direct pipeline, %d nodes per thread",
                          lbm::AV);
    if (d->fluid_model != LBM_NEWTONIAN || d->nbc != 0)
      return lbm_err::set(LBM_ERR_UNSUPPORTED, "Shan-Chen plans take no power law and no rewrite boundaries");
  }
  if (d->nbc < 0 || d->nbc > LBM_MAX_BC) return lbm_err::set(LBM_ERR_ARG, "nbc %d", d->nbc);
  if (d->nprog < 0 || d->nprog > LBM_MAX_PROG) return lbm_err::set(LBM_ERR_ARG, "nprog %d", d->nprog);
  for (int i = 0; i < d->nbc; ++i) {
    const LbmBoundary& b = d->bc[i];
    if (b.kind < LBM_BC_VELOCITY_BB || b.kind > LBM_BC_OPEN_EXTRAP || b.kind == LBM_BC_OPEN_CONV2)
      return lbm_err::set(LBM_ERR_UNSUPPORTED, "boundary kind %d has no fused form", b.kind);
    if (b.direction < 1 || b.direction > 4)
      return lbm_err::set(LBM_ERR_ARG, "boundary %d direction %d", i, b.direction);
  }
  for (int p = 0; p < d->nprog; ++p)
    for (int s = 0; s < LBM_PROG_LEN; ++s) {
      const int bi = d->prog[p][s];
      if (bi >= d->nbc) return lbm_err::set(LBM_ERR_ARG, "program %d names boundary %d", p, bi);
    }
  LbmPlan* pl = new (std::nothrow) LbmPlan();
  if (!pl) return lbm_err::set(LBM_ERR_ARG, "out of host memory");
  pl->d = *d;
  FusedParams& p = pl->base;
  std::memset(&p, 0, sizeof(p));
  p.nx = d->nx;
  p.ny = d->ny;
  p.pitch = d->pitch;
  p.nseg = (d->nx + 32 * V - 1) / (32 * V);
  p.plane = (size_t)d->ny * d->pitch;
  p.model = d->model;
  p.fluid_model = d->fluid_model;
  p.has_force = (d->gravity[0] != 0.0f || d->gravity[1] != 0.0f) ? 1 : 0;
  p.omega = 1.0f / d->tau;
  p.omega_a = d->model == LBM_TRT ? 1.0f / d->tau_antisym : 0.0f;
  p.magic = d->magic;
  p.tau_min = d->tau_min;
  p.tau_max = d->tau_max;
  p.pl_m = d->pl_m;
  p.pl_n = d->pl_n;
  for (int a = 0; a < 9; ++a) p.s[a] = d->mrt_s[a];
  p.gx = d->gravity[0];
  p.gy = d->gravity[1];
  p.nbc = d->nbc;
  std::memcpy(p.bc, d->bc, sizeof(p.bc));
  std::memcpy(p.prog, d->prog, sizeof(p.prog));
  p.sc = d->sc;
  p.g_coh = d->g_coh;
  p.sc_T = d->sc_T;
  p.eos = d->eos;
  p.tune = d->tune;
  const int e = d->fixed_exp ? d->fixed_exp : LBM_FIXED_EXP_DEFAULT;
  p.fq = std::ldexp(1.0f, -e);
  p.fiq = std::ldexp(1.0f, e);
  p.foff = std::ldexp(1.0f, 23 - e) + std::ldexp(1.0f, 15 - e);
  p.wait_cycles = d->wait_cycles ? (long long)d->wait_cycles : lbm::WAIT_CYCLES;
  if (!(d->rho_ref >= 0.0f && d->rho_ref < 1e30f))
    return lbm_err::set(LBM_ERR_ARG, "rho_ref %g must be finite and >= 0", (double)d->rho_ref);
  const float rho_ref = d->rho_ref != 0.0f ? d->rho_ref : 1.0f;
  for (int k = 0; k < 9; ++k) p.wsh[k] = d->storage == LBM_STORE_F32 ? 0.0f : lbm::W(k) * rho_ref;
  double sum = 0.0;
  for (int k = 0; k < 9; ++k) sum += p.wsh[k];
  p.rho_shift = (float)sum;
  for (int a = 0; a < 9; ++a) {
    double m = 0.0;
    for (int k = 0; k < 9; ++k) m += (double)lbm::MRT_M(a, k) * p.wsh[k];
    p.mwsh[a] = (float)m;
  }
  *out = pl;
  return LBM_OK;
}

int lbm_plan_bind(LbmPlan* pl, const LbmPlanBuffers* b) {
  if (!pl || !b) return lbm_err::set(LBM_ERR_ARG, "plan_bind: NULL argument");
  if (!b->fa || !b->fb || !b->code || !b->seg_flags)
    return lbm_err::set(LBM_ERR_ARG, "plan_bind: fa, fb, code and seg_flags are required");
  if (!b->mom_a || !b->mom_b) return lbm_err::set(LBM_ERR_ARG, "plan_bind: moment buffers are required");
  if (pl->d.fluid_model == LBM_POWERLAW && !b->tau)
    return lbm_err::set(LBM_ERR_ARG, "plan_bind: power law needs the tau state buffer");
  const size_t va = (size_t)storage_bytes(pl->d.storage) * pl->d.nodes_per_thread;
  if (!aligned(b->fa, va) || !aligned(b->fb, va) || !aligned(b->code, 16) || (b->tau && !aligned(b->tau, 16)))
    return lbm_err::set(LBM_ERR_ARG, "plan_bind: buffers must be 16-byte aligned");
  if (pl->d.pipeline == LBM_PIPE_ASYNC && (!b->status || !aligned(b->fa, 16) || !aligned(b->fb, 16)))
    return lbm_err::set(LBM_ERR_ARG, "plan_bind: the async pipeline needs a status word and 16-byte "
                                     "aligned population buffers");
  if (b->nspecial < 0 || (b->nspecial > 0 && !b->special) ||
      (int64_t)b->nspecial > (int64_t)pl->d.ny * pl->base.nseg)
    return lbm_err::set(LBM_ERR_ARG, "plan_bind: %d special segments for a %d x %d segment grid", b->nspecial,
                        pl->d.ny, pl->base.nseg);
  if (b->nlanes < 0 || (b->nlanes > 0 && !b->lanes) || (b->lanes && !b->lane_mask) ||
      (int64_t)b->nlanes > (int64_t)pl->d.ny * pl->base.nseg * 32)
    return lbm_err::set(LBM_ERR_ARG, "plan_bind: %d marked lanes for a %d x %d segment grid", b->nlanes, pl->d.ny,
                        pl->base.nseg);
  if (b->nplain < 0 || (b->nplain > 0 && !b->plain) ||
      (int64_t)b->nplain + b->nspecial > (int64_t)pl->d.ny * pl->base.nseg)
    return lbm_err::set(LBM_ERR_ARG, "plan_bind: %d plain + %d special segments for a %d x %d segment grid",
                        b->nplain, b->nspecial, pl->d.ny, pl->base.nseg);
  if (pl->d.pipeline == LBM_PIPE_PREFETCH && pl->d.nodes_per_thread != lbm::AV && !pl->d.sc &&
      !(b->special && b->plain))
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "plan_bind: the prefetch pipeline at %d nodes per thread needs the "
                        "special and plain segment lists", pl->d.nodes_per_thread);
  if (pl->d.aa) {
    if (b->fa != b->fb) return lbm_err::set(LBM_ERR_ARG, "plan_bind: the in-place step needs fa == fb");
    if ((int64_t)pl->d.ny * pl->d.pitch > INT32_MAX)  // read sites are int32 plane offsets
      return lbm_err::set(LBM_ERR_UNSUPPORTED, "plan_bind: the in-place step takes lattices below 2^31 sites");
    if (!b->special || !b->lane_mask || !b->lanes)
      return lbm_err::set(LBM_ERR_ARG, "plan_bind: the in-place step needs the lane-granular lists (special, "
                                       "lane_mask, lanes)");
    bool reads = false;  // a boundary program reads a neighbour's populations
    for (int i = 0; i < pl->d.nbc; ++i) {
      const int k = pl->d.bc[i].kind;
      reads = reads || k == LBM_BC_VELOCITY_NEEM || k == LBM_BC_PRESSURE_NEEM || k == LBM_BC_OPEN_NEUMANN ||
              k == LBM_BC_OPEN_CONV1 || k == LBM_BC_OPEN_EXTRAP;
    }
    if (b->aa_nsites < 0 || (b->aa_nsites > 0 && (!b->aa_sites || !b->aa_vals)) || (reads && b->aa_nsites == 0))
      return lbm_err::set(LBM_ERR_ARG, "plan_bind: %d boundary read sites for the in-place step%s", b->aa_nsites,
                          reads ? " (its boundaries read neighbours: the sites are required)" : "");
  }
  pl->b = *b;
  pl->bound = true;
  pl->parity = 0;
  return LBM_OK;
}

int lbm_plan_run(LbmPlan* pl, int32_t nsteps, void* stream) {
  if (!pl || !pl->bound) return lbm_err::set(LBM_ERR_STATE, "plan_run: plan not bound");
  if (nsteps < 0) return lbm_err::set(LBM_ERR_ARG, "plan_run: nsteps %d", nsteps);
  return run_steps(pl, nsteps, nullptr, 0, nullptr, (cudaStream_t)stream);
}

int lbm_plan_get_parity(const LbmPlan* pl, int32_t* parity) {
  if (!pl || !parity) return lbm_err::set(LBM_ERR_ARG, "plan_get_parity: NULL argument");
  *parity = pl->parity;
  return LBM_OK;
}

int lbm_plan_set_parity(LbmPlan* pl, int32_t parity) {
  if (!pl || (parity != 0 && parity != 1)) return lbm_err::set(LBM_ERR_ARG, "plan_set_parity: bad argument");
  pl->parity = parity;
  return LBM_OK;
}

int lbm_plan_stream(LbmPlan* pl, float* f_out, void* stream) {
  if (!pl || !pl->bound) return lbm_err::set(LBM_ERR_STATE, "plan_stream: plan not bound");
  if (!f_out) return lbm_err::set(LBM_ERR_ARG, "plan_stream: f_out is NULL");
  FusedParams p = params_for(pl);
  cudaStream_t s = (cudaStream_t)stream;
  switch (pl->d.storage) {
    case LBM_STORE_F32: return lbm::launch_stream_only<LBM_STORE_F32>(p, f_out, s);
    case LBM_STORE_F16S: return lbm::launch_stream_only<LBM_STORE_F16S>(p, f_out, s);
    case LBM_STORE_BF16S: return lbm::launch_stream_only<LBM_STORE_BF16S>(p, f_out, s);
    default: return lbm::launch_stream_only<LBM_STORE_I16S>(p, f_out, s);
  }
}

static int convert(LbmPlan* pl, const float* in, float* out, void* stream) {
  if (!pl || !pl->bound) return lbm_err::set(LBM_ERR_STATE, "plan not bound");
  FusedParams p = params_for(pl);
  cudaStream_t s = (cudaStream_t)stream;
  void* cur = pl->parity ? pl->b.fb : pl->b.fa;
  void* other = pl->parity ? pl->b.fa : pl->b.fb;
  if (in && other != cur) {  // import: the other buffer too (nodes outside the group are never written)
    int rc = LBM_OK;
    switch (pl->d.storage) {
      case LBM_STORE_F32:
        if (in != other)
          rc = lbm_err::cuda(cudaMemcpyAsync(other, in, 9 * p.plane * sizeof(float), cudaMemcpyDeviceToDevice, s),
                             "import");
        break;
      case LBM_STORE_F16S: rc = lbm::launch_convert<LBM_STORE_F16S>(p, in, other, 1, s); break;
      case LBM_STORE_BF16S: rc = lbm::launch_convert<LBM_STORE_BF16S>(p, in, other, 1, s); break;
      default: rc = lbm::launch_convert<LBM_STORE_I16S>(p, in, other, 1, s); break;
    }
    if (rc) return rc;
  }
  if (pl->d.storage == LBM_STORE_F32) {
    const size_t bytes = 9 * p.plane * sizeof(float);
    if (in && in != cur) return lbm_err::cuda(cudaMemcpyAsync(cur, in, bytes, cudaMemcpyDeviceToDevice, s), "import");
    if (out && out != cur) return lbm_err::cuda(cudaMemcpyAsync(out, cur, bytes, cudaMemcpyDeviceToDevice, s), "export");
    return LBM_OK;
  }
  if (pl->d.storage == LBM_STORE_F16S)
    return in ? lbm::launch_convert<LBM_STORE_F16S>(p, in, cur, 1, s)
              : lbm::launch_convert<LBM_STORE_F16S>(p, nullptr, out, 0, s);
  if (pl->d.storage == LBM_STORE_BF16S)
    return in ? lbm::launch_convert<LBM_STORE_BF16S>(p, in, cur, 1, s)
              : lbm::launch_convert<LBM_STORE_BF16S>(p, nullptr, out, 0, s);
  return in ? lbm::launch_convert<LBM_STORE_I16S>(p, in, cur, 1, s)
            : lbm::launch_convert<LBM_STORE_I16S>(p, nullptr, out, 0, s);
}

int lbm_plan_import(LbmPlan* pl, const float* f_post, void* stream) {
  if (!f_post) return lbm_err::set(LBM_ERR_ARG, "plan_import: NULL source");
  return convert(pl, f_post, nullptr, stream);
}

int lbm_plan_export(LbmPlan* pl, float* f_post, void* stream) {
  if (!f_post) return lbm_err::set(LBM_ERR_ARG, "plan_export: NULL destination");
  return convert(pl, nullptr, f_post, stream);
}

int lbm_plan_destroy(LbmPlan* pl) {
  if (pl) release_side(pl);
  delete pl;
  return LBM_OK;
}


int lbm_plan_momentum_exchange(LbmPlan* pl, const int32_t* links, int64_t n, double* out, void* stream) {
  if (!pl || !pl->bound) return lbm_err::set(LBM_ERR_STATE, "momentum_exchange: plan not bound");
  if (!out || n < 0 || (n > 0 && !links)) return lbm_err::set(LBM_ERR_ARG, "momentum_exchange: bad arguments");
  return mex(pl, links, n, out, (cudaStream_t)stream);
}

int lbm_plan_run_monitored(LbmPlan* pl, int32_t nsteps, const int32_t* links, int64_t n, double* series,
                           void* stream) {
  if (!pl || !pl->bound) return lbm_err::set(LBM_ERR_STATE, "run_monitored: plan not bound");
  if (nsteps < 0 || !series || n < 0 || (n > 0 && !links))
    return lbm_err::set(LBM_ERR_ARG, "run_monitored: bad arguments");
  return run_steps(pl, nsteps, links, n, series, (cudaStream_t)stream);
}

}  // extern "C"

// ------------------------------------------------------------------------
// Allocation-free moment reduction.
//
// For callers that must not allocate device memory themselves: the partial
// sums live in this file-scope device array instead of caller scratch.  It is
// 3 * LBM_NOALLOC_BLOCKS doubles (48 KiB) on every device that loads the
// library and stays allocated until the process exits.  Each block reduces a
// fixed chunk of LBM_NOALLOC_CHUNK lattice sites, so the largest lattice the
// array serves is LBM_NOALLOC_MAX_NODES sites (ny * pitch); larger ones are
// rejected.  All calls share the array and every call overwrites the slots
// it reads, so nothing needs clearing; calls whose work overlaps on the GPU
// (different streams or threads) race on it.
namespace {

static_assert(LBM_NOALLOC_MAX_NODES % LBM_NOALLOC_CHUNK == 0, "chunk must divide the limit");
constexpr int LBM_NOALLOC_BLOCKS = (int)(LBM_NOALLOC_MAX_NODES / LBM_NOALLOC_CHUNK);

__device__ __align__(256) double g_noalloc_partials[3 * LBM_NOALLOC_BLOCKS];

// Host code cannot use g_noalloc_partials as a pointer: its host-side name is
// a stand-in, not the device address.  The address is looked up once per
// device, with that device current, on the first call made on it, and kept
// for the life of the process.  It belongs to the device's primary context
// (the one the CUDA runtime and PyTorch use): after cudaDeviceReset, or from
// another driver context, the kept address no longer names the array.
constexpr int MAX_DEVICES = 64;
double* g_noalloc_ptr[MAX_DEVICES] = {nullptr};
std::mutex g_noalloc_mutex;

int noalloc_scratch(double** out) {
  int dev = 0;
  int rc = lbm_err::cuda(cudaGetDevice(&dev), "noalloc reduction: cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= MAX_DEVICES) return lbm_err::set(LBM_ERR_UNSUPPORTED, "device ordinal %d", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    rc = lbm_err::cuda(cudaGetSymbolAddress(&p, g_noalloc_partials),
                       "noalloc reduction: cudaGetSymbolAddress");
    if (rc) return rc;
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return LBM_OK;
}

// block b sums sites [b*chunk, (b+1)*chunk) of the state into partials[3b..3b+2]
template <int ST>
__global__ void __launch_bounds__(lbm::REDUCE_TPB) k_reduce_chunked(const FusedParams p, double* partials,
                                                                    int64_t chunk) {
  using S = lbm::Storage<ST>;
  using T = typename S::T;
  const T* src = reinterpret_cast<const T*>(p.src);
  const size_t n = (size_t)p.ny * p.pitch;
  const size_t lo = (size_t)blockIdx.x * chunk;
  const size_t hi = lo + chunk < n ? lo + chunk : n;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (size_t q = lo + threadIdx.x; q < hi; q += blockDim.x) {
    const int x = (int)(q % p.pitch);
    if (x >= p.nx || !(p.code[q] & LBM_CODE_ACTIVE)) continue;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double v = S::dec64(src[(size_t)k * p.plane + q], p.wsh[k], p.fq);
      a0 += v;
      if (lbm::CX(k)) a1 += lbm::CX(k) * v;
      if (lbm::CY(k)) a2 += lbm::CY(k) * v;
    }
  }
  __shared__ double sh[3][lbm::REDUCE_TPB / 32];
  a0 = lbm::warp_sum(a0);
  a1 = lbm::warp_sum(a1);
  a2 = lbm::warp_sum(a2);
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = a0;
    sh[1][threadIdx.x >> 5] = a1;
    sh[2][threadIdx.x >> 5] = a2;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int i = 0; i < lbm::REDUCE_TPB / 32; ++i) s += sh[threadIdx.x][i];
    partials[(size_t)blockIdx.x * 3 + threadIdx.x] = s;
  }
}

template <int ST>
int launch_noalloc(const FusedParams& p, double* partials, int nblocks, double* out, cudaStream_t s) {
  k_reduce_chunked<ST><<<nblocks, lbm::REDUCE_TPB, 0, s>>>(p, partials, LBM_NOALLOC_CHUNK);
  lbm::k_reduce_final<ST><<<1, 96, 0, s>>>(partials, nblocks, out);
  return lbm_err::launch("noalloc moment reduction");
}

}  // namespace

extern "C" {

int lbm_plan_reduce_moments_noalloc(LbmPlan* pl, double* out, void* stream) {
  if (!pl) return lbm_err::set(LBM_ERR_ARG, "reduce_noalloc: NULL plan");
  // the size is the descriptor's: checked before anything bound is looked at
  const int64_t sites = (int64_t)pl->d.ny * pl->d.pitch;
  if (sites > LBM_NOALLOC_MAX_NODES)
    return lbm_err::set(LBM_ERR_ARG,
                        "reduce_noalloc: lattice of %lld sites (ny * pitch) exceeds the allocation-free "
                        "limit of %lld; use lbm_plan_reduce_moments with caller scratch",
                        (long long)sites, (long long)LBM_NOALLOC_MAX_NODES);
  if (!pl->bound) return lbm_err::set(LBM_ERR_STATE, "reduce_noalloc: plan not bound");
  if (!out) return lbm_err::set(LBM_ERR_ARG, "reduce_noalloc: NULL output");
  double* partials = nullptr;
  int rc = noalloc_scratch(&partials);
  if (rc) return rc;
  const int nblocks = (int)((sites + LBM_NOALLOC_CHUNK - 1) / LBM_NOALLOC_CHUNK);
  FusedParams p = params_for(pl);
  cudaStream_t s = (cudaStream_t)stream;
  switch (pl->d.storage) {
    case LBM_STORE_F32: return launch_noalloc<LBM_STORE_F32>(p, partials, nblocks, out, s);
    case LBM_STORE_F16S: return launch_noalloc<LBM_STORE_F16S>(p, partials, nblocks, out, s);
    case LBM_STORE_BF16S: return launch_noalloc<LBM_STORE_BF16S>(p, partials, nblocks, out, s);
    default: return launch_noalloc<LBM_STORE_I16S>(p, partials, nblocks, out, s);
  }
}

int64_t lbm_reduce_scratch_doubles(void) { return (int64_t)lbm::REDUCE_BLOCKS * 3; }

int lbm_plan_reduce_moments(LbmPlan* pl, double* partials, double* out, void* stream) {
  if (!pl || !pl->bound) return lbm_err::set(LBM_ERR_STATE, "reduce: plan not bound");
  if (!partials || !out) return lbm_err::set(LBM_ERR_ARG, "reduce: NULL scratch or output");
  FusedParams p = params_for(pl);
  cudaStream_t s = (cudaStream_t)stream;
  switch (pl->d.storage) {
    case LBM_STORE_F32: return lbm::launch_reduce<LBM_STORE_F32>(p, partials, out, s);
    case LBM_STORE_F16S: return lbm::launch_reduce<LBM_STORE_F16S>(p, partials, out, s);
    case LBM_STORE_BF16S: return lbm::launch_reduce<LBM_STORE_BF16S>(p, partials, out, s);
    default: return lbm::launch_reduce<LBM_STORE_I16S>(p, partials, out, s);
  }
}

}  // extern "C"
