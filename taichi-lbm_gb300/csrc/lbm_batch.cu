// Batch of independent lattices advanced together (C ABI: lbm_batch_*).
//
// A batch holds bound plans ("members").  On the first run after a change of
// membership it groups the members by kernel kind (Shan-Chen strip, plain
// segment, flagged segment) x collision model x power law x storage x nodes
// per lane x body force, writes one device record per member (its parameters
// for both ping-pong parities) and one packed tile table, and from then on a
// step is one persistent launch per group, followed by the drag/lift monitors.
// The groups of a step run concurrently on a few worker streams (parallel
// branches of the graph when graphs are on).  The batch runs on its own
// stream, forked from and joined back to the caller's stream; with graphs on
// it captures two steps (parities 0 and 1) once per membership and replays
// them.  Membership changes never wait for the GPU: the tables are double
// buffered and written in stream order, so a rebuild is queued behind the
// steps that still read the previous tables.
#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <tuple>
#include <vector>

#include "lbm_batch.cuh"
#include "lbm_plan_internal.h"

LBM_BATCH_EXTERN(LBM_STORE_F32)
LBM_BATCH_EXTERN(LBM_STORE_F16S)
LBM_BATCH_EXTERN(LBM_STORE_BF16S)
LBM_BATCH_EXTERN(LBM_STORE_I16S)

using lbm::BatchGroup;
using lbm::BatchLattice;
using lbm::BatchMonitor;
using lbm::BatchTile;

struct BatchMember {
  LbmPlan* plan = nullptr;
  std::vector<uint32_t> masks;  // host copy of the plan's lane masks
  bool monitored = false;
  const int32_t* links = nullptr;
  int64_t nlinks = 0;
  double* series = nullptr;
  int32_t* count = nullptr;
  int32_t capacity = 0;
};

struct LbmBatch {
  std::vector<BatchMember> slots;  // plan == nullptr: free slot
  bool dirty = true;
  long long step = 0;  // steps run; parity = step & 1
  int dev = -1;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  // device tables, double buffered: set `cur` is the one launches read
  struct Tables {
    BatchLattice* lats = nullptr;
    size_t lats_cap = 0;
    BatchTile* tiles = nullptr;
    size_t tiles_cap = 0;
    BatchMonitor* mons = nullptr;
    size_t mons_cap = 0;
  } tab[2];
  int cur = 0;
  BatchLattice* d_lats = nullptr;  // tab[cur]
  BatchTile* d_tiles = nullptr;
  BatchMonitor* d_mons = nullptr;
  std::vector<BatchGroup> groups;
  // worker streams for the groups of one step
  static constexpr int NWORK = 4;
  cudaStream_t work[NWORK] = {};
  cudaEvent_t step_fork = nullptr;
  cudaEvent_t step_join[NWORK] = {};
  int mon_off[4] = {0, 0, 0, 0}, mon_cnt[4] = {0, 0, 0, 0};  // monitors per storage
  long long ntiles = 0;
  int nlats = 0;
  // graphs
  bool use_graph = false;
  cudaGraphExec_t exec = nullptr;
  bool graph_ok = false;
  // members of at least solo_nodes nodes run their own single-lattice step
  // (parameters by value, in the constant bank) instead of the packed tiles
  int64_t solo_nodes = int64_t(1) << 19;
  // rows per Shan-Chen strip (8, 16 or 32); 0 chooses from the batch's size
  int sc_rows_fixed = 0;
  // form of the lean groups (0: k_batch_lean; 1, 2: k_batch_lean_pf)
  int lean_form = 0;
  struct Solo {
    int storage, V, flip;
    lbm::FusedParams p[2];  // [parity]
  };
  std::vector<Solo> solos;
};

namespace {

int launch_group(BatchGroup& g, const BatchLattice* lats, const BatchTile* tiles, int sp, cudaStream_t s) {
  switch (g.storage) {
    case LBM_STORE_F32: return lbm::launch_batch_group<LBM_STORE_F32>(g, lats, tiles, sp, s);
    case LBM_STORE_F16S: return lbm::launch_batch_group<LBM_STORE_F16S>(g, lats, tiles, sp, s);
    case LBM_STORE_BF16S: return lbm::launch_batch_group<LBM_STORE_BF16S>(g, lats, tiles, sp, s);
    default: return lbm::launch_batch_group<LBM_STORE_I16S>(g, lats, tiles, sp, s);
  }
}

int launch_monitors(LbmBatch* b, int sp, cudaStream_t s) {
  for (int st = 0; st < 4; ++st) {
    if (!b->mon_cnt[st]) continue;
    const BatchMonitor* m = b->d_mons + b->mon_off[st];
    int rc = st == LBM_STORE_F32     ? lbm::launch_batch_monitors<LBM_STORE_F32>(b->d_lats, m, b->mon_cnt[st], sp, s)
             : st == LBM_STORE_F16S  ? lbm::launch_batch_monitors<LBM_STORE_F16S>(b->d_lats, m, b->mon_cnt[st], sp, s)
             : st == LBM_STORE_BF16S ? lbm::launch_batch_monitors<LBM_STORE_BF16S>(b->d_lats, m, b->mon_cnt[st], sp, s)
                                     : lbm::launch_batch_monitors<LBM_STORE_I16S>(b->d_lats, m, b->mon_cnt[st], sp, s);
    if (rc) return rc;
  }
  return LBM_OK;
}

int launch_solo(const LbmBatch::Solo& m, int sp, cudaStream_t s, cudaStream_t s2) {
  const lbm::FusedParams& p = m.p[(sp ^ m.flip) & 1];
  switch (m.storage) {
    case LBM_STORE_F32: return lbm::launch_fused<LBM_STORE_F32>(p, m.V, s, s2);
    case LBM_STORE_F16S: return lbm::launch_fused<LBM_STORE_F16S>(p, m.V, s, s2);
    case LBM_STORE_BF16S: return lbm::launch_fused<LBM_STORE_BF16S>(p, m.V, s, s2);
    default: return lbm::launch_fused<LBM_STORE_I16S>(p, m.V, s, s2);
  }
}

// streams a step's launches use: one per tile group, and per solo member one
// for its segments plus one for its marked lanes (the two read the same
// source and write disjoint nodes, so they overlap like the plan's own fork)
int launch_slots(const LbmBatch* b) {
  int n = (int)b->groups.size();
  for (const LbmBatch::Solo& m : b->solos) n += m.p[0].nlanes > 0 ? 2 : 1;
  return n;
}

// one batched step at parity sp on stream s: the groups and solo members on
// the worker streams (forked from s and joined back), then the monitors on s
int batch_step(LbmBatch* b, int sp, cudaStream_t s) {
  const int nslot = launch_slots(b);
  if (nslot <= 1) {
    for (BatchGroup& g : b->groups) {
      int rc = launch_group(g, b->d_lats, b->d_tiles, sp, s);
      if (rc) return rc;
    }
    for (const LbmBatch::Solo& m : b->solos) {
      int rc = launch_solo(m, sp, s, s);
      if (rc) return rc;
    }
    return launch_monitors(b, sp, s);
  }
  const int nw = nslot < LbmBatch::NWORK ? nslot : LbmBatch::NWORK;
  int rc = lbm_err::cuda(cudaEventRecord(b->step_fork, s), "batch: step fork");
  for (int w = 0; !rc && w < nw; ++w) rc = lbm_err::cuda(cudaStreamWaitEvent(b->work[w], b->step_fork, 0), "batch: step fork");
  if (rc) return rc;
  int rl = LBM_OK;
  int k = 0;
  // in key order: the plain groups (the bulk of the work) first.  Launching
  // the small groups first was measured: neutral on a fixed mix, but a
  // served stream that packs its big lattices lost a third of its rate
  for (size_t i = 0; i < b->groups.size() && !rl; ++i)
    rl = launch_group(b->groups[i], b->d_lats, b->d_tiles, sp, b->work[k++ % nw]);
  for (size_t i = 0; i < b->solos.size() && !rl; ++i) {
    const LbmBatch::Solo& m = b->solos[i];
    cudaStream_t a = b->work[k++ % nw];
    cudaStream_t c = m.p[0].nlanes > 0 ? b->work[k++ % nw] : a;
    rl = launch_solo(m, sp, a, c);
  }
  // join every worker even after a failed launch
  for (int w = 0; w < nw; ++w) {
    int rj = lbm_err::cuda(cudaEventRecord(b->step_join[w], b->work[w]), "batch: step join");
    if (!rj) rj = lbm_err::cuda(cudaStreamWaitEvent(s, b->step_join[w], 0), "batch: step join");
    if (!rc) rc = rj;
  }
  if (rl) return rl;
  if (rc) return rc;
  return launch_monitors(b, sp, s);
}

void drop_graph(LbmBatch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->graph_ok = false;
}

// stream-ordered (re)allocation: launches queued before on s keep their memory
template <typename T>
int ensure_capacity(T** ptr, size_t* cap, size_t n, cudaStream_t s, const char* what) {
  if (n <= *cap && *ptr) return LBM_OK;
  if (*ptr) cudaFreeAsync(*ptr, s);
  *ptr = nullptr;
  *cap = 0;
  const size_t want = std::max<size_t>(2 * n, 16);
  int rc = lbm_err::cuda(cudaMallocAsync(reinterpret_cast<void**>(ptr), want * sizeof(T), s), what);
  if (rc) return rc;
  *cap = want;
  return LBM_OK;
}

int ensure_stream(LbmBatch* b) {
  int dev = 0;
  int rc = lbm_err::cuda(cudaGetDevice(&dev), "batch: device");
  if (rc) return rc;
  if (b->stream && b->dev == dev) return LBM_OK;
  if (b->stream) return lbm_err::set(LBM_ERR_STATE, "batch: created on device %d, used on device %d", b->dev, dev);
  rc = lbm_err::cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "batch: stream");
  if (!rc) rc = lbm_err::cuda(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "batch: event");
  if (!rc) rc = lbm_err::cuda(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming), "batch: event");
  if (!rc) rc = lbm_err::cuda(cudaEventCreateWithFlags(&b->step_fork, cudaEventDisableTiming), "batch: event");
  for (int w = 0; !rc && w < LbmBatch::NWORK; ++w) {
    rc = lbm_err::cuda(cudaStreamCreateWithFlags(&b->work[w], cudaStreamNonBlocking), "batch: worker stream");
    if (!rc) rc = lbm_err::cuda(cudaEventCreateWithFlags(&b->step_join[w], cudaEventDisableTiming), "batch: event");
  }
  if (rc) return rc;
  b->dev = dev;
  return LBM_OK;
}

struct GroupKey {
  int kind, model, powerlaw, storage, V, force;
  bool operator<(const GroupKey& o) const {
    return std::tie(kind, storage, model, powerlaw, V, force) <
           std::tie(o.kind, o.storage, o.model, o.powerlaw, o.V, o.force);
  }
  bool operator==(const GroupKey& o) const {
    return kind == o.kind && model == o.model && powerlaw == o.powerlaw && storage == o.storage && V == o.V &&
           force == o.force;
  }
};

// rebuild the device records and tile tables from the current members
int rebuild(LbmBatch* b) {
  // the new tables go to the other buffer set, written in stream order after
  // the queued steps that still read the current set; a graph being replayed
  // is freed by the driver when its launches complete
  int rc = LBM_OK;
  drop_graph(b);
  const int sp = (int)(b->step & 1);
  std::vector<BatchLattice> lats;
  std::map<GroupKey, std::vector<BatchTile>> by_key;  // references stay valid as keys are added
  auto bucket = [&](const GroupKey& k) -> std::vector<BatchTile>& { return by_key[k]; };
  std::vector<BatchMonitor> mons[4];
  std::vector<LbmBatch::Solo> solos;
  // rows per Shan-Chen strip: the longest that still gives the GPU enough
  // strips in total (two per resident warp of 152 SMs x 12 warps)
  int sc_rows = b->sc_rows_fixed ? b->sc_rows_fixed : 2 * lbm::SC_CHUNK;
  for (; !b->sc_rows_fixed && sc_rows > lbm::SC_CHUNK / 2; sc_rows /= 2) {
    long long items = 0;
    for (const BatchMember& m : b->slots)
      if (m.plan && m.plan->d.sc)
        items += (long long)m.plan->base.nseg * ((m.plan->d.ny + sc_rows - 1) / sc_rows);
    if (items >= 2 * 152 * 12) break;
  }
  for (BatchMember& m : b->slots) {
    if (!m.plan) continue;
    LbmPlan* pl = m.plan;
    const int lat = (int)lats.size();
    BatchLattice rec;
    std::memset(&rec, 0, sizeof(rec));
    const int saved = pl->parity;
    for (int v = 0; v < 2; ++v) {
      pl->parity = v;
      rec.full[v] = lbm_plan_params(pl);
      rec.full[v].special = nullptr;  // the batch supplies its own tiles
      rec.full[v].plain = nullptr;
      rec.full[v].lane_mask = pl->b.lane_mask;
      rec.full[v].lanes = nullptr;
      rec.full[v].nlanes = 0;
      rec.lean[v] = lbm::lean_of(rec.full[v]);
      rec.lean[v].sc_rows = sc_rows;
    }
    rec.flip = saved ^ sp;
    lats.push_back(rec);
    if (!pl->d.sc && (int64_t)pl->d.nx * pl->d.ny >= b->solo_nodes && b->solo_nodes > 0 && pl->b.special &&
        pl->b.lane_mask && pl->b.lanes && pl->d.pipeline == LBM_PIPE_DIRECT) {
      LbmBatch::Solo so;
      so.storage = pl->d.storage;
      so.V = pl->d.nodes_per_thread;
      so.flip = rec.flip;
      for (int v = 0; v < 2; ++v) {
        pl->parity = v;
        so.p[v] = lbm_plan_params(pl);  // the plan's own lane-granular two-pass step
      }
      pl->parity = saved;
      solos.push_back(so);
      if (m.monitored) {
        BatchMonitor bm;
        bm.lat = lat;
        bm.nlinks = m.nlinks;
        bm.links = m.links;
        bm.series = m.series;
        bm.count = m.count;
        bm.capacity = m.capacity;
        mons[pl->d.storage].push_back(bm);
      }
      continue;
    }
    pl->parity = saved;
    const lbm::FusedParams& p = rec.full[0];
    const int pw = pl->d.fluid_model == LBM_POWERLAW ? 1 : 0;
    if (pl->d.sc) {
      auto& t = bucket({lbm::BATCH_SC, pl->d.model, 0, pl->d.storage, pl->d.nodes_per_thread, 1});
      const int chunks = (p.ny + sc_rows - 1) / sc_rows;
      for (int item = 0; item < chunks * p.nseg; ++item) t.push_back({lat, item});
    } else {
      // every segment on the plain path (fully marked ones skipped), marked lanes one by one
      const std::vector<uint32_t>& masks = m.masks;
      // lean groups hold every collision model (the kernel branches per lattice);
      // the marked-lane group also every fluid model
      auto& tl = bucket({lbm::BATCH_LEAN, -1, pw, pl->d.storage, pl->d.nodes_per_thread, p.has_force});
      auto& ts = bucket({lbm::BATCH_SPECIAL, -1, -1, pl->d.storage, pl->d.nodes_per_thread, 0});
      for (int item = 0; item < (int)masks.size(); ++item) {
        const uint32_t mk = masks[item];
        if (mk != 0xffffffffu) tl.push_back({lat, item});
        for (int l = 0; l < 32; ++l)
          if (mk >> l & 1u) ts.push_back({lat, item * 32 + l});
      }
      // whole blocks per lattice
      while (tl.size() % lbm::lean_block_tiles(b->lean_form)) tl.push_back({lat, -1});
    }
    if (m.monitored) {
      BatchMonitor bm;
      bm.lat = lat;
      bm.nlinks = m.nlinks;
      bm.links = m.links;
      bm.series = m.series;
      bm.count = m.count;
      bm.capacity = m.capacity;
      mons[pl->d.storage].push_back(bm);
    }
  }
  // plain groups first (the bulk of the work), then Shan-Chen, then flagged:
  // the key order starts with the kind
  std::vector<std::pair<GroupKey, std::vector<BatchTile>>> buckets(by_key.begin(), by_key.end());
  std::vector<BatchTile> tiles;
  b->groups.clear();
  for (auto& e : buckets) {
    if (e.second.empty()) continue;
    BatchGroup g;
    g.kind = e.first.kind;
    g.model = e.first.model;
    g.powerlaw = e.first.powerlaw;
    g.storage = e.first.storage;
    g.V = e.first.V;
    g.force = e.first.force;
    g.form = g.kind == lbm::BATCH_LEAN ? b->lean_form : 0;
    g.offset = (int)tiles.size();
    g.count = (int)e.second.size();
    g.blocks = 0;
    tiles.insert(tiles.end(), e.second.begin(), e.second.end());
    b->groups.push_back(g);
  }
  if (tiles.size() > (size_t)INT32_MAX) return lbm_err::set(LBM_ERR_UNSUPPORTED, "batch: too many tiles");
  std::vector<BatchMonitor> allm;
  for (int st = 0; st < 4; ++st) {
    b->mon_off[st] = (int)allm.size();
    b->mon_cnt[st] = (int)mons[st].size();
    allm.insert(allm.end(), mons[st].begin(), mons[st].end());
  }
  const int nt = b->cur ^ 1;
  LbmBatch::Tables& T = b->tab[nt];
  cudaStream_t s = b->stream;
  rc = ensure_capacity(&T.lats, &T.lats_cap, lats.size(), s, "batch: lattice records");
  if (!rc) rc = ensure_capacity(&T.tiles, &T.tiles_cap, tiles.size(), s, "batch: tile table");
  if (!rc) rc = ensure_capacity(&T.mons, &T.mons_cap, allm.size(), s, "batch: monitors");
  if (rc) return rc;
  // pageable sources: each call returns once its data is staged
  if (!lats.empty())
    rc = lbm_err::cuda(cudaMemcpyAsync(T.lats, lats.data(), lats.size() * sizeof(BatchLattice), cudaMemcpyHostToDevice, s),
                       "batch: upload records");
  if (!rc && !tiles.empty())
    rc = lbm_err::cuda(cudaMemcpyAsync(T.tiles, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, s),
                       "batch: upload tiles");
  if (!rc && !allm.empty())
    rc = lbm_err::cuda(cudaMemcpyAsync(T.mons, allm.data(), allm.size() * sizeof(BatchMonitor), cudaMemcpyHostToDevice, s),
                       "batch: upload monitors");
  if (rc) return rc;
  b->cur = nt;
  b->d_lats = T.lats;
  b->d_tiles = T.tiles;
  b->d_mons = T.mons;
  b->solos = std::move(solos);
  b->ntiles = (long long)tiles.size();
  b->nlats = (int)lats.size();
  b->dirty = false;
  return LBM_OK;
}

int capture(LbmBatch* b) {
  // two steps, parities 0 and 1, on the batch stream
  cudaGraph_t graph = nullptr;
  int rc = lbm_err::cuda(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "batch: begin capture");
  if (rc) return rc;
  int rs = batch_step(b, 0, b->stream);
  if (!rs) rs = batch_step(b, 1, b->stream);
  rc = lbm_err::cuda(cudaStreamEndCapture(b->stream, &graph), "batch: end capture");
  if (rs) rc = rs;
  if (!rc) rc = lbm_err::cuda(cudaGraphInstantiate(&b->exec, graph, 0), "batch: instantiate graph");
  if (graph) cudaGraphDestroy(graph);
  if (rc) {
    drop_graph(b);
    return rc;
  }
  b->graph_ok = true;
  return LBM_OK;
}

// advance the parity bookkeeping of the batch and of every member plan
void advance(LbmBatch* b, int n) {
  b->step += n;
  if (n & 1)
    for (BatchMember& m : b->slots)
      if (m.plan) m.plan->parity ^= 1;
}

int run_on_stream(LbmBatch* b, int32_t nsteps) {
  cudaStream_t s = b->stream;
  int done = 0;
  if (b->use_graph && nsteps >= 3 && b->nlats > 0) {
    if (!b->graph_ok) {  // a direct step sizes every persistent grid before the capture
      int rc = batch_step(b, (int)(b->step & 1), s);
      if (rc) return rc;
      advance(b, 1);
      ++done;
    }
    if (b->step & 1) {  // the graph starts at parity 0
      int rc = batch_step(b, 1, s);
      if (rc) return rc;
      advance(b, 1);
      ++done;
    }
    if (!b->graph_ok && nsteps - done >= 2) {
      int rc = capture(b);
      if (rc) return rc;
    }
    while (b->graph_ok && nsteps - done >= 2) {
      int rc = lbm_err::cuda(cudaGraphLaunch(b->exec, s), "batch: graph launch");
      if (rc) return rc;
      advance(b, 2);
      done += 2;
    }
  }
  while (done < nsteps) {
    int rc = batch_step(b, (int)(b->step & 1), s);
    if (rc) return rc;
    advance(b, 1);
    ++done;
  }
  return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_batch_create(LbmBatch** out) {
  if (!out) return lbm_err::set(LBM_ERR_ARG, "batch_create: NULL argument");
  *out = new (std::nothrow) LbmBatch();
  return *out ? LBM_OK : lbm_err::set(LBM_ERR_ARG, "batch_create: out of host memory");
}

int lbm_batch_add(LbmBatch* b, LbmPlan* plan, const uint32_t* host_lane_mask, int32_t* slot) {
  if (!b || !plan || !slot) return lbm_err::set(LBM_ERR_ARG, "batch_add: NULL argument");
  if (!plan->d.sc && !plan->b.lane_mask)
    return lbm_err::set(LBM_ERR_ARG, "batch_add: the plan was bound without lane masks");
  if (!plan->bound) return lbm_err::set(LBM_ERR_STATE, "batch_add: plan not bound");
  const LbmPlanDesc& d = plan->d;
  const int V = d.nodes_per_thread;
  if (d.aa) return lbm_err::set(LBM_ERR_UNSUPPORTED, "batch_add: batched members run the ping-pong step");
  if (d.sc && V != lbm::AV)
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "batch_add: Shan-Chen members run %d nodes per lane", lbm::AV);
  if (d.storage == LBM_STORE_F32 ? (V != 2 && V != 4) : (V != 4 && V != 8))
    return lbm_err::set(LBM_ERR_UNSUPPORTED, "batch_add: nodes_per_thread %d for storage %d", V, d.storage);
  for (const BatchMember& m : b->slots)
    if (m.plan == plan) return lbm_err::set(LBM_ERR_ARG, "batch_add: plan is already a member");
  size_t i = 0;
  while (i < b->slots.size() && b->slots[i].plan) ++i;
  if (i == b->slots.size()) b->slots.emplace_back();
  BatchMember m;
  m.plan = plan;
  if (!d.sc) {
    m.masks.resize((size_t)d.ny * plan->base.nseg);
    const size_t bytes = m.masks.size() * sizeof(uint32_t);
    if (host_lane_mask) {
      std::memcpy(m.masks.data(), host_lane_mask, bytes);
    } else {
      int rc = lbm_err::cuda(cudaMemcpy(m.masks.data(), plan->b.lane_mask, bytes, cudaMemcpyDeviceToHost),
                             "batch_add: lane masks");
      if (rc) return rc;
    }
  }
  b->slots[i] = std::move(m);
  b->dirty = true;
  *slot = (int32_t)i;
  return LBM_OK;
}

int lbm_batch_monitor(LbmBatch* b, int32_t slot, const int32_t* links, int64_t nlinks, double* series,
                      int32_t* count, int32_t capacity) {
  if (!b || slot < 0 || slot >= (int32_t)b->slots.size() || !b->slots[slot].plan)
    return lbm_err::set(LBM_ERR_ARG, "batch_monitor: no member in slot %d", slot);
  if (nlinks < 0 || (nlinks > 0 && !links) || !series || !count || capacity < 0)
    return lbm_err::set(LBM_ERR_ARG, "batch_monitor: bad arguments");
  BatchMember& m = b->slots[slot];
  m.monitored = true;
  m.links = links;
  m.nlinks = nlinks;
  m.series = series;
  m.count = count;
  m.capacity = capacity;
  b->dirty = true;
  return LBM_OK;
}

int lbm_batch_remove(LbmBatch* b, int32_t slot) {
  if (!b || slot < 0 || slot >= (int32_t)b->slots.size() || !b->slots[slot].plan)
    return lbm_err::set(LBM_ERR_ARG, "batch_remove: no member in slot %d", slot);
  b->slots[slot] = BatchMember();
  b->dirty = true;
  return LBM_OK;
}

int lbm_batch_set_solo(LbmBatch* b, int64_t min_nodes) {
  if (!b || min_nodes < 0) return lbm_err::set(LBM_ERR_ARG, "batch_set_solo: bad arguments");
  b->solo_nodes = min_nodes;
  b->dirty = true;
  return LBM_OK;
}

int lbm_batch_set_lean_form(LbmBatch* b, int32_t form) {
  if (!b || form < 0 || form > 2) return lbm_err::set(LBM_ERR_ARG, "batch_set_lean_form: form must be 0, 1 or 2");
  b->lean_form = form;
  b->dirty = true;
  return LBM_OK;
}

int lbm_batch_set_sc_rows(LbmBatch* b, int32_t rows) {
  if (!b || (rows != 0 && rows != lbm::SC_CHUNK / 2 && rows != lbm::SC_CHUNK && rows != 2 * lbm::SC_CHUNK))
    return lbm_err::set(LBM_ERR_ARG, "batch_set_sc_rows: rows must be 0, %d, %d or %d", lbm::SC_CHUNK / 2,
                        lbm::SC_CHUNK, 2 * lbm::SC_CHUNK);
  b->sc_rows_fixed = rows;
  b->dirty = true;
  return LBM_OK;
}

int lbm_batch_set_graph(LbmBatch* b, int32_t enable) {
  if (!b) return lbm_err::set(LBM_ERR_ARG, "batch_set_graph: NULL batch");
  b->use_graph = enable != 0;
  if (!b->use_graph) drop_graph(b);
  return LBM_OK;
}

int lbm_batch_run(LbmBatch* b, int32_t nsteps, void* stream) {
  if (!b) return lbm_err::set(LBM_ERR_ARG, "batch_run: NULL batch");
  if (nsteps < 0) return lbm_err::set(LBM_ERR_ARG, "batch_run: nsteps %d", nsteps);
  if (nsteps == 0) return LBM_OK;
  int rc = ensure_stream(b);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  rc = lbm_err::cuda(cudaEventRecord(b->fork, s), "batch_run: fork");
  if (!rc) rc = lbm_err::cuda(cudaStreamWaitEvent(b->stream, b->fork, 0), "batch_run: fork");
  if (rc) return rc;
  if (b->dirty) rc = rebuild(b);
  if (!rc) rc = run_on_stream(b, nsteps);
  // join even after a failure, so the caller's stream never runs ahead
  int rj = lbm_err::cuda(cudaEventRecord(b->join, b->stream), "batch_run: join");
  if (!rj) rj = lbm_err::cuda(cudaStreamWaitEvent(s, b->join, 0), "batch_run: join");
  return rc ? rc : rj;
}

int lbm_batch_info(const LbmBatch* b, int32_t* members, int64_t* tiles, int32_t* groups) {
  if (!b) return lbm_err::set(LBM_ERR_ARG, "batch_info: NULL batch");
  int n = 0;
  for (const BatchMember& m : b->slots) n += m.plan ? 1 : 0;
  if (members) *members = n;
  if (tiles) *tiles = b->dirty ? -1 : b->ntiles;
  if (groups) *groups = b->dirty ? -1 : (int32_t)(b->groups.size() + b->solos.size());
  return LBM_OK;
}

int lbm_batch_destroy(LbmBatch* b) {
  if (!b) return LBM_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  for (LbmBatch::Tables& t : b->tab) {
    if (t.lats) cudaFree(t.lats);
    if (t.tiles) cudaFree(t.tiles);
    if (t.mons) cudaFree(t.mons);
  }
  for (int w = 0; w < LbmBatch::NWORK; ++w) {
    if (b->work[w]) cudaStreamDestroy(b->work[w]);
    if (b->step_join[w]) cudaEventDestroy(b->step_join[w]);
  }
  if (b->step_fork) cudaEventDestroy(b->step_fork);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return LBM_OK;
}

}  // extern "C"
