// engine.cu — the out-of-memory engine behind og_engine_* / og_bfs / og_sssp /
// og_cc / og_pr (onegraph.h).
//
// One engine = one graph on one GB300, planned against a device budget:
//  * static region: vertices [0, Vs) whose whole adjacency lies in the edge
//    prefix [0, off[Vs]); that prefix is copied to HBM once
//    (GraphMeta.h:234-291 initGraphDevice, 300-360 getMaxPartitionSize);
//  * dynamic region: vertices [Vs, V); their edges stay in page-locked host
//    memory and every round the active ones are gathered by a kernel over the
//    host link into one of two device staging buffers (side stream), while the
//    previous buffer is relaxed and the static region is relaxed on the main
//    stream (CalculateOpt.h:75-188, GraphMeta.h:471-557).
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <chrono>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "batch_persist.cuh"
#include "bfs_loop.cuh"
#include "kernels.cuh"
#include "og_internal.hpp"
#include "sssp_batch.cuh"

using namespace og;

#define CK(x)                                                                          \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess)                                                             \
      return og::fail(OG_E_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, \
                      __LINE__);                                                       \
  } while (0)

#define RC(x)                    \
  do {                           \
    int r_ = (x);                \
    if (r_ != OG_OK) return r_;  \
  } while (0)

// Fragment slots of an OG_CFG_REPLACE engine (SrcF, kernels.cuh): the slot
// memory, the device slot table and its host mirror, and the policy state.
struct FragState {
  uint32_t fs = 0;          // log2 words per fragment
  uint64_t nfrag = 0;       // fragments of the packed record stream
  uint32_t nslots = 0;
  uint64_t bytes = 0;       // device bytes for slots, tables and update lists
  uint32_t *slots_d = nullptr;
  int32_t *slot_of_d = nullptr;
  uint32_t *visits_d = nullptr;  // records listed per fragment since the last step
  unsigned long long *miss_d = nullptr;  // of those, records of slotted fragments read from the host
  unsigned long long *miss_h = nullptr;  // page-locked
  uint2 *pairs_d = nullptr;      // one update: (fragment, slot)
  uint32_t *evict_d = nullptr;   // one update: the fragment each slot held before
  uint32_t max_pairs = 0;
  uint32_t *visits_h = nullptr;  // page-locked
  uint2 *pairs_h = nullptr;      // page-locked
  uint32_t *evict_h = nullptr;   // page-locked
  cudaEvent_t ev_ready = nullptr;  // slot updates done (the dynamic stream waits on it)
  std::vector<int32_t> slot_of;  // host mirror of slot_of_d
  std::vector<uint32_t> owner;   // fragment held by each slot (UINT32_MAX: none)
  std::vector<float> score;      // records listed per fragment, halved every step
  std::vector<void *> dallocs, hallocs;
  uint64_t dalloc_bytes = 0;
  bool broken = false;     // a layout failed: queries through the slots are refused
  uint64_t since = 0;      // dynamic records listed since the last policy step
  uint64_t step_min = 0;   // records between policy steps (as many as the slots hold)
  og_fragment_stats st{};
};

struct og_engine {
  og_graph *g = nullptr;
  og_config cfg{};
  og_plan plan{};
  int dev = 0;
  int sms = 0;
  bool pr_enabled = false;
  bool registered = false;
  uint32_t V = 0, Vs = 0;
  uint64_t nwords = 0;

  cudaStream_t s_main = nullptr, s_dyn = nullptr, s_gat = nullptr;
  cudaEvent_t ev_round = nullptr, ev_cs = nullptr, ev_cd = nullptr, ev_dyn_done = nullptr;
  cudaEvent_t ev_gat[2] = {nullptr, nullptr}, ev_rel[2] = {nullptr, nullptr};
  cudaEvent_t t_s0 = nullptr, t_s1 = nullptr, t_d0 = nullptr;
  std::vector<cudaEvent_t> t_gat;  // start/end pairs around each gather launch

  uint64_t *off_d = nullptr;
  // edges as bit-packed records (host copy and static region) and as
  // unpacked u32 columns + weights of wbytes (1, 2, 4) in the staging buffers
  uint32_t *spk_d = nullptr;                 // static region records (HBM)
  uint32_t bpe = 0, bc = 0, wmin = 0;        // record layout
  uint32_t *stage_col[2] = {nullptr, nullptr};  // staging buffers (columns)
  void *stage_w[2] = {nullptr, nullptr};        // staging buffers (weights)
  const uint32_t *hpk_d = nullptr;           // page-locked host records, device view
  uint32_t wbytes = 0;
  uint32_t *value_d = nullptr;
  uint32_t *bm[3] = {nullptr, nullptr, nullptr};
  uint32_t *list_d[2] = {nullptr, nullptr};
  uint64_t *pref_d[2] = {nullptr, nullptr};
  uint32_t *tile_d[2] = {nullptr, nullptr};
  uint64_t list_cap[2] = {0, 0}, tile_cap[2] = {0, 0};
  Lookback lb[2]{};
  uint32_t lb_tiles = 0;
  // counts of the two regions followed by their two far keys (u64), one D2H
  Counts *counts_d = nullptr, *counts_h = nullptr;
  uint32_t epoch = 0;  // look-back epoch of the last compaction launch
  uint32_t *err_d = nullptr, *err_h = nullptr;
  uint32_t *active_d = nullptr;

  // PageRank state
  float *contrib_d = nullptr, *sum_d = nullptr, *cont_d = nullptr, *carry_d = nullptr;
  uint32_t *outdeg_d = nullptr, *carry_idx_d = nullptr;
  double *part_d = nullptr, *l1_d = nullptr, *l1_h = nullptr;
  uint32_t part_n = 0;
  uint64_t pr_tiles = 0;

  // batched BFS state
  bool batch_enabled = false;
  unsigned long long *bmask[3] = {nullptr, nullptr, nullptr};  // visited, cur, next
  unsigned long long *hist_d = nullptr, *hist_h = nullptr;
  uint32_t *srcs_d = nullptr, *srcs_h = nullptr;
  // persistent kernel state
  uint32_t *ptile_d = nullptr;
  uint64_t ptile_cap = 0;
  uint32_t *cta_n = nullptr;
  unsigned long long *cta_e = nullptr;
  unsigned long long *smf_d = nullptr;  // batched BFS: per-source frontier degree sums
  uint32_t *bar_d = nullptr;   // [0..1] barrier, [2] error, [3] levels, [4..11] 4 x u64 stats
  uint32_t *pmisc_h = nullptr;  // host copy of bar_d
  int tuned = -1;               // index into kPersistConfigs chosen by the autotuner
  cudaGraphExec_t graph = nullptr;
  // device-driven BFS level loop: state, its host mirror, one graph per
  // frontier parity (captured for the direction mode `bfs_exec_dopt`)
  BfsLoop *loop_d = nullptr, *loop_h = nullptr;
  cudaGraphExec_t bfs_exec[2] = {nullptr, nullptr};
  int bfs_exec_dopt = -1;
  uint32_t dev_epoch = 1u << 29;  // epochs of device-driven compactions: [2^29, 2^30)
  uint32_t bfs_levels_hint = 4;   // levels of the last BFS (launched before the first check)
  uint32_t level_loop = 0;        // OG_LOOP_AUTO / OG_LOOP_HOST
  uint32_t relax_timer = 0;       // OG_PARAM_RELAX_TIMER
  // device-driven SSSP / CC rounds: state, host mirror, round graphs captured
  // for (algorithm, split) = min_exec_key
  MinLoop *mloop_d = nullptr, *mloop_h = nullptr;
  cudaGraphExec_t min_exec[2] = {nullptr, nullptr};
  int min_exec_key = -1;
  uint32_t min_rounds_hint[2] = {16, 4};  // SSSP, CC
  uint32_t graph_n = 0;
  int graph_cfg = -1;
  int graph_dopt = -1;
  bool graph_broken = false;

  // batched BFS depth matrix (n x V u32, outside the budget), kept between
  // calls that ask for depths; its byte form for og_bfs_batch_u8
  uint32_t *depth_d = nullptr;
  uint64_t depth_cap = 0;  // entries
  uint8_t *depth8_d = nullptr;
  uint64_t depth8_cap = 0;

  // multi-source SSSP (og_sssp_batch, sssp_batch.cuh): sb_k sources per pass
  // in rows of sb_ks slots; its rows, pending masks and near masks share
  // `arena` with the batched BFS masks
  uint32_t sb_k = 0, sb_ks = 0;
  unsigned char *arena = nullptr;
  uint32_t *sb_dist = nullptr, *sb_pend = nullptr, *sb_lmask = nullptr;
  uint32_t *sb_masks = nullptr;  // device: [0] pending slots seen, [1] waiting slots, [2..3] spare
  uint32_t *sb_io_h = nullptr;   // page-locked: sources [0, 32), slots [32, 64), masks [64, 68)
  uint32_t *sb_io_d = nullptr;
  unsigned long long *sb_ck_d = nullptr, *sb_ck_h = nullptr;  // per-slot checks (2 x 32)
  uint32_t sb_thr = 0, sb_far_min = 0;
  uint32_t sb_delta = 0;  // OG_PARAM_SSSP_BATCH_DELTA: near/far width of the batch (0: every round)
  bool sb_advance = false;
  uint32_t sb_dirty = 0;  // slots whose distances are not all unreached
  bool sb_session = false;  // a session is open: no other query ran since og_sssp_batch_begin

  // batched BFS level by level (og_bfs_batch_begin ... _fetch): up to 64
  // slots over the batch masks; a slot's depths are offset by the level it
  // joined at, and a finished slot's visited bits are cleared when it is
  // joined again
  uint32_t *bb_io_d = nullptr, *bb_io_h = nullptr;  // sources [0,64), slots [64,128), depth offsets [128,192)
  bool bb_session = false;  // no other query ran since og_bfs_batch_begin
  bool bb_record = false;   // depths recorded in depth_d (64 x V)
  uint32_t bb_level = 1;    // depth of the frontier the next step expands, for a source at depth 1 at begin
  uint32_t bb_par = 0;      // frontier parity: cur = bmask[1 + par], cur_any = bm[par]
  uint64_t bb_used = 0;     // slots joined and not finished
  uint64_t bb_dirty = 0;    // finished slots whose visited bits are still set
  uint32_t bb_off[64] = {};
  uint64_t bb_reached[64] = {}, bb_dsum[64] = {};

  FragState *frag = nullptr;  // OG_CFG_REPLACE: fragment slots of the dynamic region

  og_engine *parent = nullptr;  // set on clones: resident state belongs to the parent
  int clones = 0;               // live clones of this engine
  uint64_t resident_bytes = 0;  // device bytes of the shared resident state
  unsigned long long *sum64_d = nullptr;  // result checksum scratch

  uint32_t sssp_delta = 0;  // near/far split width (0: plain frontier relaxation)
  uint32_t cc_method = 0;   // OG_CC_AUTO / OG_CC_LABEL_PROPAGATION / OG_CC_UNION_FIND
  uint32_t bfs_direction = 0;  // OG_BFS_AUTO / OG_BFS_TOP_DOWN

  int last_algo = -1;
  uint64_t launches = 0;  // kernels launched since the query began
  std::vector<void *> dallocs;
  uint64_t dbytes = 0;
};

namespace {

constexpr int kGatherMult = 2;  // gather tiles of 4096 positions
constexpr uint32_t kMaxPersistCtas = 2048;

template <class T>
int dalloc(og_engine *e, T **p, uint64_t count) {
  const uint64_t bytes = std::max<uint64_t>(count * sizeof(T), 256);
  void *q = nullptr;
  cudaError_t err = cudaMalloc(&q, bytes);
  if (err != cudaSuccess)
    return fail(OG_E_CUDA, "cudaMalloc(%llu B) failed: %s (engine holds %llu B)",
                (unsigned long long)bytes, cudaGetErrorString(err), (unsigned long long)e->dbytes);
  e->dallocs.push_back(q);
  e->dbytes += bytes;
  *p = (T *)q;
  return OG_OK;
}

int grid_for(uint64_t n, int sms) {
  const uint64_t g = (n + kThreads - 1) / kThreads;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)sms * 8));
}

// ------------------------------------------------------- fragment slots
//
// Static-region replacement (OG_CFG_REPLACE).  The reference declares its
// pieces and never defines them: recordFragmentVisit (per-fragment visit
// records), setFragmentData / setStaticFragmentData (which static fragments
// may be swapped) and bfs_kernelStaticSwap (BFS/oneGraph_BFS/gpu_kernels.h:
// 46-66,153-176, FragmentData in globals.h:22-33).  Here the swappable part
// is a set of slots carved from the static region's bytes; the relax counts
// the records it lists per fragment (SrcF::note) and frag_step, after every
// round, moves the most-read fragments without a slot into the slots whose
// fragments were read least.

void frag_release(og_engine *e) {
  FragState &F = *e->frag;
  for (void *p : F.dallocs) cudaFree(p);
  for (void *p : F.hallocs) cudaFreeHost(p);
  F.dallocs.clear();
  F.hallocs.clear();
  e->dbytes -= F.dalloc_bytes;
  if (!e->parent) e->resident_bytes -= std::min(e->resident_bytes, F.dalloc_bytes);
  F.dalloc_bytes = 0;
  F.slots_d = nullptr;
  F.slot_of_d = nullptr;
  F.visits_d = nullptr;
  F.miss_d = nullptr;
  F.miss_h = nullptr;
  F.pairs_d = nullptr;
  F.evict_d = nullptr;
  F.visits_h = nullptr;
  F.pairs_h = nullptr;
  F.evict_h = nullptr;
}

template <class T>
int frag_dalloc(og_engine *e, T **p, uint64_t count) {
  const uint64_t bytes = std::max<uint64_t>(count * sizeof(T), 256);
  void *q = nullptr;
  CK(cudaMalloc(&q, bytes));
  e->frag->dallocs.push_back(q);
  e->frag->dalloc_bytes += bytes;
  e->dbytes += bytes;
  *p = (T *)q;
  return OG_OK;
}

template <class T>
int frag_halloc(og_engine *e, T **p, uint64_t count) {
  void *q = nullptr;
  CK(cudaHostAlloc(&q, std::max<uint64_t>(count * sizeof(T), 64), cudaHostAllocDefault));
  e->frag->hallocs.push_back(q);
  *p = (T *)q;
  return OG_OK;
}

// Default fragment size: the power of two nearest packed words / 4096,
// clamped to [2^8, 2^14] words.
uint32_t frag_default_shift(uint64_t packed_words) {
  const double x = std::log2(std::max<double>(1.0, (double)packed_words / 4096.0));
  return (uint32_t)std::min(14.0, std::max(8.0, std::floor(x + 0.5)));
}

// Lays out slots of 2^fs + kFragPad words, the slot table, the visit counts
// and the update lists inside F.bytes of device memory.
// Device bytes of the tables and update lists for fragments of 2^fs words,
// and the most pairs one step moves (a quarter of the slots, at most 4096).
uint64_t frag_fixed_bytes(const FragState &F, uint64_t nfrag, uint32_t fs, uint32_t *max_pairs) {
  const uint64_t slot_words = (1ull << fs) + kFragPad;
  *max_pairs = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(4096, F.bytes / (4 * slot_words) / 4));
  return nfrag * 8 + (uint64_t)*max_pairs * 12 + 5 * 256;
}

// 0 when slots of 2^fs words fit F.bytes (checked before anything is freed).
int frag_fits(const og_engine *e, uint32_t fs) {
  const FragState &F = *e->frag;
  const uint64_t nfrag = (e->g->packed_words + (1ull << fs) - 1) >> fs;
  uint32_t mp;
  const uint64_t slot_words = (1ull << fs) + kFragPad;
  if (F.bytes < frag_fixed_bytes(F, nfrag, fs, &mp) + 4 * slot_words)
    return fail(OG_E_BUDGET, "fragment slots: %llu B of static region cannot hold one %llu-word slot and the "
                "%llu-fragment tables", (unsigned long long)F.bytes, (unsigned long long)slot_words,
                (unsigned long long)nfrag);
  return OG_OK;
}

int frag_layout(og_engine *e, uint32_t fs) {
  FragState &F = *e->frag;
  RC(frag_fits(e, fs));
  frag_release(e);
  F.broken = true;  // until the layout below completes
  const og_graph *g = e->g;
  F.fs = fs;
  F.nfrag = (g->packed_words + (1ull << fs) - 1) >> fs;
  const uint64_t slot_words = (1ull << fs) + kFragPad;
  const uint64_t fixed = frag_fixed_bytes(F, F.nfrag, fs, &F.max_pairs);
  const uint64_t ns = std::min<uint64_t>((F.bytes - fixed) / (4 * slot_words), std::min<uint64_t>(F.nfrag, 0x7fffffffull));
  F.nslots = (uint32_t)ns;
  RC(frag_dalloc(e, &F.slots_d, ns * slot_words));
  RC(frag_dalloc(e, &F.slot_of_d, F.nfrag));
  RC(frag_dalloc(e, &F.visits_d, F.nfrag));
  RC(frag_dalloc(e, &F.miss_d, 1));
  RC(frag_dalloc(e, &F.pairs_d, F.max_pairs));
  RC(frag_dalloc(e, &F.evict_d, F.max_pairs));
  if (!e->parent) e->resident_bytes += F.dalloc_bytes;
  RC(frag_halloc(e, &F.visits_h, F.nfrag));
  RC(frag_halloc(e, &F.miss_h, 1));
  RC(frag_halloc(e, &F.pairs_h, F.max_pairs));
  RC(frag_halloc(e, &F.evict_h, F.max_pairs));
  F.slot_of.assign(F.nfrag, -1);
  F.owner.assign(F.nslots, 0xffffffffu);
  F.score.assign(F.nfrag, 0.0f);
  F.since = 0;
  F.step_min = (uint64_t)((double)F.nslots * (double)(1ull << fs) * 32.0 / e->bpe);
  F.st = og_fragment_stats{};
  F.st.fragments = F.nfrag;
  F.st.slots = F.nslots;
  F.st.fragment_words = 1u << fs;
  F.broken = false;
  return OG_OK;
}

// Copies n (fragment, slot) pairs from F.pairs_h / F.evict_h into the slots
// and the table on stream s.
int frag_apply(og_engine *e, uint32_t n, cudaStream_t s) {
  FragState &F = *e->frag;
  if (n == 0) return OG_OK;
  CK(cudaMemcpyAsync(F.pairs_d, F.pairs_h, 8ull * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(F.evict_d, F.evict_h, 4ull * n, cudaMemcpyHostToDevice, s));
  k_frag_fill<<<n, kThreads, 0, s>>>(e->hpk_d, e->g->packed_words, F.slots_d, F.pairs_d, n, F.fs);
  k_frag_table<<<(n + 255) / 256, 256, 0, s>>>(F.slot_of_d, F.pairs_d, F.evict_d, n);
  e->launches += 2;
  CK(cudaGetLastError());
  return OG_OK;
}

// Empties the slots, then fills them with the fragments that follow the
// static prefix (the records a larger static prefix would hold).
int frag_reset(og_engine *e) {
  FragState &F = *e->frag;
  cudaStream_t s = e->s_main;
  F.broken = true;  // until every fill below is queued
  CK(cudaMemsetAsync(F.slot_of_d, 0xff, 4 * F.nfrag, s));
  CK(cudaMemsetAsync(F.visits_d, 0, 4 * F.nfrag, s));
  CK(cudaMemsetAsync(F.miss_d, 0, 8, s));
  const uint64_t f0 = (e->plan.static_edges * e->bpe >> 5) >> F.fs;
  uint32_t filled = 0;
  while (filled < F.nslots && f0 + filled < F.nfrag) {
    uint32_t n = 0;
    for (; n < F.max_pairs && filled < F.nslots && f0 + filled < F.nfrag; n++, filled++) {
      const uint32_t f = (uint32_t)(f0 + filled);
      F.pairs_h[n] = make_uint2(f, filled);
      F.evict_h[n] = 0xffffffffu;
      F.slot_of[f] = (int32_t)filled;
      F.owner[filled] = f;
    }
    RC(frag_apply(e, n, s));
    CK(cudaStreamSynchronize(s));  // the page-locked lists are reused
  }
  if (!F.ev_ready) CK(cudaEventCreateWithFlags(&F.ev_ready, cudaEventDisableTiming));
  F.broken = false;
  return OG_OK;
}

// After a compaction (the previous round's relax has finished), once as many
// records as the slots hold have been listed since the last step, or when
// `force` (a compaction that lists nothing, e.g. the query's last): reads
// the visit counts, moves the records served from slots out of the
// host-link bytes, and replaces slots.  Ascetic's rule: fragments read in
// this round that have no slot take the slots of fragments that were read
// least; scores are records listed, halved every step; a fragment comes in
// only if its score is at least a quarter of its records and above twice the
// evicted one's; the copies of one step read at most a quarter of the
// round's host-link bytes.  The dynamic stream waits for the updates.
int frag_step(og_engine *e, og_stats &st, bool force) {
  FragState &F = *e->frag;
  if (!force && F.since < F.step_min) return OG_OK;  // counts keep adding up on the device
  F.since = 0;
  cudaStream_t s = e->s_main;
  CK(cudaMemcpyAsync(F.visits_h, F.visits_d, 4 * F.nfrag, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(F.miss_h, F.miss_d, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemsetAsync(F.visits_d, 0, 4 * F.nfrag, s));
  CK(cudaMemsetAsync(F.miss_d, 0, 8, s));
  CK(cudaStreamSynchronize(s));
  uint64_t in_slots = 0, in_host = 0;
  std::vector<uint32_t> cand;
  const float min_score = (float)((double)(1ull << F.fs) * 32.0 / e->bpe / 4.0);
  for (uint64_t f = 0; f < F.nfrag; f++) {
    const uint32_t v = F.visits_h[f];
    F.score[f] = 0.5f * F.score[f] + (float)v;
    if (!v) continue;
    if (F.slot_of[f] >= 0) {
      in_slots += v;
    } else {
      in_host += v;
      if (F.score[f] >= min_score) cand.push_back((uint32_t)f);
    }
  }
  // records of slotted fragments that a range over a fragment end read from the host
  const uint64_t miss = std::min<uint64_t>(*F.miss_h, in_slots);
  in_slots -= miss;
  in_host += miss;
  F.st.records_slots += in_slots;
  F.st.records_host += in_host;
  const uint64_t slot_link = (in_slots * e->bpe) / 8;
  st.link_bytes -= std::min(st.link_bytes, slot_link);
  const uint64_t frag_bytes = 4ull * ((1ull << F.fs) + kFragPad);
  const uint64_t cap = (in_host * e->bpe / 8) / 4 / frag_bytes;
  uint32_t n = (uint32_t)std::min<uint64_t>({cap, (uint64_t)F.max_pairs, (uint64_t)F.nslots, (uint64_t)cand.size()});
  if (n == 0) return OG_OK;
  auto hot = [&](uint32_t a, uint32_t b) { return F.score[a] > F.score[b] || (F.score[a] == F.score[b] && a < b); };
  std::partial_sort(cand.begin(), cand.begin() + n, cand.end(), hot);
  std::vector<uint32_t> vict(F.nslots);
  for (uint32_t i = 0; i < F.nslots; i++) vict[i] = i;
  auto vscore = [&](uint32_t sl) { return F.owner[sl] == 0xffffffffu ? -1.0f : F.score[F.owner[sl]]; };
  std::partial_sort(vict.begin(), vict.begin() + n, vict.end(), [&](uint32_t a, uint32_t b) {
    return vscore(a) < vscore(b) || (vscore(a) == vscore(b) && a < b);
  });
  uint32_t m = 0;
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t f = cand[i], sl = vict[i];
    if (F.score[f] <= 2.0f * vscore(sl) + 1.0f) break;
    const uint32_t old = F.owner[sl];
    F.pairs_h[m] = make_uint2(f, sl);
    F.evict_h[m] = old;
    if (old != 0xffffffffu) F.slot_of[old] = -1;
    F.slot_of[f] = (int32_t)sl;
    F.owner[sl] = f;
    m++;
  }
  if (m == 0) return OG_OK;
  RC(frag_apply(e, m, s));
  CK(cudaEventRecord(F.ev_ready, s));
  CK(cudaStreamWaitEvent(e->s_dyn, F.ev_ready, 0));
  F.st.swaps += m;
  F.st.swap_bytes += m * frag_bytes;
  st.link_bytes += m * frag_bytes;
  return OG_OK;
}

void destroy(og_engine *e) {
  if (!e) return;
  cudaSetDevice(e->dev);
  if (e->s_main) cudaStreamSynchronize(e->s_main);
  if (e->s_dyn) cudaStreamSynchronize(e->s_dyn);
  if (e->s_gat) cudaStreamSynchronize(e->s_gat);
  if (e->frag) {
    frag_release(e);
    if (e->frag->ev_ready) cudaEventDestroy(e->frag->ev_ready);
    delete e->frag;
    e->frag = nullptr;
  }
  for (void *p : e->dallocs) cudaFree(p);
  if (e->depth_d) cudaFree(e->depth_d);
  if (e->depth8_d) cudaFree(e->depth8_d);
  if (e->counts_h) cudaFreeHost(e->counts_h);
  if (e->hist_h) cudaFreeHost(e->hist_h);
  if (e->srcs_h) cudaFreeHost(e->srcs_h);
  if (e->sb_io_h) cudaFreeHost(e->sb_io_h);
  if (e->bb_io_h) cudaFreeHost(e->bb_io_h);
  if (e->sb_ck_h) cudaFreeHost(e->sb_ck_h);
  if (e->pmisc_h) cudaFreeHost(e->pmisc_h);
  if (e->graph) cudaGraphExecDestroy(e->graph);
  for (int p = 0; p < 2; p++)
    if (e->bfs_exec[p]) cudaGraphExecDestroy(e->bfs_exec[p]);
  if (e->loop_h) cudaFreeHost(e->loop_h);
  for (int p = 0; p < 2; p++)
    if (e->min_exec[p]) cudaGraphExecDestroy(e->min_exec[p]);
  if (e->mloop_h) cudaFreeHost(e->mloop_h);
  if (e->err_h) cudaFreeHost(e->err_h);
  if (e->l1_h) cudaFreeHost(e->l1_h);
  cudaEvent_t evs[] = {e->ev_round, e->ev_cs, e->ev_cd, e->ev_dyn_done, e->ev_gat[0], e->ev_gat[1],
                       e->ev_rel[0], e->ev_rel[1], e->t_s0, e->t_s1, e->t_d0};
  for (auto ev : evs)
    if (ev) cudaEventDestroy(ev);
  for (auto ev : e->t_gat) cudaEventDestroy(ev);
  if (e->s_main) cudaStreamDestroy(e->s_main);
  if (e->s_dyn) cudaStreamDestroy(e->s_dyn);
  if (e->s_gat) cudaStreamDestroy(e->s_gat);
  if (e->registered && e->g) {
    if (--e->g->registered == 0) {
      cudaHostUnregister(e->g->packed);
    }
  }
  if (e->parent) e->parent->clones--;
  cudaGetLastError();  // a failure while tearing down is not the next call's error
  delete e;
}

// Per-query state: streams, events, frontier/list arrays, staging buffers and
// the PageRank / batched-BFS working arrays.  A parent engine and each of its
// clones own one set; the resident graph (offsets, static edges, out-degrees,
// page-locked host CSR) is shared.
int create_query_state(og_engine *e) {
  const og_plan &P = e->plan;
  const uint64_t V = e->V;
  // A fully resident graph's queries are short and HBM-bound; an
  // out-of-memory graph's kernels wait on the host link with many CTAs
  // resident.  When both share the GPU (several engines, the server), the
  // resident graph's streams get the highest priority so that the block
  // scheduler places its CTAs first as SMs free up, instead of behind a
  // link-bound grid of millions of CTAs.
  int prio_lo = 0, prio_hi = 0;
  CK(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
  const int prio = P.dynamic_edges == 0 ? prio_hi : prio_lo;
  CK(cudaStreamCreateWithPriority(&e->s_main, cudaStreamNonBlocking, prio));
  CK(cudaStreamCreateWithPriority(&e->s_dyn, cudaStreamNonBlocking, prio));
  CK(cudaStreamCreateWithPriority(&e->s_gat, cudaStreamNonBlocking, prio));
  cudaEvent_t *evs[] = {&e->ev_round, &e->ev_cs, &e->ev_cd, &e->ev_dyn_done, &e->ev_gat[0],
                        &e->ev_gat[1], &e->ev_rel[0], &e->ev_rel[1], &e->t_s0, &e->t_s1, &e->t_d0};
  for (auto ev : evs) CK(cudaEventCreate(ev));
  RC(dalloc(e, &e->value_d, V + 1));
  for (int i = 0; i < 3; i++) RC(dalloc(e, &e->bm[i], e->nwords));
  e->list_cap[0] = std::max<uint64_t>(e->Vs, 1);
  e->list_cap[1] = std::max<uint64_t>(V - e->Vs, 1);
  e->tile_cap[0] = P.static_edges / kTile + 2;
  e->tile_cap[1] = P.dynamic_edges / kTile + 2;
  // one allocation per array, the dynamic region's part after the static one,
  // so the batched kernel can also use them as a single list over [0, V)
  RC(dalloc(e, &e->list_d[0], e->list_cap[0] + e->list_cap[1]));
  RC(dalloc(e, &e->pref_d[0], e->list_cap[0] + e->list_cap[1] + 2));
  RC(dalloc(e, &e->tile_d[0], e->tile_cap[0] + e->tile_cap[1]));
  e->list_d[1] = e->list_d[0] + e->list_cap[0];
  e->pref_d[1] = e->pref_d[0] + e->list_cap[0] + 1;
  e->tile_d[1] = e->tile_d[0] + e->tile_cap[0];
  e->lb_tiles = (uint32_t)((e->nwords + kWordsPerCompactTile - 1) / kWordsPerCompactTile + 1);
  for (int r = 0; r < 2; r++) {
    RC(dalloc(e, &e->lb[r].status, e->lb_tiles + 1));
    e->lb[r].ticket = e->lb[r].status + e->lb_tiles;
    RC(dalloc(e, &e->lb[r].agg_n, e->lb_tiles));
    RC(dalloc(e, &e->lb[r].agg_e, e->lb_tiles));
    RC(dalloc(e, &e->lb[r].inc_n, e->lb_tiles));
    RC(dalloc(e, &e->lb[r].inc_e, e->lb_tiles));
  }
  for (int r = 0; r < 2; r++)  // epochs start at 1: zeroed status words are "empty"
    CK(cudaMemsetAsync(e->lb[r].status, 0, sizeof(uint32_t) * (e->lb_tiles + 1), e->s_main));
  RC(dalloc(e, &e->counts_d, 3));  // Counts[2] + u64 far key[2]
  CK(cudaMemsetAsync(e->counts_d, 0, 3 * sizeof(Counts), e->s_main));
  RC(dalloc(e, &e->err_d, 4));
  e->active_d = e->err_d + 1;
  RC(dalloc(e, &e->sum64_d, 3ull * e->sms * 8 + 4));
  CK(cudaMallocHost(&e->counts_h, 3 * sizeof(Counts)));
  RC(dalloc(e, (char **)&e->loop_d, sizeof(BfsLoop)));
  CK(cudaMallocHost(&e->loop_h, sizeof(BfsLoop)));
  RC(dalloc(e, (char **)&e->mloop_d, sizeof(MinLoop)));
  CK(cudaMallocHost(&e->mloop_h, sizeof(MinLoop)));
  CK(cudaMallocHost(&e->err_h, 4 * sizeof(uint32_t)));
  CK(cudaMallocHost(&e->l1_h, sizeof(double)));
  if (P.chunk_edges && !(e->cfg.flags & OG_CFG_DIRECT)) {
    for (int b = 0; b < 2; b++) {
      RC(dalloc(e, &e->stage_col[b], P.chunk_edges));
      if (e->wbytes) RC(dalloc(e, (char **)&e->stage_w[b], P.chunk_edges * e->wbytes));
    }
  }
  // PageRank's contributions and sums live in the batch arena when the
  // engine has one (a context runs one computation at a time)
  const bool arena = e->batch_enabled || e->sb_k;
  if (e->pr_enabled) {
    if (!arena) {
      RC(dalloc(e, &e->contrib_d, V + 1));
      RC(dalloc(e, &e->sum_d, V + 1));
    }
    e->pr_tiles = e->tile_cap[0] + e->tile_cap[1];
    RC(dalloc(e, &e->cont_d, e->pr_tiles));
    RC(dalloc(e, &e->carry_d, e->pr_tiles));
    RC(dalloc(e, &e->carry_idx_d, e->pr_tiles));
    e->part_n = (uint32_t)e->sms * 8;
    RC(dalloc(e, &e->part_d, e->part_n));
    RC(dalloc(e, &e->l1_d, 1));
  }
  if (arena) {
    // one arena for the batched BFS masks (24 B per vertex), the
    // multi-source SSSP rows (4 sb_ks + 8 B per vertex) and PageRank's
    // contributions and sums (8 B per vertex): a context runs one at a time
    uint64_t per = std::max<uint64_t>(e->batch_enabled ? 24 : 0, e->sb_k ? 4ull * e->sb_ks + 8 : 0);
    if (e->pr_enabled) per = std::max<uint64_t>(per, 8);
    RC(dalloc(e, &e->arena, per * (V + 1)));
    if (e->pr_enabled) {
      e->contrib_d = (float *)e->arena;
      e->sum_d = e->contrib_d + (V + 1);
    }
    if (e->batch_enabled)
      for (int i = 0; i < 3; i++) e->bmask[i] = (unsigned long long *)e->arena + (uint64_t)i * (V + 1);
    if (e->sb_k) {
      e->sb_dist = (uint32_t *)e->arena;
      e->sb_pend = e->sb_dist + (V + 1) * e->sb_ks;
      e->sb_lmask = e->sb_pend + (V + 1);  // list_cap[0] + list_cap[1] <= V + 1 entries
      RC(dalloc(e, &e->sb_masks, 4));
      RC(dalloc(e, &e->sb_io_d, 128));
      RC(dalloc(e, &e->sb_ck_d, 2 * kSbMaxSources));
      CK(cudaMallocHost(&e->sb_io_h, 128 * sizeof(uint32_t)));
      CK(cudaMallocHost(&e->sb_ck_h, 2 * kSbMaxSources * sizeof(unsigned long long)));
    }
  }
  if (e->batch_enabled) {
    RC(dalloc(e, &e->hist_d, (uint64_t)kMaxBatchLevels * 64));
    RC(dalloc(e, &e->srcs_d, 64));
    RC(dalloc(e, &e->bb_io_d, 192));
    CK(cudaMallocHost(&e->bb_io_h, 192 * sizeof(uint32_t)));
    e->ptile_cap = e->g->E / 1024 + 8;
    RC(dalloc(e, &e->ptile_d, e->ptile_cap));
    RC(dalloc(e, &e->cta_n, kMaxPersistCtas));
    RC(dalloc(e, &e->cta_e, kMaxPersistCtas));
    RC(dalloc(e, &e->smf_d, 2 * 64));
    RC(dalloc(e, &e->bar_d, 16));  // barrier (2), error, levels, stats (6 u64)
    CK(cudaMallocHost(&e->hist_h, (size_t)kMaxBatchLevels * 64 * sizeof(unsigned long long)));
    CK(cudaMallocHost(&e->srcs_h, 64 * sizeof(uint32_t)));
    CK(cudaMallocHost(&e->pmisc_h, 16 * sizeof(uint32_t)));
  }
  CK(cudaMemsetAsync(e->err_d, 0, 16, e->s_main));
  CK(cudaStreamSynchronize(e->s_main));
  return OG_OK;
}

int create(og_graph *g, const og_config *cfg, og_engine *e) {
  e->g = g;
  e->cfg = *cfg;
  e->dev = cfg->device;
  e->V = g->V;
  e->pr_enabled = g->kind == OG_GRAPH_PR || (cfg->flags & OG_CFG_PR);
  e->batch_enabled = (cfg->flags & OG_CFG_BATCH) != 0;
  e->sb_k = sb_sources(cfg->flags);
  if (e->sb_k > kSbMaxSources) return fail(OG_E_ARG, "OG_CFG_SSSP_BATCH(%u): at most %u sources", e->sb_k, kSbMaxSources);
  if (e->sb_k && g->kind != OG_GRAPH_WEIGHTED) return fail(OG_E_UNSUPPORTED, "multi-source SSSP needs a weighted graph");
  e->sb_ks = e->sb_k ? sb_row_slots(e->sb_k) : 0;
  CK(cudaSetDevice(e->dev));
  CK(cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, e->dev));
  RC(graph_prepare(g));
  // default near/far width: a sixteenth of the weight range's midpoint sum
  // (4 for weights in [1, 64]), at least 1
  e->sssp_delta = g->kind == OG_GRAPH_WEIGHTED ? std::max<uint32_t>(1, (uint32_t)(((uint64_t)g->wmin + g->wmax) / 16)) : 0;
  e->wbytes = g->wbytes;
  e->bpe = g->bpe;
  e->bc = g->bc;
  e->wmin = g->wmin;
  RC(plan_compute(g->V, g->E, g->off, g->kind, cfg->budget_bytes, cfg->advisek, cfg->flags, &e->plan,
                  g->bpe, 4 + g->wbytes));
  if (cfg->flags & OG_CFG_REPLACE) {
    // half of the static prefix's bytes become fragment slots (the same split
    // og_graph_plan reports)
    uint64_t slot_bytes = 0;
    RC(plan_replace_split(g, cfg->flags, &e->plan, &slot_bytes));
    e->frag = new FragState;
    e->frag->bytes = slot_bytes;
  }
  const og_plan &P = e->plan;
  size_t free_b = 0, total_b = 0;
  CK(cudaMemGetInfo(&free_b, &total_b));
  if (P.budget_bytes > free_b)
    return fail(OG_E_BUDGET, "budget %llu B exceeds free device memory %llu B",
                (unsigned long long)P.budget_bytes, (unsigned long long)free_b);
  e->Vs = P.static_vertices;
  e->nwords = ((uint64_t)g->V + 31) / 32 + 2 * kWordsPerCompactTile;

  // kernels with more than 48 KB of shared memory opt in once per process
  const int gsm = (int)gather_smem_bytes<kGatherMult>();
  CK(cudaFuncSetAttribute(k_gather<SrcP<false>, DstU, kGatherMult>,
                          cudaFuncAttributeMaxDynamicSharedMemorySize, gsm));
  CK(cudaFuncSetAttribute(k_gather<SrcP<true>, DstW<uint8_t>, kGatherMult>,
                          cudaFuncAttributeMaxDynamicSharedMemorySize, gsm));
  CK(cudaFuncSetAttribute(k_gather<SrcP<true>, DstW<uint16_t>, kGatherMult>,
                          cudaFuncAttributeMaxDynamicSharedMemorySize, gsm));
  CK(cudaFuncSetAttribute(k_gather<SrcP<true>, DstW<uint32_t>, kGatherMult>,
                          cudaFuncAttributeMaxDynamicSharedMemorySize, gsm));
  // The SSSP relax reads each packed record as two overlapping words; the
  // second mostly hits L1, so it runs best with a large L1: 58 % of the
  // unified L1/shared storage as shared memory (3 CTAs of 38 KB per SM,
  // ~124 KB of L1).  Measured on R-MAT 27: 9.55 queries/s with the CUDA driver's
  // choice, 9.85 at 58 %, 6.77 at 86 %, 8.06 at 30 %.
  CK(cudaFuncSetAttribute(k_lbs_pair<SrcP<true>, SrcP<true>, MinOp<true>>,
                          cudaFuncAttributePreferredSharedMemoryCarveout, 58));
  CK(cudaFuncSetAttribute(k_lbs_pair_dev<SrcP<true>, SrcP<true>, MinOp<true>>,
                          cudaFuncAttributePreferredSharedMemoryCarveout, 58));
  if (cfg->flags & OG_CFG_REPLACE) {  // the same relax reading fragment slots
    CK(cudaFuncSetAttribute(k_lbs_pair<SrcP<true>, SrcF<true>, MinOp<true>>,
                            cudaFuncAttributePreferredSharedMemoryCarveout, 58));
    CK(cudaFuncSetAttribute(k_lbs<SrcF<true>, MinOp<true>>, cudaFuncAttributePreferredSharedMemoryCarveout, 58));
  }
  // Same for the PageRank pull (29 KB tiles: 4 CTAs per SM at 58 %).  R-MAT 26
  // directed: 58.5 iterations/s with the CUDA driver's choice, 69.6 at 58 %,
  // 68.4 at 44 %, 63.2 at 30 %, 34.0 at 86 %.
  CK(cudaFuncSetAttribute(k_pr_pull<SrcP<false>>, cudaFuncAttributePreferredSharedMemoryCarveout, 58));
  CK(cudaFuncSetAttribute(k_pr_pull_pair<SrcP<false>, SrcP<false>>,
                          cudaFuncAttributePreferredSharedMemoryCarveout, 58));

  // host CSR: page-lock so kernels can gather from it over the link
  if (P.dynamic_edges > 0) {
    if (cfg->flags & OG_CFG_NO_PIN) {
      int pageable = 0;
      CK(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, e->dev));
      if (!pageable) return fail(OG_E_UNSUPPORTED, "device cannot read pageable host memory");
      e->hpk_d = g->packed;
    } else {
      if (g->registered == 0) {
        int ro = 0;
        cudaDeviceGetAttribute(&ro, cudaDevAttrHostRegisterReadOnlySupported, e->dev);
        CK(cudaHostRegister(g->packed, g->packed_words * 4,
                            cudaHostRegisterMapped | (ro ? cudaHostRegisterReadOnly : 0)));
      }
      g->registered++;
      e->registered = true;
      void *dp = nullptr;
      CK(cudaHostGetDevicePointer(&dp, g->packed, 0));
      e->hpk_d = (const uint32_t *)dp;
    }
  }

  // resident graph state shared with clones
  const uint64_t V = g->V;
  RC(dalloc(e, &e->off_d, V + 1));
  if (P.static_edges) RC(dalloc(e, &e->spk_d, g->packed_words_for(P.static_edges)));
  if (e->pr_enabled) RC(dalloc(e, &e->outdeg_d, V + 1));
  e->resident_bytes = e->dbytes;
  if (e->frag) RC(frag_layout(e, frag_default_shift(g->packed_words)));
  RC(create_query_state(e));
  if (e->dbytes > P.budget_bytes)
    return fail(OG_E_BUDGET, "engine allocated %llu B, above the %llu B budget",
                (unsigned long long)e->dbytes, (unsigned long long)P.budget_bytes);

  // initGraphDevice: offsets, the static edge prefix, PageRank out-degrees
  CK(cudaMemcpyAsync(e->off_d, g->off, 8 * (V + 1), cudaMemcpyHostToDevice, e->s_main));
  if (P.static_edges)
    CK(cudaMemcpyAsync(e->spk_d, g->packed, 4 * g->packed_words_for(P.static_edges),
                       cudaMemcpyHostToDevice, e->s_main));
  if (e->pr_enabled) {
    if (g->kind == OG_GRAPH_PR) {
      CK(cudaMemcpyAsync(e->outdeg_d, g->outdeg, 4 * V, cudaMemcpyHostToDevice, e->s_main));
    } else {
      k_degree_from_offsets<<<grid_for(V, e->sms), kThreads, 0, e->s_main>>>(V, e->off_d, e->outdeg_d);
      e->launches++;
    }
  }
  if (e->frag) RC(frag_reset(e));
  CK(cudaStreamSynchronize(e->s_main));
  CK(cudaGetLastError());
  return OG_OK;
}

// A query context on the parent's resident graph (nothing resident is copied).
int clone(og_engine *parent, og_engine *e) {
  e->parent = parent;
  e->g = parent->g;
  e->cfg = parent->cfg;
  e->plan = parent->plan;
  e->dev = parent->dev;
  e->sms = parent->sms;
  e->pr_enabled = parent->pr_enabled;
  e->batch_enabled = parent->batch_enabled;
  e->sb_k = parent->sb_k;
  e->sb_ks = parent->sb_ks;
  e->sb_delta = parent->sb_delta;
  e->V = parent->V;
  e->Vs = parent->Vs;
  e->nwords = parent->nwords;
  e->off_d = parent->off_d;
  e->spk_d = parent->spk_d;
  e->hpk_d = parent->hpk_d;
  e->bpe = parent->bpe;
  e->bc = parent->bc;
  e->wmin = parent->wmin;
  e->wbytes = parent->wbytes;
  e->outdeg_d = parent->outdeg_d;
  e->tuned = parent->tuned;
  e->sssp_delta = parent->sssp_delta;
  e->cc_method = parent->cc_method;
  e->bfs_direction = parent->bfs_direction;
  e->level_loop = parent->level_loop;
  e->relax_timer = parent->relax_timer;
  CK(cudaSetDevice(e->dev));
  RC(create_query_state(e));
  parent->clones++;
  return OG_OK;
}

// ------------------------------------------------------------------ rounds

// Near/far split (SplitArgs::on): list only vertices with value < thr; the
// waiting ones go to far_bits (when not null) and their minimum to the
// region's Counts::far_min; listed ones are cleared from clear_bits.
struct SplitArgs {
  // device-driven loops: epoch read from device memory, launch gated by a flag
  const uint32_t *epoch_ptr = nullptr;
  const uint32_t *run_flag = nullptr;
  const uint32_t *thr_ptr = nullptr;
  bool on = false;
  uint32_t thr = 0;
  uint32_t *far_bits = nullptr;
  uint32_t *clear_bits = nullptr;
};

int launch_compact(og_engine *e, int r, const uint32_t *bits, uint32_t vb, uint32_t ve,
                   cudaStream_t s, const SplitArgs &sp = SplitArgs()) {
  if (ve <= vb) {  // empty region: no kernel writes its counts
    CK(cudaMemsetAsync(e->counts_d + r, 0, sizeof(Counts), s));
    return OG_OK;
  }
  CompactArgs a{};
  a.bits = bits;
  a.v_begin = vb;
  a.v_end = ve;
  a.w_begin = vb / 32;
  a.w_end = (uint32_t)(((uint64_t)ve + 31) / 32);
  a.ntiles = (a.w_end - a.w_begin + kWordsPerCompactTile - 1) / kWordsPerCompactTile;
  a.off = e->off_d;
  a.list = e->list_d[r];
  a.pref = e->pref_d[r];
  a.tile_first = e->tile_d[r];
  a.counts = e->counts_d + r;
  a.lb = e->lb[r];
  a.err = e->err_d;
  a.list_cap = e->list_cap[r];
  a.tile_cap = e->tile_cap[r];
  a.value = e->value_d;
  a.thr = sp.thr;
  a.split = sp.on ? 1u : 0u;
  a.far_bits = sp.far_bits;
  a.far_key = (unsigned long long *)(e->counts_d + 2) + r;
  a.clear_bits = sp.clear_bits;
  a.epoch = e->epoch;
  a.epoch_ptr = sp.epoch_ptr;
  a.run_flag = sp.run_flag;
  a.thr_ptr = sp.thr_ptr;
  if (a.ntiles + 1 > e->lb_tiles) return fail(OG_E_STATE, "compaction scratch too small");
  k_compact<<<a.ntiles, kThreads, 0, s>>>(a);
  e->launches++;
  return OG_OK;
}

LbsArgs lbs_args(og_engine *e, int r, uint64_t pos_begin, uint64_t pos_end, bool csr,
                 uint64_t edge_bound) {
  LbsArgs a;
  a.list = e->list_d[r];
  a.pref = e->pref_d[r];
  a.tile_first = e->tile_d[r];
  a.n = e->counts_h[r].n;
  a.total = e->counts_h[r].total;
  a.pos_begin = pos_begin;
  a.pos_end = pos_end;
  a.off = csr ? e->off_d : nullptr;
  a.stage_base = pos_begin;
  a.edge_bound = edge_bound;
  a.err = e->err_d;
  return a;
}

unsigned lbs_grid(uint64_t pb, uint64_t pe) { return (unsigned)((pe - pb + kTile - 1) / kTile); }

int check_device_error(og_engine *e) {
  const uint32_t err = *e->err_h;
  if (!err) return OG_OK;
  if (err & kErrLookback) return fail(OG_E_TIMEOUT, "frontier compaction look-back wait gave up");
  return fail(OG_E_DEVICE, "kernel reported an out-of-range index (flags 0x%x)", err);
}

// Edge views of an engine: EK<void> reads columns only (BFS, CC, PageRank,
// batched BFS), EK<W> columns and weights (SSSP, W = staging weight type).
// The static region and the host copy are packed records (PSrc); staging
// buffers hold unpacked edges (Src / Dst).
template <class W>
struct EK {
  static constexpr bool kFrag = false;
  using PSrc = SrcP<true>;
  using Src = SrcW<W>;
  using Dst = DstW<W>;
  static PSrc stat(const og_engine *e) { return PSrc{e->spk_d, e->bpe, e->bc, e->wmin}; }
  static PSrc host(const og_engine *e) { return PSrc{e->hpk_d, e->bpe, e->bc, e->wmin}; }
  static Src stage(const og_engine *e, int b) { return Src{e->stage_col[b], (const W *)e->stage_w[b]}; }
  static Dst stage_dst(const og_engine *e, int b) { return Dst{e->stage_col[b], (W *)e->stage_w[b]}; }
};
template <>
struct EK<void> {
  static constexpr bool kFrag = false;
  using PSrc = SrcP<false>;
  using Src = SrcU;
  using Dst = DstU;
  static PSrc stat(const og_engine *e) { return PSrc{e->spk_d, e->bpe, e->bc, e->wmin}; }
  static PSrc host(const og_engine *e) { return PSrc{e->hpk_d, e->bpe, e->bc, e->wmin}; }
  static Src stage(const og_engine *e, int b) { return Src{e->stage_col[b]}; }
  static Dst stage_dst(const og_engine *e, int b) { return Dst{e->stage_col[b]}; }
};
using EKU = EK<void>;
// An OG_CFG_REPLACE engine's views: the dynamic region is read through the
// fragment slots (direct mode only: there are no staging buffers).
template <class W>
struct EKF : EK<W> {
  static constexpr bool kFrag = true;
  using HSrc = SrcF<!std::is_void<W>::value>;
  static HSrc host(const og_engine *e) {
    HSrc h;
    h.words = e->hpk_d;
    h.bpe = e->bpe;
    h.bc = e->bc;
    h.wmin = e->wmin;
    h.slots = e->frag->slots_d;
    h.slot_of = e->frag->slot_of_d;
    h.visits = e->frag->visits_d;
    h.miss = e->frag->miss_d;
    h.fs = e->frag->fs;
    return h;
  }
};

// Relax op factory per algorithm; `level` is the BFS depth of the frontier.
struct RoundOps {
  int algo;
  uint32_t level;
};

template <class Src0, class Src1>
int launch_relax_pair(og_engine *e, const RoundOps &ro, const LbsArgs &a0, Src0 s0, const LbsArgs &a1,
                      Src1 s1, uint32_t *next, cudaStream_t s) {
  const uint64_t n0 = lbs_grid(a0.pos_begin, a0.pos_end), n1 = lbs_grid(a1.pos_begin, a1.pos_end);
  const uint64_t n = n0 + n1;
  if (n == 0) return OG_OK;
  if (n > 0x7fffffffull) return fail(OG_E_STATE, "relax grid of %llu tiles", (unsigned long long)n);
  if (ro.algo == OG_ALGO_BFS) {
    BfsOp op{e->bm[2], next, e->value_d, e->err_d, e->V, ro.level + 1};
    k_lbs_pair<Src0, Src1, BfsOp><<<(unsigned)n, kThreads, 0, s>>>(a0, s0, a1, s1, op, n0, n);
  } else if (ro.algo == OG_ALGO_SSSP) {
    MinOp<true> op{e->value_d, next, e->err_d, e->V};
    k_lbs_pair<Src0, Src1, MinOp<true>><<<(unsigned)n, kThreads, 0, s>>>(a0, s0, a1, s1, op, n0, n);
  } else {
    MinOp<false> op{e->value_d, next, e->err_d, e->V};
    k_lbs_pair<Src0, Src1, MinOp<false>><<<(unsigned)n, kThreads, 0, s>>>(a0, s0, a1, s1, op, n0, n);
  }
  e->launches++;
  return OG_OK;
}

template <class Src>
int launch_relax(og_engine *e, const RoundOps &ro, const LbsArgs &a, Src src, uint32_t *next,
                 cudaStream_t s) {
  const unsigned grid = lbs_grid(a.pos_begin, a.pos_end);
  if (grid == 0) return OG_OK;
  if (ro.algo == OG_ALGO_BFS) {
    BfsOp op{e->bm[2], next, e->value_d, e->err_d, e->V, ro.level + 1};
    k_lbs<Src, BfsOp><<<grid, kThreads, 0, s>>>(a, src, op);
  } else if (ro.algo == OG_ALGO_SSSP) {
    MinOp<true> op{e->value_d, next, e->err_d, e->V};
    k_lbs<Src, MinOp<true>><<<grid, kThreads, 0, s>>>(a, src, op);
  } else {
    MinOp<false> op{e->value_d, next, e->err_d, e->V};
    k_lbs<Src, MinOp<false>><<<grid, kThreads, 0, s>>>(a, src, op);
  }
  e->launches++;
  return OG_OK;
}

template <class K>
int launch_gather(og_engine *e, const LbsArgs &a, int buf, cudaStream_t s) {
  constexpr uint64_t T = (uint64_t)kGatherMult * kTile;
  const unsigned grid = (unsigned)((a.pos_end - a.pos_begin + T - 1) / T);
  if (grid == 0) return OG_OK;
  k_gather<typename K::PSrc, typename K::Dst, kGatherMult>
      <<<grid, kThreads, gather_smem_bytes<kGatherMult>(), s>>>(a, K::host(e), K::stage_dst(e, buf));
  e->launches++;
  return OG_OK;
}

struct Timing {
  bool pend_s = false, pend_d = false;
  uint32_t pend_g = 0;  // gather launches whose event pair is still to be read
};

// Event pair g of the gather timing list, created on first use.
int gather_events(og_engine *e, uint32_t g, cudaEvent_t *b, cudaEvent_t *en) {
  while (e->t_gat.size() < 2ull * (g + 1)) {
    cudaEvent_t ev;
    CK(cudaEventCreate(&ev));
    e->t_gat.push_back(ev);
  }
  *b = e->t_gat[2 * g];
  *en = e->t_gat[2 * g + 1];
  return OG_OK;
}

void collect_timing(og_engine *e, Timing &t, og_stats *st) {
  float ms;
  if (t.pend_s && cudaEventElapsedTime(&ms, e->t_s0, e->t_s1) == cudaSuccess) st->ms_static += ms;
  if (t.pend_d && cudaEventElapsedTime(&ms, e->t_d0, e->ev_dyn_done) == cudaSuccess)
    st->ms_dynamic += ms;
  for (uint32_t g = 0; g < t.pend_g; g++)
    if (cudaEventElapsedTime(&ms, e->t_gat[2 * g], e->t_gat[2 * g + 1]) == cudaSuccess)
      st->ms_gather += ms;
  t.pend_s = t.pend_d = false;
  t.pend_g = 0;
}

struct NoPair {};

// One round's region work given the compaction counts (already on the host).
// `static_fn(a)` / `dyn_fn(a, src, stream)` launch the per-region kernel;
// `pair_fn(a0, src0, a1, src1, stream)`, when given, launches both regions
// as one interleaved kernel (direct mode with both regions non-empty): the
// static tiles then overlap the link-bound dynamic ones instead of taking the
// SMs first.  Its time is counted as dynamic-region time.
template <class K, class StaticFn, class DynFn, class PairFn = NoPair>
int run_regions(og_engine *e, og_stats &st, Timing &tm, StaticFn static_fn, DynFn dyn_fn,
                PairFn pair_fn = PairFn()) {
  const Counts cs = e->counts_h[0], cd = e->counts_h[1];
  if constexpr (!std::is_same<PairFn, NoPair>::value) {
    if (cs.n && cd.n && (e->cfg.flags & OG_CFG_DIRECT)) {
      CK(cudaEventRecord(e->t_d0, e->s_main));
      RC(pair_fn(lbs_args(e, 0, 0, cs.total, true, e->plan.static_edges), K::stat(e),
                 lbs_args(e, 1, 0, cd.total, true, e->g->E), K::host(e), e->s_main));
      CK(cudaEventRecord(e->ev_dyn_done, e->s_main));
      tm.pend_d = true;
      st.chunks += 1;
      st.edges_static += cs.total;
      st.edges_dynamic += cd.total;
      st.link_bytes += (cd.total * e->bpe + 7) / 8;
      return OG_OK;
    }
  }
  if (cs.n) {
    CK(cudaEventRecord(e->t_s0, e->s_main));
    RC(static_fn(lbs_args(e, 0, 0, cs.total, true, e->plan.static_edges)));
    CK(cudaEventRecord(e->t_s1, e->s_main));
    tm.pend_s = true;
    st.edges_static += cs.total;
  }
  if (cd.n) {
    CK(cudaEventRecord(e->t_d0, e->s_dyn));
    if (K::kFrag || (e->cfg.flags & OG_CFG_DIRECT)) {
      RC(dyn_fn(lbs_args(e, 1, 0, cd.total, true, e->g->E), K::host(e), e->s_dyn));
      st.chunks += 1;
    } else if constexpr (!K::kFrag) {
      const uint64_t C = e->plan.chunk_edges;
      const uint64_t nch = (cd.total + C - 1) / C;
      for (uint64_t c = 0; c < nch; c++) {
        const int buf = (int)(c & 1);
        const uint64_t b = c * C, en = std::min(b + C, cd.total);
        CK(cudaStreamWaitEvent(e->s_gat, e->ev_cd, 0));
        if (c >= 2) CK(cudaStreamWaitEvent(e->s_gat, e->ev_rel[buf], 0));
        cudaEvent_t g0, g1;
        RC(gather_events(e, tm.pend_g, &g0, &g1));
        CK(cudaEventRecord(g0, e->s_gat));
        RC(launch_gather<K>(e, lbs_args(e, 1, b, en, true, e->g->E), buf, e->s_gat));
        CK(cudaEventRecord(g1, e->s_gat));
        tm.pend_g++;
        CK(cudaEventRecord(e->ev_gat[buf], e->s_gat));
        CK(cudaStreamWaitEvent(e->s_dyn, e->ev_gat[buf], 0));
        RC(dyn_fn(lbs_args(e, 1, b, en, false, C), K::stage(e, buf), e->s_dyn));
        CK(cudaEventRecord(e->ev_rel[buf], e->s_dyn));
      }
      st.chunks += (uint32_t)nch;
    }
    CK(cudaEventRecord(e->ev_dyn_done, e->s_dyn));
    CK(cudaStreamWaitEvent(e->s_main, e->ev_dyn_done, 0));
    tm.pend_d = true;
    st.edges_dynamic += cd.total;
    st.link_bytes += (cd.total * e->bpe + 7) / 8;
  }
  return OG_OK;
}

// Compacts both regions of `cur` and brings the counts (and the error word) to
// the host.  Returns the number of listed vertices through *n.
// Smallest waiting value the last compaction of region r saw, or UINT32_MAX
// (its far key carries the launch epoch; another epoch means "none").
uint32_t far_of(const og_engine *e, int r) {
  const uint64_t key = ((const uint64_t *)(e->counts_h + 2))[r];
  return (uint32_t)(key >> 32) == e->epoch ? ~(uint32_t)key : 0xffffffffu;
}

int compact_round(og_engine *e, const uint32_t *cur, og_stats &st, Timing &tm, uint64_t *n,
                  const SplitArgs &sp = SplitArgs()) {
  if (++e->epoch >= (1u << 30)) {  // epoch wrap: clear the status words and far keys once
    for (int r = 0; r < 2; r++)
      CK(cudaMemsetAsync(e->lb[r].status, 0, sizeof(uint32_t) * e->lb_tiles, e->s_main));
    CK(cudaMemsetAsync(e->counts_d + 2, 0, sizeof(Counts), e->s_main));
    e->epoch = 1;
  }
  CK(cudaEventRecord(e->ev_round, e->s_main));
  RC(launch_compact(e, 0, cur, 0, e->Vs, e->s_main, sp));
  CK(cudaEventRecord(e->ev_cs, e->s_main));
  CK(cudaStreamWaitEvent(e->s_dyn, e->ev_round, 0));
  RC(launch_compact(e, 1, cur, e->Vs, e->V, e->s_dyn, sp));
  CK(cudaEventRecord(e->ev_cd, e->s_dyn));
  CK(cudaStreamWaitEvent(e->s_dyn, e->ev_cs, 0));
  CK(cudaMemcpyAsync(e->counts_h, e->counts_d, 3 * sizeof(Counts), cudaMemcpyDeviceToHost, e->s_dyn));
  CK(cudaMemcpyAsync(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost, e->s_dyn));
  CK(cudaStreamSynchronize(e->s_dyn));
  collect_timing(e, tm, &st);
  float ms;
  if (cudaEventElapsedTime(&ms, e->ev_round, e->ev_cd) == cudaSuccess) st.ms_compact += ms;
  RC(check_device_error(e));
  *n = (uint64_t)e->counts_h[0].n + e->counts_h[1].n;
  return OG_OK;
}

template <class K>
int run_frontier(og_engine *e, int algo, uint32_t src, og_stats &st) {
  const uint64_t V = e->V;
  uint32_t *cur = e->bm[0], *next = e->bm[1];
  cudaStream_t s = e->s_main;
  const int g = grid_for(V, e->sms);
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  CK(cudaMemsetAsync(cur, 0, 4 * e->nwords, s));
  CK(cudaMemsetAsync(next, 0, 4 * e->nwords, s));
  if (algo == OG_ALGO_BFS) {
    CK(cudaMemsetAsync(e->bm[2], 0, 4 * e->nwords, s));
    k_fill_u32<<<g, kThreads, 0, s>>>(e->value_d, V, (uint32_t)(V + 1));  // GraphMeta.h:378
    k_set_source<<<1, 1, 0, s>>>(e->value_d, src, 1u, cur, e->bm[2]);
    e->launches += 2;
  } else if (algo == OG_ALGO_SSSP) {
    if (e->sssp_delta > 0) CK(cudaMemsetAsync(e->bm[2], 0, 4 * e->nwords, s));  // waiting set
    // far keys: a device-driven query leaves keys of higher epochs, which
    // atomicMax would keep over this query's
    CK(cudaMemsetAsync(e->counts_d + 2, 0, sizeof(Counts), s));
    k_fill_u32<<<g, kThreads, 0, s>>>(e->value_d, V, 0xFFFFFFFFu);  // SSSP GraphMeta.h:377
    k_set_source<<<1, 1, 0, s>>>(e->value_d, src, 1u, cur, nullptr);
    e->launches += 2;
  } else {
    k_iota_u32<<<g, kThreads, 0, s>>>(e->value_d, V);  // CC GraphMeta.h:341-345
    k_fill_bits<<<g, kThreads, 0, s>>>(cur, e->nwords, V);
    e->launches += 2;
  }
  CK(cudaGetLastError());
  Timing tm;
  RoundOps ro{algo, 1};
  // SSSP near/far split (two-bucket delta stepping): a round expands only
  // frontier vertices closer than thr; the others move to the waiting set
  // (bm[2]) and are not looked at again until no near vertex is left.  Then
  // thr moves to the smallest waiting distance + delta and one scan of the
  // waiting set lists the vertices below it.  far_min is the minimum over
  // the waiting set as of the last scan, lowered by every insertion since; a
  // vertex listed from the frontier leaves the waiting set, so the minimum
  // may be stale-low, in which case the scan lists nothing and returns the
  // true minimum for the next try.
  const bool split = algo == OG_ALGO_SSSP && e->sssp_delta > 0;
  uint32_t *waiting = e->bm[2];
  uint64_t thr = 1ull + e->sssp_delta;
  uint32_t far_min = 0xffffffffu;
  bool advance = false;
  // Direction-optimizing BFS (symmetric graphs): a level is expanded bottom-up
  // when its frontier's edges exceed unexplored / kAlpha (unexplored = the
  // degrees of the vertices that have not been a frontier yet), and top-down
  // again once the frontier falls below V / kBeta while shrinking.
  constexpr uint64_t kAlpha = 14, kBeta = 24;
  const bool dopt = algo == OG_ALGO_BFS && e->bfs_direction == OG_BFS_AUTO && e->g->symmetric == 1;
  uint64_t unexplored = e->g->E;
  bool bottom = false, counted = false;
  uint64_t fn = 0;  // frontier size when it came from a bottom-up level
  for (;;) {
    uint64_t n = 0;
    if (dopt && bottom) {
      unsigned long long *cnt = e->sum64_d;  // reached, their degrees, host records, static records
      CK(cudaMemsetAsync(cnt, 0, 32, s));  // next is all zero here, as at every level start
      CK(cudaEventRecord(e->t_d0, s));
      k_bfs_bottom_up<EKU::PSrc><<<grid_for(V, e->sms), kThreads, 0, s>>>(
          e->off_d, (uint32_t)V, e->Vs, EKU::stat(e), EKU::host(e), cur, e->bm[2], next, e->value_d,
          ro.level + 1, cnt, e->err_d);
      e->launches++;
      CK(cudaEventRecord(e->ev_dyn_done, s));
      unsigned long long c4[4];
      CK(cudaMemcpyAsync(c4, cnt, 32, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      RC(check_device_error(e));
      float ms = 0;
      if (cudaEventElapsedTime(&ms, e->t_d0, e->ev_dyn_done) == cudaSuccess) st.ms_dynamic += ms;
      st.iterations++;
      st.frontier_sum += fn;
      st.edges_dynamic += c4[2];
      st.edges_static += c4[3];
      st.link_bytes += (c4[2] * e->bpe + 7) / 8;
      unexplored -= std::min<uint64_t>(unexplored, c4[1]);
      std::swap(cur, next);
      CK(cudaMemsetAsync(next, 0, 4 * e->nwords, s));  // the level just expanded
      ro.level++;
      if (c4[0] == 0) break;
      if (c4[0] < V / kBeta && c4[0] < fn) bottom = false;  // next level: compaction + top-down
      fn = c4[0];
      counted = true;
      continue;
    }
    SplitArgs sp;
    sp.on = split;
    sp.thr = (uint32_t)std::min<uint64_t>(thr, 0xffffffffull);
    sp.clear_bits = split ? waiting : nullptr;
    sp.far_bits = split && !advance ? waiting : nullptr;
    RC(compact_round(e, advance ? waiting : cur, st, tm, &n, sp));
    if constexpr (K::kFrag) RC(frag_step(e, st, n == 0));
    if (split) {
      const uint32_t fm = std::min(far_of(e, 0), far_of(e, 1));
      far_min = advance ? fm : std::min(far_min, fm);
    }
    if (n == 0) {
      if (!split || far_min == 0xffffffffu) break;
      thr = (uint64_t)far_min + e->sssp_delta;
      advance = true;
      continue;
    }
    advance = false;
    if (dopt) {
      const uint64_t mf = e->counts_h[0].total + e->counts_h[1].total;
      if (!counted) unexplored -= std::min(unexplored, mf);
      counted = false;
      if (mf > unexplored / kAlpha) {  // expand this frontier bottom-up
        bottom = true;
        fn = n;
        counted = true;
        continue;
      }
    }
    st.iterations++;
    st.frontier_sum += n;
    st.static_vertices += e->counts_h[0].n;
    auto sfn = [&](const LbsArgs &a) { return launch_relax(e, ro, a, K::stat(e), next, e->s_main); };
    auto dfn = [&](const LbsArgs &a, auto src, cudaStream_t ds) {
      return launch_relax(e, ro, a, src, next, ds);
    };
    auto pfn = [&](const LbsArgs &a0, auto s0, const LbsArgs &a1, auto s1, cudaStream_t ps) {
      return launch_relax_pair(e, ro, a0, s0, a1, s1, next, ps);
    };
    RC((run_regions<K>(e, st, tm, sfn, dfn, pfn)));
    if constexpr (K::kFrag) e->frag->since += e->counts_h[1].total;
    CK(cudaStreamWaitEvent(e->s_main, e->ev_cd, 0));
    CK(cudaMemsetAsync(cur, 0, 4 * e->nwords, e->s_main));
    std::swap(cur, next);
    ro.level++;
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(e->s_main));
  CK(cudaMemcpy(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost));
  RC(check_device_error(e));
  e->last_algo = algo;
  return OG_OK;
}

// ------------------------------------------------------- device-driven BFS

// Captures one BFS level for the frontier in bm[p] (next in bm[1 - p]).
int capture_bfs_level(og_engine *e, int p, int dopt, cudaGraphExec_t *out) {
  cudaStream_t s = e->s_main;
  uint32_t *cur = e->bm[p], *next = e->bm[1 - p];
  BfsLoop *L = e->loop_d;
  cudaGraph_t gr = nullptr;
  const uint64_t before = e->launches;
  int per_sm = 0;  // fixed grid of the top-down relax: every CTA resident
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lbs_pair_dev<EKU::PSrc, EKU::PSrc, BfsOp>, kThreads, 0));
  const unsigned grid = (unsigned)std::max(1, per_sm) * (unsigned)e->sms;
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = OG_OK;
  auto body = [&]() -> int {
    SplitArgs sp;
    sp.epoch_ptr = &L->epoch;
    sp.run_flag = &L->compact_go;
    CK(cudaEventRecord(e->ev_round, s));
    CK(cudaStreamWaitEvent(e->s_dyn, e->ev_round, 0));
    RC(launch_compact(e, 0, cur, 0, e->Vs, s, sp));
    RC(launch_compact(e, 1, cur, e->Vs, e->V, e->s_dyn, sp));
    CK(cudaEventRecord(e->ev_cd, e->s_dyn));
    CK(cudaStreamWaitEvent(s, e->ev_cd, 0));
    k_bfs_ctl_mid<<<1, 32, 0, s>>>(L, e->counts_d, dopt);
    BfsOp op{e->bm[2], next, e->value_d, e->err_d, e->V, 0};
    if (e->relax_timer) k_stamp<<<1, 1, 0, s>>>(&L->td_go, L->relax_timer, 0);
    k_lbs_pair_dev<EKU::PSrc, EKU::PSrc, BfsOp><<<grid, kThreads, 0, s>>>(
        lbs_args(e, 0, 0, 0, true, e->plan.static_edges), EKU::stat(e), lbs_args(e, 1, 0, 0, true, e->g->E),
        EKU::host(e), op, e->counts_d, &L->td_go, &L->level, &L->tile_next);
    if (e->relax_timer) k_stamp<<<1, 1, 0, s>>>(&L->td_go, L->relax_timer, 1);
    k_bfs_bottom_up<EKU::PSrc><<<grid_for(e->V, e->sms), kThreads, 0, s>>>(
        e->off_d, e->V, e->Vs, EKU::stat(e), EKU::host(e), cur, e->bm[2], next, e->value_d, 0, L->bu,
        e->err_d, &L->bu_go, &L->level);
    k_bfs_ctl_end<<<1, 32, 0, s>>>(L, e->V);
    CK(cudaMemsetAsync(cur, 0, 4 * e->nwords, s));  // the expanded frontier: next level's "next"
    return OG_OK;
  };
  rc = body();
  const cudaError_t ce = cudaStreamEndCapture(s, &gr);
  e->launches = before;  // captured, not launched
  if (rc != OG_OK || ce != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    cudaGetLastError();
    return rc != OG_OK ? rc : fail(OG_E_CUDA, "BFS level capture: %s", cudaGetErrorString(ce));
  }
  const cudaError_t ie = cudaGraphInstantiate(out, gr, 0);
  cudaGraphDestroy(gr);
  if (ie != cudaSuccess) return fail(OG_E_CUDA, "BFS level graph: %s", cudaGetErrorString(ie));
  return OG_OK;
}

// Single-source BFS with the device-driven level loop (see bfs_loop.cuh):
// the two level graphs alternate; the host checks the done flag after as many
// levels as the previous query took, then every two levels.
int run_bfs_dev(og_engine *e, uint32_t src, og_stats &st) {
  const uint64_t V = e->V;
  cudaStream_t s = e->s_main;
  const int g = grid_for(V, e->sms);
  // the captured graphs depend on the direction mode and the relax timer
  const int dopt = (e->bfs_direction == OG_BFS_AUTO && e->g->symmetric == 1) | (e->relax_timer ? 2 : 0);
  if (dopt != e->bfs_exec_dopt) {
    for (int p = 0; p < 2; p++)
      if (e->bfs_exec[p]) {
        cudaGraphExecDestroy(e->bfs_exec[p]);
        e->bfs_exec[p] = nullptr;
      }
    for (int p = 0; p < 2; p++) RC(capture_bfs_level(e, p, dopt & 1, &e->bfs_exec[p]));
    e->bfs_exec_dopt = dopt;
  }
  if (e->dev_epoch > (1u << 30) - (1u << 20)) {  // epoch wrap: clear the status words once
    for (int r = 0; r < 2; r++)
      CK(cudaMemsetAsync(e->lb[r].status, 0, sizeof(uint32_t) * e->lb_tiles, s));
    e->dev_epoch = 1u << 29;
  }
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  CK(cudaMemsetAsync(e->bm[0], 0, 4 * e->nwords, s));
  CK(cudaMemsetAsync(e->bm[1], 0, 4 * e->nwords, s));
  CK(cudaMemsetAsync(e->bm[2], 0, 4 * e->nwords, s));
  k_fill_u32<<<g, kThreads, 0, s>>>(e->value_d, V, (uint32_t)(V + 1));  // GraphMeta.h:378
  k_set_source<<<1, 1, 0, s>>>(e->value_d, src, 1u, e->bm[0], e->bm[2]);
  BfsLoop &h = *e->loop_h;
  memset(&h, 0, sizeof h);
  h.level = 1;
  h.need_compact = 1;
  h.compact_go = 1;
  h.epoch = e->dev_epoch;
  h.unexplored = e->g->E;
  CK(cudaMemcpyAsync(e->loop_d, &h, sizeof h, cudaMemcpyHostToDevice, s));
  CK(cudaEventRecord(e->t_d0, s));
  uint32_t launched = 0, batch = std::max<uint32_t>(2, e->bfs_levels_hint + 1);
  for (;;) {
    for (uint32_t i = 0; i < batch; i++, launched++) CK(cudaGraphLaunch(e->bfs_exec[launched & 1], s));
    CK(cudaMemcpyAsync(&h.done, &e->loop_d->done, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (h.done) break;
    if (launched > 4 * V + 64) return fail(OG_E_STATE, "BFS did not end after %u levels", launched);
    batch = 2;
  }
  CK(cudaEventRecord(e->ev_dyn_done, s));
  CK(cudaMemcpyAsync(&h, e->loop_d, sizeof h, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  RC(check_device_error(e));
  float ms = 0;
  if (cudaEventElapsedTime(&ms, e->t_d0, e->ev_dyn_done) == cudaSuccess) st.ms_dynamic += ms;
  st.iterations += (uint32_t)h.iterations;
  st.frontier_sum += h.frontier_sum;
  st.edges_static += h.edges_static;
  st.edges_dynamic += h.edges_dynamic;
  st.link_bytes += (h.edges_dynamic * e->bpe + 7) / 8;
  st.chunks += (uint32_t)h.iterations;
  st.ms_relax += h.relax_timer[1] / 1e6;
  e->launches += 2 + (7ull + (e->relax_timer ? 2 : 0)) * launched;
  e->bfs_levels_hint = (uint32_t)h.iterations;
  e->dev_epoch = h.epoch + 1;
  e->last_algo = OG_ALGO_BFS;
  return OG_OK;
}

// Captures one SSSP / CC round for the frontier in bm[p] (next in bm[1 - p],
// waiting set in bm[2]); see bfs_loop.cuh.
template <class K, bool kW>
int capture_min_round(og_engine *e, int p, bool split, cudaGraphExec_t *out) {
  cudaStream_t s = e->s_main;
  uint32_t *cur = e->bm[p], *next = e->bm[1 - p], *waiting = e->bm[2];
  MinLoop *L = e->mloop_d;
  const unsigned long long *keys = (const unsigned long long *)(e->counts_d + 2);
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, k_lbs_pair_dev<typename K::PSrc, typename K::PSrc, MinOp<kW>>, kThreads, 0));
  const unsigned grid = (unsigned)std::max(1, per_sm) * (unsigned)e->sms;
  cudaGraph_t gr = nullptr;
  const uint64_t before = e->launches;
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  auto compact_both = [&](const uint32_t *bits, const SplitArgs &sp) -> int {
    CK(cudaEventRecord(e->ev_round, s));
    CK(cudaStreamWaitEvent(e->s_dyn, e->ev_round, 0));
    RC(launch_compact(e, 0, bits, 0, e->Vs, s, sp));
    RC(launch_compact(e, 1, bits, e->Vs, e->V, e->s_dyn, sp));
    CK(cudaEventRecord(e->ev_cd, e->s_dyn));
    CK(cudaStreamWaitEvent(s, e->ev_cd, 0));
    return OG_OK;
  };
  auto body = [&]() -> int {
    SplitArgs sr;
    sr.epoch_ptr = &L->epoch;
    sr.run_flag = &L->round_go;
    sr.thr_ptr = &L->thr;
    sr.on = split;
    sr.far_bits = split ? waiting : nullptr;
    sr.clear_bits = split ? waiting : nullptr;
    RC(compact_both(cur, sr));
    k_min_ctl_a<<<1, 32, 0, s>>>(L, e->counts_d, keys);
    if (split) {
      SplitArgs sa = sr;
      sa.run_flag = &L->adv_go;
      sa.far_bits = nullptr;
      RC(compact_both(waiting, sa));
      k_min_ctl_b<<<1, 32, 0, s>>>(L, e->counts_d, keys);
    }
    MinOp<kW> op{e->value_d, next, e->err_d, e->V};
    if (e->relax_timer) k_stamp<<<1, 1, 0, s>>>(&L->relax_go, L->relax_timer, 0);
    k_lbs_pair_dev<typename K::PSrc, typename K::PSrc, MinOp<kW>><<<grid, kThreads, 0, s>>>(
        lbs_args(e, 0, 0, 0, true, e->plan.static_edges), K::stat(e), lbs_args(e, 1, 0, 0, true, e->g->E),
        K::host(e), op, e->counts_d, &L->relax_go, nullptr, &L->tile_next);
    if (e->relax_timer) k_stamp<<<1, 1, 0, s>>>(&L->relax_go, L->relax_timer, 1);
    k_min_ctl_end<<<1, 32, 0, s>>>(L);
    CK(cudaMemsetAsync(cur, 0, 4 * e->nwords, s));
    return OG_OK;
  };
  const int rc = body();
  const cudaError_t ce = cudaStreamEndCapture(s, &gr);
  e->launches = before;  // captured, not launched
  if (rc != OG_OK || ce != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    cudaGetLastError();
    return rc != OG_OK ? rc : fail(OG_E_CUDA, "round capture: %s", cudaGetErrorString(ce));
  }
  const cudaError_t ie = cudaGraphInstantiate(out, gr, 0);
  cudaGraphDestroy(gr);
  if (ie != cudaSuccess) return fail(OG_E_CUDA, "round graph: %s", cudaGetErrorString(ie));
  return OG_OK;
}

// SSSP (algo OG_ALGO_SSSP) or label-propagation CC with device-driven rounds.
int run_min_dev(og_engine *e, int algo, uint32_t src, og_stats &st) {
  const uint64_t V = e->V;
  cudaStream_t s = e->s_main;
  const int g = grid_for(V, e->sms);
  const bool sssp = algo == OG_ALGO_SSSP;
  const bool split = sssp && e->sssp_delta > 0;
  const int key = (sssp ? 2 : 0) + (split ? 1 : 0) + (e->relax_timer ? 4 : 0);
  if (key != e->min_exec_key) {
    for (int p = 0; p < 2; p++)
      if (e->min_exec[p]) {
        cudaGraphExecDestroy(e->min_exec[p]);
        e->min_exec[p] = nullptr;
      }
    for (int p = 0; p < 2; p++)
      RC((sssp ? capture_min_round<EK<uint8_t>, true>(e, p, split, &e->min_exec[p])
               : capture_min_round<EKU, false>(e, p, false, &e->min_exec[p])));
    e->min_exec_key = key;
  }
  if (e->dev_epoch > (1u << 30) - (1u << 20)) {  // epoch wrap: clear the status words once
    for (int r = 0; r < 2; r++)
      CK(cudaMemsetAsync(e->lb[r].status, 0, sizeof(uint32_t) * e->lb_tiles, s));
    CK(cudaMemsetAsync(e->counts_d + 2, 0, sizeof(Counts), s));
    e->dev_epoch = 1u << 29;
  }
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  CK(cudaMemsetAsync(e->bm[0], 0, 4 * e->nwords, s));
  CK(cudaMemsetAsync(e->bm[1], 0, 4 * e->nwords, s));
  if (sssp) {
    if (split) CK(cudaMemsetAsync(e->bm[2], 0, 4 * e->nwords, s));  // waiting set
    CK(cudaMemsetAsync(e->counts_d + 2, 0, sizeof(Counts), s));    // far keys of earlier queries
    k_fill_u32<<<g, kThreads, 0, s>>>(e->value_d, V, 0xFFFFFFFFu);  // SSSP GraphMeta.h:377
    k_set_source<<<1, 1, 0, s>>>(e->value_d, src, 1u, e->bm[0], nullptr);
  } else {
    k_iota_u32<<<g, kThreads, 0, s>>>(e->value_d, V);  // CC GraphMeta.h:341-345
    k_fill_bits<<<g, kThreads, 0, s>>>(e->bm[0], e->nwords, V);
  }
  MinLoop &h = *e->mloop_h;
  memset(&h, 0, sizeof h);
  h.epoch = e->dev_epoch;
  const uint64_t thr = 1ull + e->sssp_delta;
  h.thr = thr > 0xffffffffull ? 0xffffffffu : (uint32_t)thr;
  h.round_go = 1;
  h.far_min = 0xffffffffu;
  h.delta = e->sssp_delta;
  h.split = split ? 1 : 0;
  CK(cudaMemcpyAsync(e->mloop_d, &h, sizeof h, cudaMemcpyHostToDevice, s));
  CK(cudaEventRecord(e->t_d0, s));
  uint32_t &hint = e->min_rounds_hint[sssp ? 0 : 1];
  uint32_t launched = 0, batch = std::max<uint32_t>(2, hint + 2);
  for (;;) {
    for (uint32_t i = 0; i < batch; i++, launched++) CK(cudaGraphLaunch(e->min_exec[launched & 1], s));
    CK(cudaMemcpyAsync(&h.done, &e->mloop_d->done, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (h.done) break;
    if (launched > 8 * V + 64) return fail(OG_E_STATE, "rounds did not end after %u", launched);
    batch = 8;
  }
  CK(cudaEventRecord(e->ev_dyn_done, s));
  CK(cudaMemcpyAsync(&h, e->mloop_d, sizeof h, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  RC(check_device_error(e));
  float ms = 0;
  if (cudaEventElapsedTime(&ms, e->t_d0, e->ev_dyn_done) == cudaSuccess) st.ms_dynamic += ms;
  st.iterations += (uint32_t)h.iterations;
  st.frontier_sum += h.frontier_sum;
  st.edges_static += h.edges_static;
  st.edges_dynamic += h.edges_dynamic;
  st.link_bytes += (h.edges_dynamic * e->bpe + 7) / 8;
  st.chunks += (uint32_t)h.iterations;
  st.ms_relax += h.relax_timer[1] / 1e6;
  e->launches += 2 + ((split ? 11ull : 7ull) + (e->relax_timer ? 2 : 0)) * launched;
  hint = h.rounds;  // rounds this query needed (the next one is launched that far before its first check)
  e->dev_epoch = h.epoch + 1;
  e->last_algo = algo;
  return OG_OK;
}

// ------------------------------------------------------------------ batched BFS

// The n x V depth matrix (outside the budget), allocated on first use and
// kept for later calls; it grows when a call needs more sources.
int depth_matrix(og_engine *e, uint32_t n, uint32_t **out) {
  const uint64_t need = (uint64_t)n * e->V;
  if (need > e->depth_cap) {
    if (e->depth_d) cudaFree(e->depth_d);
    e->depth_d = nullptr;
    e->depth_cap = 0;
    CK(cudaMalloc(&e->depth_d, 4 * need));
    e->depth_cap = need;
  }
  *out = e->depth_d;
  return OG_OK;
}

int run_batch(og_engine *e, const uint32_t *srcs, uint32_t n, uint32_t *out, uint64_t *checks,
              og_stats &st) {
  const uint64_t V = e->V;
  uint32_t *cur_any = e->bm[0], *next_any = e->bm[1];
  unsigned long long *visited = e->bmask[0], *cur = e->bmask[1], *next = e->bmask[2];
  cudaStream_t s = e->s_main;
  uint32_t *depth_d = nullptr;
  if (out) {
    RC(depth_matrix(e, n, &depth_d));
    k_fill_u32<<<grid_for(n * V, e->sms), kThreads, 0, s>>>(depth_d, (uint64_t)n * V, (uint32_t)(V + 1));
    e->launches++;
  }
  std::vector<uint64_t> reached(n, 1), dsum(n, 1);  // each source: itself at depth 1
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  CK(cudaMemsetAsync(cur_any, 0, 4 * e->nwords, s));
  CK(cudaMemsetAsync(next_any, 0, 4 * e->nwords, s));
  for (int i = 0; i < 3; i++) CK(cudaMemsetAsync(e->bmask[i], 0, 8 * (V + 1), s));
  CK(cudaMemcpyAsync(e->srcs_d, srcs, 4 * n, cudaMemcpyHostToDevice, s));
  k_batch_init<<<1, 64, 0, s>>>(e->srcs_d, n, visited, cur, cur_any, depth_d, V);
  e->launches++;
  CK(cudaGetLastError());
  Timing tm;
  for (uint32_t level = 1;; level++) {
    uint64_t nl = 0;
    RC(compact_round(e, cur_any, st, tm, &nl));
    if (nl == 0) break;
    st.iterations++;
    st.frontier_sum += nl;
    st.static_vertices += e->counts_h[0].n;
    BatchOp op{visited, cur, next, next_any, e->err_d, e->V};
    auto launch = [&](const LbsArgs &a, auto src, cudaStream_t ls) {
      const unsigned grid = lbs_grid(a.pos_begin, a.pos_end);
      if (grid) {
        k_lbs<decltype(src), BatchOp><<<grid, kThreads, 0, ls>>>(a, src, op);
        e->launches++;
      }
      return (int)OG_OK;
    };
    auto sfn = [&](const LbsArgs &a) { return launch(a, EKU::stat(e), e->s_main); };
    auto pfn = [&](const LbsArgs &a0, auto s0, const LbsArgs &a1, auto s1, cudaStream_t ps) {
      const uint64_t n0 = lbs_grid(a0.pos_begin, a0.pos_end), n1 = lbs_grid(a1.pos_begin, a1.pos_end);
      if (n0 + n1 > 0x7fffffffull) return fail(OG_E_STATE, "relax grid too large");
      k_lbs_pair<decltype(s0), decltype(s1), BatchOp><<<(unsigned)(n0 + n1), kThreads, 0, ps>>>(
          a0, s0, a1, s1, op, n0, n0 + n1);
      e->launches++;
      return (int)OG_OK;
    };
    RC((run_regions<EKU>(e, st, tm, sfn, launch, pfn)));
    CK(cudaMemsetAsync(e->hist_d, 0, 64 * 8, s));
    k_batch_level<<<grid_for(e->nwords, e->sms), kThreads, 0, s>>>(next_any, next, e->nwords, n,
                                                                 e->hist_d, depth_d, V, level + 1);
    e->launches++;
    CK(cudaMemcpyAsync(e->hist_h, e->hist_d, 64 * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamWaitEvent(s, e->ev_cd, 0));
    CK(cudaMemsetAsync(cur_any, 0, 4 * e->nwords, s));
    CK(cudaMemsetAsync(cur, 0, 8 * (V + 1), s));
    CK(cudaStreamSynchronize(s));
    for (uint32_t i = 0; i < n; i++) {
      reached[i] += e->hist_h[i];
      dsum[i] += (uint64_t)(level + 1) * e->hist_h[i];
    }
    std::swap(cur_any, next_any);
    std::swap(cur, next);
    CK(cudaGetLastError());
  }
  CK(cudaMemcpy(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost));
  RC(check_device_error(e));
  if (out) CK(cudaMemcpy(out, depth_d, 4ull * n * V, cudaMemcpyDeviceToHost));
  if (checks)
    for (uint32_t i = 0; i < n; i++) {
      checks[2 * i] = reached[i];
      checks[2 * i + 1] = dsum[i];
    }
  e->last_algo = -1;  // the engine's value array holds no single result
  return OG_OK;
}

// ------------------------------------------------- batched BFS, level by level

// Opens a session: no slot in use, empty masks and frontier; with `record`
// the 64 x V depth matrix (outside the budget) is kept for og_bfs_batch_fetch.
int bb_begin_impl(og_engine *e, bool record) {
  const uint64_t V = e->V;
  cudaStream_t s = e->s_main;
  e->sb_session = false;  // the masks share the arena with the SSSP rows
  e->bb_session = false;
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  CK(cudaMemsetAsync(e->bm[0], 0, 4 * e->nwords, s));
  CK(cudaMemsetAsync(e->bm[1], 0, 4 * e->nwords, s));
  for (int i = 0; i < 3; i++) CK(cudaMemsetAsync(e->bmask[i], 0, 8 * (V + 1), s));
  e->bb_record = record;
  if (record) {
    uint32_t *d = nullptr;
    RC(depth_matrix(e, 64, &d));
    k_fill_u32<<<grid_for(64 * V, e->sms), kThreads, 0, s>>>(d, 64 * V, (uint32_t)(V + 1));
    e->launches++;
  }
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  e->bb_level = 1;
  e->bb_par = 0;
  e->bb_used = e->bb_dirty = 0;
  e->bb_session = true;
  return OG_OK;
}

// Seeds slots[i] with srcs[i] at the current level boundary.
int bb_join_impl(og_engine *e, const uint32_t *srcs, const uint32_t *slots, uint32_t n) {
  if (n == 0) return OG_OK;
  if (n > 64) return fail(OG_E_ARG, "%u sources joined, a batch holds 64", n);
  uint64_t cols = 0;
  for (uint32_t i = 0; i < n; i++) {
    if (srcs[i] >= e->V) return fail(OG_E_ARG, "source %u >= V %u", srcs[i], e->V);
    if (slots[i] >= 64) return fail(OG_E_ARG, "slot %u >= 64", slots[i]);
    const uint64_t b = 1ull << slots[i];
    if (cols & b) return fail(OG_E_ARG, "slot %u joined twice", slots[i]);
    if (e->bb_used & b) return fail(OG_E_STATE, "slot %u is still in flight", slots[i]);
    cols |= b;
  }
  const uint64_t V = e->V;
  cudaStream_t s = e->s_main;
  if (cols & e->bb_dirty) {
    k_batch_clear_bits<<<grid_for(V + 1, e->sms), kThreads, 0, s>>>(e->bmask[0], V + 1, cols & e->bb_dirty);
    e->launches++;
    e->bb_dirty &= ~cols;
  }
  if (e->bb_record)
    for (uint32_t i = 0; i < n; i++) {
      k_fill_u32<<<grid_for(V, e->sms), kThreads, 0, s>>>(e->depth_d + (uint64_t)slots[i] * V, V,
                                                         (uint32_t)(V + 1));
      e->launches++;
    }
  for (uint32_t i = 0; i < n; i++) {
    e->bb_off[slots[i]] = e->bb_level - 1;
    e->bb_reached[slots[i]] = 1;  // the source itself, at depth 1
    e->bb_dsum[slots[i]] = 1;
  }
  CK(cudaStreamSynchronize(s));  // the page-locked buffer is rewritten only after the previous upload ran
  memcpy(e->bb_io_h, srcs, 4 * n);
  memcpy(e->bb_io_h + 64, slots, 4 * n);
  memcpy(e->bb_io_h + 128, e->bb_off, 4 * 64);
  CK(cudaMemcpyAsync(e->bb_io_d, e->bb_io_h, 192 * 4, cudaMemcpyHostToDevice, s));
  k_batch_init<<<1, 64, 0, s>>>(e->bb_io_d, n, e->bmask[0], e->bmask[1 + e->bb_par], e->bm[e->bb_par],
                                e->bb_record ? e->depth_d : nullptr, V, nullptr, e->bb_io_d + 64);
  e->launches++;
  CK(cudaGetLastError());
  e->bb_used |= cols;
  return OG_OK;
}

// One level: expands the frontier of every slot in flight.  A slot that
// reached no new vertex has finished: it leaves *pending, its checks are
// final and it may be joined again.
int bb_step_impl(og_engine *e, uint64_t *pending, bool *done, og_stats &st, Timing &tm) {
  const uint64_t V = e->V;
  cudaStream_t s = e->s_main;
  const uint32_t par = e->bb_par;
  uint32_t *cur_any = e->bm[par], *next_any = e->bm[1 - par];
  unsigned long long *visited = e->bmask[0], *cur = e->bmask[1 + par], *next = e->bmask[2 - par];
  uint64_t nl = 0;
  RC(compact_round(e, cur_any, st, tm, &nl));
  if (nl == 0) {  // nothing in flight
    e->bb_dirty |= e->bb_used;
    e->bb_used = 0;
    *pending = 0;
    *done = true;
    return OG_OK;
  }
  st.iterations++;
  st.frontier_sum += nl;
  st.static_vertices += e->counts_h[0].n;
  BatchOp op{visited, cur, next, next_any, e->err_d, e->V};
  auto launch = [&](const LbsArgs &a, auto src, cudaStream_t ls) {
    const unsigned grid = lbs_grid(a.pos_begin, a.pos_end);
    if (grid) {
      k_lbs<decltype(src), BatchOp><<<grid, kThreads, 0, ls>>>(a, src, op);
      e->launches++;
    }
    return (int)OG_OK;
  };
  auto sfn = [&](const LbsArgs &a) { return launch(a, EKU::stat(e), s); };
  auto pfn = [&](const LbsArgs &a0, auto s0, const LbsArgs &a1, auto s1, cudaStream_t ps) {
    const uint64_t n0 = lbs_grid(a0.pos_begin, a0.pos_end), n1 = lbs_grid(a1.pos_begin, a1.pos_end);
    if (n0 + n1 > 0x7fffffffull) return fail(OG_E_STATE, "relax grid too large");
    k_lbs_pair<decltype(s0), decltype(s1), BatchOp><<<(unsigned)(n0 + n1), kThreads, 0, ps>>>(
        a0, s0, a1, s1, op, n0, n0 + n1);
    e->launches++;
    return (int)OG_OK;
  };
  RC((run_regions<EKU>(e, st, tm, sfn, launch, pfn)));
  CK(cudaMemsetAsync(e->hist_d, 0, 64 * 8, s));
  const uint32_t depth = e->bb_level + 1;  // of the vertices this level reaches, for a source joined at begin
  k_batch_level<<<grid_for(e->nwords, e->sms), kThreads, 0, s>>>(next_any, next, e->nwords, 64, e->hist_d,
                                                               e->bb_record ? e->depth_d : nullptr, V, depth,
                                                               e->bb_io_d + 128);
  e->launches++;
  CK(cudaMemcpyAsync(e->hist_h, e->hist_d, 64 * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamWaitEvent(s, e->ev_cd, 0));
  CK(cudaMemsetAsync(cur_any, 0, 4 * e->nwords, s));
  CK(cudaMemsetAsync(cur, 0, 8 * (V + 1), s));
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  for (uint32_t i = 0; i < 64; i++) {
    const uint64_t b = 1ull << i;
    if (!(e->bb_used & b)) continue;
    const uint64_t c = e->hist_h[i];
    if (c == 0) {
      e->bb_used &= ~b;
      e->bb_dirty |= b;
    } else {
      e->bb_reached[i] += c;
      e->bb_dsum[i] += (uint64_t)(depth - e->bb_off[i]) * c;
    }
  }
  e->bb_par ^= 1u;
  e->bb_level++;
  *pending = e->bb_used;
  *done = e->bb_used == 0;
  return OG_OK;
}

// ------------------------------------------------------- persistent batched BFS

struct PersistCfg {
  int block, items;
};
// candidate (CTA size, edge positions per thread); the tile is their product
constexpr PersistCfg kPersistConfigs[] = {{256, 8}, {128, 8}, {256, 4}, {512, 4}, {128, 16}};
constexpr int kNumPersistConfigs = 5;

template <int B, int I>
int launch_persist_cfg(og_engine *e, const PersistArgs &a, cudaStream_t s) {
  auto kern = k_batch_persistent<B, I>;
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, B, 0));
  if (occ < 1) return fail(OG_E_UNSUPPORTED, "persistent kernel does not fit an SM");
  const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)occ * e->sms, kMaxPersistCtas);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(B);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // all CTAs co-resident: the grid barriers rely on it
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CK(cudaLaunchKernelEx(&cfg, kern, a));
  e->launches++;
  return OG_OK;
}

int launch_persist(og_engine *e, int ci, const PersistArgs &a, cudaStream_t s) {
  switch (ci) {
    case 0: return launch_persist_cfg<256, 8>(e, a, s);
    case 1: return launch_persist_cfg<128, 8>(e, a, s);
    case 2: return launch_persist_cfg<256, 4>(e, a, s);
    case 3: return launch_persist_cfg<512, 4>(e, a, s);
    default: return launch_persist_cfg<128, 16>(e, a, s);
  }
}

// Bottom-up levels need the graph's reverse edges: only a symmetric graph has
// them in its own records.
uint32_t batch_dopt(const og_engine *e) {
  return e->bfs_direction == OG_BFS_AUTO && e->g->symmetric == 1 ? 1u : 0u;
}

// Enqueues one whole batch on s_main: clear state, upload the sources from the
// page-locked buffer, seed, run every level in one cooperative kernel, copy
// the per-level counts and the status words back to page-locked memory.
int enqueue_persist(og_engine *e, uint32_t n, int ci, uint32_t *depth_d, uint8_t *depth8_d = nullptr) {
  const uint64_t V = e->V;
  cudaStream_t s = e->s_main;
  for (int i = 0; i < 3; i++) CK(cudaMemsetAsync(e->bmask[i], 0, 8 * (V + 1), s));
  CK(cudaMemsetAsync(e->bm[0], 0, 4 * e->nwords, s));
  CK(cudaMemsetAsync(e->bm[1], 0, 4 * e->nwords, s));
  CK(cudaMemsetAsync(e->bm[2], 0, 4 * e->nwords, s));  // deferred bottom-up vertices
  CK(cudaMemsetAsync(e->smf_d, 0, 8 * 2 * 64, s));
  CK(cudaMemsetAsync(e->hist_d, 0, 8ull * kMaxBatchLevels * 64, s));
  CK(cudaMemsetAsync(e->bar_d, 0, 64, s));
  CK(cudaMemcpyAsync(e->srcs_d, e->srcs_h, 4 * n, cudaMemcpyHostToDevice, s));
  k_batch_init<<<1, 64, 0, s>>>(e->srcs_d, n, e->bmask[0], e->bmask[1], e->bm[0], depth_d, V, depth8_d);
  e->launches++;
  PersistArgs a;
  a.V = e->V;
  a.nwords = e->nwords;
  a.off = e->off_d;
  a.ssrc = EKU::stat(e);
  a.hsrc = EKU::host(e);
  a.static_edges = e->plan.static_edges;
  a.E = e->g->E;
  a.visited = e->bmask[0];
  a.cur = e->bmask[1];
  a.next = e->bmask[2];
  a.cur_any = e->bm[0];
  a.next_any = e->bm[1];
  a.list = e->list_d[0];
  a.pref = e->pref_d[0];
  a.tile_first = e->ptile_d;
  a.list_cap = e->list_cap[0] + e->list_cap[1];
  a.tile_cap = e->ptile_cap;
  a.cta_n = e->cta_n;
  a.cta_e = e->cta_e;
  a.bar = e->bar_d;
  a.hist = e->hist_d;
  a.depth = depth_d;
  a.depth8 = depth8_d;
  a.n_src = n;
  a.err = e->bar_d + 2;
  a.levels = e->bar_d + 3;
  a.stat = (unsigned long long *)(e->bar_d + 4);
  a.smf = e->smf_d;
  a.defer = e->bm[2];
  a.Vs = e->Vs;
  a.dopt = batch_dopt(e);
  RC(launch_persist(e, ci, a, s));
  CK(cudaMemcpyAsync(e->hist_h, e->hist_d, 8ull * kMaxBatchLevels * 64, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(e->pmisc_h, e->bar_d, 64, cudaMemcpyDeviceToHost, s));
  return OG_OK;
}

// Captures enqueue_persist for (n, config) as a CUDA graph once and replays it.
int run_persist_graph(og_engine *e, uint32_t n, int ci, bool *used_graph) {
  *used_graph = false;
  const int dopt = (int)batch_dopt(e);
  if (!e->graph_broken &&
      !(e->graph && e->graph_n == n && e->graph_cfg == ci && e->graph_dopt == dopt)) {
    if (e->graph) {
      cudaGraphExecDestroy(e->graph);
      e->graph = nullptr;
    }
    cudaGraph_t gr = nullptr;
    bool ok = cudaStreamBeginCapture(e->s_main, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    const uint64_t before = e->launches;
    const int rc = ok ? enqueue_persist(e, n, ci, nullptr) : OG_E_CUDA;
    e->launches = before;  // captured, not launched
    if (ok) ok = cudaStreamEndCapture(e->s_main, &gr) == cudaSuccess && rc == OG_OK;
    if (ok) ok = cudaGraphInstantiate(&e->graph, gr, 0) == cudaSuccess;
    if (gr) cudaGraphDestroy(gr);
    if (!ok) {
      cudaGetLastError();
      e->graph = nullptr;
      e->graph_broken = true;  // fall back to direct launches from now on
    } else {
      e->graph_n = n;
      e->graph_cfg = ci;
      e->graph_dopt = dopt;
    }
  }
  if (e->graph) {
    CK(cudaGraphLaunch(e->graph, e->s_main));
    e->launches += 2;  // the seed kernel and the persistent kernel
    *used_graph = true;
    return OG_OK;
  }
  return enqueue_persist(e, n, ci, nullptr);
}

// out: V u32 depths per source (out_bytes 4) or byte depths (out_bytes 1).
// outs (og_bfs_batch_to): source i's V u32 depths go to outs[i] instead.
// The kernel then writes byte depths (an n x V byte matrix, a quarter of the
// u32 one) and each row is widened into its output; if some depth reaches
// 255, the outputs are filled by single-source runs instead.
int run_batch_persist(og_engine *e, const uint32_t *srcs, uint32_t n, void *out, int out_bytes,
                      uint64_t *clamped, uint64_t *checks, og_stats &st, int ci,
                      uint32_t *const *outs = nullptr) {
  const uint64_t V = e->V;
  memcpy(e->srcs_h, srcs, 4 * n);
  uint32_t *depth_d = nullptr;
  uint8_t *depth8_d = nullptr;
  bool graph = false;
  if (out && out_bytes == 4) {
    RC(depth_matrix(e, n, &depth_d));
    k_fill_u32<<<grid_for(n * V, e->sms), kThreads, 0, e->s_main>>>(depth_d, (uint64_t)n * V,
                                                                 (uint32_t)(V + 1));
    e->launches++;
  } else if (out || outs) {  // byte depths, written by the kernel itself (0 = unreached)
    const uint64_t need = (uint64_t)n * V;
    if (need > e->depth8_cap) {
      if (e->depth8_d) cudaFree(e->depth8_d);
      e->depth8_d = nullptr;
      e->depth8_cap = 0;
      CK(cudaMalloc(&e->depth8_d, need));
      e->depth8_cap = need;
    }
    depth8_d = e->depth8_d;
    CK(cudaMemsetAsync(depth8_d, 0, need, e->s_main));
  }
  // events outside any captured graph: they bracket the whole batch on s_main
  CK(cudaEventRecord(e->t_s0, e->s_main));
  if (out || outs) {
    RC(enqueue_persist(e, n, ci, depth_d, depth8_d));
  } else {
    RC(run_persist_graph(e, n, ci, &graph));
  }
  CK(cudaEventRecord(e->t_s1, e->s_main));
  CK(cudaStreamSynchronize(e->s_main));
  CK(cudaGetLastError());
  const uint32_t err = e->pmisc_h[2], levels = e->pmisc_h[3];
  const unsigned long long *stat = (const unsigned long long *)(e->pmisc_h + 4);
  if (err & kErrBarrier) return fail(OG_E_TIMEOUT, "batched BFS grid barrier wait gave up");
  if (err & kErrLevels) return fail(OG_E_STATE, "batched BFS needs more than %u levels", kMaxBatchLevels);
  if (err) return fail(OG_E_DEVICE, "batched BFS kernel reported an out-of-range index (0x%x)", err);
  float ms = 0;
  if (cudaEventElapsedTime(&ms, e->t_s0, e->t_s1) == cudaSuccess) st.ms_static += ms;
  st.iterations = levels;
  st.frontier_sum = stat[0];
  st.edges_static = stat[1] - stat[2];
  st.edges_dynamic = stat[2];
  st.link_bytes = (stat[2] * e->bpe + 7) / 8;  // packed records read over the link
  st.chunks = graph ? 1u : 0u;  // 1: replayed from the captured CUDA graph
  if (checks)
    for (uint32_t i = 0; i < n; i++) {
      uint64_t r = 1, d = 1;
      for (uint32_t L = 1; L <= levels && L < kMaxBatchLevels; L++) {
        const uint64_t c = e->hist_h[(uint64_t)L * 64 + i];
        r += c;
        d += (uint64_t)(L + 1) * c;
      }
      checks[2 * i] = r;
      checks[2 * i + 1] = d;
    }
  if (outs) {
    // entries at depth >= 255 do not fit a byte: single-source runs fill the
    // outputs (no n x V u32 matrix is needed for that)
    uint64_t c = 0;
    for (uint32_t L = 254; L <= levels && L < kMaxBatchLevels; L++)
      for (uint32_t i = 0; i < n; i++) c += e->hist_h[(uint64_t)L * 64 + i];
    if (c) {
      for (uint32_t i = 0; i < n; i++) {
        og_stats one;
        memset(&one, 0, sizeof one);
        RC(run_frontier<EKU>(e, OG_ALGO_BFS, srcs[i], one));
        CK(cudaMemcpyAsync(outs[i], e->value_d, 4ull * V, cudaMemcpyDeviceToHost, e->s_main));
        CK(cudaStreamSynchronize(e->s_main));
      }
      e->last_algo = -1;
      return OG_OK;
    }
    // widened into a V-entry device buffer, then one DMA copy per source
    // (kernel stores straight into page-locked memory measured several
    // times slower than the copy engine)
    uint32_t *stage = nullptr;
    RC(depth_matrix(e, 1, &stage));
    for (uint32_t i = 0; i < n; i++) {
      k_depth_expand<<<grid_for((V + 3) / 4, e->sms), kThreads, 0, e->s_main>>>(depth8_d + (uint64_t)i * V, V,
                                                                                (uint32_t)(V + 1), stage);
      e->launches++;
      CK(cudaMemcpyAsync(outs[i], stage, 4ull * V, cudaMemcpyDeviceToHost, e->s_main));
    }
    CK(cudaGetLastError());
  } else if (out && out_bytes == 4) {
    CK(cudaMemcpyAsync(out, depth_d, 4ull * n * V, cudaMemcpyDeviceToHost, e->s_main));
  } else if (out) {
    CK(cudaMemcpyAsync(out, depth8_d, (uint64_t)n * V, cudaMemcpyDeviceToHost, e->s_main));
    if (clamped) {  // entries at depth L + 1 >= 255, from the per-level counts
      uint64_t c = 0;
      for (uint32_t L = 254; L <= levels && L < kMaxBatchLevels; L++)
        for (uint32_t i = 0; i < n; i++) c += e->hist_h[(uint64_t)L * 64 + i];
      *clamped = c;
    }
  }
  CK(cudaStreamSynchronize(e->s_main));
  e->last_algo = -1;
  return OG_OK;
}

// ------------------------------------------------------------ multi-source SSSP

// Launches k_compact_sb for region r over the active (scan_wait = false) or
// waiting bitmap.
int launch_compact_sb(og_engine *e, int r, uint32_t *bits, uint32_t vb, uint32_t ve, bool scan_wait,
                      cudaStream_t s) {
  if (ve <= vb) {
    CK(cudaMemsetAsync(e->counts_d + r, 0, sizeof(Counts), s));
    return OG_OK;
  }
  SbCompactArgs a{};
  a.bits = bits;
  a.wait = e->bm[2];
  a.v_begin = vb;
  a.v_end = ve;
  a.w_begin = vb / 32;
  a.w_end = (uint32_t)(((uint64_t)ve + 31) / 32);
  a.ntiles = (a.w_end - a.w_begin + kWordsPerCompactTile - 1) / kWordsPerCompactTile;
  a.off = e->off_d;
  a.list = e->list_d[r];
  a.pref = e->pref_d[r];
  a.tile_first = e->tile_d[r];
  a.lmask = e->sb_lmask + (e->list_d[r] - e->list_d[0]);
  a.counts = e->counts_d + r;
  a.lb = e->lb[r];
  a.err = e->err_d;
  a.list_cap = e->list_cap[r];
  a.tile_cap = e->tile_cap[r];
  a.pend = e->sb_pend;
  a.dist = e->sb_dist;
  a.ks = e->sb_ks;
  a.thr = e->sb_thr;
  a.scan_wait = scan_wait ? 1u : 0u;
  a.far_key = (unsigned long long *)(e->counts_d + 2) + r;
  a.masks = e->sb_masks;
  a.epoch = e->epoch;
  if (a.ntiles + 1 > e->lb_tiles) return fail(OG_E_STATE, "compaction scratch too small");
  k_compact_sb<<<a.ntiles, kThreads, 0, s>>>(a);
  e->launches++;
  return OG_OK;
}

// Clears the batch: no slot in use, no vertex active or waiting.
int sb_reset(og_engine *e) {
  if (!e->sb_k) return fail(OG_E_STATE, "engine created without OG_CFG_SSSP_BATCH");
  const uint64_t V = e->V;
  cudaStream_t s = e->s_main;
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  CK(cudaMemsetAsync(e->bm[0], 0, 4 * e->nwords, s));  // active
  CK(cudaMemsetAsync(e->bm[2], 0, 4 * e->nwords, s));  // waiting
  CK(cudaMemsetAsync(e->sb_pend, 0, 4 * (V + 1), s));
  CK(cudaMemsetAsync(e->sb_masks, 0, 16, s));
  CK(cudaMemsetAsync(e->counts_d + 2, 0, sizeof(Counts), s));  // far keys of earlier queries
  k_fill_u32<<<grid_for((V + 1) * e->sb_ks, e->sms), kThreads, 0, s>>>(e->sb_dist, (V + 1) * e->sb_ks,
                                                                      0xffffffffu);
  e->launches++;
  const uint64_t thr = 1ull + e->sb_delta;
  e->sb_thr = e->sb_delta == 0 || thr > 0xffffffffull ? 0xffffffffu : (uint32_t)thr;
  e->sb_far_min = 0xffffffffu;
  e->sb_advance = false;
  e->sb_dirty = 0;
  e->sb_session = true;
  e->bb_session = false;  // the batch arena now holds SSSP rows
  CK(cudaGetLastError());
  return OG_OK;
}

// Seeds slots[i] with srcs[i] (their columns are reset first when a finished
// source left distances there).  A source may join while others are in
// flight: its distances start below any threshold, so it is expanded every
// round until it has caught up; the result is the same.
int sb_join_impl(og_engine *e, const uint32_t *srcs, const uint32_t *slots, uint32_t n) {
  if (n == 0) return OG_OK;
  if (n > e->sb_k) return fail(OG_E_ARG, "%u sources joined, the engine holds %u", n, e->sb_k);
  uint32_t cols = 0;
  for (uint32_t i = 0; i < n; i++) {
    if (srcs[i] >= e->V) return fail(OG_E_ARG, "source %u >= V %u", srcs[i], e->V);
    if (slots[i] >= e->sb_k) return fail(OG_E_ARG, "slot %u >= %u", slots[i], e->sb_k);
    if (cols & (1u << slots[i])) return fail(OG_E_ARG, "slot %u joined twice", slots[i]);
    cols |= 1u << slots[i];
  }
  cudaStream_t s = e->s_main;
  if (cols & e->sb_dirty) {
    k_sb_clear_cols<<<grid_for(e->V + 1, e->sms), kThreads, 0, s>>>(e->sb_dist, e->V + 1, e->sb_ks,
                                                                   cols & e->sb_dirty);
    e->launches++;
  }
  e->sb_dirty |= cols;
  // the page-locked buffer is rewritten only after the previous upload ran
  CK(cudaStreamSynchronize(s));
  memcpy(e->sb_io_h, srcs, 4 * n);
  memcpy(e->sb_io_h + 32, slots, 4 * n);
  CK(cudaMemcpyAsync(e->sb_io_d, e->sb_io_h, 256, cudaMemcpyHostToDevice, s));
  k_sb_seed<<<1, 32, 0, s>>>(e->sb_io_d, e->sb_io_d + 32, n, e->sb_dist, e->sb_ks, e->sb_pend, e->bm[0],
                             e->V, e->err_d);
  e->launches++;
  CK(cudaGetLastError());
  return OG_OK;
}

// One round: compaction of the active set (or of the waiting set after a
// threshold advance) in both regions, then the relax of the listed near
// pairs.  *pending receives the slots that still have work as of this
// round's compaction (a slot outside it has final distances); *done is set
// when nothing is active or waiting.
template <class K>
int sb_round(og_engine *e, og_stats &st, Timing &tm, uint32_t *pending, bool *done) {
  *done = false;
  if (++e->epoch >= (1u << 30)) {  // epoch wrap: clear the status words and far keys once
    for (int r = 0; r < 2; r++)
      CK(cudaMemsetAsync(e->lb[r].status, 0, sizeof(uint32_t) * e->lb_tiles, e->s_main));
    CK(cudaMemsetAsync(e->counts_d + 2, 0, sizeof(Counts), e->s_main));
    e->epoch = 1;
  }
  const bool adv = e->sb_advance;
  uint32_t *bits = adv ? e->bm[2] : e->bm[0];
  // masks[0] is per round; masks[1] (slots waiting) accumulates until the
  // waiting set is scanned again
  CK(cudaMemsetAsync(e->sb_masks, 0, adv ? 8 : 4, e->s_main));
  CK(cudaEventRecord(e->ev_round, e->s_main));
  RC(launch_compact_sb(e, 0, bits, 0, e->Vs, adv, e->s_main));
  CK(cudaEventRecord(e->ev_cs, e->s_main));
  CK(cudaStreamWaitEvent(e->s_dyn, e->ev_round, 0));
  RC(launch_compact_sb(e, 1, bits, e->Vs, e->V, adv, e->s_dyn));
  CK(cudaEventRecord(e->ev_cd, e->s_dyn));
  CK(cudaStreamWaitEvent(e->s_dyn, e->ev_cs, 0));
  CK(cudaMemcpyAsync(e->counts_h, e->counts_d, 3 * sizeof(Counts), cudaMemcpyDeviceToHost, e->s_dyn));
  CK(cudaMemcpyAsync(e->sb_io_h + 64, e->sb_masks, 8, cudaMemcpyDeviceToHost, e->s_dyn));
  CK(cudaMemcpyAsync(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost, e->s_dyn));
  CK(cudaStreamSynchronize(e->s_dyn));
  collect_timing(e, tm, &st);
  float ms;
  if (cudaEventElapsedTime(&ms, e->ev_round, e->ev_cd) == cudaSuccess) st.ms_compact += ms;
  RC(check_device_error(e));
  *pending = e->sb_io_h[64] | e->sb_io_h[65];
  const uint32_t fm = std::min(far_of(e, 0), far_of(e, 1));
  e->sb_far_min = adv ? fm : std::min(e->sb_far_min, fm);
  const uint64_t n = (uint64_t)e->counts_h[0].n + e->counts_h[1].n;
  if (n == 0) {
    if (e->sb_far_min == 0xffffffffu) {
      *done = true;
      *pending = 0;
      return OG_OK;
    }
    const uint64_t t = (uint64_t)e->sb_far_min + e->sb_delta;
    e->sb_thr = t > 0xffffffffull ? 0xffffffffu : (uint32_t)t;
    e->sb_advance = true;
    return OG_OK;
  }
  e->sb_advance = false;
  st.iterations++;
  st.frontier_sum += n;
  st.static_vertices += e->counts_h[0].n;
  SbOp op{e->list_d[0], e->sb_lmask, e->sb_dist, e->sb_pend, e->bm[0], e->err_d, e->V, e->sb_ks};
  auto launch = [&](const LbsArgs &a, auto src, cudaStream_t ls) {
    const unsigned grid = lbs_grid(a.pos_begin, a.pos_end);
    if (grid) {
      using S = decltype(src);
      if (e->sb_ks == 4) k_sb_relax<S, 4><<<grid, kThreads, 0, ls>>>(a, src, op);
      else if (e->sb_ks == 8) k_sb_relax<S, 8><<<grid, kThreads, 0, ls>>>(a, src, op);
      else if (e->sb_ks == 16) k_sb_relax<S, 16><<<grid, kThreads, 0, ls>>>(a, src, op);
      else k_sb_relax<S, 32><<<grid, kThreads, 0, ls>>>(a, src, op);
      e->launches++;
    }
    return (int)OG_OK;
  };
  auto sfn = [&](const LbsArgs &a) { return launch(a, K::stat(e), e->s_main); };
  auto pfn = [&](const LbsArgs &a0, auto s0, const LbsArgs &a1, auto s1, cudaStream_t ps) {
    const uint64_t n0 = lbs_grid(a0.pos_begin, a0.pos_end), n1 = lbs_grid(a1.pos_begin, a1.pos_end);
    if (n0 + n1 > 0x7fffffffull) return fail(OG_E_STATE, "relax grid too large");
    using S0 = decltype(s0);
    using S1 = decltype(s1);
    const unsigned grid = (unsigned)(n0 + n1);
    if (e->sb_ks == 4) k_sb_relax_pair<S0, S1, 4><<<grid, kThreads, 0, ps>>>(a0, s0, a1, s1, op, n0, n0 + n1);
    else if (e->sb_ks == 8) k_sb_relax_pair<S0, S1, 8><<<grid, kThreads, 0, ps>>>(a0, s0, a1, s1, op, n0, n0 + n1);
    else if (e->sb_ks == 16) k_sb_relax_pair<S0, S1, 16><<<grid, kThreads, 0, ps>>>(a0, s0, a1, s1, op, n0, n0 + n1);
    else k_sb_relax_pair<S0, S1, 32><<<grid, kThreads, 0, ps>>>(a0, s0, a1, s1, op, n0, n0 + n1);
    e->launches++;
    return (int)OG_OK;
  };
  RC((run_regions<K>(e, st, tm, sfn, launch, pfn)));
  CK(cudaStreamWaitEvent(e->s_main, e->ev_cd, 0));
  CK(cudaGetLastError());
  return OG_OK;
}

int sb_round_any(og_engine *e, og_stats &st, Timing &tm, uint32_t *pending, bool *done) {
  if (e->wbytes == 1) return sb_round<EK<uint8_t>>(e, st, tm, pending, done);
  if (e->wbytes == 2) return sb_round<EK<uint16_t>>(e, st, tm, pending, done);
  return sb_round<EK<uint32_t>>(e, st, tm, pending, done);
}

// {reached, sum of distances} of every slot in cols, indexed by slot.
int sb_checks_impl(og_engine *e, uint32_t cols, uint64_t *out) {
  cudaStream_t s = e->s_main;
  CK(cudaMemsetAsync(e->sb_ck_d, 0, 16 * kSbMaxSources, s));
  k_sb_checks<<<(unsigned)e->sms * 4, kThreads, 0, s>>>(e->sb_dist, e->V, e->sb_ks, cols, e->sb_ck_d);
  e->launches++;
  CK(cudaMemcpyAsync(e->sb_ck_h, e->sb_ck_d, 16 * kSbMaxSources, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (uint32_t i = 0; i < 2 * kSbMaxSources; i++) out[i] = e->sb_ck_h[i];
  return OG_OK;
}

// Distances of slot `slot` into out (V entries of host memory), through the
// engine's value array.
int sb_fetch_impl(og_engine *e, uint32_t slot, uint32_t *out) {
  if (slot >= e->sb_k) return fail(OG_E_ARG, "slot %u >= %u", slot, e->sb_k);
  cudaStream_t s = e->s_main;
  k_sb_column<<<grid_for(e->V, e->sms), kThreads, 0, s>>>(e->sb_dist, e->V, e->sb_ks, slot, e->value_d);
  e->launches++;
  CK(cudaMemcpyAsync(out, e->value_d, 4ull * e->V, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  e->last_algo = -1;  // the value array holds no single-source result
  return OG_OK;
}

int run_sssp_batch(og_engine *e, const uint32_t *srcs, uint32_t n, uint32_t *out, uint64_t *checks,
                   og_stats &st) {
  RC(sb_reset(e));
  uint32_t slots[kSbMaxSources];
  for (uint32_t i = 0; i < n; i++) slots[i] = i;
  RC(sb_join_impl(e, srcs, slots, n));
  Timing tm;
  for (uint64_t r = 0;; r++) {
    uint32_t pending = 0;
    bool done = false;
    RC(sb_round_any(e, st, tm, &pending, &done));
    if (done) break;
    if (r > 16ull * e->V + 64) return fail(OG_E_STATE, "multi-source SSSP did not end after %llu rounds",
                                           (unsigned long long)r);
  }
  CK(cudaStreamSynchronize(e->s_main));
  collect_timing(e, tm, &st);
  CK(cudaMemcpy(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost));
  RC(check_device_error(e));
  if (checks) {
    uint64_t ck[2 * kSbMaxSources];
    RC(sb_checks_impl(e, (n >= 32 ? 0xffffffffu : (1u << n) - 1u), ck));
    for (uint32_t i = 0; i < 2 * n; i++) checks[i] = ck[i];
  }
  if (out)
    for (uint32_t i = 0; i < n; i++) RC(sb_fetch_impl(e, i, out + (uint64_t)i * e->V));
  e->last_algo = -1;
  return OG_OK;
}

// ------------------------------------------------------------------ PageRank

int pr_sums(og_engine *e, og_stats &st, Timing &tm) {
  PrArgs p;
  p.contrib = e->contrib_d;
  p.sum = e->sum_d;
  p.V = e->V;
  // static tiles use [0, tile_cap0), dynamic tiles [tile_cap0, ...)
  const uint64_t toff[2] = {0, e->tile_cap[0]};
  CK(cudaMemsetAsync(e->carry_idx_d, 0xff, 4 * e->pr_tiles, e->s_main));
  CK(cudaEventRecord(e->ev_round, e->s_main));
  CK(cudaStreamWaitEvent(e->s_dyn, e->ev_round, 0));
  CK(cudaStreamWaitEvent(e->s_gat, e->ev_round, 0));
  auto args_for = [&](int r) {
    PrArgs q = p;
    q.cont = e->cont_d + toff[r];
    q.carry = e->carry_d + toff[r];
    q.carry_idx = e->carry_idx_d + toff[r];
    return q;
  };
  auto sfn = [&](const LbsArgs &a) {
    const unsigned grid = lbs_grid(a.pos_begin, a.pos_end);
    if (grid) {
      k_pr_pull<EKU::PSrc><<<grid, kThreads, 0, e->s_main>>>(a, EKU::stat(e), args_for(0));
      e->launches++;
    }
    return (int)OG_OK;
  };
  auto dfn = [&](const LbsArgs &a, auto src, cudaStream_t ds) {
    const unsigned grid = lbs_grid(a.pos_begin, a.pos_end);
    if (grid) {
      k_pr_pull<decltype(src)><<<grid, kThreads, 0, ds>>>(a, src, args_for(1));
      e->launches++;
    }
    return (int)OG_OK;
  };
  auto pfn = [&](const LbsArgs &a0, auto s0, const LbsArgs &a1, auto s1, cudaStream_t ps) {
    const uint64_t n0 = lbs_grid(a0.pos_begin, a0.pos_end), n1 = lbs_grid(a1.pos_begin, a1.pos_end);
    if (n0 + n1 > 0x7fffffffull) return fail(OG_E_STATE, "pull grid too large");
    k_pr_pull_pair<decltype(s0), decltype(s1)><<<(unsigned)(n0 + n1), kThreads, 0, ps>>>(
        a0, s0, args_for(0), a1, s1, args_for(1), n0, n0 + n1);
    e->launches++;
    return (int)OG_OK;
  };
  RC((run_regions<EKU>(e, st, tm, sfn, dfn, pfn)));
  for (int r = 0; r < 2; r++) {
    const Counts c = e->counts_h[r];
    if (!c.n) continue;
    const uint64_t nt = (c.total + kTile - 1) / kTile;
    k_pr_fixup<<<(unsigned)((nt + kThreads - 1) / kThreads), kThreads, 0, e->s_main>>>(
        e->list_d[r], e->pref_d[r], 0, nt, args_for(r));
    e->launches++;
  }
  CK(cudaGetLastError());
  return OG_OK;
}

int run_pr_delta(og_engine *e, float thresh, int max_rounds, og_stats &st) {
  const uint64_t V = e->V;
  uint32_t *cur = e->bm[0], *next = e->bm[1];
  cudaStream_t s = e->s_main;
  const int g = grid_for(V, e->sms);
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  k_pr_init<<<g, kThreads, 0, s>>>(V, (float *)e->value_d, e->contrib_d, e->sum_d, e->outdeg_d,
                                   1.0f);  // PR/OneGraph/GraphMeta.h:354-357
  k_fill_bits<<<g, kThreads, 0, s>>>(cur, e->nwords, V);
  e->launches += 2;
  CK(cudaGetLastError());
  Timing tm;
  for (int round = 0; max_rounds <= 0 || round < max_rounds; round++) {
    uint64_t n = 0;
    RC(compact_round(e, cur, st, tm, &n));
    st.iterations++;
    st.frontier_sum += n;
    st.static_vertices += e->counts_h[0].n;
    RC(pr_sums(e, st, tm));
    CK(cudaMemsetAsync(e->active_d, 0, 4, s));
    k_pr_update_delta<<<grid_for(e->nwords, e->sms), kThreads, 0, s>>>(
        cur, next, e->nwords, (float *)e->value_d, e->contrib_d, e->sum_d, e->outdeg_d, thresh,
        e->active_d);
    e->launches++;
    CK(cudaMemcpyAsync(e->err_h, e->err_d, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    RC(check_device_error(e));
    std::swap(cur, next);
    if (e->err_h[1] == 0) break;
  }
  CK(cudaStreamSynchronize(s));
  collect_timing(e, tm, &st);
  e->last_algo = OG_ALGO_PR;
  return OG_OK;
}

int run_pr_l1(og_engine *e, float damping, double tol, int max_iter, og_stats &st) {
  const uint64_t V = e->V;
  uint32_t *cur = e->bm[0];
  cudaStream_t s = e->s_main;
  const int g = grid_for(V, e->sms);
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  k_pr_init<<<g, kThreads, 0, s>>>(V, (float *)e->value_d, e->contrib_d, e->sum_d, e->outdeg_d,
                                   (float)(1.0 / (double)V));
  e->launches++;
  k_fill_bits<<<g, kThreads, 0, s>>>(cur, e->nwords, V);
  e->launches++;
  CK(cudaGetLastError());
  Timing tm;
  uint64_t n = 0;
  RC(compact_round(e, cur, st, tm, &n));  // every vertex with in-edges, once
  const float teleport = (float)((1.0 - (double)damping) / (double)V);
  for (int it = 0; it < max_iter; it++) {
    st.iterations++;
    st.frontier_sum += n;
    st.static_vertices += e->counts_h[0].n;
    RC(pr_sums(e, st, tm));
    k_pr_update_l1<<<e->part_n, kThreads, 0, s>>>(V, (float *)e->value_d, e->contrib_d, e->sum_d,
                                                  e->outdeg_d, teleport, damping, e->part_d);
    e->launches++;
    k_reduce_f64<<<1, kThreads, 0, s>>>(e->part_d, e->part_n, e->l1_d);
    e->launches++;
    CK(cudaMemcpyAsync(e->l1_h, e->l1_d, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    RC(check_device_error(e));
    collect_timing(e, tm, &st);
    st.residual = *e->l1_h;
    if (*e->l1_h < tol) break;
  }
  e->last_algo = OG_ALGO_PR;
  return OG_OK;
}

// og_pr_l1_push: the graph holds out-edges; sums by scattered atomic adds.
int run_pr_l1_push(og_engine *e, float damping, double tol, int max_iter, og_stats &st) {
  const uint64_t V = e->V;
  uint32_t *cur = e->bm[0];
  cudaStream_t s = e->s_main;
  const int g = grid_for(V, e->sms);
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  k_pr_init<<<g, kThreads, 0, s>>>(V, (float *)e->value_d, e->contrib_d, e->sum_d, e->outdeg_d,
                                   (float)(1.0 / (double)V));
  e->launches++;
  k_fill_bits<<<g, kThreads, 0, s>>>(cur, e->nwords, V);
  e->launches++;
  CK(cudaGetLastError());
  Timing tm;
  uint64_t n = 0;
  RC(compact_round(e, cur, st, tm, &n));  // every vertex with out-edges, once
  const float teleport = (float)((1.0 - (double)damping) / (double)V);
  const PushOp op{e->contrib_d, e->sum_d, e->err_d, (uint32_t)V};
  auto launch = [&](const LbsArgs &a, auto src, cudaStream_t ls) {
    const unsigned grid = lbs_grid(a.pos_begin, a.pos_end);
    if (grid) {
      k_lbs<decltype(src), PushOp><<<grid, kThreads, 0, ls>>>(a, src, op);
      e->launches++;
    }
    return (int)OG_OK;
  };
  auto sfn = [&](const LbsArgs &a) { return launch(a, EKU::stat(e), e->s_main); };
  auto pfn = [&](const LbsArgs &a0, auto s0, const LbsArgs &a1, auto s1, cudaStream_t ps) {
    const uint64_t n0 = lbs_grid(a0.pos_begin, a0.pos_end), n1 = lbs_grid(a1.pos_begin, a1.pos_end);
    if (n0 + n1 > 0x7fffffffull) return fail(OG_E_STATE, "push grid too large");
    k_lbs_pair<decltype(s0), decltype(s1), PushOp><<<(unsigned)(n0 + n1), kThreads, 0, ps>>>(a0, s0, a1, s1, op,
                                                                                        n0, n0 + n1);
    e->launches++;
    return (int)OG_OK;
  };
  for (int it = 0; it < max_iter; it++) {
    st.iterations++;
    st.frontier_sum += n;
    st.static_vertices += e->counts_h[0].n;
    CK(cudaMemsetAsync(e->sum_d, 0, 4 * V, s));
    RC((run_regions<EKU>(e, st, tm, sfn, launch, pfn)));
    k_pr_update_l1<<<e->part_n, kThreads, 0, s>>>(V, (float *)e->value_d, e->contrib_d, e->sum_d,
                                                  e->outdeg_d, teleport, damping, e->part_d);
    e->launches++;
    k_reduce_f64<<<1, kThreads, 0, s>>>(e->part_d, e->part_n, e->l1_d);
    e->launches++;
    CK(cudaMemcpyAsync(e->l1_h, e->l1_d, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    RC(check_device_error(e));
    collect_timing(e, tm, &st);
    st.residual = *e->l1_h;
    if (*e->l1_h < tol) break;
  }
  e->last_algo = OG_ALGO_PR;
  return OG_OK;
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

int fetch(og_engine *e, void *out) {
  CK(cudaSetDevice(e->dev));
  CK(cudaMemcpyAsync(out, e->value_d, 4ull * e->V, cudaMemcpyDeviceToHost, e->s_main));
  CK(cudaStreamSynchronize(e->s_main));
  return OG_OK;
}

template <class F>
int guarded(F f) {
  try {
    return f();
  } catch (const std::bad_alloc &) {
    return fail(OG_E_NOMEM, "host allocation failed");
  } catch (...) {
    return fail(OG_E_STATE, "unexpected exception");
  }
}

int query_common(og_engine *e, int algo, og_stats *st_out, void *out,
                 int (*body)(og_engine *, og_stats &, void *), void *ctx) {
  if (!e) return fail(OG_E_ARG, "null engine");
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    cudaGetLastError();  // drop a stale error left by an unrelated earlier call
    og_stats st;
    memset(&st, 0, sizeof st);
    e->launches = 0;
    // every query reuses the frontier bitmaps, lists and arena of an open
    // multi-source SSSP or batched BFS session: the session ends here
    e->sb_session = false;
    e->bb_session = false;
    const double t0 = now_ms();
    RC(body(e, st, ctx));
    st.launches = e->launches;
    if (out) RC(fetch(e, out));
    st.ms_total = now_ms() - t0;
    if (st_out) *st_out = st;
    (void)algo;
    return OG_OK;
  });
}

}  // namespace

// ====================================================================== C ABI

extern "C" int og_engine_create(og_graph *g, const og_config *cfg, og_engine **out) {
  clear_error();
  if (!g || !out) return fail(OG_E_ARG, "og_engine_create: null argument");
  *out = nullptr;
  og_config c;
  memset(&c, 0, sizeof c);
  if (cfg) c = *cfg;
  return guarded([&]() -> int {
    og_engine *e = new og_engine;
    int rc = create(g, &c, e);
    if (rc != OG_OK) {
      std::string keep = og_last_error();
      destroy(e);
      return fail(rc, "%s", keep.c_str());
    }
    *out = e;
    return OG_OK;
  });
}

extern "C" int og_engine_clone(og_engine *parent, og_engine **out) {
  clear_error();
  if (!parent || !out) return fail(OG_E_ARG, "og_engine_clone: null argument");
  if (parent->parent) return fail(OG_E_ARG, "og_engine_clone: clone a parent engine, not a clone");
  if (parent->frag) return fail(OG_E_UNSUPPORTED, "og_engine_clone: an OG_CFG_REPLACE engine has no clones");
  *out = nullptr;
  return guarded([&]() -> int {
    og_engine *e = new og_engine;
    int rc = clone(parent, e);
    if (rc != OG_OK) {
      std::string keep = og_last_error();
      destroy(e);
      return fail(rc, "%s", keep.c_str());
    }
    *out = e;
    return OG_OK;
  });
}

extern "C" int og_engine_set_param(og_engine *e, int param, double value) {
  if (!e) return fail(OG_E_ARG, "og_engine_set_param: null engine");
  if (param == OG_PARAM_SSSP_DELTA) {
    if (value < 0 || value > 4294967295.0) return fail(OG_E_ARG, "delta out of range");
    e->sssp_delta = (uint32_t)value;
    return OG_OK;
  }
  if (param == OG_PARAM_CC_METHOD) {
    if (value != OG_CC_AUTO && value != OG_CC_LABEL_PROPAGATION && value != OG_CC_UNION_FIND)
      return fail(OG_E_ARG, "unknown CC method %g", value);
    e->cc_method = (uint32_t)value;
    return OG_OK;
  }
  if (param == OG_PARAM_BFS_DIRECTION) {
    if (value != OG_BFS_AUTO && value != OG_BFS_TOP_DOWN) return fail(OG_E_ARG, "unknown BFS direction %g", value);
    e->bfs_direction = (uint32_t)value;
    return OG_OK;
  }
  if (param == OG_PARAM_LEVEL_LOOP) {
    if (value != OG_LOOP_AUTO && value != OG_LOOP_HOST) return fail(OG_E_ARG, "unknown level loop %g", value);
    e->level_loop = (uint32_t)value;
    return OG_OK;
  }
  if (param == OG_PARAM_RELAX_TIMER) {
    if (value != 0 && value != 1) return fail(OG_E_ARG, "relax timer must be 0 or 1, not %g", value);
    e->relax_timer = (uint32_t)value;
    return OG_OK;
  }
  if (param == OG_PARAM_SSSP_BATCH_DELTA) {
    if (value < 0 || value > 4294967295.0) return fail(OG_E_ARG, "delta out of range");
    e->sb_delta = (uint32_t)value;
    return OG_OK;
  }
  if (param == OG_PARAM_FRAGMENT_WORDS) {
    if (!e->frag) return fail(OG_E_STATE, "fragment words: the engine was created without OG_CFG_REPLACE");
    uint32_t fs = 8;
    while (fs <= 20 && (double)(1u << fs) != value) fs++;
    if (fs > 20) return fail(OG_E_ARG, "fragment words must be a power of two in [2^8, 2^20], not %g", value);
    return guarded([&]() -> int {
      CK(cudaSetDevice(e->dev));
      CK(cudaStreamSynchronize(e->s_main));
      CK(cudaStreamSynchronize(e->s_dyn));
      RC(frag_layout(e, fs));  // checks the fit before releasing the old layout
      RC(frag_reset(e));
      CK(cudaStreamSynchronize(e->s_main));
      return (int)OG_OK;
    });
  }
  return fail(OG_E_ARG, "unknown parameter %d", param);
}

extern "C" int og_engine_get_param(const og_engine *e, int param, double *value) {
  if (!e || !value) return fail(OG_E_ARG, "og_engine_get_param: null argument");
  if (param == OG_PARAM_SSSP_DELTA) {
    *value = e->sssp_delta;
    return OG_OK;
  }
  if (param == OG_PARAM_CC_METHOD) {
    *value = e->cc_method;
    return OG_OK;
  }
  if (param == OG_PARAM_BFS_DIRECTION) {
    *value = e->bfs_direction;
    return OG_OK;
  }
  if (param == OG_PARAM_LEVEL_LOOP) {
    *value = e->level_loop;
    return OG_OK;
  }
  if (param == OG_PARAM_RELAX_TIMER) {
    *value = e->relax_timer;
    return OG_OK;
  }
  if (param == OG_PARAM_SSSP_BATCH_DELTA) {
    *value = e->sb_delta;
    return OG_OK;
  }
  if (param == OG_PARAM_FRAGMENT_WORDS) {
    if (!e->frag) return fail(OG_E_STATE, "fragment words: the engine was created without OG_CFG_REPLACE");
    *value = (double)(1u << e->frag->fs);
    return OG_OK;
  }
  return fail(OG_E_ARG, "unknown parameter %d", param);
}

extern "C" int og_engine_fragment_stats(const og_engine *e, og_fragment_stats *out) {
  if (!e || !out) return fail(OG_E_ARG, "og_engine_fragment_stats: null argument");
  if (!e->frag) return fail(OG_E_STATE, "the engine was created without OG_CFG_REPLACE");
  *out = e->frag->st;
  return OG_OK;
}

extern "C" int og_engine_bytes(const og_engine *e, uint64_t *resident, uint64_t *context) {
  if (!e) return fail(OG_E_ARG, "og_engine_bytes: null engine");
  if (resident) *resident = e->parent ? 0 : e->resident_bytes;
  if (context) *context = e->parent ? e->dbytes : e->dbytes - e->resident_bytes;
  return OG_OK;
}

extern "C" int og_engine_plan(const og_engine *e, og_plan *out) {
  if (!e || !out) return fail(OG_E_ARG, "og_engine_plan: null argument");
  *out = e->plan;
  return OG_OK;
}

extern "C" void og_engine_destroy(og_engine *e) { destroy(e); }

extern "C" int og_bfs(og_engine *e, uint32_t src, uint32_t *out_depth, og_stats *st) {
  if (e && src >= e->V) return fail(OG_E_ARG, "source %u >= V %u", src, e->V);
  return query_common(e, OG_ALGO_BFS, st, out_depth, [](og_engine *en, og_stats &s, void *c) {
    const uint32_t src_ = *(uint32_t *)c;
    if (en->frag && en->frag->broken)
      return fail(OG_E_STATE, "the fragment slots were not laid out (a failed OG_PARAM_FRAGMENT_WORDS change)");
    if (en->frag) return run_frontier<EKF<void>>(en, OG_ALGO_BFS, src_, s);
    // the device-driven loop needs no staging pipeline: direct mode or a
    // fully resident graph
    const bool dev = en->level_loop == OG_LOOP_AUTO &&
                     (en->plan.dynamic_edges == 0 || (en->cfg.flags & OG_CFG_DIRECT));
    return dev ? run_bfs_dev(en, src_, s) : run_frontier<EKU>(en, OG_ALGO_BFS, src_, s);
  }, &src);
}

extern "C" int og_sssp(og_engine *e, uint32_t src, uint32_t *out_dist, og_stats *st) {
  if (e && src >= e->V) return fail(OG_E_ARG, "source %u >= V %u", src, e->V);
  if (e && e->g->kind != OG_GRAPH_WEIGHTED) return fail(OG_E_UNSUPPORTED, "SSSP needs a weighted graph");
  return query_common(e, OG_ALGO_SSSP, st, out_dist, [](og_engine *en, og_stats &s, void *c) {
    const uint32_t src_ = *(uint32_t *)c;
    if (en->frag && en->frag->broken)
      return fail(OG_E_STATE, "the fragment slots were not laid out (a failed OG_PARAM_FRAGMENT_WORDS change)");
    if (en->frag) return run_frontier<EKF<uint8_t>>(en, OG_ALGO_SSSP, src_, s);
    if (en->level_loop == OG_LOOP_AUTO && (en->plan.dynamic_edges == 0 || (en->cfg.flags & OG_CFG_DIRECT)))
      return run_min_dev(en, OG_ALGO_SSSP, src_, s);
    if (en->wbytes == 1) return run_frontier<EK<uint8_t>>(en, OG_ALGO_SSSP, src_, s);
    if (en->wbytes == 2) return run_frontier<EK<uint16_t>>(en, OG_ALGO_SSSP, src_, s);
    return run_frontier<EK<uint32_t>>(en, OG_ALGO_SSSP, src_, s);
  }, &src);
}

// ------------------------------------------------------------ union-find CC
//
// Symmetric graphs only (the result equals label propagation's there): two
// sampling passes over every vertex's first two edges, compression, the giant
// component picked from 1024 sampled roots, then one edge-balanced pass over
// the edges of the vertices outside it (both regions, interleaved), and a
// final compression.  parent[] lives in value_d and ends as the labels.
int run_cc_uf(og_engine *e, og_stats &st) {
  const uint32_t V = e->V;
  cudaStream_t s = e->s_main;
  const int g = grid_for(V, e->sms);
  uint32_t *par = e->value_d;
  unsigned long long *reads = e->sum64_d;  // [0] host records, [1] static records
  uint32_t *roots_d = (uint32_t *)(e->sum64_d + 2);
  constexpr uint32_t kRoots = 1024;
  CK(cudaMemsetAsync(e->err_d, 0, 16, s));
  CK(cudaMemsetAsync(reads, 0, 16, s));
  k_iota_u32<<<g, kThreads, 0, s>>>(par, V);
  e->launches++;
  cudaEvent_t t0 = e->t_d0, t1 = e->ev_dyn_done;
  CK(cudaEventRecord(t0, s));
  for (uint32_t r = 0; r < 2; r++) {
    k_uf_sample<EKU::PSrc><<<g, kThreads, 0, s>>>(e->off_d, V, e->plan.static_edges, EKU::stat(e),
                                                  EKU::host(e), r, par, reads, e->err_d);
    k_uf_compress<<<g, kThreads, 0, s>>>(par, V, e->err_d);
    e->launches += 2;
    st.iterations++;
  }
  k_uf_roots<<<(kRoots + kThreads - 1) / kThreads, kThreads, 0, s>>>(par, V, kRoots, roots_d);
  e->launches++;
  CK(cudaEventRecord(t1, s));
  std::vector<uint32_t> roots(kRoots);
  unsigned long long rd[2] = {0, 0};
  CK(cudaMemcpyAsync(roots.data(), roots_d, 4 * kRoots, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(rd, reads, 16, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  float ms = 0;
  if (cudaEventElapsedTime(&ms, t0, t1) == cudaSuccess) st.ms_dynamic += ms;
  st.link_bytes += (rd[0] * e->bpe + 7) / 8;
  st.edges_dynamic += rd[0];
  st.edges_static += rd[1];
  std::sort(roots.begin(), roots.end());
  uint32_t c = roots[0], best = 0;
  for (uint32_t i = 0; i < kRoots;) {
    uint32_t j = i;
    while (j < kRoots && roots[j] == roots[i]) j++;
    if (j - i > best) {
      best = j - i;
      c = roots[i];
    }
    i = j;
  }
  // final pass over the vertices outside c
  uint32_t *cur = e->bm[0];
  k_uf_mark<<<grid_for(e->nwords * 32, e->sms), kThreads, 0, s>>>(e->off_d, par, V, c, cur, e->nwords);
  e->launches++;
  Timing tm;
  uint64_t n = 0;
  RC(compact_round(e, cur, st, tm, &n));
  if (n) {
    st.iterations++;
    st.frontier_sum += n;
    st.static_vertices += e->counts_h[0].n;
    UnionOp op{par, e->err_d, V};
    auto launch = [&](const LbsArgs &a, auto src, cudaStream_t ls) {
      const unsigned grid = lbs_grid(a.pos_begin, a.pos_end);
      if (grid) {
        k_lbs<decltype(src), UnionOp><<<grid, kThreads, 0, ls>>>(a, src, op);
        e->launches++;
      }
      return (int)OG_OK;
    };
    auto sfn = [&](const LbsArgs &a) { return launch(a, EKU::stat(e), e->s_main); };
    auto pfn = [&](const LbsArgs &a0, auto s0, const LbsArgs &a1, auto s1, cudaStream_t ps) {
      const uint64_t n0 = lbs_grid(a0.pos_begin, a0.pos_end), n1 = lbs_grid(a1.pos_begin, a1.pos_end);
      if (n0 + n1 > 0x7fffffffull) return fail(OG_E_STATE, "relax grid too large");
      k_lbs_pair<decltype(s0), decltype(s1), UnionOp><<<(unsigned)(n0 + n1), kThreads, 0, ps>>>(
          a0, s0, a1, s1, op, n0, n0 + n1);
      e->launches++;
      return (int)OG_OK;
    };
    RC((run_regions<EKU>(e, st, tm, sfn, launch, pfn)));
    CK(cudaStreamWaitEvent(e->s_main, e->ev_cd, 0));
  }
  k_uf_compress<<<g, kThreads, 0, s>>>(par, V, e->err_d);
  e->launches++;
  CK(cudaStreamSynchronize(s));
  collect_timing(e, tm, &st);
  CK(cudaMemcpy(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost));
  RC(check_device_error(e));
  e->last_algo = OG_ALGO_CC;
  return OG_OK;
}

extern "C" int og_cc(og_engine *e, uint32_t *out_label, og_stats *st) {
  uint32_t dummy = 0;
  return query_common(e, OG_ALGO_CC, st, out_label, [](og_engine *en, og_stats &s, void *) {
    const bool uf = en->cc_method == OG_CC_UNION_FIND ||
                    (en->cc_method == OG_CC_AUTO && en->g->symmetric == 1);
    if (en->cc_method == OG_CC_UNION_FIND && en->g->symmetric != 1)
      return fail(OG_E_ARG, "union-find CC needs a graph known to be symmetric (og_graph_symmetric)");
    if (uf) return run_cc_uf(en, s);
    if (en->frag && en->frag->broken)
      return fail(OG_E_STATE, "the fragment slots were not laid out (a failed OG_PARAM_FRAGMENT_WORDS change)");
    if (en->frag) return run_frontier<EKF<void>>(en, OG_ALGO_CC, 0, s);
    if (en->level_loop == OG_LOOP_AUTO && (en->plan.dynamic_edges == 0 || (en->cfg.flags & OG_CFG_DIRECT)))
      return run_min_dev(en, OG_ALGO_CC, 0, s);
    return run_frontier<EKU>(en, OG_ALGO_CC, 0, s);
  }, &dummy);
}

namespace {
struct PrCtx {
  double a, b;
  int n;
};
}  // namespace

extern "C" int og_pr(og_engine *e, float *out_rank, double threshold, int max_rounds, og_stats *st) {
  if (e && !e->pr_enabled) return fail(OG_E_UNSUPPORTED, "engine has no PageRank state (OG_CFG_PR)");
  PrCtx c{threshold, 0, max_rounds};
  return query_common(e, OG_ALGO_PR, st, out_rank, [](og_engine *en, og_stats &s, void *cx) {
    const PrCtx &p = *(PrCtx *)cx;
    return run_pr_delta(en, (float)p.a, p.n, s);
  }, &c);
}

extern "C" int og_pr_l1(og_engine *e, float *out_rank, double damping, double tol, int max_iter,
                        og_stats *st) {
  if (e && !e->pr_enabled) return fail(OG_E_UNSUPPORTED, "engine has no PageRank state (OG_CFG_PR)");
  if (max_iter <= 0) return fail(OG_E_ARG, "max_iter must be positive");
  PrCtx c{damping, tol, max_iter};
  return query_common(e, OG_ALGO_PR, st, out_rank, [](og_engine *en, og_stats &s, void *cx) {
    const PrCtx &p = *(PrCtx *)cx;
    return run_pr_l1(en, (float)p.a, p.b, p.n, s);
  }, &c);
}

extern "C" int og_pr_l1_push(og_engine *e, float *out_rank, double damping, double tol, int max_iter,
                             og_stats *st) {
  if (e && !e->pr_enabled) return fail(OG_E_UNSUPPORTED, "engine has no PageRank state (OG_CFG_PR)");
  if (max_iter <= 0) return fail(OG_E_ARG, "max_iter must be positive");
  PrCtx c{damping, tol, max_iter};
  return query_common(e, OG_ALGO_PR, st, out_rank, [](og_engine *en, og_stats &s, void *cx) {
    const PrCtx &p = *(PrCtx *)cx;
    return run_pr_l1_push(en, (float)p.a, p.b, p.n, s);
  }, &c);
}

namespace {
struct BatchCtx {
  const uint32_t *srcs;
  uint32_t n;
  uint32_t *out;
  uint64_t *checks;
  int mode;  // 0 persistent (tuned configuration), 1 host-driven levels, 2+k persistent config k
  uint8_t *out8 = nullptr;  // og_bfs_batch_u8
  uint64_t *clamped = nullptr;
  uint32_t *const *outs = nullptr;  // og_bfs_batch_to
};

int batch_body(og_engine *en, og_stats &s, void *cx) {
  const BatchCtx &b = *(BatchCtx *)cx;
  if (b.mode == 1) return run_batch(en, b.srcs, b.n, b.out, b.checks, s);
  const int ci = b.mode >= 2 ? b.mode - 2 : (en->tuned >= 0 ? en->tuned : 0);
  if (b.out8) return run_batch_persist(en, b.srcs, b.n, b.out8, 1, b.clamped, b.checks, s, ci);
  return run_batch_persist(en, b.srcs, b.n, b.out, 4, nullptr, b.checks, s, ci, b.outs);
}

int batch_checks(og_engine *e, const uint32_t *srcs, int n) {
  if (!e || !srcs) return fail(OG_E_ARG, "og_bfs_batch: null argument");
  if (n < 1 || n > 64) return fail(OG_E_ARG, "og_bfs_batch: %d sources (1..64)", n);
  if (!e->batch_enabled) return fail(OG_E_UNSUPPORTED, "engine created without OG_CFG_BATCH");
  for (int i = 0; i < n; i++)
    if (srcs[i] >= e->V) return fail(OG_E_ARG, "source %u >= V %u", srcs[i], e->V);
  return OG_OK;
}
}  // namespace

extern "C" int og_bfs_batch(og_engine *e, const uint32_t *srcs, int n, uint32_t *out,
                            uint64_t *checks, og_stats *st) {
  RC(batch_checks(e, srcs, n));
  BatchCtx c{srcs, (uint32_t)n, out, checks, (e->cfg.flags & OG_CFG_BATCH_LEVELS) ? 1 : 0};
  return query_common(e, OG_ALGO_BFS, st, nullptr, batch_body, &c);
}

extern "C" int og_bfs_batch_to(og_engine *e, const uint32_t *srcs, int n, uint32_t *const *outs,
                               uint64_t *checks, og_stats *st) {
  RC(batch_checks(e, srcs, n));
  if (!outs) return fail(OG_E_ARG, "og_bfs_batch_to: null output list");
  for (int i = 0; i < n; i++)
    if (!outs[i]) return fail(OG_E_ARG, "og_bfs_batch_to: output %d is null", i);
  if (e->cfg.flags & OG_CFG_BATCH_LEVELS)
    return fail(OG_E_UNSUPPORTED, "og_bfs_batch_to runs the persistent kernel (engine has OG_CFG_BATCH_LEVELS)");
  BatchCtx c{srcs, (uint32_t)n, nullptr, checks, 0};
  c.outs = outs;
  return query_common(e, OG_ALGO_BFS, st, nullptr, batch_body, &c);
}

extern "C" int og_bfs_batch_u8(og_engine *e, const uint32_t *srcs, int n, uint8_t *out, uint64_t *clamped,
                               uint64_t *checks, og_stats *st) {
  RC(batch_checks(e, srcs, n));
  if (!out) return fail(OG_E_ARG, "og_bfs_batch_u8: null output");
  BatchCtx c{srcs, (uint32_t)n, nullptr, checks, 0, out, clamped};
  return query_common(e, OG_ALGO_BFS, st, nullptr, batch_body, &c);
}

extern "C" int og_host_alloc(uint64_t bytes, void **out) {
  clear_error();
  if (!out || bytes == 0) return fail(OG_E_ARG, "og_host_alloc: bad argument");
  *out = nullptr;
  CK(cudaHostAlloc(out, bytes, cudaHostAllocPortable));
  return OG_OK;
}

extern "C" void og_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

extern "C" int og_bfs_batch_tune(og_engine *e, const uint32_t *srcs, int n, int reps,
                                 og_tune_result *res) {
  RC(batch_checks(e, srcs, n));
  if (reps < 1) reps = 1;
  og_tune_result r;
  memset(&r, 0, sizeof r);
  r.configs = kNumPersistConfigs;
  float best = 1e30f;
  for (int i = 0; i < kNumPersistConfigs; i++) {
    r.block[i] = kPersistConfigs[i].block;
    r.items[i] = kPersistConfigs[i].items;
    float tmin = 1e30f;
    for (int k = 0; k <= reps; k++) {  // the first run warms up
      og_stats st{};
      BatchCtx c{srcs, (uint32_t)n, nullptr, nullptr, 2 + i};
      RC(query_common(e, OG_ALGO_BFS, &st, nullptr, batch_body, &c));
      if (k > 0) tmin = std::min(tmin, (float)st.ms_static);
    }
    r.ms[i] = tmin;
    if (tmin < best) {
      best = tmin;
      r.best = i;
    }
  }
  e->tuned = r.best;
  if (res) *res = r;
  return OG_OK;
}

extern "C" int og_bfs_batch_set_config(og_engine *e, int config) {
  if (!e) return fail(OG_E_ARG, "null engine");
  if (config < -1 || config >= kNumPersistConfigs) return fail(OG_E_ARG, "config %d out of range", config);
  e->tuned = config;
  return OG_OK;
}

extern "C" int og_sssp_batch(og_engine *e, const uint32_t *srcs, int n, uint32_t *out, uint64_t *checks,
                             og_stats *st) {
  if (!e || !srcs) return fail(OG_E_ARG, "og_sssp_batch: null argument");
  if (e->g->kind != OG_GRAPH_WEIGHTED) return fail(OG_E_UNSUPPORTED, "SSSP needs a weighted graph");
  if (!e->sb_k) return fail(OG_E_STATE, "engine created without OG_CFG_SSSP_BATCH");
  if (n < 1 || n > (int)e->sb_k) return fail(OG_E_ARG, "n = %d, the engine holds 1..%u sources", n, e->sb_k);
  for (int i = 0; i < n; i++)
    if (srcs[i] >= e->V) return fail(OG_E_ARG, "source %u >= V %u", srcs[i], e->V);
  struct Ctx {
    const uint32_t *srcs;
    uint32_t n;
    uint32_t *out;
    uint64_t *checks;
  } c{srcs, (uint32_t)n, out, checks};
  return query_common(e, OG_ALGO_SSSP, st, nullptr, [](og_engine *en, og_stats &s, void *cx) {
    Ctx &q = *(Ctx *)cx;
    return run_sssp_batch(en, q.srcs, q.n, q.out, q.checks, s);
  }, &c);
}

extern "C" int og_sssp_batch_begin(og_engine *e) {
  if (!e) return fail(OG_E_ARG, "null engine");
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    e->launches = 0;
    return sb_reset(e);
  });
}

extern "C" int og_sssp_batch_join(og_engine *e, const uint32_t *srcs, const uint32_t *slots, int n) {
  if (!e || n < 0 || (n && (!srcs || !slots))) return fail(OG_E_ARG, "og_sssp_batch_join: bad argument");
  if (!e->sb_k) return fail(OG_E_STATE, "engine created without OG_CFG_SSSP_BATCH");
  if (!e->sb_session)
    return fail(OG_E_STATE, "no open multi-source SSSP session: og_sssp_batch_begin first (any other query on "
                            "the engine ends a session)");
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    return sb_join_impl(e, srcs, slots, (uint32_t)n);
  });
}

extern "C" int og_sssp_batch_step(og_engine *e, uint32_t *pending, int *done, og_stats *st) {
  if (!e || !pending || !done) return fail(OG_E_ARG, "og_sssp_batch_step: null argument");
  if (!e->sb_k) return fail(OG_E_STATE, "engine created without OG_CFG_SSSP_BATCH");
  if (!e->sb_session)
    return fail(OG_E_STATE, "no open multi-source SSSP session: og_sssp_batch_begin first (any other query on "
                            "the engine ends a session)");
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    og_stats s;
    memset(&s, 0, sizeof s);
    const uint64_t l0 = e->launches;
    const double t0 = now_ms();
    Timing tm;
    bool d = false;
    RC(sb_round_any(e, s, tm, pending, &d));
    CK(cudaStreamSynchronize(e->s_main));
    collect_timing(e, tm, &s);
    CK(cudaMemcpy(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost));
    RC(check_device_error(e));
    s.launches = e->launches - l0;
    s.ms_total = now_ms() - t0;
    if (st) *st = s;
    *done = d ? 1 : 0;
    e->last_algo = -1;
    return OG_OK;
  });
}

extern "C" int og_sssp_batch_checks(og_engine *e, uint32_t slots, uint64_t *out) {
  if (!e || !out) return fail(OG_E_ARG, "og_sssp_batch_checks: null argument");
  if (!e->sb_k) return fail(OG_E_STATE, "engine created without OG_CFG_SSSP_BATCH");
  if (!e->sb_session)
    return fail(OG_E_STATE, "no open multi-source SSSP session: og_sssp_batch_begin first (any other query on "
                            "the engine ends a session)");
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    return sb_checks_impl(e, slots, out);
  });
}

extern "C" int og_sssp_batch_fetch(og_engine *e, uint32_t slot, uint32_t *out) {
  if (!e || !out) return fail(OG_E_ARG, "og_sssp_batch_fetch: null argument");
  if (!e->sb_k) return fail(OG_E_STATE, "engine created without OG_CFG_SSSP_BATCH");
  if (!e->sb_session)
    return fail(OG_E_STATE, "no open multi-source SSSP session: og_sssp_batch_begin first (any other query on "
                            "the engine ends a session)");
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    return sb_fetch_impl(e, slot, out);
  });
}

namespace {
int bb_session_ok(og_engine *e) {
  if (!e->batch_enabled) return fail(OG_E_UNSUPPORTED, "engine created without OG_CFG_BATCH");
  if (!e->bb_session)
    return fail(OG_E_STATE, "no open batched BFS session: og_bfs_batch_begin first (any other query on the "
                            "engine ends a session)");
  return OG_OK;
}
}  // namespace

extern "C" int og_bfs_batch_begin(og_engine *e, int record_depths) {
  if (!e) return fail(OG_E_ARG, "null engine");
  if (!e->batch_enabled) return fail(OG_E_UNSUPPORTED, "engine created without OG_CFG_BATCH");
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    cudaGetLastError();
    e->launches = 0;
    e->last_algo = -1;
    return bb_begin_impl(e, record_depths != 0);
  });
}

extern "C" int og_bfs_batch_join(og_engine *e, const uint32_t *srcs, const uint32_t *slots, int n) {
  if (!e || n < 0 || (n && (!srcs || !slots))) return fail(OG_E_ARG, "og_bfs_batch_join: bad argument");
  RC(bb_session_ok(e));
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    return bb_join_impl(e, srcs, slots, (uint32_t)n);
  });
}

extern "C" int og_bfs_batch_step(og_engine *e, uint64_t *pending, int *done, og_stats *st) {
  if (!e || !pending || !done) return fail(OG_E_ARG, "og_bfs_batch_step: null argument");
  RC(bb_session_ok(e));
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    og_stats s;
    memset(&s, 0, sizeof s);
    const uint64_t l0 = e->launches;
    const double t0 = now_ms();
    Timing tm;
    bool d = false;
    RC(bb_step_impl(e, pending, &d, s, tm));
    collect_timing(e, tm, &s);
    CK(cudaMemcpy(e->err_h, e->err_d, 4, cudaMemcpyDeviceToHost));
    RC(check_device_error(e));
    s.launches = e->launches - l0;
    s.ms_total = now_ms() - t0;
    if (st) *st = s;
    *done = d ? 1 : 0;
    e->last_algo = -1;
    return OG_OK;
  });
}

extern "C" int og_bfs_batch_checks(og_engine *e, uint64_t slots, uint64_t *out) {
  if (!e || !out) return fail(OG_E_ARG, "og_bfs_batch_checks: null argument");
  RC(bb_session_ok(e));
  for (uint32_t i = 0; i < 64; i++) {
    const bool on = (slots >> i) & 1u;
    out[2 * i] = on ? e->bb_reached[i] : 0;
    out[2 * i + 1] = on ? e->bb_dsum[i] : 0;
  }
  return OG_OK;
}

extern "C" int og_bfs_batch_fetch(og_engine *e, uint32_t slot, uint32_t *out) {
  if (!e || !out) return fail(OG_E_ARG, "og_bfs_batch_fetch: null argument");
  RC(bb_session_ok(e));
  if (slot >= 64) return fail(OG_E_ARG, "slot %u >= 64", slot);
  if (!e->bb_record) return fail(OG_E_STATE, "the session was opened without depth recording");
  if ((e->bb_used >> slot) & 1u) return fail(OG_E_STATE, "slot %u is still in flight", slot);
  return guarded([&]() -> int {
    clear_error();
    CK(cudaSetDevice(e->dev));
    CK(cudaMemcpyAsync(out, e->depth_d + (uint64_t)slot * e->V, 4ull * e->V, cudaMemcpyDeviceToHost, e->s_main));
    CK(cudaStreamSynchronize(e->s_main));
    return OG_OK;
  });
}

extern "C" int og_result_checksum(og_engine *e, int algo, uint64_t *out) {
  if (!e || !out) return fail(OG_E_ARG, "og_result_checksum: null argument");
  if (e->last_algo != algo) return fail(OG_E_STATE, "no result of algorithm %d on the device", algo);
  return guarded([&]() -> int {
    CK(cudaSetDevice(e->dev));
    const int mode = algo == OG_ALGO_CC ? 1 : (algo == OG_ALGO_PR ? 2 : 0);
    const uint32_t unreached = algo == OG_ALGO_BFS ? e->V + 1 : 0xFFFFFFFFu;
    const uint32_t nb = (uint32_t)e->sms * 8;
    unsigned long long *fin = e->sum64_d + 3ull * nb;
    k_checksum<<<nb, kThreads, 0, e->s_main>>>(e->value_d, e->V, mode, unreached, e->sum64_d);
    k_checksum_final<<<1, 32, 0, e->s_main>>>(e->sum64_d, nb, mode, fin);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(e->counts_h, fin, 16, cudaMemcpyDeviceToHost, e->s_main));
    CK(cudaStreamSynchronize(e->s_main));
    memcpy(out, e->counts_h, 16);
    return OG_OK;
  });
}

extern "C" int og_result_fetch(og_engine *e, int algo, void *out) {
  if (!e || !out) return fail(OG_E_ARG, "og_result_fetch: null argument");
  if (e->last_algo != algo) return fail(OG_E_STATE, "no result of algorithm %d on the device", algo);
  return guarded([&]() { return fetch(e, out); });
}

// ------------------------------------------------------- kernel launchers

namespace {

uint32_t compact_tiles(uint32_t v_begin, uint32_t v_end) {
  const uint32_t wb = v_begin / 32, we = (uint32_t)(((uint64_t)v_end + 31) / 32);
  return (we - wb + kWordsPerCompactTile - 1) / kWordsPerCompactTile;
}

// Launches k_compact over [v_begin, v_end) with the given look-back scratch
// (already cleared) and error word.
void compact_launch(const uint32_t *bits, uint32_t v_begin, uint32_t v_end, const uint64_t *off,
                    uint32_t *list, uint64_t *pref, uint64_t list_cap, uint32_t *tile,
                    uint64_t tile_cap, Counts *counts, const Lookback &lb, uint32_t *err,
                    cudaStream_t s) {
  CompactArgs a{};
  a.bits = bits;
  a.v_begin = v_begin;
  a.v_end = v_end;
  a.w_begin = v_begin / 32;
  a.w_end = (uint32_t)(((uint64_t)v_end + 31) / 32);
  a.ntiles = compact_tiles(v_begin, v_end);
  a.off = off;
  a.list = list;
  a.pref = pref;
  a.tile_first = tile;
  a.counts = counts;
  a.lb = lb;
  a.err = err;
  a.list_cap = list_cap;
  a.tile_cap = tile_cap;
  a.value = nullptr;
  a.thr = 0;
  a.split = 0;
  a.far_bits = nullptr;
  a.far_key = nullptr;
  a.clear_bits = nullptr;
  a.epoch = 1;  // the caller's scratch is zeroed before every launch
  k_compact<<<a.ntiles, kThreads, 0, s>>>(a);
}

// Look-back scratch of `ntiles` tiles carved out of one allocation:
// status[ntiles] + ticket, agg_n, inc_n (u32) and agg_e, inc_e (u64).
uint64_t lookback_bytes(uint32_t ntiles) {
  const uint64_t n = ntiles;
  return 4 * (n + 1) + 8 * n + 8 * n + 4 * n + 4 * n + 64;
}

Lookback lookback_carve(void *base, uint32_t ntiles) {
  const uint64_t n = ntiles;
  char *p = (char *)base;
  Lookback lb;
  lb.agg_e = (unsigned long long *)p;
  lb.inc_e = (unsigned long long *)(p + 8 * n);
  lb.agg_n = (uint32_t *)(p + 16 * n);
  lb.inc_n = (uint32_t *)(p + 20 * n);
  lb.status = (uint32_t *)(p + 24 * n);
  lb.ticket = lb.status + n;
  return lb;
}

int compact_args_ok(const uint32_t *bits, uint32_t v_begin, uint32_t v_end, const uint64_t *off,
                    uint32_t *out_list, uint64_t *out_pref, uint64_t list_cap, uint32_t *out_tile,
                    uint64_t tile_cap, og_counts *out_counts) {
  if (!bits || !off || !out_list || !out_pref || !out_tile || !out_counts)
    return fail(OG_E_ARG, "og_k_compact: null pointer");
  if (v_end < v_begin) return fail(OG_E_ARG, "og_k_compact: v_end < v_begin");
  if (list_cap == 0 || tile_cap == 0) return fail(OG_E_ARG, "og_k_compact: zero capacity");
  static_assert(sizeof(og_counts) == sizeof(Counts), "og_counts layout");
  static_assert(kCompactWords == kWordsPerCompactTile, "planner and kernel compaction tiles differ");
  return OG_OK;
}

int compact_status(uint32_t err) {
  if (!err) return OG_OK;
  if (err & kErrLookback) return fail(OG_E_TIMEOUT, "compaction look-back wait gave up");
  return fail(OG_E_DEVICE, "compaction output capacity too small (flags 0x%x)", err);
}

}  // namespace

extern "C" int og_k_compact(const uint32_t *bits, uint32_t v_begin, uint32_t v_end,
                            const uint64_t *off, uint32_t *out_list, uint64_t *out_pref,
                            uint64_t list_cap, uint32_t *out_tile, uint64_t tile_cap,
                            og_counts *out_counts, void *stream) {
  clear_error();
  RC(compact_args_ok(bits, v_begin, v_end, off, out_list, out_pref, list_cap, out_tile, tile_cap,
                     out_counts));
  cudaGetLastError();  // drop a stale error left by an unrelated earlier call
  cudaStream_t s = (cudaStream_t)stream;
  CK(cudaMemsetAsync(out_counts, 0, sizeof(og_counts), s));
  CK(cudaMemsetAsync(out_pref, 0, sizeof(uint64_t), s));
  if (v_end == v_begin) {
    CK(cudaStreamSynchronize(s));
    return OG_OK;
  }
  const uint32_t nt = compact_tiles(v_begin, v_end);
  void *scratch = nullptr;
  CK(cudaMalloc(&scratch, lookback_bytes(nt) + 256));
  char *err_d = (char *)scratch + lookback_bytes(nt);
  Lookback lb = lookback_carve(scratch, nt);
  uint32_t err = 0;
  cudaError_t ce = cudaMemsetAsync(scratch, 0, lookback_bytes(nt) + 256, s);
  if (ce == cudaSuccess) {
    compact_launch(bits, v_begin, v_end, off, out_list, out_pref, list_cap, out_tile, tile_cap,
                   (Counts *)out_counts, lb, (uint32_t *)err_d, s);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&err, err_d, 4, cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  cudaFree(scratch);
  if (ce != cudaSuccess) return fail(OG_E_CUDA, "og_k_compact: %s", cudaGetErrorString(ce));
  return compact_status(err);
}

// ------------------------------------------------ allocation-free variant
//
// og_k_compact_noalloc runs the same compaction with its look-back scratch in
// a fixed array that is part of the loaded library instead of memory it asks
// the CUDA runtime for.  Limit: kNoAllocTiles compaction tiles of 1024 bitmap
// words, counted from the word holding v_begin: 2^28 vertices when v_begin is
// a multiple of 32, 2^28 - 32 otherwise.  The array (229,700 bytes) lives on
// every device that loads the library, for as long as the process runs.

namespace {

constexpr uint32_t kNoAllocTiles = 8192;
constexpr uint64_t kNoAllocErrOffset = 4 * (kNoAllocTiles + 1ull) + 24ull * kNoAllocTiles + 64;
constexpr uint64_t kNoAllocBytes = kNoAllocErrOffset + 256;

static __device__ __align__(256) unsigned char g_compact_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_compact_scratch on the current device.  Host code may
// not use the symbol itself: on the host it names a stand-in, not device
// memory.  Looked up once per device, the first time that device calls.
int scratch_address(void **out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(OG_E_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_compact_scratch));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return OG_OK;
}

}  // namespace

extern "C" int og_k_compact_noalloc(const uint32_t *bits, uint32_t v_begin, uint32_t v_end,
                                    const uint64_t *off, uint32_t *out_list, uint64_t *out_pref,
                                    uint64_t list_cap, uint32_t *out_tile, uint64_t tile_cap,
                                    og_counts *out_counts, void *stream) {
  clear_error();
  RC(compact_args_ok(bits, v_begin, v_end, off, out_list, out_pref, list_cap, out_tile, tile_cap,
                     out_counts));
  const uint32_t nt = v_end > v_begin ? compact_tiles(v_begin, v_end) : 0;
  if (nt > kNoAllocTiles)
    return fail(OG_E_ARG,
                "og_k_compact_noalloc: range of %u vertices needs %u scratch tiles, the fixed "
                "scratch holds %u (2^28 vertices per call from a multiple of 32)",
                v_end - v_begin, nt, kNoAllocTiles);
  void *base = nullptr;
  RC(scratch_address(&base));
  cudaGetLastError();  // drop a stale error left by an unrelated earlier call
  cudaStream_t s = (cudaStream_t)stream;
  CK(cudaMemsetAsync(out_counts, 0, sizeof(og_counts), s));
  CK(cudaMemsetAsync(out_pref, 0, sizeof(uint64_t), s));
  if (nt == 0) {
    CK(cudaStreamSynchronize(s));
    return OG_OK;
  }
  // the previous call's look-back state and error word must not leak in
  uint32_t *err_d = (uint32_t *)((char *)base + kNoAllocErrOffset);
  CK(cudaMemsetAsync(base, 0, lookback_bytes(nt), s));
  CK(cudaMemsetAsync(err_d, 0, sizeof(uint32_t), s));
  compact_launch(bits, v_begin, v_end, off, out_list, out_pref, list_cap, out_tile, tile_cap,
                 (Counts *)out_counts, lookback_carve(base, nt), err_d, s);
  CK(cudaGetLastError());
  uint32_t err = 0;
  CK(cudaMemcpyAsync(&err, err_d, sizeof err, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return compact_status(err);
}

extern "C" void og_graph_free(og_graph *g) {
  if (!g) return;
  if (g->registered) {
    cudaHostUnregister(g->packed);
  }
  og::graph_delete(g);
}

// Kernel-level launchers of include/onegraph_kernels.h (same translation unit).
#include "kernel_abi.cuh"
