// server.cpp — the serving loop behind og_server_* (onegraph.h).
//
// Several graphs stay resident (one parent engine each: offsets + static edge
// prefix in HBM, the host CSR page-locked).  Requests (BFS / SSSP / CC /
// PageRank) are queued as they arrive; worker threads admit them when a query
// context of the request's graph is free or a new one fits the server's
// device-memory budget, run them (each context has its own streams, so the
// work of different requests overlaps on the GPU), and post responses.
// Continuous batching:
//  * SSSP requests of a graph run as one multi-source pass
//    (og_sssp_batch_begin / _join / _step): the worker that admits one takes
//    the queued SSSP requests of that graph into free slots, and between
//    rounds it takes the requests that arrived meanwhile; a request is
//    answered as soon as its slot has no pending work, and its slot is then
//    free for the next one.  So requests join and leave a pass in flight.
//  * when a worker admits a BFS request it also takes the BFS requests for
//    the same graph that queued up meanwhile (up to max_batch) and serves
//    them in one og_bfs_batch pass (og_bfs_batch_to when the requests carry
//    result buffers, at most 8 GiB of depths per pass); with OG_SERVER_BFS_JOIN the pass runs
//    level by level (og_bfs_batch_begin / _join / _step) and BFS requests
//    queued meanwhile join it at every level boundary, as SSSP requests join
//    SSSP passes;
//  * queued PageRank requests for the same graph share one computation.
// Built on the public C ABI (and the flag helpers of og_internal.hpp).
// No reference counterpart: the reference runs one query per process run.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "og_internal.hpp"

namespace {

struct Pending {
  og_request r;
  uint64_t ticket;
  double t_submit;
};

struct GraphSlot {
  og_graph *g = nullptr;
  og_engine *parent = nullptr;
  uint64_t ctx_bytes = 0;            // device bytes of one extra query context
  std::vector<og_engine *> idle;     // contexts ready for a request
  std::vector<og_engine *> clones;   // every clone created (destroyed with the server)
  bool batch = false, pagerank = false;
  uint32_t sssp_slots = 0;  // sources per multi-source SSSP pass (0: one at a time)
};

double now_ms(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct og_server {
  og_server_config cfg{};
  std::chrono::steady_clock::time_point t0;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending> queue;
  std::deque<og_response> done;
  std::vector<GraphSlot> graphs;
  std::vector<std::thread> workers;
  bool stop = false;
  bool started = false;
  uint64_t used_bytes = 0;
  uint64_t next_ticket = 1;
  uint64_t in_flight = 0;  // submitted and not yet responded
  og_server_stats st{};
};

namespace {

using og::fail;

// Device bytes of the byte-depth matrix of one batched pass of BFS requests
// that carry result buffers (og_bfs_batch_to; outside the server's budget,
// like og_bfs_batch's): 64 sources of 2^27 vertices.
constexpr uint64_t kBfsOutMatrixBytes = 8ull << 30;

struct Job {
  std::vector<Pending> reqs;
  og_engine *ctx = nullptr;
  int graph = -1;
  bool sssp_pass = false;  // a multi-source SSSP pass that admits requests while it runs
  bool bfs_pass = false;   // a level-by-level BFS pass that admits requests while it runs
};

// Moves up to `room` queued requests of graph g for `algo` (FIFO) into out;
// BFS requests only when they need no result array.  Called with the lock
// held.
void take_algo(og_server *s, int g, int algo, size_t room, std::vector<Pending> &out) {
  for (auto jt = s->queue.begin(); jt != s->queue.end() && room > 0;) {
    if (jt->r.graph == g && jt->r.algo == algo && (algo != OG_ALGO_BFS || !jt->r.out)) {
      out.push_back(*jt);
      jt = s->queue.erase(jt);
      room--;
    } else {
      ++jt;
    }
  }
}

// Takes the first admissible request (FIFO with skipping) and, for BFS, the
// queued BFS requests of the same graph.  Called with the lock held.
bool pick(og_server *s, Job &job) {
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
    GraphSlot &gs = s->graphs[it->r.graph];
    og_engine *ctx = nullptr;
    if (!gs.idle.empty()) {
      ctx = gs.idle.back();
      gs.idle.pop_back();
    } else if (s->cfg.budget_bytes == 0 || s->used_bytes + gs.ctx_bytes <= s->cfg.budget_bytes) {
      // admission by free memory: a new context only if it fits the budget
      if (og_engine_clone(gs.parent, &ctx) != OG_OK) {
        ctx = nullptr;
      } else {
        gs.clones.push_back(ctx);
        s->used_bytes += gs.ctx_bytes;
        s->st.contexts_created++;
      }
    }
    if (!ctx) continue;
    job.ctx = ctx;
    job.graph = it->r.graph;
    if (it->r.algo == OG_ALGO_SSSP && gs.sssp_slots > 1 && s->cfg.max_batch > 1) {
      job.sssp_pass = true;
      job.reqs.push_back(*it);
      s->queue.erase(it);
      take_algo(s, job.graph, OG_ALGO_SSSP, std::min<size_t>(gs.sssp_slots, s->cfg.max_batch) - 1, job.reqs);
      return true;
    }
    if (it->r.algo == OG_ALGO_BFS && gs.batch && s->cfg.max_batch > 1 && !it->r.out &&
        (s->cfg.flags & OG_SERVER_BFS_JOIN)) {
      job.bfs_pass = true;
      job.reqs.push_back(*it);
      s->queue.erase(it);
      take_algo(s, job.graph, OG_ALGO_BFS, std::min<size_t>(64, s->cfg.max_batch) - 1, job.reqs);
      return true;
    }
    job.reqs.push_back(*it);
    // BFS requests with result buffers share a pass too (og_bfs_batch_to);
    // its n x V depth matrix is kept within kBfsOutMatrixBytes
    const bool with_out = it->r.out != nullptr;
    const int bfs_cap = with_out ? (int)std::min<uint64_t>(64, kBfsOutMatrixBytes / (uint64_t)gs.g->V) : 64;
    const bool bfs_batch = it->r.algo == OG_ALGO_BFS && gs.batch && s->cfg.max_batch > 1 && bfs_cap > 1;
    // PageRank does not depend on a source: queued PR requests for the same
    // graph and iteration count are answered by one computation
    const bool pr_share = it->r.algo == OG_ALGO_PR && s->cfg.max_batch > 1;
    const int iters = it->r.iterations;
    const int limit = bfs_batch ? std::min(s->cfg.max_batch, bfs_cap) : s->cfg.max_batch;
    it = s->queue.erase(it);
    if (bfs_batch || pr_share) {
      for (auto jt = s->queue.begin(); jt != s->queue.end() && (int)job.reqs.size() < limit;) {
        const bool same_bfs = bfs_batch && jt->r.algo == OG_ALGO_BFS && (jt->r.out != nullptr) == with_out;
        const bool same_pr = pr_share && jt->r.algo == OG_ALGO_PR && jt->r.iterations == iters;
        if (jt->r.graph == job.graph && (same_bfs || same_pr)) {
          job.reqs.push_back(*jt);
          jt = s->queue.erase(jt);
        } else {
          ++jt;
        }
      }
    }
    return true;
  }
  return false;
}

og_response make_response(const Pending &p, int status, const uint64_t *ck, uint32_t batch, double t_start) {
  og_response r;
  memset(&r, 0, sizeof r);
  r.ticket = p.ticket;
  r.user = p.r.user;
  r.status = status;
  r.graph = p.r.graph;
  r.algo = p.r.algo;
  r.source = p.r.source;
  r.batch = batch;
  r.t_submit_ms = p.t_submit;
  r.t_start_ms = t_start;
  if (ck) {
    r.checksum[0] = ck[0];
    r.checksum[1] = ck[1];
  }
  return r;
}

void count_launches(og_server *s, const og_stats &st) {
  std::lock_guard<std::mutex> lk(s->m);
  s->st.launches += st.launches;
}

// Posts finished responses (stamps their completion time).
void post(og_server *s, std::vector<og_response> &rs) {
  if (rs.empty()) return;
  const double t_done = now_ms(s->t0);
  std::lock_guard<std::mutex> lk(s->m);
  for (auto &r : rs) {
    r.t_done_ms = t_done;
    s->done.push_back(r);
  }
  s->in_flight -= rs.size();
  s->st.completed += rs.size();
  s->cv_done.notify_all();
  rs.clear();
}

// A multi-source SSSP pass on job.ctx: the admitted requests take slots,
// every round frees the slots whose sources are final (their requests are
// answered at once) and fills free slots with SSSP requests of the same graph
// that queued up meanwhile.  Ends when no slot is in use and none is waiting.
void run_sssp_pass(og_server *s, Job &job) {
  og_engine *e = job.ctx;
  const uint32_t k = std::min<uint32_t>(s->graphs[job.graph].sssp_slots, (uint32_t)s->cfg.max_batch);
  struct Slot {
    bool used = false;
    Pending p;
    double t_start = 0;
  };
  std::vector<Slot> slot(k);
  std::vector<og_response> out;
  uint32_t served = 0;
  auto fail_all = [&](int rc) {
    for (auto &sl : slot)
      if (sl.used) {
        out.push_back(make_response(sl.p, rc, nullptr, served, sl.t_start));
        sl.used = false;
      }
    post(s, out);
  };
  auto join = [&](std::vector<Pending> &reqs) -> int {
    std::vector<uint32_t> srcs, ids;
    const double t = now_ms(s->t0);
    size_t q = 0;
    for (uint32_t i = 0; i < k && q < reqs.size(); i++)
      if (!slot[i].used) {
        slot[i].used = true;
        slot[i].p = reqs[q++];
        slot[i].t_start = t;
        srcs.push_back(slot[i].p.r.source);
        ids.push_back(i);
      }
    reqs.clear();
    return og_sssp_batch_join(e, srcs.data(), ids.data(), (int)srcs.size());
  };
  int rc = og_sssp_batch_begin(e);
  if (rc == OG_OK) rc = join(job.reqs);
  if (rc != OG_OK) return fail_all(rc);
  for (;;) {
    uint32_t pending = 0;
    int done = 0;
    og_stats st;
    rc = og_sssp_batch_step(e, &pending, &done, &st);
    if (rc != OG_OK) return fail_all(rc);
    count_launches(s, st);
    uint32_t fin = 0, used = 0;
    for (uint32_t i = 0; i < k; i++)
      if (slot[i].used) {
        used++;
        if (!((pending >> i) & 1u)) fin |= 1u << i;
      }
    if (fin) {
      uint64_t ck[64];
      rc = og_sssp_batch_checks(e, fin, ck);
      for (uint32_t i = 0; i < k; i++) {
        if (!((fin >> i) & 1u)) continue;
        int rq = rc;
        if (rq == OG_OK && slot[i].p.r.out) rq = og_sssp_batch_fetch(e, i, (uint32_t *)slot[i].p.r.out);
        served++;
        out.push_back(make_response(slot[i].p, rq, rq == OG_OK ? &ck[2 * i] : nullptr, served, slot[i].t_start));
        slot[i].used = false;
        used--;
      }
      post(s, out);
    }
    // admit the SSSP requests of this graph that arrived meanwhile
    std::vector<Pending> more;
    if (used < k) {
      std::lock_guard<std::mutex> lk(s->m);
      take_algo(s, job.graph, OG_ALGO_SSSP, k - used, more);
      if (!more.empty()) s->st.batched_requests += more.size();
    }
    if (!more.empty()) {
      used += (uint32_t)more.size();
      rc = join(more);
      if (rc != OG_OK) return fail_all(rc);
    }
    if (used == 0) break;
  }
}

// A level-by-level BFS pass on job.ctx: the admitted requests take slots,
// every level answers the requests whose sources have finished and seeds
// the freed slots with BFS requests of the same graph that queued up
// meanwhile.  Ends when no slot is in use and none is waiting.
void run_bfs_pass(og_server *s, Job &job) {
  og_engine *e = job.ctx;
  const uint32_t k = (uint32_t)std::min(64, s->cfg.max_batch);
  struct Slot {
    bool used = false;
    Pending p;
    double t_start = 0;
  };
  std::vector<Slot> slot(k);
  std::vector<og_response> out;
  uint32_t served = 0;
  auto fail_all = [&](int rc) {
    for (auto &sl : slot)
      if (sl.used) {
        out.push_back(make_response(sl.p, rc, nullptr, served, sl.t_start));
        sl.used = false;
      }
    post(s, out);
  };
  auto join = [&](std::vector<Pending> &reqs) -> int {
    std::vector<uint32_t> srcs, ids;
    const double t = now_ms(s->t0);
    size_t q = 0;
    for (uint32_t i = 0; i < k && q < reqs.size(); i++)
      if (!slot[i].used) {
        slot[i].used = true;
        slot[i].p = reqs[q++];
        slot[i].t_start = t;
        srcs.push_back(slot[i].p.r.source);
        ids.push_back(i);
      }
    reqs.clear();
    return og_bfs_batch_join(e, srcs.data(), ids.data(), (int)srcs.size());
  };
  int rc = og_bfs_batch_begin(e, 0);
  if (rc == OG_OK) rc = join(job.reqs);
  if (rc != OG_OK) return fail_all(rc);
  for (;;) {
    uint64_t pending = 0;
    int done = 0;
    og_stats st;
    rc = og_bfs_batch_step(e, &pending, &done, &st);
    if (rc != OG_OK) return fail_all(rc);
    count_launches(s, st);
    uint64_t fin = 0;
    uint32_t used = 0;
    for (uint32_t i = 0; i < k; i++)
      if (slot[i].used) {
        used++;
        if (!((pending >> i) & 1u)) fin |= 1ull << i;
      }
    if (fin) {
      uint64_t ck[128];
      rc = og_bfs_batch_checks(e, fin, ck);
      for (uint32_t i = 0; i < k; i++) {
        if (!((fin >> i) & 1u)) continue;
        served++;
        out.push_back(make_response(slot[i].p, rc, rc == OG_OK ? &ck[2 * i] : nullptr, served, slot[i].t_start));
        slot[i].used = false;
        used--;
      }
      post(s, out);
    }
    // admit the BFS requests of this graph that arrived meanwhile
    std::vector<Pending> more;
    if (used < k) {
      std::lock_guard<std::mutex> lk(s->m);
      take_algo(s, job.graph, OG_ALGO_BFS, k - used, more);
      if (!more.empty()) s->st.batched_requests += more.size();
    }
    if (!more.empty()) {
      used += (uint32_t)more.size();
      rc = join(more);
      if (rc != OG_OK) return fail_all(rc);
    }
    if (used == 0) break;
  }
}

void run_job(og_server *s, Job &job) {
  if (job.sssp_pass) return run_sssp_pass(s, job);
  if (job.bfs_pass) return run_bfs_pass(s, job);
  const double t_start = now_ms(s->t0);
  og_engine *e = job.ctx;
  og_stats st;
  memset(&st, 0, sizeof st);
  std::vector<og_response> out;
  auto respond = [&](const Pending &p, int status, const uint64_t *ck) {
    out.push_back(make_response(p, status, ck, (uint32_t)job.reqs.size(), t_start));
  };
  if (job.reqs.size() > 1 && job.reqs[0].r.algo == OG_ALGO_PR) {
    const Pending &p = job.reqs[0];
    int rc = og_pr_l1(e, nullptr, 0.85, 0.0, p.r.iterations > 0 ? p.r.iterations : 5, &st);
    uint64_t ck[2] = {0, 0};
    if (rc == OG_OK) rc = og_result_checksum(e, OG_ALGO_PR, ck);
    for (auto &q : job.reqs) {
      int rq = rc;
      if (rq == OG_OK && q.r.out) rq = og_result_fetch(e, OG_ALGO_PR, q.r.out);
      respond(q, rq, rq == OG_OK ? ck : nullptr);
    }
  } else if (job.reqs.size() > 1) {
    std::vector<uint32_t> srcs;
    std::vector<uint32_t *> outs;
    for (auto &p : job.reqs) {
      srcs.push_back(p.r.source);
      outs.push_back((uint32_t *)p.r.out);
    }
    std::vector<uint64_t> checks(2 * srcs.size());
    const int rc = outs[0] ? og_bfs_batch_to(e, srcs.data(), (int)srcs.size(), outs.data(), checks.data(), &st)
                           : og_bfs_batch(e, srcs.data(), (int)srcs.size(), nullptr, checks.data(), &st);
    for (size_t i = 0; i < job.reqs.size(); i++) respond(job.reqs[i], rc, rc == OG_OK ? &checks[2 * i] : nullptr);
  } else {
    const Pending &p = job.reqs[0];
    int rc;
    switch (p.r.algo) {
      case OG_ALGO_BFS: rc = og_bfs(e, p.r.source, (uint32_t *)p.r.out, &st); break;
      case OG_ALGO_SSSP: rc = og_sssp(e, p.r.source, (uint32_t *)p.r.out, &st); break;
      case OG_ALGO_CC: rc = og_cc(e, (uint32_t *)p.r.out, &st); break;
      case OG_ALGO_PR:
        rc = og_pr_l1(e, (float *)p.r.out, 0.85, 0.0, p.r.iterations > 0 ? p.r.iterations : 5, &st);
        break;
      default: rc = OG_E_ARG;
    }
    uint64_t ck[2] = {0, 0};
    if (rc == OG_OK) rc = og_result_checksum(e, p.r.algo, ck);
    respond(p, rc, rc == OG_OK ? ck : nullptr);
  }
  count_launches(s, st);
  post(s, out);
}

void worker_loop(og_server *s) {
  cudaSetDevice(s->cfg.device);
  std::unique_lock<std::mutex> lk(s->m);
  for (;;) {
    Job job;
    while (!s->stop && !pick(s, job)) s->cv_work.wait(lk);
    if (job.reqs.empty()) break;  // stop requested, nothing admitted
    s->st.gpu_passes++;
    if (job.reqs.size() > 1) s->st.batched_requests += job.reqs.size();
    lk.unlock();
    run_job(s, job);  // posts its responses as they finish
    lk.lock();
    s->graphs[job.graph].idle.push_back(job.ctx);
    s->cv_work.notify_all();  // a context came back: something may be admissible
  }
}

void start_workers(og_server *s) {
  if (s->started) return;
  s->started = true;
  for (int i = 0; i < s->cfg.workers; i++) s->workers.emplace_back(worker_loop, s);
}

}  // namespace

// ====================================================================== C ABI

extern "C" int og_server_create(const og_server_config *cfg, og_server **out) {
  og::clear_error();
  if (!cfg || !out) return fail(OG_E_ARG, "og_server_create: null argument");
  if (cfg->workers < 1 || cfg->workers > 64) return fail(OG_E_ARG, "workers must be 1..64");
  if (cfg->max_batch < 1 || cfg->max_batch > 64) return fail(OG_E_ARG, "max_batch must be 1..64");
  og_server *s = new (std::nothrow) og_server;
  if (!s) return fail(OG_E_NOMEM, "cannot allocate the server");
  s->cfg = *cfg;
  s->t0 = std::chrono::steady_clock::now();
  *out = s;
  return OG_OK;
}

extern "C" int og_server_add_graph(og_server *s, og_graph *g, const og_config *gcfg, int *graph_id) {
  og::clear_error();
  if (!s || !g || !gcfg) return fail(OG_E_ARG, "og_server_add_graph: null argument");
  std::lock_guard<std::mutex> lk(s->m);
  if (s->started) return fail(OG_E_STATE, "graphs must be added before the first request");
  og_config c = *gcfg;
  c.device = s->cfg.device;
  if (s->cfg.max_batch > 1) c.flags |= OG_CFG_BATCH;
  og_engine *e = nullptr;
  int rc = og_engine_create(g, &c, &e);
  if (rc != OG_OK) return rc;
  uint64_t resident = 0, ctx = 0;
  og_engine_bytes(e, &resident, &ctx);
  if (s->cfg.budget_bytes && s->used_bytes + resident + ctx > s->cfg.budget_bytes) {
    og_engine_destroy(e);
    return fail(OG_E_BUDGET, "graph does not fit the server budget (%llu B used of %llu B)",
                (unsigned long long)s->used_bytes, (unsigned long long)s->cfg.budget_bytes);
  }
  GraphSlot gs;
  gs.g = g;
  gs.parent = e;
  gs.ctx_bytes = ctx;
  gs.idle.push_back(e);  // the parent is the first context
  gs.batch = (c.flags & OG_CFG_BATCH) != 0;
  gs.sssp_slots = g->kind == OG_GRAPH_WEIGHTED ? og::sb_sources(c.flags) : 0;
  gs.pagerank = g->kind == OG_GRAPH_PR || (c.flags & OG_CFG_PR);
  s->used_bytes += resident + ctx;
  s->graphs.push_back(std::move(gs));
  if (graph_id) *graph_id = (int)s->graphs.size() - 1;
  return OG_OK;
}

extern "C" int og_server_submit(og_server *s, const og_request *r, uint64_t *ticket) {
  if (!s || !r) return fail(OG_E_ARG, "og_server_submit: null argument");
  std::lock_guard<std::mutex> lk(s->m);
  if (r->graph < 0 || r->graph >= (int)s->graphs.size()) return fail(OG_E_ARG, "unknown graph %d", r->graph);
  const GraphSlot &gs = s->graphs[r->graph];
  if (r->algo < OG_ALGO_BFS || r->algo > OG_ALGO_PR) return fail(OG_E_ARG, "unknown algorithm %d", r->algo);
  if ((r->algo == OG_ALGO_BFS || r->algo == OG_ALGO_SSSP) && r->source >= gs.g->V)
    return fail(OG_E_ARG, "source %u >= V", r->source);
  if (r->algo == OG_ALGO_SSSP && gs.g->kind != OG_GRAPH_WEIGHTED)
    return fail(OG_E_UNSUPPORTED, "SSSP needs a weighted graph");
  if (r->algo == OG_ALGO_PR && !gs.pagerank) return fail(OG_E_UNSUPPORTED, "graph has no PageRank state");
  Pending p;
  p.r = *r;
  p.ticket = s->next_ticket++;
  p.t_submit = now_ms(s->t0);
  s->queue.push_back(p);
  s->in_flight++;
  s->st.submitted++;
  if (ticket) *ticket = p.ticket;
  start_workers(s);
  s->cv_work.notify_one();
  return OG_OK;
}

extern "C" int og_server_poll(og_server *s, og_response *out, int max, int *n, int wait_ms) {
  if (!s || !out || !n || max < 1) return fail(OG_E_ARG, "og_server_poll: bad argument");
  std::unique_lock<std::mutex> lk(s->m);
  if (s->done.empty() && wait_ms != 0) {
    auto pred = [&] { return !s->done.empty() || s->in_flight == 0; };
    if (wait_ms < 0) s->cv_done.wait(lk, pred);
    else s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), pred);
  }
  int k = 0;
  while (k < max && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  *n = k;
  return OG_OK;
}

extern "C" int og_server_drain(og_server *s, int timeout_ms) {
  if (!s) return fail(OG_E_ARG, "og_server_drain: null server");
  std::unique_lock<std::mutex> lk(s->m);
  auto pred = [&] { return s->in_flight == 0; };
  if (timeout_ms < 0) s->cv_done.wait(lk, pred);
  else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
    return fail(OG_E_TIMEOUT, "%llu requests still in flight", (unsigned long long)s->in_flight);
  return OG_OK;
}

extern "C" int og_server_get_stats(og_server *s, og_server_stats *out) {
  if (!s || !out) return fail(OG_E_ARG, "og_server_get_stats: null argument");
  std::lock_guard<std::mutex> lk(s->m);
  *out = s->st;
  out->used_bytes = s->used_bytes;
  return OG_OK;
}

extern "C" void og_server_destroy(og_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto &t : s->workers) t.join();
  for (auto &gs : s->graphs) {
    for (og_engine *c : gs.clones) og_engine_destroy(c);
    og_engine_destroy(gs.parent);
  }
  delete s;
}
