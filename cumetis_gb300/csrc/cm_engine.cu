// cm_engine.cu -- many independent partitions on one GPU: the batched form
// (cm_part_batch) and the served form (cm_engine_*: submit / wait with
// admission by device-memory footprint).  Neither has a counterpart in the
// reference, which partitions one graph per process (cuMetis.cu:3874).
//
// Design: one scheduler thread owns a context and a batch coarsener.  Jobs
// admitted by footprint join the batch before its next level; each level
// coarsens every graph still coarsening in one set of launches (the graphs
// laid side by side as one disjoint union, cm_batch.cu), and a graph whose
// stop rule ends its coarsening leaves the batch at once -- continuous
// batching at level granularity.  A pool of worker threads, each owning a
// context and its own stream, then takes the coarsened jobs and runs the
// rest of the pipeline (the initial partition on the worker's host thread,
// projection and refinement on its stream), smallest coarsest graph first
// unless a job has waited longer than kReadyAgeMs.  Graphs are read from the
// caller's host arrays, which must stay valid until the job is waited for.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "cm.h"
#include "cm_batch.h"
#include "cm_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Job {
  int64_t id = 0;
  cm_graph g{};
  int32_t nparts = 0;
  cm_part_params params{};
  int32_t *part = nullptr;
  int64_t footprint = 0;
  int32_t objval = 0;
  int status = CM_OK;
  std::string error;
  cm_part_stats stats{};
  Clock::time_point t_submit, t_start, t_end;
  Clock::time_point t_batch, t_coarsened;  // joined the batch / left it coarsened
  cm_hierarchy *h = nullptr;               // its levels once coarsened
  int32_t coarsest = 0;                    // vertices of its coarsest level
  bool done = false;
  bool waited = false;  // a thread is in cm_engine_wait for this job
};

// A coarsened job that waited this long is taken before smaller ones.
constexpr double kReadyAgeMs = 250.0;

// Device bytes a job holds while it runs: the level graphs (input and coarse
// levels, each with match and cmap), the context workspace of the finest
// level and the refinement arrays.
int64_t footprint_bytes(int64_t n, int64_t m, int32_t k) {
  return 40 * m + 96 * n + 4 * (int64_t)k * (n / 1024 + 2) + (4 << 20);
}

}  // namespace

struct cm_engine {
  int device = 0;
  int64_t budget = 0;
  int32_t max_queue = 0;       // <= 0: unbounded
  std::vector<cm_ctx *> ctxs;  // workers' contexts
  cm_ctx *sched_ctx = nullptr; // the scheduler's context (batch coarsening)
  std::vector<std::thread> threads;
  std::thread sched;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_sched;
  std::deque<Job *> pending;   // submitted, waiting for admission (FIFO by footprint)
  std::vector<Job *> admitted; // admitted, to join the batch before its next level
  std::vector<Job *> ready;    // coarsened, waiting for a worker
  std::unordered_map<int64_t, std::unique_ptr<Job>> jobs;
  int64_t inflight = 0;        // footprint of admitted jobs not yet finished
  int64_t next_id = 1;
  bool stop = false;
  int waiters = 0;             // threads inside cm_engine_wait
  // statistics
  int64_t completed = 0;
  std::vector<double> latencies;

  void admit_locked() {
    bool any = false;
    while (!pending.empty()) {
      Job *j = pending.front();
      const bool fits = budget <= 0 || inflight + j->footprint <= budget || inflight == 0;
      if (!fits) break;
      pending.pop_front();
      inflight += j->footprint;
      admitted.push_back(j);
      any = true;
    }
    if (any) cv_sched.notify_one();
  }

  void finish_locked(Job *j, int rc, const std::string &err) {
    j->t_end = Clock::now();
    j->status = rc;
    j->error = err;
    j->done = true;
    inflight -= j->footprint;
    ++completed;
    latencies.push_back(ms_between(j->t_submit, j->t_end));
    admit_locked();
  }

  // The next coarsened job for a worker: the oldest if it waited longer than
  // kReadyAgeMs, else the one with the smallest coarsest graph.
  Job *take_ready_locked() {
    if (ready.empty()) return nullptr;
    const auto now = Clock::now();
    size_t pick = 0, oldest = 0;
    for (size_t i = 1; i < ready.size(); ++i) {
      if (ready[i]->t_coarsened < ready[oldest]->t_coarsened) oldest = i;
      if (ready[i]->coarsest < ready[pick]->coarsest) pick = i;
    }
    if (ms_between(ready[oldest]->t_coarsened, now) > kReadyAgeMs) pick = oldest;
    Job *j = ready[pick];
    ready.erase(ready.begin() + pick);
    return j;
  }

  void scheduler() {
    auto B = std::make_unique<cm::BatchCoarsener>(sched_ctx, sched_ctx->stream);
    std::unordered_map<int64_t, Job *> inbatch;
    std::vector<std::pair<int64_t, cm_hierarchy *>> fin;
    auto fail_all = [&](int rc) {
      const std::string err = cm_last_error();
      std::lock_guard<std::mutex> lk(mu);
      for (auto &kv : inbatch) finish_locked(kv.second, rc, err);
      inbatch.clear();
      cv_done.notify_all();
    };
    for (;;) {
      std::vector<Job *> add;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_sched.wait(lk, [&] { return stop || !admitted.empty() || !B->empty(); });
        if (stop) break;
        add.swap(admitted);
      }
      fin.clear();
      int rc = CM_OK;
      if (!add.empty()) {
        std::vector<cm_graph> gs(add.size());
        std::vector<cm_coarsen_params> ps(add.size());
        std::vector<int64_t> tags(add.size());
        const auto now = Clock::now();
        for (size_t i = 0; i < add.size(); ++i) {
          Job *j = add[i];
          j->t_batch = now;
          gs[i] = j->g;
          cm_coarsen_default_params(j->g.nvtxs, j->nparts, &ps[i]);
          if (j->params.coarsen_to > 0) ps[i].coarsen_to = j->params.coarsen_to;
          ps[i].match_mode = j->params.match_mode;
          tags[i] = j->id;
          inbatch[j->id] = j;
        }
        rc = B->add((int32_t)add.size(), gs.data(), ps.data(), tags.data(), fin);
      }
      if (rc == CM_OK && !B->empty()) rc = B->step(fin);
      if (rc == CM_OK) rc = cm::cuda_status(cudaStreamSynchronize(sched_ctx->stream), "batch level");
      if (rc != CM_OK) {
        for (auto &f : fin) cm_hierarchy_free(f.second);
        fail_all(rc);
        B = std::make_unique<cm::BatchCoarsener>(sched_ctx, sched_ctx->stream);  // frees what it held
        continue;
      }
      if (fin.empty()) continue;
      const auto now = Clock::now();
      std::lock_guard<std::mutex> lk(mu);
      for (auto &f : fin) {
        Job *j = inbatch[f.first];
        inbatch.erase(f.first);
        j->h = f.second;
        j->t_coarsened = now;
        cm_graph cg{};
        cm_hierarchy_level(j->h, cm_hierarchy_levels(j->h) - 1, &cg, nullptr, nullptr);
        j->coarsest = cg.nvtxs;
        ready.push_back(j);
      }
      cv_work.notify_all();
    }
    // shutting down: jobs still coarsening or admitted are dropped
    B.reset();
    std::lock_guard<std::mutex> lk(mu);
    for (auto &kv : inbatch) finish_locked(kv.second, CM_ERR_INVALID, "cm_engine_wait: the engine was destroyed before the job ran");
    for (Job *j : admitted) finish_locked(j, CM_ERR_INVALID, "cm_engine_wait: the engine was destroyed before the job ran");
    admitted.clear();
    cv_done.notify_all();
  }

  void worker(int w) {
    cm_ctx *ctx = ctxs[w];
    for (;;) {
      Job *j = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || !ready.empty(); });
        if (stop && ready.empty()) return;
        j = take_ready_locked();
        if (!j) continue;
        j->t_start = Clock::now();
      }
      int32_t obj = 0;
      cm_part_stats st{};
      st.coarsen_ms = ms_between(j->t_batch, j->t_coarsened);
      cm_hierarchy *h = j->h;
      j->h = nullptr;
      h->stream = ctx->stream;  // frees of its own blocks and waits go to this worker's stream
      int rc = CM_OK;
      if (j->nparts == 1 || h->levels[0].g.nvtxs == 0) {
        for (int i = 0; i < h->levels[0].g.nvtxs; ++i) j->part[i] = 0;
        cm_hierarchy_free(h);
      } else {
        rc = part_hierarchy(ctx, h, j->nparts, j->params, j->part, &obj, &st);
      }
      st.total_ms = ms_between(j->t_batch, Clock::now());
      std::string err = rc == CM_OK ? std::string() : std::string(cm_last_error());
      {
        std::lock_guard<std::mutex> lk(mu);
        j->objval = obj;
        j->stats = st;
        finish_locked(j, rc, err);
      }
      cv_done.notify_all();
    }
  }
};

extern "C" int cm_engine_create(int device, int32_t nworkers, int64_t hbm_budget_bytes, int32_t max_queue,
                                int64_t reserve_nvtxs, int64_t reserve_nedges, cm_engine **out) {
  if (!out || nworkers < 1 || nworkers > 256) return cm_fail(CM_ERR_INVALID, "cm_engine_create: bad arguments");
  *out = nullptr;
  auto e = std::make_unique<cm_engine>();
  e->device = device;
  e->budget = hbm_budget_bytes;
  e->max_queue = max_queue;
  for (int w = 0; w < nworkers; ++w) {
    cm_ctx *c = nullptr;
    int rc = cm_ctx_create(device, &c);
    if (rc == CM_OK && (reserve_nvtxs > 0 || reserve_nedges > 0)) rc = cm_ctx_reserve(c, reserve_nvtxs, reserve_nedges);
    if (rc != CM_OK) {
      if (c) cm_ctx_destroy(c);
      for (cm_ctx *x : e->ctxs) cm_ctx_destroy(x);
      return rc;
    }
    e->ctxs.push_back(c);
  }
  int rc = cm_ctx_create(device, &e->sched_ctx);
  if (rc == CM_OK && (reserve_nvtxs > 0 || reserve_nedges > 0)) rc = cm_ctx_reserve(e->sched_ctx, reserve_nvtxs, reserve_nedges);
  if (rc != CM_OK) {
    if (e->sched_ctx) cm_ctx_destroy(e->sched_ctx);
    for (cm_ctx *x : e->ctxs) cm_ctx_destroy(x);
    return rc;
  }
  cm_engine *raw = e.get();
  e->sched = std::thread([raw] { raw->scheduler(); });
  for (int w = 0; w < nworkers; ++w) e->threads.emplace_back([raw, w] { raw->worker(w); });
  *out = e.release();
  return CM_OK;
}

extern "C" void cm_engine_destroy(cm_engine *e) {
  if (!e) return;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    e->stop = true;
    // Jobs not started are dropped: they end with an error, and their
    // waiters wake up.  Running jobs finish.
    auto drop = [&](Job *j) {
      j->status = CM_ERR_INVALID;
      j->error = "cm_engine_wait: the engine was destroyed before the job ran";
      j->t_start = j->t_end = Clock::now();
      j->done = true;
    };
    for (Job *j : e->pending) drop(j);
    for (Job *j : e->ready) {
      drop(j);
      e->inflight -= j->footprint;
    }
    e->pending.clear();
    e->ready.clear();
  }
  e->cv_work.notify_all();
  e->cv_done.notify_all();
  e->cv_sched.notify_all();
  e->sched.join();
  for (auto &t : e->threads) t.join();
  {
    // threads still inside cm_engine_wait leave before the engine goes away
    std::unique_lock<std::mutex> lk(e->mu);
    e->cv_done.wait(lk, [&] { return e->waiters == 0; });
  }
  for (cm_ctx *c : e->ctxs) cm_ctx_destroy(c);
  cm_ctx_destroy(e->sched_ctx);
  delete e;
}

extern "C" int cm_engine_submit(cm_engine *e, const cm_graph *g, int32_t nparts, const cm_part_params *params,
                                int32_t *part, int64_t *job_id) {
  if (!e || !g || !part || !job_id || nparts < 1 || g->nvtxs < 0)
    return cm_fail(CM_ERR_INVALID, "cm_engine_submit: bad arguments");
  auto j = std::make_unique<Job>();
  j->g = *g;
  j->nparts = nparts;
  if (params) j->params = *params;
  else cm_part_default_params(&j->params);
  j->part = part;
  j->footprint = footprint_bytes(g->nvtxs, g->nedges, nparts);
  j->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(e->mu);
  if (e->stop) return cm_fail(CM_ERR_INVALID, "cm_engine_submit: engine is shutting down");
  if (e->max_queue > 0 && (int64_t)(e->pending.size() + e->ready.size()) >= e->max_queue)
    return cm_fail(CM_ERR_LIMIT, "cm_engine_submit: queue full (%d waiting jobs)", e->max_queue);
  j->id = e->next_id++;
  *job_id = j->id;
  e->pending.push_back(j.get());
  e->jobs.emplace(j->id, std::move(j));
  e->admit_locked();
  return CM_OK;
}

extern "C" int cm_engine_wait(cm_engine *e, int64_t job_id, int32_t *objval, cm_job_info *info) {
  if (!e) return cm_fail(CM_ERR_INVALID, "cm_engine_wait: null engine");
  std::unique_lock<std::mutex> lk(e->mu);
  auto it = e->jobs.find(job_id);
  if (it == e->jobs.end()) return cm_fail(CM_ERR_INVALID, "cm_engine_wait: unknown job %lld", (long long)job_id);
  Job *j = it->second.get();
  if (j->waited) return cm_fail(CM_ERR_INVALID, "cm_engine_wait: job %lld already has a waiter", (long long)job_id);
  j->waited = true;
  ++e->waiters;
  e->cv_done.wait(lk, [&] { return j->done; });
  --e->waiters;
  if (objval) *objval = j->objval;
  if (info) {
    info->queue_ms = ms_between(j->t_submit, j->t_start);
    info->run_ms = ms_between(j->t_start, j->t_end);
    info->latency_ms = ms_between(j->t_submit, j->t_end);
    info->stats = j->stats;
    info->status = j->status;
  }
  const int rc = j->status;
  const std::string err = j->error;
  e->jobs.erase(it);
  lk.unlock();
  e->cv_done.notify_all();  // a destroy may be waiting for the waiters to leave
  if (rc != CM_OK) return cm_fail(rc, "%s", err.c_str());
  return CM_OK;
}

extern "C" int cm_engine_poll(cm_engine *e, int64_t job_id, int32_t *done) {
  if (!e || !done) return cm_fail(CM_ERR_INVALID, "cm_engine_poll: bad arguments");
  std::lock_guard<std::mutex> lk(e->mu);
  auto it = e->jobs.find(job_id);
  if (it == e->jobs.end()) return cm_fail(CM_ERR_INVALID, "cm_engine_poll: unknown job %lld", (long long)job_id);
  *done = it->second->done ? 1 : 0;
  return CM_OK;
}

extern "C" int cm_engine_stats(cm_engine *e, int64_t *completed, double *p50_ms, double *p99_ms, int reset) {
  if (!e) return cm_fail(CM_ERR_INVALID, "cm_engine_stats: null engine");
  std::lock_guard<std::mutex> lk(e->mu);
  std::vector<double> v = e->latencies;
  std::sort(v.begin(), v.end());
  auto pct = [&](double q) {
    if (v.empty()) return 0.0;
    const size_t i = std::min(v.size() - 1, (size_t)(q * (double)(v.size() - 1) + 0.5));
    return v[i];
  };
  if (completed) *completed = e->completed;
  if (p50_ms) *p50_ms = pct(0.50);
  if (p99_ms) *p99_ms = pct(0.99);
  if (reset) {
    e->latencies.clear();
    e->completed = 0;
  }
  return CM_OK;
}

extern "C" int cm_part_batch(int device, int32_t nworkers, int32_t nbatch, const cm_graph *graphs,
                             const int32_t *nparts, int32_t *const *parts, int32_t *objvals,
                             const cm_part_params *params, cm_batch_stats *stats) {
  if (nbatch < 0 || (nbatch > 0 && (!graphs || !nparts || !parts)) || nworkers < 1)
    return cm_fail(CM_ERR_INVALID, "cm_part_batch: bad arguments");
  const auto t0 = Clock::now();
  int64_t max_n = 0, max_m = 0, sum_m = 0;
  for (int i = 0; i < nbatch; ++i) {
    max_n = std::max<int64_t>(max_n, graphs[i].nvtxs);
    max_m = std::max<int64_t>(max_m, graphs[i].nedges);
    sum_m += graphs[i].nedges;
  }
  cm_engine *e = nullptr;
  int rc = cm_engine_create(device, std::min(nworkers, std::max(nbatch, 1)), 0, 0, max_n, max_m, &e);
  if (rc != CM_OK) return rc;
  const auto t1 = Clock::now();
  std::vector<int64_t> ids(nbatch);
  for (int i = 0; i < nbatch && rc == CM_OK; ++i)
    rc = cm_engine_submit(e, &graphs[i], nparts[i], params, parts[i], &ids[i]);
  int first_err = rc;
  std::string first_msg = rc == CM_OK ? std::string() : std::string(cm_last_error());
  int64_t cut_sum = 0;
  double sum_coarsen = 0, sum_init = 0, sum_uncoarsen = 0;
  for (int i = 0; i < nbatch; ++i) {
    if (ids[i] == 0) continue;
    int32_t obj = 0;
    cm_job_info info{};
    const int r = cm_engine_wait(e, ids[i], &obj, &info);
    if (objvals) objvals[i] = obj;
    cut_sum += obj;
    sum_coarsen += info.stats.coarsen_ms;
    sum_init += info.stats.init_ms;
    sum_uncoarsen += info.stats.uncoarsen_ms;
    if (r != CM_OK && first_err == CM_OK) {
      first_err = r;
      first_msg = cm_last_error();
    }
  }
  const auto t2 = Clock::now();
  cm_engine_destroy(e);
  if (stats) {
    stats->setup_ms = ms_between(t0, t1);
    stats->run_ms = ms_between(t1, t2);
    stats->graphs = nbatch;
    stats->sum_nedges = sum_m;
    stats->sum_cut = cut_sum;
    stats->sum_coarsen_ms = sum_coarsen;
    stats->sum_init_ms = sum_init;
    stats->sum_uncoarsen_ms = sum_uncoarsen;
  }
  if (first_err != CM_OK) return cm_fail(first_err, "%s", first_msg.c_str());
  return CM_OK;
}
