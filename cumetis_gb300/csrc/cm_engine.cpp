// cm_engine.cpp -- many independent partitions on one GPU: the batched form
// (cm_part_batch) and the served form (cm_engine_*: submit / wait with
// admission by device-memory footprint).  Neither has a counterpart in the
// reference, which partitions one graph per process (cuMetis.cu:3874).
//
// Design: a pool of worker threads, each owning a cm_ctx (workspace, status
// block, its own non-blocking stream).  A worker takes the oldest admitted
// job and runs the whole pipeline for it (cm_part_graph: coarsening and
// refinement on the worker's stream, the initial partition on the worker's
// host thread).  Jobs of different workers overlap on the GPU through their
// streams, and their host steps run in parallel on the host cores.  A job is
// admitted while the estimated device memory of the running jobs stays within
// the budget (a job larger than the budget runs alone).  Graphs are read from
// the caller's host arrays, which must stay valid until the job is waited for.
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
  bool done = false;
  bool waited = false;  // a thread is in cm_engine_wait for this job
};

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
  std::vector<cm_ctx *> ctxs;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job *> pending;   // submitted, waiting for admission (FIFO)
  std::deque<Job *> ready;     // admitted, waiting for a worker
  std::unordered_map<int64_t, std::unique_ptr<Job>> jobs;
  int64_t inflight = 0;        // footprint of admitted jobs not yet finished
  int64_t next_id = 1;
  bool stop = false;
  int waiters = 0;             // threads inside cm_engine_wait
  // statistics
  int64_t completed = 0;
  std::vector<double> latencies;

  void admit_locked() {
    while (!pending.empty()) {
      Job *j = pending.front();
      const bool fits = budget <= 0 || inflight + j->footprint <= budget || inflight == 0;
      if (!fits) break;
      pending.pop_front();
      inflight += j->footprint;
      ready.push_back(j);
      cv_work.notify_one();
    }
  }

  void worker(int w) {
    cm_ctx *ctx = ctxs[w];
    for (;;) {
      Job *j = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || !ready.empty(); });
        if (ready.empty()) return;  // stop requested and nothing left
        j = ready.front();
        ready.pop_front();
        j->t_start = Clock::now();
      }
      int32_t obj = 0;
      cm_part_stats st{};
      const int rc = cm_part_graph(ctx, j->g.nvtxs, j->g.xadj, j->g.adjncy, j->g.vwgt, j->g.adjwgt, j->nparts,
                                   nullptr, nullptr, &obj, j->part, &j->params, &st);
      std::string err = rc == CM_OK ? std::string() : std::string(cm_last_error());
      {
        std::lock_guard<std::mutex> lk(mu);
        j->t_end = Clock::now();
        j->status = rc;
        j->error = err;
        j->objval = obj;
        j->stats = st;
        j->done = true;
        inflight -= j->footprint;
        ++completed;
        latencies.push_back(ms_between(j->t_submit, j->t_end));
        admit_locked();
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
  cm_engine *raw = e.get();
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
  for (auto &t : e->threads) t.join();
  {
    // threads still inside cm_engine_wait leave before the engine goes away
    std::unique_lock<std::mutex> lk(e->mu);
    e->cv_done.wait(lk, [&] { return e->waiters == 0; });
  }
  for (cm_ctx *c : e->ctxs) cm_ctx_destroy(c);
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
