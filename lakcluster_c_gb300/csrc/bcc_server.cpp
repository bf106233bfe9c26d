// Many bcc solves at once on one GPU: a batch entry point and a serving loop.
// (No counterpart in the reference, which runs one solve per process.)
//
// Each worker thread drives whole solves through the same driver and kernels
// as lakgb_bcc_solve.  The library gives every host thread its own CUDA stream
// and staging arena, so the kernels, copies and host-side stages of different
// solves overlap: while one solve sorts its scores on the host, another's
// Gram runs on the device.
//
// Serving is continuous batching rather than a queue in front of one solver:
// a request is admitted as soon as a worker is idle and its estimated device
// footprint fits the HBM budget beside the solves already running; requests
// that arrive while others are on the GPU join them as slots free up, in
// arrival order except that a request which does not fit yet does not hold
// back smaller ones behind it.  A solve's result does not depend on what runs
// beside it: solves share no mutable state (each owns its buffers, mirrors,
// stream and staging arena), so every result is identical to the same solve
// alone.
#include <string.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lakcluster_gb300.h"
#include "bcc_driver.h"
#include "bcc_model.h"

namespace {

using Clock = std::chrono::steady_clock;

// A deep copy of a problem, so the caller's buffers may be freed after submit.
struct OwnedProblem {
  lakgb_bcc_problem p{};
  std::vector<lakgb_bcc_bin> bins;
  std::vector<std::vector<unsigned char>> store;
  std::string qc, qr;

  explicit OwnedProblem(const lakgb_bcc_problem &src) {
    p = src;
    const long rb = (long)src.row_bytes;
    bins.assign(src.bins, src.bins + src.nbins);
    auto keep = [&](const unsigned char *ptr, size_t n) -> const unsigned char * {
      if (!ptr) return nullptr;
      store.emplace_back(ptr, ptr + n);
      return store.back().data();
    };
    store.reserve((size_t)src.nbins * 6 + 1);
    for (auto &b : bins) {
      b.A_rows = keep(b.A_rows, (size_t)b.A_nrows * rb);
      b.Z_rows = keep(b.Z_rows, (size_t)b.Z_nrows * rb);
      b.A_mr_b = keep(b.A_mr_b, (size_t)(b.A_nrows + 15) / 16 * 2);
      b.Z_mr_b = keep(b.Z_mr_b, (size_t)(b.Z_nrows + 15) / 16 * 2);
      const size_t tch = (size_t)((src.T_ncols > 0 ? src.T_ncols : 1) + 15) / 16 * 2;
      b.T_rows = keep(b.T_rows, (size_t)b.A_nrows * tch);
      b.S_rows = keep(b.S_rows, (size_t)b.Z_nrows * tch);
    }
    p.mc_b = keep(src.mc_b, (size_t)(src.ncols + 15) / 16 * 2);
    if (src.QC_strategy) {
      qc = src.QC_strategy;
      p.QC_strategy = qc.c_str();
    }
    if (src.QR_strategy) {
      qr = src.QR_strategy;
      p.QR_strategy = qr.c_str();
    }
    p.bins = bins.data();
  }
};

// Device bytes a solve holds at its peak (an upper estimate): the packed
// matrices and their transposes, the FP64 Gram matrices of every bin pair
// with their low-rank updates (kept on the device for the whole solve), the
// bit planes of the initial loop product, and the SNP x SNP low-rank blocks.
long long footprint(const lakgb_bcc_problem &p) {
  const long long m = lakbcc::bsize(p.ncols) * 8;  // padded columns
  long long bytes = 0, rows_total = 0;
  for (int i = 0; i < p.nbins; ++i) rows_total += p.bins[i].A_nrows + p.bins[i].Z_nrows;
  bytes += 2 * rows_total * m / 8;                              // rows and transposes
  for (int a = 0; a < p.nbins; ++a)
    for (int b = 0; b < p.nbins; ++b) {
      const long long na = p.bins[a].A_nrows, nz = p.bins[b].Z_nrows, nb = p.bins[b].A_nrows;
      bytes += 8 * 2 * (na * nz + na * nb);                      // AnZt, AnAt and their updates
      bytes += 8 * 3 * (na * nz + na * nb) / 4;                  // low-rank Gram blocks
      bytes += (long long)(p.B_MLT + 1) * (nz + nb) * lakbcc::bsize(na);  // planes
    }
  const long long cdrop = p.ncols / 8 + 1;
  bytes += 8 * 3 * (long long)p.ncols * cdrop * p.nbins;        // SNP x SNP blocks
  if (p.QR_strategy && strstr(p.QR_strategy, "condense"))
    bytes += 8 * (rows_total + rows_total) * cdrop;             // dense removed columns, their uploads
  return bytes + (64ll << 20);                                // staging arena, scratch
}

struct Job {
  long long id = 0;
  std::unique_ptr<OwnedProblem> prob;
  long long bytes = 0;
  Clock::time_point t_submit, t_start, t_end;
  bool has_deadline = false;
  Clock::time_point deadline;
  std::atomic<int> cancel{0};  // set by lakgb_server_cancel / destroy
  int rc = 0;
  std::string err;
  lakgb_bcc_result res{};
  bool running = false, done = false;
};

// The stop check of a worker's solve (lakbcc::set_stop_check): cancellation
// first, then the deadline.
int job_stop_check(void *ctx, const char **why) {
  Job *j = static_cast<Job *>(ctx);
  if (j->cancel.load()) {
    *why = "cancelled";
    return LAKGB_E_CANCELLED;
  }
  if (j->has_deadline && Clock::now() > j->deadline) {
    *why = "deadline passed while solving";
    return LAKGB_E_DEADLINE;
  }
  return 0;
}

}  // namespace

struct lakgb_server {
  int workers = 1;
  long long budget = 0, in_use = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job *> pending;
  std::map<long long, std::unique_ptr<Job>> jobs;
  std::vector<std::thread> threads;
  long long next_id = 1;
  int running = 0, peak_running = 0;
  int waiters = 0;  // threads inside lakgb_server_wait
  bool stop = false;

  // A queued job that will not run: completed at once with `rc`.
  void fail_pending_locked(Job *j, int rc, const char *why) {
    j->rc = rc;
    j->err = why;
    j->t_start = j->t_end = Clock::now();
    j->done = true;
    j->prob.reset();
  }

  // Next admissible job: the oldest that fits the budget (continuous
  // batching with first-fit admission).  Queued jobs past their deadline are
  // failed on the way.
  Job *admit_locked() {
    const Clock::time_point now = Clock::now();
    bool failed = false;
    for (auto it = pending.begin(); it != pending.end();) {
      Job *j = *it;
      if (j->has_deadline && now > j->deadline) {
        fail_pending_locked(j, LAKGB_E_DEADLINE, "deadline passed while queued");
        it = pending.erase(it);
        failed = true;
        continue;
      }
      if (running == 0 || in_use + j->bytes <= budget) {
        pending.erase(it);
        in_use += j->bytes;
        ++running;
        if (running > peak_running) peak_running = running;
        j->running = true;
        if (failed) cv_done.notify_all();
        return j;
      }
      ++it;
    }
    if (failed) cv_done.notify_all();
    return nullptr;
  }

  void worker() {
    for (;;) {
      Job *j = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || (j = admit_locked()) != nullptr; });
        if (!j) return;
      }
      j->t_start = Clock::now();
      lakbcc::set_stop_check(job_stop_check, j);
      j->rc = lakgb_bcc_solve(&j->prob->p, &j->res);
      lakbcc::set_stop_check(nullptr, nullptr);
      if (j->rc) {
        char msg[512];
        lakgb_bcc_last_error(msg, sizeof msg);
        j->err = msg;
      }
      j->t_end = Clock::now();
      {
        std::lock_guard<std::mutex> lk(mu);
        j->done = true;
        j->running = false;
        in_use -= j->bytes;
        --running;
        j->prob.reset();
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }
};

extern "C" lakgb_server *lakgb_server_create(int workers, long long hbm_budget_bytes) {
  auto *s = new lakgb_server();
  s->workers = workers > 0 ? workers : 1;
  s->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : (1ll << 62);
  for (int i = 0; i < s->workers; ++i) s->threads.emplace_back([s] { s->worker(); });
  return s;
}

extern "C" long long lakgb_server_submit_deadline(lakgb_server *s, const struct lakgb_bcc_problem *p,
                                                  double deadline_s) {
  if (!s || !p) return -1;
  auto j = std::make_unique<Job>();
  j->prob = std::make_unique<OwnedProblem>(*p);
  j->bytes = footprint(*p);
  j->t_submit = Clock::now();
  if (deadline_s > 0) {
    j->has_deadline = true;
    j->deadline = j->t_submit + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(deadline_s));
  }
  long long id;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return -1;
    id = j->id = s->next_id++;
    s->pending.push_back(j.get());
    s->jobs[id] = std::move(j);
  }
  s->cv_work.notify_all();
  return id;
}

extern "C" long long lakgb_server_submit(lakgb_server *s, const struct lakgb_bcc_problem *p) {
  return lakgb_server_submit_deadline(s, p, 0.0);
}

extern "C" int lakgb_server_wait_msg(lakgb_server *s, long long id, struct lakgb_bcc_result *r, double *times,
                                     char *msg, int msg_len) {
  if (msg && msg_len > 0) msg[0] = 0;
  if (r) memset(r, 0, sizeof(*r));
  std::unique_ptr<Job> j;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return -1;
    Job *raw = it->second.get();
    ++s->waiters;
    // A queued job fails at its deadline even while every worker is busy.
    while (!raw->done) {
      if (raw->has_deadline && !raw->running) {
        s->cv_done.wait_until(lk, raw->deadline + std::chrono::milliseconds(1));
        if (!raw->done && !raw->running && Clock::now() > raw->deadline) {
          for (auto p = s->pending.begin(); p != s->pending.end(); ++p)
            if (*p == raw) { s->pending.erase(p); break; }
          s->fail_pending_locked(raw, LAKGB_E_DEADLINE, "deadline passed while queued");
        }
      } else {
        s->cv_done.wait(lk);
      }
    }
    it = s->jobs.find(id);
    if (it != s->jobs.end()) {  // another waiter on the same id may have taken it
      j = std::move(it->second);
      s->jobs.erase(it);
    }
    --s->waiters;
    s->cv_done.notify_all();  // destroy may be waiting for the waiters to leave
  }
  if (!j) return -1;
  if (r) *r = j->res;
  else lakgb_bcc_result_free(&j->res);
  if (times) {
    times[0] = std::chrono::duration<double>(j->t_start - j->t_submit).count();  // queueing
    times[1] = std::chrono::duration<double>(j->t_end - j->t_start).count();     // solving
    times[2] = std::chrono::duration<double>(j->t_end - j->t_submit).count();    // latency
  }
  if (msg && msg_len > 0) {
    strncpy(msg, j->err.c_str(), (size_t)msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  return j->rc;
}

extern "C" int lakgb_server_wait(lakgb_server *s, long long id, struct lakgb_bcc_result *r, double *times) {
  return lakgb_server_wait_msg(s, id, r, times, nullptr, 0);
}

extern "C" int lakgb_server_cancel(lakgb_server *s, long long id) {
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end() || it->second->done) return -1;
  Job *j = it->second.get();
  j->cancel.store(1);
  if (!j->running) {
    for (auto p = s->pending.begin(); p != s->pending.end(); ++p)
      if (*p == j) { s->pending.erase(p); break; }
    s->fail_pending_locked(j, LAKGB_E_CANCELLED, "cancelled while queued");
    s->cv_done.notify_all();
  }
  return 0;
}

extern "C" int lakgb_server_peak_concurrency(lakgb_server *s) {
  std::lock_guard<std::mutex> lk(s->mu);
  return s->peak_running;
}

extern "C" long long lakgb_bcc_footprint(const struct lakgb_bcc_problem *p) { return footprint(*p); }

extern "C" void lakgb_server_destroy(lakgb_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (Job *j : s->pending) s->fail_pending_locked(j, LAKGB_E_CANCELLED, "server shut down");
    s->pending.clear();
    for (auto &kv : s->jobs)
      if (kv.second->running) kv.second->cancel.store(1);
  }
  s->cv_work.notify_all();
  s->cv_done.notify_all();
  for (auto &t : s->threads) t.join();
  {
    // every job is done now; let the threads inside wait collect theirs
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.notify_all();
    s->cv_done.wait(lk, [&] { return s->waiters == 0; });
  }
  for (auto &kv : s->jobs) lakgb_bcc_result_free(&kv.second->res);
  delete s;
}

extern "C" int lakgb_bcc_solve_many(const struct lakgb_bcc_problem *ps, int n, struct lakgb_bcc_result *rs,
                                    int *rcs, int workers, long long hbm_budget_bytes) {
  lakgb_server *s = lakgb_server_create(workers, hbm_budget_bytes);
  std::vector<long long> ids(n);
  for (int i = 0; i < n; ++i) ids[i] = lakgb_server_submit(s, &ps[i]);
  int bad = 0;
  for (int i = 0; i < n; ++i) {
    const int rc = lakgb_server_wait(s, ids[i], &rs[i], nullptr);
    if (rcs) rcs[i] = rc;
    bad += rc != 0;
  }
  lakgb_server_destroy(s);
  return bad;
}
