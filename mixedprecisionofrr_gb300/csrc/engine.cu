// Solve engine: many independent eigen/SVD solves sharing one GPU.
//
// Small problems (n of a few hundred, b ~ 16) cannot fill 152 SMs on their own, and a serving
// process receives requests at random times.  The engine runs a fixed set of worker threads, each
// owning an ofrr_ctx (its own non-blocking stream, cuBLAS handle and cached workspace), so solves
// overlap on the GPU.  Requests wait in a FIFO queue; admission charges each request an estimate of
// its device workspace against an HBM budget, and a request starts only when its charge fits (the
// head of the queue is never overtaken, so a large request cannot starve).  A worker whose cached
// workspace exceeds its share of the budget releases it after a solve.  The library's own kernels reduce
// in a fixed order; a request's result in the mix matches its result alone bit for bit on small solves
// and within its tolerance on large dense SVDs (whose certification fallback and FP64 continuation use
// the library GEMM), where the last bits can differ.
//
// Batched form (ofrr_batch_si_eig): submit every problem, then wait for all of them.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ofrr_internal.cuh"

namespace ofrr {
namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Job {
  uint64_t ticket = 0;
  ofrr_request req{};
  size_t charge = 0;
  int status = OFRR_SUCCESS;
  bool done = false;
  double t_submit = 0, t_start = 0, t_end = 0;
};

// device workspace a request may hold at its peak (bytes), from the sizes of its operator and bases
size_t request_charge(const ofrr_request& r) {
  const ofrr_operator& A = r.A;
  const size_t m = (size_t)A.nrows, n = (size_t)A.ncols;
  const size_t b = (size_t)(r.opt.block > 0 ? r.opt.block : 1);
  size_t bytes = (size_t)64 << 20;  // small matrices, flags, first workspace chunk
  if (A.kind == OFRR_OP_DENSE) {
    // 16-bit copies of A and A', exact-slice digit stacks of both orientations, an FP64 A' transient
    bytes += m * n * (2 + 2 + 10 + 10 + 8);
  } else {
    bytes += (size_t)A.csr.nnz * 8;
  }
  const size_t kb = (r.kind == OFRR_REQ_ARNOLDI_EIG) ? (size_t)(r.opt.kdim > 0 ? r.opt.kdim : r.opt.maxiter) + 1 : b;
  bytes += (m + n) * kb * 8 * 8;  // bases, products and their 16-bit / sliced copies
  return bytes;
}

}  // namespace
}  // namespace ofrr

struct ofrr_serve {
  int device = 0;
  size_t budget = 0;
  size_t charged = 0;
  std::vector<ofrr_ctx*> ctxs;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<ofrr::Job*> queue;
  std::unordered_map<uint64_t, ofrr::Job*> jobs;
  uint64_t next_ticket = 1;
  bool stopping = false;
  // statistics
  uint64_t completed = 0, failed = 0;
  double busy_ms = 0, first_submit = -1, last_end = 0;
  std::vector<double> latencies;
};

namespace ofrr {
namespace {

int run_request(ofrr_ctx* ctx, const ofrr_request& r) {
  switch (r.kind) {
    case OFRR_REQ_SI_EIG:
      return ofrr_si_eig(ctx, &r.A, &r.opt, r.V, r.ldv, r.values, r.resid, r.info);
    case OFRR_REQ_SI_SVD:
      return ofrr_si_svd(ctx, &r.A, &r.opt, r.U, r.ldu, r.values, r.V, r.ldv, r.resid, r.info);
    case OFRR_REQ_ARNOLDI_EIG:
      return ofrr_arnoldi_eig(ctx, &r.A, &r.opt, r.v0, r.V, r.ldv, r.values, r.resid, r.info);
    default:
      return OFRR_ERR_INVALID_ARGUMENT;
  }
}

void worker_loop(ofrr_serve* s, int w) {
  ofrr_ctx* ctx = s->ctxs[w];
  cudaSetDevice(s->device);
  const size_t share = s->budget / (s->ctxs.empty() ? 1 : s->ctxs.size());
  while (true) {
    Job* job = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] {
        return s->stopping || (!s->queue.empty() && s->charged + s->queue.front()->charge <= s->budget) ||
               (!s->queue.empty() && s->charged == 0);  // a request larger than the budget runs alone
      });
      if (s->queue.empty() && s->stopping) return;
      if (s->queue.empty()) continue;
      job = s->queue.front();
      s->queue.pop_front();
      s->charged += job->charge;
      job->t_start = now_ms();
    }
    int st = run_request(ctx, job->req);
    const int sst = ofrr_ctx_synchronize(ctx);
    if (st == OFRR_SUCCESS) st = sst;
    if (ofrr_ctx_workspace_bytes(ctx) > share) ofrr_ctx_trim(ctx);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      job->status = st;
      job->t_end = now_ms();
      job->done = true;
      s->charged -= job->charge;
      s->completed++;
      if (st != OFRR_SUCCESS && st != OFRR_ERR_SOLVER_MAX_ITERATIONS) s->failed++;
      s->busy_ms += job->t_end - job->t_start;
      s->last_end = job->t_end;
      s->latencies.push_back(job->t_end - job->t_submit);
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

}  // namespace
}  // namespace ofrr

using namespace ofrr;

extern "C" {

int ofrr_serve_create(ofrr_serve** out, int device, int workers, size_t hbm_budget_bytes) {
  if (!out || workers < 1 || workers > 64) return OFRR_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  ofrr_serve* s = new ofrr_serve();
  s->device = device;
  if (hbm_budget_bytes == 0) {
    size_t fr = 0, tot = 0;
    OFRR_CUDA(cudaSetDevice(device));
    OFRR_CUDA(cudaMemGetInfo(&fr, &tot));
    hbm_budget_bytes = fr / 2;
  }
  s->budget = hbm_budget_bytes;
  for (int w = 0; w < workers; ++w) {
    ofrr_ctx* c = nullptr;
    const int st = ofrr_ctx_create(&c, device, nullptr);
    if (st != OFRR_SUCCESS) {
      for (ofrr_ctx* x : s->ctxs) ofrr_ctx_destroy(x);
      delete s;
      return st;
    }
    s->ctxs.push_back(c);
  }
  for (int w = 0; w < workers; ++w) s->threads.emplace_back(worker_loop, s, w);
  *out = s;
  return OFRR_SUCCESS;
}

int ofrr_serve_destroy(ofrr_serve* s) {
  if (!s) return OFRR_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
  }
  s->cv_work.notify_all();
  for (std::thread& t : s->threads) t.join();
  for (ofrr_ctx* c : s->ctxs) ofrr_ctx_destroy(c);
  for (auto& kv : s->jobs) delete kv.second;
  delete s;
  return OFRR_SUCCESS;
}

int ofrr_serve_submit(ofrr_serve* s, const ofrr_request* r, uint64_t* ticket) {
  if (!s || !r || !ticket) return OFRR_ERR_INVALID_ARGUMENT;
  if (r->kind != OFRR_REQ_SI_EIG && r->kind != OFRR_REQ_SI_SVD && r->kind != OFRR_REQ_ARNOLDI_EIG)
    return OFRR_ERR_INVALID_ARGUMENT;
  Job* j = new Job();
  j->req = *r;
  j->charge = request_charge(*r);
  j->t_submit = now_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) {
      delete j;
      return OFRR_ERR_INVALID_ARGUMENT;
    }
    j->ticket = s->next_ticket++;
    s->jobs[j->ticket] = j;
    s->queue.push_back(j);
    if (s->first_submit < 0) s->first_submit = j->t_submit;
    *ticket = j->ticket;
  }
  s->cv_work.notify_all();
  return OFRR_SUCCESS;
}

int ofrr_serve_poll(ofrr_serve* s, uint64_t ticket, int* done, int* status) {
  if (!s || !done) return OFRR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return OFRR_ERR_INVALID_ARGUMENT;
  *done = it->second->done ? 1 : 0;
  if (status) *status = it->second->done ? it->second->status : OFRR_SUCCESS;
  return OFRR_SUCCESS;
}

int ofrr_serve_wait(ofrr_serve* s, uint64_t ticket, int* status, double* latency_ms) {
  if (!s) return OFRR_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return OFRR_ERR_INVALID_ARGUMENT;
  Job* j = it->second;
  s->cv_done.wait(lk, [&] { return j->done; });
  if (status) *status = j->status;
  if (latency_ms) *latency_ms = j->t_end - j->t_submit;
  s->jobs.erase(it);  // a ticket is released once its result has been collected
  delete j;
  return OFRR_SUCCESS;
}

int ofrr_serve_stats(ofrr_serve* s, ofrr_serve_report* out) {
  if (!s || !out) return OFRR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  out->completed = s->completed;
  out->failed = s->failed;
  out->queued = s->queue.size();
  out->charged_bytes = s->charged;
  out->budget_bytes = s->budget;
  out->wall_ms = (s->first_submit >= 0) ? s->last_end - s->first_submit : 0.0;
  out->busy_ms = s->busy_ms;
  std::vector<double> l = s->latencies;
  std::sort(l.begin(), l.end());
  out->p50_ms = l.empty() ? 0.0 : l[l.size() / 2];
  out->p99_ms = l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t)(0.99 * (double)l.size()))];
  return OFRR_SUCCESS;
}

int ofrr_batch_si_eig(ofrr_serve* s, int count, const ofrr_operator* ops, const ofrr_options* opt, void* const* V,
                      const int64_t* ldv, double* const* evals, double* const* resid, ofrr_info* infos,
                      int* statuses) {
  if (!s || count < 0 || (count > 0 && (!ops || !opt || !V || !ldv || !evals || !statuses)))
    return OFRR_ERR_INVALID_ARGUMENT;
  std::vector<uint64_t> tickets(count, 0);
  int first_err = OFRR_SUCCESS;
  for (int i = 0; i < count; ++i) {
    ofrr_request r{};
    r.kind = OFRR_REQ_SI_EIG;
    r.A = ops[i];
    r.opt = *opt;
    r.V = V[i];
    r.ldv = ldv[i];
    r.values = evals[i];
    r.resid = resid ? resid[i] : nullptr;
    r.info = infos ? &infos[i] : nullptr;
    const int st = ofrr_serve_submit(s, &r, &tickets[i]);
    if (st != OFRR_SUCCESS) {
      statuses[i] = st;
      tickets[i] = 0;
      if (first_err == OFRR_SUCCESS) first_err = st;
    }
  }
  for (int i = 0; i < count; ++i) {
    if (!tickets[i]) continue;
    int st = OFRR_SUCCESS;
    OFRR_TRY(ofrr_serve_wait(s, tickets[i], &st, nullptr));
    statuses[i] = st;
  }
  return first_err;
}

}  // extern "C"
