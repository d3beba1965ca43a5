// Per-solve phase tracing: NVTX ranges always (free without a tool attached) and, when a trace sink is
// set on the context, CUDA events at every phase boundary on the context's stream.  At the end of a
// solve the events are read back and one JSON line is appended to the sink:
//   {"solver": "si_svd", "m": .., "n": .., "block": .., "step_size": .., "status": .., "iterations": ..,
//    "max_residual": .., "launches": .., "total_ms": .., "phases": {"power": {"ms": .., "n": ..}, ...}}
// Phase times are event-to-event on the main stream (work forked to the auxiliary stream is inside
// the phase that joins it).  The sink is the file named by ofrr_ctx_set_trace, or by the environment
// variable OFRR_TRACE_FILE when a context is created.
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ofrr_internal.cuh"

namespace ofrr {

struct Tracer {
  std::string path;
  struct Rec {
    const char* name;
    cudaEvent_t e0, e1;
  };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;  // events reused across solves
  size_t used = 0;

  cudaEvent_t take() {
    if (used == pool.size()) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      pool.push_back(e);
    }
    return pool[used++];
  }
  ~Tracer() {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};

static int trace_open(ofrr_ctx* c, const char* name) {
  nvtxRangePushA(name);
  Tracer* t = c ? c->tracer : nullptr;
  if (!t) return -1;
  cudaEvent_t e0 = t->take(), e1 = t->take();
  if (!e0 || !e1) return -1;
  cudaEventRecord(e0, c->stream);
  t->recs.push_back(Tracer::Rec{name, e0, e1});
  return (int)t->recs.size() - 1;
}

static void trace_close(ofrr_ctx* c, int idx) {
  if (idx >= 0 && c->tracer && idx < (int)c->tracer->recs.size())
    cudaEventRecord(c->tracer->recs[(size_t)idx].e1, c->stream);
  nvtxRangePop();
}

TraceScope::TraceScope(ofrr_ctx* c, const char* name) : ctx(c) { idx = trace_open(c, name); }
TraceScope::~TraceScope() { trace_close(ctx, idx); }
void TraceScope::next(const char* name) {
  trace_close(ctx, idx);
  idx = trace_open(ctx, name);
}

void trace_begin_solve(ofrr_ctx* ctx) {
  if (!ctx || !ctx->tracer) return;
  ctx->tracer->recs.clear();
  ctx->tracer->used = 0;
}

void trace_end_solve(ofrr_ctx* ctx, const char* solver, int64_t m, int64_t n, const ofrr_options* opt, int status,
                     const ofrr_info* info, unsigned long long launches) {
  Tracer* t = ctx ? ctx->tracer : nullptr;
  if (!t || t->recs.empty()) return;
  cudaEventSynchronize(t->recs.back().e1);
  std::map<std::string, std::pair<double, int>> agg;
  std::vector<std::string> order;
  for (const Tracer::Rec& r : t->recs) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.e0, r.e1) != cudaSuccess) ms = 0.f;
    auto it = agg.find(r.name);
    if (it == agg.end()) {
      order.push_back(r.name);
      agg[r.name] = {ms, 1};
    } else {
      it->second.first += ms;
      it->second.second += 1;
    }
  }
  float total = 0.f;
  cudaEventElapsedTime(&total, t->recs.front().e0, t->recs.back().e1);
  double inside = 0;  // top-level phases only are disjoint; nested ones (certify) are counted once
  for (const auto& kv : agg) inside += kv.second.first;
  cudaGetLastError();
  std::string line = "{\"solver\": \"" + std::string(solver) + "\"";
  char buf[512];
  snprintf(buf, sizeof buf, ", \"m\": %lld, \"n\": %lld, \"block\": %d, \"step_size\": %d, \"status\": %d", (long long)m,
           (long long)n, opt ? opt->block : 0, opt ? opt->step_size : 0, status);
  line += buf;
  if (info) {
    snprintf(buf, sizeof buf, ", \"iterations\": %d, \"max_residual\": %.6e, \"escalations\": %d", info->iterations,
             info->max_residual, info->escalations);
    line += buf;
  }
  snprintf(buf, sizeof buf, ", \"launches\": %llu, \"total_ms\": %.4f, \"between_phases_ms\": %.4f, \"phases\": {",
           launches, (double)total, std::max(0.0, (double)total - inside));
  line += buf;
  for (size_t i = 0; i < order.size(); ++i) {
    const auto& a = agg[order[i]];
    snprintf(buf, sizeof buf, "%s\"%s\": {\"ms\": %.4f, \"n\": %d}", i ? ", " : "", order[i].c_str(), a.first,
             a.second);
    line += buf;
  }
  line += "}}\n";
  static std::mutex mu;  // several contexts may share one sink
  std::lock_guard<std::mutex> lk(mu);
  if (FILE* f = fopen(t->path.c_str(), "a")) {
    fputs(line.c_str(), f);
    fclose(f);
  }
  t->recs.clear();
  t->used = 0;
}

void trace_destroy(ofrr_ctx* ctx) {
  if (ctx && ctx->tracer) {
    delete ctx->tracer;
    ctx->tracer = nullptr;
  }
}

}  // namespace ofrr

using namespace ofrr;

extern "C" int ofrr_ctx_set_trace(ofrr_ctx* ctx, const char* path) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  if (!path || !*path) {
    trace_destroy(ctx);
    return OFRR_SUCCESS;
  }
  if (!ctx->tracer) ctx->tracer = new (std::nothrow) Tracer();
  if (!ctx->tracer) return OFRR_ERR_OUT_OF_MEMORY;
  ctx->tracer->path = path;
  return OFRR_SUCCESS;
}
