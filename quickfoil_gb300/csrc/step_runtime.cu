// step_runtime.cu -- replaying batched steps from CUDA graphs, and a serving
// loop that runs literal-scoring requests of many rule searches concurrently.
//
// Graphs.  A refinement step's host work (planning, relation key tables,
// scratch sizing, descriptor building) is done once; its device work -- ~50
// memsets, scans, partition passes and evaluation launches -- is captured
// into a CUDA graph with its own workspace and replayed with one
// cudaGraphLaunch.  The graph reads the binding set at replay time, so new
// binding data of the same shape (the same binding set refilled in place) is
// evaluated by a replay.
//
// Serving.  A server owns `slots` workspaces, each with its own stream and
// pinned count buffers.  Requests (a device-resident binding set plus a batch
// of candidate literals) are admitted in arrival order when a slot has room
// and the scratch they need fits the server's HBM budget next to the
// requests in flight; admitted requests run concurrently on their slots'
// streams, and requests that arrive meanwhile are admitted as slots and
// memory free up (continuous batching).  A slot holds up to `depth`
// requests (QFG_OPT_SERVER_DEPTH): the ones after the first are queued on
// its stream behind it, so consecutive requests of a slot follow each other
// on the GPU without a host turnaround between them, sharing the slot's
// workspace in stream order.  Completion is stamped on the host by a stream
// callback; latency = completion - submission.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <chrono>
#include <cstring>
#include <deque>
#include <vector>

#include "eval_common.cuh"

using namespace qfg;

extern "C" int qfg_step_scratch_bytes(qfg_ctx* c, const qfg_bindings* b, int32_t n,
                                      const qfg_literal* lits, int64_t* bytes) {
  if (c == nullptr || b == nullptr || bytes == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  QFG_TRY(validate_literals(ctx, b, n, lits));
  return step_scratch_bytes(ctx, b, n, lits, bytes);
}

struct qfg_step_graph {
  Workspace ws;
  cudaStream_t capture_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t launches_per_replay = 0;
  DevBuf own_counts;  // counts of a graph kept in the context's cache
};

namespace qfg {

void step_graph_free(Ctx* ctx, qfg_step_graph* g) {
  if (g == nullptr) return;
  cudaStreamSynchronize(ctx->stream);
  if (g->exec != nullptr) cudaGraphExecDestroy(g->exec);
  if (g->graph != nullptr) cudaGraphDestroy(g->graph);
  if (g->capture_stream != nullptr) cudaStreamSynchronize(g->capture_stream);
  g->ws.release();
  g->own_counts.release();
  if (g->capture_stream != nullptr) cudaStreamDestroy(g->capture_stream);
  delete g;
}

// Prepares the step in the graph's own workspace, runs it once uncaptured
// (which sizes every scratch buffer it touches, so the captured run
// allocates nothing), then captures the zeroing of the counts and the step's
// device work.
int step_graph_build(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                     unsigned long long* counts, qfg_step_graph* g) {
  if (cudaStreamCreateWithFlags(&g->capture_stream, cudaStreamNonBlocking) != cudaSuccess)
    return cuda_error(ctx, cudaGetLastError(), "cudaStreamCreate");
  g->ws.stream = g->capture_stream;
  const bool timing = ctx->stage_timing;
  int st = QFG_OK;
  {
    WorkspaceScope scope(ctx, &g->ws);
    PreparedStep* ps = prepared_step_new();
    st = prepare_step(ctx, b, n, lits, counts, ps);
    if (st == QFG_OK) st = upload_prepared(ctx, ps, true);
    if (st == QFG_OK) {
      ctx->stage_timing = false;
      st = enqueue_step(ctx, ps);
    }
    if (st == QFG_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      st = cuda_error(ctx, cudaGetLastError(), "warm-up run");
    if (st == QFG_OK) {
      const int64_t before = ctx->launches;
      cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) {
        st = cuda_error(ctx, e, "cudaStreamBeginCapture");
      } else {
        if (n > 0) e = cudaMemsetAsync(counts, 0, sizeof(int64_t) * 4 * (size_t)n, ctx->stream);
        int st2 = e == cudaSuccess ? enqueue_step(ctx, ps) : cuda_error(ctx, e, "memset");
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(ctx->stream, &graph);
        g->graph = graph;
        if (st2 != QFG_OK) st = st2;
        else if (e != cudaSuccess) st = cuda_error(ctx, e, "cudaStreamEndCapture");
        g->launches_per_replay = ctx->launches - before;
      }
    }
    ctx->stage_timing = timing;
    prepared_step_free(ps);
  }
  if (st != QFG_OK) return st;
  QFG_CUDA(ctx, cudaGraphInstantiate(&g->exec, g->graph, 0));
  return QFG_OK;
}

int step_graph_replay(Ctx* ctx, qfg_step_graph* g) {
  if (g->exec == nullptr) return QFG_OK;
  QFG_CUDA(ctx, cudaGraphLaunch(g->exec, ctx->stream));
  ctx->launches += g->launches_per_replay;
  return QFG_OK;
}

void graph_cache_clear(Ctx* ctx) {
  for (auto& kv : ctx->graph_cache) step_graph_free(ctx, kv.second);
  ctx->graph_cache.clear();
}

namespace {

constexpr size_t kGraphCacheEntries = 8;

template <typename T>
void append_bytes(std::string* key, const T& v) {
  key->append(reinterpret_cast<const char*>(&v), sizeof(T));
}

}  // namespace

int evaluate_step_cached(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                         unsigned long long* counts) {
  const int64_t nb = b->num_positive + b->num_negative;
  std::string key;
  append_bytes(&key, b);
  append_bytes(&key, b->num_positive);
  append_bytes(&key, b->num_negative);
  for (const int32_t* c : b->columns) append_bytes(&key, c);
  append_bytes(&key, n);
  key.append(reinterpret_cast<const char*>(lits), sizeof(qfg_literal) * (size_t)n);
  append_bytes(&key, step_partition_bits(ctx, nb));
  append_bytes(&key, ctx->shard_index);
  append_bytes(&key, ctx->shard_count);
  auto it = ctx->graph_cache.find(key);
  qfg_step_graph* g = nullptr;
  if (it != ctx->graph_cache.end()) {
    g = it->second;
  } else {
    if (ctx->graph_cache.size() >= kGraphCacheEntries) graph_cache_clear(ctx);
    g = new qfg_step_graph();
    int st = g->own_counts.reserve(ctx, sizeof(int64_t) * 4 * (size_t)std::max(n, 1));
    if (st == QFG_OK)
      st = step_graph_build(ctx, b, n, lits, g->own_counts.as<unsigned long long>(), g);
    if (st != QFG_OK) {
      step_graph_free(ctx, g);
      return st;
    }
    ctx->graph_cache[key] = g;
  }
  QFG_TRY(step_graph_replay(ctx, g));
  if (n > 0)
    QFG_CUDA(ctx, cudaMemcpyAsync(counts, g->own_counts.ptr(), sizeof(int64_t) * 4 * (size_t)n,
                                  cudaMemcpyDeviceToDevice, ctx->stream));
  return QFG_OK;
}

}  // namespace qfg

extern "C" int qfg_step_graph_destroy(qfg_ctx* c, qfg_step_graph* g) {
  if (c == nullptr || g == nullptr) return QFG_ERR_INVALID;
  step_graph_free(&c->impl, g);
  return QFG_OK;
}

extern "C" int qfg_step_graph_create(qfg_ctx* c, const qfg_bindings* b, int32_t n,
                                     const qfg_literal* lits, int64_t* counts_dev,
                                     qfg_step_graph** out) {
  if (c == nullptr || b == nullptr || out == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  *out = nullptr;
  QFG_TRY(validate_literals(ctx, b, n, lits));
  if (n > 0 && counts_dev == nullptr) return set_error(ctx, QFG_ERR_INVALID, "null counts");
  auto g = new qfg_step_graph();
  const int st = step_graph_build(ctx, b, n, lits, reinterpret_cast<unsigned long long*>(counts_dev), g);
  if (st != QFG_OK) {
    step_graph_free(ctx, g);
    return st;
  }
  *out = g;
  return QFG_OK;
}

extern "C" int qfg_step_graph_launch(qfg_ctx* c, qfg_step_graph* g) {
  if (c == nullptr || g == nullptr) return QFG_ERR_INVALID;
  return step_graph_replay(&c->impl, g);
}

// ---------------------------------------------------------------------------
// Serving loop.

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  const qfg_bindings* bindings = nullptr;
  std::vector<qfg_literal> literals;
  int64_t* host_counts = nullptr;
  int64_t scratch_bytes = 0;
  Clock::time_point submitted;
  Clock::time_point finished;
  std::atomic<int> done{0};  // set by the stream callback after `finished`
  int slot = -1;
  int status = QFG_OK;
  // Recorded on the context stream at submission: work queued there before
  // (e.g. the upload of this request's binding set) precedes the request.
  cudaEvent_t ready = nullptr;
  // Recorded on the slot stream after the completion callback: a wait for
  // this request alone (the slot's stream may hold requests queued behind).
  cudaEvent_t complete = nullptr;
  int buf = -1;           // the slot's pinned count buffer it uses
  bool retired = false;   // counts copied out, slot room given back
  ~Request() {
    if (ready != nullptr) cudaEventDestroy(ready);
    if (complete != nullptr) cudaEventDestroy(complete);
  }
};

struct PinnedCounts {
  int64_t* p = nullptr;
  size_t cap = 0;  // int64 values
};

struct Slot {
  Workspace ws;
  cudaStream_t stream = nullptr;
  // One pinned count buffer per request the slot can hold, used in turn:
  // requests of a slot retire in admission order, so a buffer comes round
  // again only after its previous request retired.
  std::vector<PinnedCounts> counts;
  int next_buf = 0;
  std::deque<Request*> running;  // admitted, in stream order
};

void CUDART_CB mark_done(void* user) {
  Request* r = static_cast<Request*>(user);
  r->finished = Clock::now();
  r->done.store(1, std::memory_order_release);
}

}  // namespace

struct qfg_server {
  Ctx* ctx = nullptr;
  int64_t budget = 0;
  int depth = 1;  // requests a slot holds at once
  std::vector<Slot> slots;
  std::deque<Request*> queue;
  std::vector<Request*> all;
  int64_t next_id = 1;
  int64_t in_flight_bytes = 0;
  int64_t peak_in_flight = 0;
  std::vector<double> latencies_ms;
  std::deque<int64_t> finished;  // retired ids not yet returned by poll
};

namespace {

int server_admit(qfg_server* s) {
  Ctx* ctx = s->ctx;
  while (!s->queue.empty()) {
    Request* r = s->queue.front();
    // The slot holding the fewest requests, if it has room.
    int free_slot = -1;
    size_t fewest = (size_t)s->depth;
    int running = 0;
    for (size_t i = 0; i < s->slots.size(); ++i) {
      const size_t k = s->slots[i].running.size();
      running += (int)k;
      if (k < fewest) {
        fewest = k;
        free_slot = (int)i;
      }
    }
    if (free_slot < 0) return QFG_OK;
    if (running > 0 && s->in_flight_bytes + r->scratch_bytes > s->budget) return QFG_OK;
    s->queue.pop_front();
    if (running == 0 && r->scratch_bytes > s->budget) {
      // Can never run: it fails alone instead of blocking the queue.
      r->status = set_error(ctx, QFG_ERR_BUDGET,
                            "request needs more scratch than the server's HBM budget");
      r->finished = Clock::now();
      r->done.store(1, std::memory_order_release);
      r->retired = true;
      s->finished.push_back(r->id);
      continue;
    }
    Slot& slot = s->slots[free_slot];
    r->slot = free_slot;
    r->buf = slot.next_buf;
    slot.next_buf = (slot.next_buf + 1) % s->depth;
    slot.running.push_back(r);
    s->in_flight_bytes += r->scratch_bytes;
    s->peak_in_flight = std::max<int64_t>(s->peak_in_flight, running + 1);
    // Idle slots give their cached scratch back when it would not fit.
    int64_t held = 0;
    for (const Slot& o : s->slots) held += o.ws.bytes();
    if (held - slot.ws.bytes() + r->scratch_bytes > s->budget) {
      for (Slot& o : s->slots)
        if (o.running.empty() && &o != &slot) o.ws.release();
    }
    const int n = (int)r->literals.size();
    int st = QFG_OK;
    PinnedCounts& pc = slot.counts[r->buf];
    if ((size_t)std::max(n, 1) * 4 > pc.cap) {
      if (pc.p != nullptr) cudaFreeHost(pc.p);
      pc.p = nullptr;
      pc.cap = 0;
      cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&pc.p),
                                    sizeof(int64_t) * 4 * (size_t)std::max(n, 1), cudaHostAllocDefault);
      if (e != cudaSuccess) st = cuda_error(ctx, e, "cudaHostAlloc");
      else pc.cap = (size_t)std::max(n, 1) * 4;
    }
    if (st == QFG_OK && r->ready != nullptr) {
      const cudaError_t e = cudaStreamWaitEvent(slot.stream, r->ready, 0);
      if (e != cudaSuccess) st = cuda_error(ctx, e, "cudaStreamWaitEvent");
    }
    if (st == QFG_OK) {
      WorkspaceScope scope(ctx, &slot.ws);
      unsigned long long* dev = nullptr;
      st = ctx->scratch[kScrCounts].reserve(ctx, sizeof(int64_t) * 4 * (size_t)std::max(n, 1));
      if (st == QFG_OK) {
        dev = ctx->scratch[kScrCounts].as<unsigned long long>();
        cudaError_t e = cudaMemsetAsync(dev, 0, sizeof(int64_t) * 4 * (size_t)std::max(n, 1),
                                        ctx->stream);
        if (e != cudaSuccess) st = cuda_error(ctx, e, "memset");
      }
      if (st == QFG_OK && n > 0) {
        PreparedStep* ps = prepared_step_new();
        st = prepare_step(ctx, r->bindings, n, r->literals.data(), dev, ps);
        if (st == QFG_OK) st = upload_prepared(ctx, ps, false);
        if (st == QFG_OK) st = enqueue_step(ctx, ps);
        prepared_step_free(ps);
        if (st == QFG_OK) {
          cudaError_t e = cudaMemcpyAsync(pc.p, dev, sizeof(int64_t) * 4 * (size_t)n,
                                          cudaMemcpyDeviceToHost, ctx->stream);
          if (e != cudaSuccess) st = cuda_error(ctx, e, "count download");
        }
      }
      if (st == QFG_OK) {
        cudaError_t e = cudaLaunchHostFunc(ctx->stream, mark_done, r);
        if (e != cudaSuccess) st = cuda_error(ctx, e, "cudaLaunchHostFunc");
      }
      if (st == QFG_OK) {
        // After the callback in stream order: complete means done is set.
        cudaError_t e = cudaEventCreateWithFlags(&r->complete, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(r->complete, ctx->stream);
        if (e != cudaSuccess) st = cuda_error(ctx, e, "cudaEventRecord");
      }
    }
    if (st != QFG_OK) {
      r->status = st;
      r->finished = Clock::now();
      r->done.store(1, std::memory_order_release);
    }
  }
  return QFG_OK;
}

// Retires finished requests, each slot's in admission order: copies their
// counts out and gives their room in the slot back.
int server_reap(qfg_server* s) {
  for (Slot& slot : s->slots) {
    while (!slot.running.empty()) {
      Request* r = slot.running.front();
      if (!r->done.load(std::memory_order_acquire)) break;
      if (r->status == QFG_OK && !r->literals.empty())
        memcpy(r->host_counts, slot.counts[r->buf].p, sizeof(int64_t) * 4 * r->literals.size());
      s->in_flight_bytes -= r->scratch_bytes;
      slot.running.pop_front();
      r->retired = true;
      s->latencies_ms.push_back(
          std::chrono::duration<double, std::milli>(r->finished - r->submitted).count());
      s->finished.push_back(r->id);
    }
  }
  return QFG_OK;
}

}  // namespace

extern "C" int qfg_server_create(qfg_ctx* c, int32_t slots, int64_t hbm_budget_bytes,
                                 qfg_server** out) {
  if (c == nullptr || out == nullptr || slots < 1 || slots > 1024) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  auto s = new qfg_server();
  s->ctx = ctx;
  s->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : ctx->budget / 2;
  s->depth = std::max(1, ctx->server_depth);
  s->slots.resize(slots);
  for (Slot& slot : s->slots) {
    slot.counts.resize((size_t)s->depth);
    if (cudaStreamCreateWithFlags(&slot.stream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      for (Slot& o : s->slots)
        if (o.stream != nullptr) cudaStreamDestroy(o.stream);
      delete s;
      return set_error(ctx, QFG_ERR_CUDA, "cudaStreamCreate failed");
    }
    slot.ws.stream = slot.stream;
  }
  *out = s;
  return QFG_OK;
}

extern "C" int qfg_server_submit(qfg_server* s, const qfg_bindings* b, int32_t n,
                                 const qfg_literal* lits, int64_t* host_counts,
                                 int64_t* request_id) {
  if (s == nullptr || b == nullptr || (n > 0 && host_counts == nullptr)) return QFG_ERR_INVALID;
  Ctx* ctx = s->ctx;
  QFG_TRY(validate_literals(ctx, b, n, lits));
  auto r = new Request();
  r->id = s->next_id++;
  r->bindings = b;
  r->literals.assign(lits, lits + n);
  r->host_counts = host_counts;
  r->submitted = Clock::now();
  int st = step_scratch_bytes(ctx, b, n, lits, &r->scratch_bytes);
  if (st == QFG_OK) {
    cudaError_t e = cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(r->ready, ctx->stream);
    if (e != cudaSuccess) st = cuda_error(ctx, e, "cudaEventRecord");
  }
  if (st != QFG_OK) {
    delete r;
    return st;
  }
  s->all.push_back(r);
  s->queue.push_back(r);
  if (request_id != nullptr) *request_id = r->id;
  QFG_TRY(server_reap(s));
  return server_admit(s);
}

extern "C" int qfg_server_poll(qfg_server* s, int64_t* done_ids, int32_t max, int32_t* num_done) {
  if (s == nullptr) return QFG_ERR_INVALID;
  QFG_TRY(server_reap(s));
  int32_t k = 0;
  while (k < max && done_ids != nullptr && !s->finished.empty()) {
    done_ids[k++] = s->finished.front();
    s->finished.pop_front();
  }
  if (num_done != nullptr) *num_done = k;
  return server_admit(s);
}

extern "C" int qfg_server_wait(qfg_server* s, int64_t request_id) {
  if (s == nullptr) return QFG_ERR_INVALID;
  Request* target = nullptr;
  for (Request* r : s->all)
    if (r->id == request_id) target = r;
  if (target == nullptr) return set_error(s->ctx, QFG_ERR_NOT_FOUND, "unknown request id");
  for (;;) {
    QFG_TRY(server_reap(s));
    QFG_TRY(server_admit(s));
    if (target->retired) break;
    // Block on the request itself once it is admitted, else on the oldest
    // request of a busy slot (its retirement makes room).  A request whose
    // admission failed has no event: it is done and retires once the
    // requests ahead of it in its slot do.
    Request* w = nullptr;
    if (target->slot >= 0) {
      const Slot& sl = s->slots[target->slot];
      w = target->complete != nullptr ? target : (sl.running.empty() ? nullptr : sl.running.front());
    } else {
      for (Slot& slot : s->slots)
        if (w == nullptr && !slot.running.empty()) w = slot.running.front();
      if (w == nullptr) return set_error(s->ctx, QFG_ERR_INVALID, "request cannot be admitted");
    }
    if (w == nullptr) break;
    if (w->complete != nullptr) QFG_CUDA(s->ctx, cudaEventSynchronize(w->complete));
  }
  return target->status;
}

extern "C" int qfg_server_drain(qfg_server* s) {
  if (s == nullptr) return QFG_ERR_INVALID;
  for (;;) {
    QFG_TRY(server_reap(s));
    QFG_TRY(server_admit(s));
    bool busy = false;
    for (Slot& slot : s->slots)
      if (!slot.running.empty()) {
        busy = true;
        QFG_CUDA(s->ctx, cudaStreamSynchronize(slot.stream));
      }
    if (!busy && s->queue.empty()) break;
  }
  return QFG_OK;
}

extern "C" int qfg_server_stats(qfg_server* s, double* p50_ms, double* p99_ms, int64_t* completed,
                                int64_t* peak_in_flight) {
  if (s == nullptr) return QFG_ERR_INVALID;
  std::vector<double> v = s->latencies_ms;
  std::sort(v.begin(), v.end());
  auto pct = [&](double q) {
    if (v.empty()) return 0.0;
    const size_t i = (size_t)std::min<double>(v.size() - 1, std::ceil(q * v.size()) - 1);
    return v[i];
  };
  if (p50_ms) *p50_ms = pct(0.50);
  if (p99_ms) *p99_ms = pct(0.99);
  if (completed) *completed = (int64_t)v.size();
  if (peak_in_flight) *peak_in_flight = s->peak_in_flight;
  return QFG_OK;
}

extern "C" int qfg_server_reset_stats(qfg_server* s) {
  if (s == nullptr) return QFG_ERR_INVALID;
  s->latencies_ms.clear();
  int64_t running = 0;
  for (const Slot& slot : s->slots) running += (int64_t)slot.running.size();
  s->peak_in_flight = running;
  return QFG_OK;
}

extern "C" int qfg_server_destroy(qfg_server* s) {
  if (s == nullptr) return QFG_ERR_INVALID;
  qfg_server_drain(s);
  for (Slot& slot : s->slots) {
    slot.ws.release();
    for (PinnedCounts& pc : slot.counts)
      if (pc.p != nullptr) cudaFreeHost(pc.p);
    if (slot.stream != nullptr) cudaStreamDestroy(slot.stream);
  }
  for (Request* r : s->all) delete r;
  delete s;
  return QFG_OK;
}
