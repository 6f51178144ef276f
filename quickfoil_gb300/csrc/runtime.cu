// runtime.cu -- context, HBM budget, relations and binding sets of libqfgpu.
//
// The reference keeps relations as host int32 columns owned by FoilPredicate
// (schema/FoilPredicate.hpp:21-68) and binding sets as host blocks owned by
// FoilClause (schema/FoilClause.hpp:72-109).  Here both live in device memory
// charged against a per-context HBM budget; derived structures (relation
// partitions and key tables) are cached per relation for the whole run, as
// the reference caches relation partitions on its TableView.
#include <cstring>
#include <new>

#include "qfg_common.cuh"

namespace qfg {

int set_error(Ctx* ctx, int status, const std::string& msg) {
  if (ctx != nullptr) ctx->last_error = msg;
  return status;
}

int cuda_error(Ctx* ctx, cudaError_t e, const char* what) {
  std::string msg = std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                    cudaGetErrorString(e) + ")";
  if (e == cudaErrorMemoryAllocation) return set_error(ctx, QFG_ERR_OOM, msg);
  return set_error(ctx, QFG_ERR_CUDA, msg);
}

DevBuf::~DevBuf() { release(); }

DevBuf& DevBuf::operator=(DevBuf&& o) noexcept {
  if (this != &o) {
    release();
    ctx_ = o.ctx_;
    ptr_ = o.ptr_;
    bytes_ = o.bytes_;
    pooled_ = o.pooled_;
    o.ctx_ = nullptr;
    o.ptr_ = nullptr;
    o.bytes_ = 0;
    o.pooled_ = false;
  }
  return *this;
}

constexpr size_t kBindingPoolBlocks = 2;

static void free_binding_pool(Ctx* ctx) {
  for (auto& blk : ctx->binding_pool) {
    cudaFree(blk.first);
    ctx->used -= (int64_t)blk.second;
  }
  ctx->binding_pool.clear();
}

void DevBuf::release() {
  if (ptr_ != nullptr) {
    // Work queued on the context stream may still read this buffer.
    if (ctx_ != nullptr) cudaStreamSynchronize(ctx_->stream);
    if (pooled_ && ctx_ != nullptr && ctx_->binding_pool.size() < kBindingPoolBlocks) {
      ctx_->binding_pool.emplace_back(ptr_, bytes_);
    } else {
      cudaFree(ptr_);
      if (ctx_ != nullptr) ctx_->used -= (int64_t)bytes_;
    }
  }
  ptr_ = nullptr;
  bytes_ = 0;
  pooled_ = false;
}

int DevBuf::reserve_pooled(Ctx* ctx, size_t bytes) {
  if (bytes <= bytes_ && ptr_ != nullptr) return QFG_OK;
  int best = -1;
  for (size_t i = 0; i < ctx->binding_pool.size(); ++i) {
    const size_t sz = ctx->binding_pool[i].second;
    if (sz >= bytes && (best < 0 || sz < ctx->binding_pool[best].second)) best = (int)i;
  }
  if (best >= 0) {
    release();
    ctx_ = ctx;
    ptr_ = ctx->binding_pool[best].first;
    bytes_ = ctx->binding_pool[best].second;
    ctx->binding_pool.erase(ctx->binding_pool.begin() + best);
    pooled_ = true;
    return QFG_OK;
  }
  QFG_TRY(reserve(ctx, bytes));
  pooled_ = true;
  return QFG_OK;
}

int DevBuf::reserve(Ctx* ctx, size_t bytes) {
  if (bytes <= bytes_ && ptr_ != nullptr) return QFG_OK;
  if (bytes == 0) bytes = 256;
  // Round up so repeated growth does not reallocate for small increases.
  size_t want = (bytes + 255) & ~size_t(255);
  if (ptr_ != nullptr) want = std::max(want, bytes_ + bytes_ / 4);
  if (ctx->used - (int64_t)bytes_ + (int64_t)want > ctx->budget) free_binding_pool(ctx);
  const int64_t after = ctx->used - (int64_t)bytes_ + (int64_t)want;
  if (after > ctx->budget) {
    want = (bytes + 255) & ~size_t(255);
    if (ctx->used - (int64_t)bytes_ + (int64_t)want > ctx->budget)
      return set_error(ctx, QFG_ERR_BUDGET,
                       "allocation of " + std::to_string(want) + " bytes exceeds the HBM budget (" +
                           std::to_string(ctx->used) + " of " + std::to_string(ctx->budget) +
                           " bytes in use)");
  }
  release();
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_error(ctx, e, "cudaMalloc");
  }
  ctx_ = ctx;
  ptr_ = p;
  bytes_ = want;
  ctx->used += (int64_t)want;
  return QFG_OK;
}

WorkspaceScope::WorkspaceScope(Ctx* ctx, Workspace* ws) : ctx_(ctx), ws_(ws) {
  for (int i = 0; i < kNumScratch; ++i) std::swap(ctx_->scratch[i], ws_->scratch[i]);
  std::swap(ctx_->stream, ws_->stream);
}

WorkspaceScope::~WorkspaceScope() {
  for (int i = 0; i < kNumScratch; ++i) std::swap(ctx_->scratch[i], ws_->scratch[i]);
  std::swap(ctx_->stream, ws_->stream);
}

int upload_small(Ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return QFG_OK;
  const int slot = ctx->staging_next;
  ctx->staging_next ^= 1;
  if (ctx->staging_done[slot] == nullptr)
    QFG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->staging_done[slot], cudaEventDisableTiming));
  else
    QFG_CUDA(ctx, cudaEventSynchronize(ctx->staging_done[slot]));  // slot's last copy finished
  if (ctx->staging_cap[slot] < bytes) {
    if (ctx->staging_host[slot] != nullptr) cudaFreeHost(ctx->staging_host[slot]);
    ctx->staging_host[slot] = nullptr;
    ctx->staging_cap[slot] = 0;
    const size_t cap = std::max<size_t>(bytes, 64 * 1024);
    QFG_CUDA(ctx, cudaHostAlloc(&ctx->staging_host[slot], cap, cudaHostAllocDefault));
    ctx->staging_cap[slot] = cap;
  }
  memcpy(ctx->staging_host[slot], src, bytes);
  QFG_CUDA(ctx, cudaMemcpyAsync(dst, ctx->staging_host[slot], bytes, cudaMemcpyHostToDevice,
                                ctx->stream));
  QFG_CUDA(ctx, cudaEventRecord(ctx->staging_done[slot], ctx->stream));
  return QFG_OK;
}

int find_relation(Ctx* ctx, int32_t id, Relation** out) {
  auto it = ctx->relations.find(id);
  if (it == ctx->relations.end())
    return set_error(ctx, QFG_ERR_NOT_FOUND, "unknown relation id " + std::to_string(id));
  *out = it->second.get();
  return QFG_OK;
}

// ---------------------------------------------------------------------------
// Device-wide exclusive scan (reduce-then-scan, recursive over block sums).

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot,
                                                         uint32_t* block_total) {
  const int lane = lane_id(), warp = warp_id();
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(kFullMask, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t t = lane < nw ? warp_tot[lane] : 0;
    uint32_t s = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFullMask, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) warp_tot[lane] = s - t;
    if (lane == nw - 1) *block_total = s;
  }
  __syncthreads();
  return x - v + warp_tot[warp];
}

__global__ void scan_tiles_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                  int64_t n, uint32_t* __restrict__ tile_sums) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t total;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k;
    v[k] = i < n ? in[i] : 0u;
    sum += v[k];
  }
  uint32_t run = block_exclusive_scan(sum, warp_tot, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (threadIdx.x == 0 && tile_sums != nullptr) tile_sums[blockIdx.x] = total;
}

__global__ void scan_add_kernel(uint32_t* __restrict__ out, int64_t n,
                                const uint32_t* __restrict__ tile_offsets) {
  const uint32_t add = tile_offsets[blockIdx.x];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  for (int k = threadIdx.x; k < kScanTile; k += blockDim.x) {
    const int64_t i = base + k;
    if (i < n) out[i] += add;
  }
}

__global__ void scan_total_kernel(const uint32_t* in_last, const uint32_t* out_last,
                                  uint32_t* total) {
  *total = *in_last + *out_last;
}

static int scan_level(Ctx* ctx, const uint32_t* in, uint32_t* out, int64_t n, uint32_t* pool,
                      size_t pool_words) {
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles <= 1) {
    scan_tiles_kernel<<<1, kScanThreads, 0, ctx->stream>>>(in, out, n, nullptr);
    QFG_LAUNCHED(ctx);
    return QFG_OK;
  }
  if ((size_t)tiles > pool_words) return set_error(ctx, QFG_ERR_INVALID, "scan pool too small");
  uint32_t* sums = pool;
  scan_tiles_kernel<<<(unsigned)tiles, kScanThreads, 0, ctx->stream>>>(in, out, n, sums);
  QFG_LAUNCHED(ctx);
  QFG_TRY(scan_level(ctx, sums, sums, tiles, pool + tiles, pool_words - tiles));
  scan_add_kernel<<<(unsigned)tiles, kScanThreads, 0, ctx->stream>>>(out, n, sums);
  QFG_LAUNCHED(ctx);
  return QFG_OK;
}

int exclusive_scan_u32(Ctx* ctx, const uint32_t* in, uint32_t* out, int64_t n,
                       uint32_t* total_dev) {
  if (n <= 0) return QFG_OK;
  // Pool for the per-level tile sums (sum of ceil(n/T^k)) plus the total.
  size_t words = 64;
  for (int64_t m = n; m > 1; m = (m + kScanTile - 1) / kScanTile) words += (size_t)(m / kScanTile + 2);
  QFG_TRY(ctx->scratch[kScrScan].reserve(ctx, words * sizeof(uint32_t)));
  uint32_t* pool = ctx->scratch[kScrScan].as<uint32_t>();
  uint32_t* last_in = pool;  // remember the last input before an in-place scan
  if (total_dev != nullptr) {
    QFG_CUDA(ctx, cudaMemcpyAsync(last_in, in + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                                  ctx->stream));
  }
  QFG_TRY(scan_level(ctx, in, out, n, pool + 1, words - 1));
  if (total_dev != nullptr) {
    scan_total_kernel<<<1, 1, 0, ctx->stream>>>(last_in, out + n - 1, total_dev);
    QFG_LAUNCHED(ctx);
  }
  return QFG_OK;
}

int stage_collect(Ctx* ctx) {
  for (int s = 0; s < QFG_NUM_STAGES; ++s) {
    if (!ctx->stage_pending[s]) continue;
    QFG_CUDA(ctx, cudaEventSynchronize(ctx->stage_events[2 * s + 1]));
    float ms = 0.f;
    QFG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->stage_events[2 * s], ctx->stage_events[2 * s + 1]));
    ctx->stage_ms[s] += ms;
    ctx->stage_calls[s] += 1;
    ctx->stage_pending[s] = false;
  }
  return QFG_OK;
}

int stage_begin(Ctx* ctx, int stage) {
  if (!ctx->stage_timing) return QFG_OK;
  if (ctx->stage_pending[stage]) QFG_TRY(stage_collect(ctx));
  if (ctx->stage_events[2 * stage] == nullptr) {
    QFG_CUDA(ctx, cudaEventCreate(&ctx->stage_events[2 * stage]));
    QFG_CUDA(ctx, cudaEventCreate(&ctx->stage_events[2 * stage + 1]));
  }
  QFG_CUDA(ctx, cudaEventRecord(ctx->stage_events[2 * stage], ctx->stream));
  return QFG_OK;
}

int stage_end(Ctx* ctx, int stage) {
  if (!ctx->stage_timing) return QFG_OK;
  QFG_CUDA(ctx, cudaEventRecord(ctx->stage_events[2 * stage + 1], ctx->stream));
  ctx->stage_pending[stage] = true;
  return QFG_OK;
}

}  // namespace qfg

using namespace qfg;

// ---------------------------------------------------------------------------
// C ABI: library and context.

extern "C" int qfg_version(void) { return 1; }

extern "C" const char* qfg_status_string(int status) {
  switch (status) {
    case QFG_OK: return "ok";
    case QFG_ERR_INVALID: return "invalid argument";
    case QFG_ERR_OOM: return "device out of memory";
    case QFG_ERR_BUDGET: return "HBM budget exceeded";
    case QFG_ERR_CUDA: return "CUDA error";
    case QFG_ERR_TIMEOUT: return "device wait timed out";
    case QFG_ERR_NOT_FOUND: return "not found";
    case QFG_ERR_MISMATCH: return "row count mismatch";
    default: return "unknown status";
  }
}

extern "C" int qfg_ctx_create(int device, int64_t hbm_budget_bytes, qfg_ctx** out) {
  if (out == nullptr) return QFG_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return QFG_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) return QFG_ERR_CUDA;
  qfg_ctx* c = new (std::nothrow) qfg_ctx();
  if (c == nullptr) return QFG_ERR_OOM;
  Ctx* ctx = &c->impl;
  ctx->device = device;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    delete c;
    return QFG_ERR_CUDA;
  }
  ctx->num_sms = prop.multiProcessorCount;
  ctx->smem_optin = prop.sharedMemPerBlockOptin;
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  ctx->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : (int64_t)(0.9 * (double)free_b);
  if (cudaMalloc(&ctx->error_flag, sizeof(int)) != cudaSuccess ||
      cudaMemset(ctx->error_flag, 0, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return QFG_ERR_CUDA;
  }
  *out = c;
  return QFG_OK;
}

extern "C" int qfg_ctx_destroy(qfg_ctx* c) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  cudaStreamSynchronize(ctx->stream);
  graph_cache_clear(ctx);
  ctx->relations.clear();
  for (auto& s : ctx->scratch) s.release();
  free_binding_pool(ctx);
  for (int i = 0; i < 2; ++i) {
    if (ctx->staging_host[i] != nullptr) cudaFreeHost(ctx->staging_host[i]);
    if (ctx->staging_done[i] != nullptr) cudaEventDestroy(ctx->staging_done[i]);
  }
  if (ctx->error_flag != nullptr) cudaFree(ctx->error_flag);
  for (auto& e : ctx->stage_events)
    if (e != nullptr) cudaEventDestroy(e);
  delete c;
  return QFG_OK;
}

extern "C" const char* qfg_ctx_last_error(const qfg_ctx* c) {
  return c == nullptr ? "null context" : c->impl.last_error.c_str();
}

extern "C" int qfg_ctx_set_stream(qfg_ctx* c, void* stream) {
  if (c == nullptr) return QFG_ERR_INVALID;
  c->impl.stream = static_cast<cudaStream_t>(stream);
  return QFG_OK;
}

extern "C" int qfg_ctx_synchronize(qfg_ctx* c) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return QFG_OK;
}

extern "C" int qfg_ctx_set_option(qfg_ctx* c, int option, int64_t value) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  switch (option) {
    case QFG_OPT_NUM_RADIX_BITS:
      if (value < 1 || value > QFG_MAX_RADIX_BITS)
        return set_error(ctx, QFG_ERR_INVALID, "num_radix_bits out of range [1, 15]");
      ctx->num_radix_bits = (int)value;
      return QFG_OK;
    case QFG_OPT_EVAL_BITS:
      if (value < 0 || value > 16)
        return set_error(ctx, QFG_ERR_INVALID, "eval bits out of range [0, 16]");
      ctx->eval_bits = (int)value;
      return QFG_OK;
    case QFG_OPT_WAIT_LIMIT:
      if (value < 1) return set_error(ctx, QFG_ERR_INVALID, "wait limit must be positive");
      ctx->wait_limit = value;
      return QFG_OK;
    case QFG_OPT_USE_GRAPHS:
      ctx->use_graphs = value != 0;
      return QFG_OK;
    case QFG_OPT_STAGE_TIMING:
      ctx->stage_timing = value != 0;
      return QFG_OK;
    case QFG_OPT_SHARD_INDEX:
      if (value < 0 || value >= 65536)
        return set_error(ctx, QFG_ERR_INVALID, "shard index out of range");
      ctx->shard_index = (int)value;
      return QFG_OK;
    case QFG_OPT_SHARD_COUNT:
      if (value < 1 || value > 65536)
        return set_error(ctx, QFG_ERR_INVALID, "shard count out of range [1, 65536]");
      ctx->shard_count = (int)value;
      return QFG_OK;
    case QFG_OPT_AUTOTUNE:
      ctx->autotune = value != 0;
      return QFG_OK;
    case QFG_OPT_PASS1_BITS:
      if (value < 0 || value > 8)
        return set_error(ctx, QFG_ERR_INVALID, "pass-1 bits out of range [0, 8]");
      ctx->eval_cbits = (int)value;
      return QFG_OK;
    case QFG_OPT_SERVER_DEPTH:
      if (value < 1 || value > 8)
        return set_error(ctx, QFG_ERR_INVALID, "server depth out of range [1, 8]");
      ctx->server_depth = (int)value;
      return QFG_OK;
    case QFG_OPT_TEST_WITHHOLD_COPIES:
      ctx->withhold_copies = value != 0;
      return QFG_OK;
    case QFG_OPT_COVERAGE_COMPAT:
      ctx->coverage_compat = value != 0;
      return QFG_OK;
    case QFG_OPT_EVAL_MODE:
      if (value < 0 || value > 2)
        return set_error(ctx, QFG_ERR_INVALID, "evaluation mode out of range [0, 2]");
      ctx->eval_mode = (int)value;
      graph_cache_clear(ctx);
      return QFG_OK;
    default:
      return set_error(ctx, QFG_ERR_INVALID, "unknown option " + std::to_string(option));
  }
}

extern "C" int qfg_ctx_memory(const qfg_ctx* c, int64_t* used, int64_t* budget) {
  if (c == nullptr) return QFG_ERR_INVALID;
  if (used) *used = c->impl.used;
  if (budget) *budget = c->impl.budget;
  return QFG_OK;
}

extern "C" int qfg_ctx_kernel_launches(const qfg_ctx* c, int64_t* launches) {
  if (c == nullptr || launches == nullptr) return QFG_ERR_INVALID;
  *launches = c->impl.launches;
  return QFG_OK;
}

extern "C" int qfg_ctx_stage_times(qfg_ctx* c, double* ms, int64_t* calls, int reset_after) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  QFG_TRY(stage_collect(ctx));
  for (int s = 0; s < QFG_NUM_STAGES; ++s) {
    if (ms) ms[s] = ctx->stage_ms[s];
    if (calls) calls[s] = ctx->stage_calls[s];
    if (reset_after) {
      ctx->stage_ms[s] = 0.0;
      ctx->stage_calls[s] = 0;
    }
  }
  return QFG_OK;
}

// ---------------------------------------------------------------------------
// Column upload helper: copies (or borrows) ncols columns of n rows.

static int load_columns(Ctx* ctx, int32_t ncols, const int32_t* const* cols, int64_t n,
                        int64_t dst_offset, int64_t dst_rows, int flags, DevBuf* storage,
                        std::vector<const int32_t*>* out_ptrs) {
  if (flags == QFG_DEVICE_BORROW) {
    out_ptrs->assign(cols, cols + ncols);
    return QFG_OK;
  }
  const cudaMemcpyKind kind =
      flags == QFG_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  int32_t* base = storage->as<int32_t>();
  for (int c = 0; c < ncols; ++c) {
    if (n > 0)
      QFG_CUDA(ctx, cudaMemcpyAsync(base + (int64_t)c * dst_rows + dst_offset, cols[c],
                                    sizeof(int32_t) * (size_t)n, kind, ctx->stream));
  }
  out_ptrs->resize(ncols);
  for (int c = 0; c < ncols; ++c) (*out_ptrs)[c] = base + (int64_t)c * dst_rows;
  return QFG_OK;
}

// ---------------------------------------------------------------------------
// C ABI: relations.

extern "C" int qfg_relation_register(qfg_ctx* c, int32_t relation_id, int32_t num_columns,
                                     const int32_t* const* columns, int64_t num_tuples,
                                     int flags) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_columns < 1 || num_columns > QFG_MAX_ARITY || num_tuples < 0 ||
      num_tuples > INT32_MAX || columns == nullptr ||
      (flags != QFG_HOST && flags != QFG_DEVICE_COPY && flags != QFG_DEVICE_BORROW))
    return set_error(ctx, QFG_ERR_INVALID, "invalid relation descriptor");
  for (int i = 0; i < num_columns; ++i)
    if (columns[i] == nullptr && num_tuples > 0)
      return set_error(ctx, QFG_ERR_INVALID, "null relation column");
  auto rel = std::make_unique<Relation>();
  rel->id = relation_id;
  rel->num_columns = num_columns;
  rel->num_tuples = num_tuples;
  rel->borrowed = flags == QFG_DEVICE_BORROW;
  if (!rel->borrowed)
    QFG_TRY(rel->storage.reserve(ctx, sizeof(int32_t) * (size_t)num_columns *
                                          (size_t)std::max<int64_t>(num_tuples, 1)));
  QFG_TRY(load_columns(ctx, num_columns, columns, num_tuples, 0, num_tuples, flags,
                       &rel->storage, &rel->columns));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->relations.count(relation_id)) graph_cache_clear(ctx);
  ctx->relations[relation_id] = std::move(rel);
  return QFG_OK;
}

extern "C" int qfg_relation_release(qfg_ctx* c, int32_t relation_id) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  auto it = ctx->relations.find(relation_id);
  if (it == ctx->relations.end())
    return set_error(ctx, QFG_ERR_NOT_FOUND, "unknown relation id " + std::to_string(relation_id));
  cudaStreamSynchronize(ctx->stream);
  graph_cache_clear(ctx);
  ctx->relations.erase(it);
  return QFG_OK;
}

// ---------------------------------------------------------------------------
// C ABI: binding sets.

static int bindings_common(Ctx* ctx, int32_t num_columns, int64_t num_positive,
                           int64_t num_negative, int flags) {
  if (num_columns < 1 || num_columns > 1024 || num_positive < 0 || num_negative < 0 ||
      num_positive + num_negative > INT32_MAX ||
      (flags != QFG_HOST && flags != QFG_DEVICE_COPY && flags != QFG_DEVICE_BORROW))
    return set_error(ctx, QFG_ERR_INVALID, "invalid binding-set descriptor");
  return QFG_OK;
}

extern "C" int qfg_bindings_create(qfg_ctx* c, int32_t num_columns, const int32_t* const* columns,
                                   int64_t num_positive, int64_t num_negative, int flags,
                                   qfg_bindings** out) {
  if (c == nullptr || out == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  *out = nullptr;
  QFG_TRY(bindings_common(ctx, num_columns, num_positive, num_negative, flags));
  if (columns == nullptr) return set_error(ctx, QFG_ERR_INVALID, "null binding columns");
  const int64_t n = num_positive + num_negative;
  for (int i = 0; i < num_columns; ++i)
    if (columns[i] == nullptr && n > 0)
      return set_error(ctx, QFG_ERR_INVALID, "null binding column");
  auto b = std::make_unique<qfg_bindings>();
  b->num_columns = num_columns;
  b->num_positive = num_positive;
  b->num_negative = num_negative;
  b->borrowed = flags == QFG_DEVICE_BORROW;
  if (!b->borrowed)
    QFG_TRY(b->storage.reserve_pooled(ctx, sizeof(int32_t) * (size_t)num_columns *
                                               (size_t)std::max<int64_t>(n, 1)));
  QFG_TRY(load_columns(ctx, num_columns, columns, n, 0, n, flags, &b->storage, &b->columns));
  *out = b.release();
  return QFG_OK;
}

extern "C" int qfg_bindings_create_split(qfg_ctx* c, int32_t num_columns,
                                         const int32_t* const* positive_columns,
                                         int64_t num_positive,
                                         const int32_t* const* negative_columns,
                                         int64_t num_negative, int flags, qfg_bindings** out) {
  if (c == nullptr || out == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  *out = nullptr;
  QFG_TRY(bindings_common(ctx, num_columns, num_positive, num_negative, flags));
  if (flags == QFG_DEVICE_BORROW)
    return set_error(ctx, QFG_ERR_INVALID, "split binding sets are always copied");
  if (positive_columns == nullptr || negative_columns == nullptr)
    return set_error(ctx, QFG_ERR_INVALID, "null binding columns");
  const int64_t n = num_positive + num_negative;
  auto b = std::make_unique<qfg_bindings>();
  b->num_columns = num_columns;
  b->num_positive = num_positive;
  b->num_negative = num_negative;
  QFG_TRY(b->storage.reserve_pooled(ctx, sizeof(int32_t) * (size_t)num_columns *
                                             (size_t)std::max<int64_t>(n, 1)));
  QFG_TRY(load_columns(ctx, num_columns, positive_columns, num_positive, 0, n, flags,
                       &b->storage, &b->columns));
  QFG_TRY(load_columns(ctx, num_columns, negative_columns, num_negative, num_positive, n, flags,
                       &b->storage, &b->columns));
  *out = b.release();
  return QFG_OK;
}

extern "C" int qfg_bindings_destroy(qfg_ctx* c, qfg_bindings* b) {
  if (c == nullptr || b == nullptr) return QFG_ERR_INVALID;
  cudaStreamSynchronize(c->impl.stream);
  delete b;
  return QFG_OK;
}

extern "C" int qfg_bindings_info(const qfg_bindings* b, int32_t* num_columns,
                                 int64_t* num_positive, int64_t* num_negative) {
  if (b == nullptr) return QFG_ERR_INVALID;
  if (num_columns) *num_columns = b->num_columns;
  if (num_positive) *num_positive = b->num_positive;
  if (num_negative) *num_negative = b->num_negative;
  return QFG_OK;
}

extern "C" int qfg_bindings_column(const qfg_bindings* b, int32_t column,
                                   const int32_t** device_ptr) {
  if (b == nullptr || device_ptr == nullptr || column < 0 || column >= b->num_columns)
    return QFG_ERR_INVALID;
  *device_ptr = b->columns[column];
  return QFG_OK;
}

extern "C" int qfg_bindings_download(qfg_ctx* c, const qfg_bindings* b,
                                     int32_t* const* host_columns) {
  if (c == nullptr || b == nullptr || host_columns == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  const int64_t n = b->num_positive + b->num_negative;
  for (int i = 0; i < b->num_columns; ++i) {
    if (n > 0)
      QFG_CUDA(ctx, cudaMemcpyAsync(host_columns[i], b->columns[i], sizeof(int32_t) * (size_t)n,
                                    cudaMemcpyDeviceToHost, ctx->stream));
  }
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return QFG_OK;
}
