// qfg_common.cuh -- shared definitions of the GB300 candidate-literal engine.
//
// Host side: the context (qfg_ctx), device buffers under an HBM budget,
// registered relations with their cached derived structures, binding sets,
// and status plumbing.  Device side: warp helpers and the hash mix used for
// the engine's own partitioning.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/qfgpu.h"

struct qfg_step_graph;

namespace qfg {

constexpr unsigned kFullMask = 0xffffffffu;

// ---------------------------------------------------------------------------
// Device helpers.

// MurmurHash3's 32-bit finalizer (Austin Appleby, public domain): a bijective
// avalanche mix.  The engine's own partitions take its top bits, so keys
// with structured low bits still spread evenly.
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

// Reference hash (utility/Hash.hpp:20-28): identity on int32, boost-style
// combine for multi-column keys.
__host__ __device__ __forceinline__ uint32_t ref_hash(int32_t v) { return (uint32_t)v; }
__host__ __device__ __forceinline__ uint32_t ref_hash_combine(uint32_t seed, int32_t v) {
  return seed ^ ((uint32_t)v + 0x9e3779b9u + (seed << 6) + (seed >> 2));
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ int warp_id() { return threadIdx.x >> 5; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ long long warp_sum(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
  return v;
}

__device__ __forceinline__ unsigned long long as_ull(long long v) {
  return (unsigned long long)v;
}

// ---------------------------------------------------------------------------
// Host side.

struct Ctx;

// Grow-only scratch buffers per context (and per workspace); see ScratchSlot.
constexpr int kNumScratch = 17;

// A device allocation charged against the context's HBM budget.
class DevBuf {
 public:
  DevBuf() = default;
  ~DevBuf();
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { *this = std::move(o); }
  DevBuf& operator=(DevBuf&& o) noexcept;

  // Ensures at least `bytes` (grow-only); contents are not preserved.
  int reserve(Ctx* ctx, size_t bytes);
  // Like reserve, but takes a block from the context's pool of released
  // binding-set storage when one is large enough, and returns its block to
  // that pool on release (binding sets uploaded step after step then
  // allocate nothing).
  int reserve_pooled(Ctx* ctx, size_t bytes);
  void release();
  template <typename T>
  T* as() const { return static_cast<T*>(ptr_); }
  void* ptr() const { return ptr_; }
  size_t bytes() const { return bytes_; }

 private:
  Ctx* ctx_ = nullptr;
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
  bool pooled_ = false;
};

// Relation tuples projected onto an ordered list of argument positions,
// deduplicated to (key tuple, multiplicity) and grouped by the engine's
// partition function (top kRelPartitionBits of mix32(first key)).
struct KeyTable {
  int num_keys = 0;
  int64_t num_entries = 0;      // distinct key tuples
  int64_t max_partition = 0;    // largest partition (entries)
  DevBuf keys;                  // num_keys SoA columns of num_entries int32
  DevBuf mult;                  // num_entries int32
  DevBuf offsets;               // (1 << kRelPartitionBits) + 1 uint32
};
constexpr int kRelPartitionBits = 16;

// A column in the reference partition layout: PartitionTuple{value, tid}
// grouped by ((uint32)v) & (2^bits-1), stable.
struct PartitionedColumn {
  int bits = 0;
  int64_t n = 0;
  int64_t max_partition = 0;
  DevBuf tuples;   // 2*n int32
  DevBuf offsets;  // 2^bits + 1 int64
};

// Open-addressing set of the relation's distinct key tuples over a list of
// argument positions: slot -> a relation row holding the tuple (-1 empty).
struct KeySet {
  uint32_t mask = 0;  // slots - 1 (slots >= 2 * tuples, a power of two)
  DevBuf owner;
  int64_t distinct = 0;  // distinct key tuples (inline form)
  DevBuf filter;         // hashed-bit filter of the key tuples, or empty
  int gbits = 0;         // bits (log2) of the larger filter kept in global memory, or 0
  DevBuf gfilter;
};

// The relation as the build side of a binding-set extension, over a list of
// argument positions: its key set (slot -> representative row), the rows
// sorted stably by representative, and each representative's segment in
// that order.
struct ExtensionBuild {
  uint32_t mask = 0;
  DevBuf owner;      // mask + 1 int32
  DevBuf sorted;     // n int32: relation rows by representative
  DevBuf seg_first;  // n int32, indexed by representative row
  DevBuf seg_last;   // n int32
};

struct Relation {
  int32_t id = 0;
  int32_t num_columns = 0;
  int64_t num_tuples = 0;
  bool borrowed = false;
  DevBuf storage;                          // owned columns (num_columns * num_tuples)
  std::vector<const int32_t*> columns;     // device column pointers
  std::map<std::vector<int>, std::unique_ptr<KeyTable>> key_tables;
  std::map<std::pair<int, int>, std::unique_ptr<PartitionedColumn>> partitions;  // (col, bits)
  std::map<std::vector<int>, std::unique_ptr<KeySet>> key_sets;  // by argument positions
  std::map<std::vector<int>, std::unique_ptr<ExtensionBuild>> ext_builds;  // by argument positions
};

struct Ctx {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  int64_t budget = 0;
  int64_t used = 0;
  std::string last_error;
  int num_radix_bits = 5;
  int eval_bits = 0;
  int64_t wait_limit = 1 << 26;
  bool withhold_copies = false;  // QFG_OPT_TEST_WITHHOLD_COPIES
  bool coverage_compat = false;  // QFG_OPT_COVERAGE_COMPAT
  int eval_mode = 0;             // QFG_OPT_EVAL_MODE (0 automatic, 1 tiled, 2 streamed)
  // Autotuner's evaluation mode and streamed-path bits offset per
  // binding-size class; stream_bias is the offset a tuning trial uses.
  std::map<int, std::pair<int, int>> tuned_mode;
  int stream_bias = 0;
  int use_graphs = 0;
  // QFG_OPT_USE_GRAPHS: captured steps by key (see step_runtime.cu).
  std::map<std::string, qfg_step_graph*> graph_cache;
  // QFG_OPT_AUTOTUNE: partition bits and pass-1 bits chosen per
  // binding-size class; eval_cbits fixes the pass-1 bits (0 = automatic).
  bool autotune = false;
  std::map<int, std::pair<int, int>> tuned_bits;
  int eval_cbits = 0;
  int server_depth = 1;  // QFG_OPT_SERVER_DEPTH: requests a server slot holds
  int shard_index = 0;
  int shard_count = 1;
  int64_t launches = 0;
  std::map<int32_t, std::unique_ptr<Relation>> relations;
  // Released binding-set storage kept for reuse (still charged to `used`).
  std::vector<std::pair<void*, size_t>> binding_pool;
  // Grow-only scratch, reused by every call on this context.
  DevBuf scratch[kNumScratch];
  // Double-buffered pinned staging for small host->device uploads
  // (descriptors), so an upload never waits on the stream.
  void* staging_host[2] = {nullptr, nullptr};
  size_t staging_cap[2] = {0, 0};
  cudaEvent_t staging_done[2] = {nullptr, nullptr};
  int staging_next = 0;
  int* error_flag = nullptr;  // device word: nonzero when a bounded wait gave up
  // Stage timing (QFG_OPT_STAGE_TIMING): CUDA events around each stage of
  // an evaluation, accumulated per stage in milliseconds.
  bool stage_timing = false;
  cudaEvent_t stage_events[2 * QFG_NUM_STAGES] = {};
  bool stage_pending[QFG_NUM_STAGES] = {};
  double stage_ms[QFG_NUM_STAGES] = {};
  int64_t stage_calls[QFG_NUM_STAGES] = {};
};

// Records the start / end of a stage on the context stream (no-op unless
// stage timing is on).  stage_end folds the previous measurement of that
// stage in before re-arming, so a stage may run many times per call.
int stage_begin(Ctx* ctx, int stage);
// Drops the graphs cached under QFG_OPT_USE_GRAPHS (relations changed).
void graph_cache_clear(Ctx* ctx);
int stage_end(Ctx* ctx, int stage);
int stage_collect(Ctx* ctx);

enum ScratchSlot {
  kScrScan = 0,
  kScrHist = 1,
  kScrTmpA = 2,
  kScrTmpB = 3,
  kScrTmpC = 4,
  kScrCounts = 5,
  kScrBindPart = 6,
  kScrBindOffsets = 7,
  kScrWork = 8,
  kScrDedup = 9,
  kScrMisc = 10,
  kScrSortA = 11,
  kScrSortB = 12,
  kScrJoin = 13,
  kScrJoin2 = 14,
  kScrLits = 15,
  kScrEntries = 16,
};
static_assert(kScrEntries + 1 == kNumScratch, "scratch slot count");

// An independent set of scratch buffers and a stream.  Evaluation code uses
// ctx->scratch and ctx->stream; a WorkspaceScope swaps a workspace's buffers
// and stream in for its lifetime, so that a captured graph or a serving slot
// owns scratch that no other call touches.
struct Workspace {
  DevBuf scratch[kNumScratch];
  cudaStream_t stream = nullptr;
  int64_t bytes() const {
    int64_t t = 0;
    for (const DevBuf& d : scratch) t += (int64_t)d.bytes();
    return t;
  }
  void release() {
    for (DevBuf& d : scratch) d.release();
  }
};

class WorkspaceScope {
 public:
  WorkspaceScope(Ctx* ctx, Workspace* ws);
  ~WorkspaceScope();
  WorkspaceScope(const WorkspaceScope&) = delete;
  WorkspaceScope& operator=(const WorkspaceScope&) = delete;

 private:
  Ctx* ctx_;
  Workspace* ws_;
};

int set_error(Ctx* ctx, int status, const std::string& msg);

// Copies `bytes` of host data to device `dst` on the context stream through
// pinned staging memory; returns once the data is staged.
int upload_small(Ctx* ctx, void* dst, const void* src, size_t bytes);
int cuda_error(Ctx* ctx, cudaError_t e, const char* what);

#define QFG_CUDA(ctx, expr)                                   \
  do {                                                        \
    cudaError_t _e = (expr);                                  \
    if (_e != cudaSuccess) return ::qfg::cuda_error((ctx), _e, #expr); \
  } while (0)

#define QFG_TRY(expr)          \
  do {                         \
    int _s = (expr);           \
    if (_s != QFG_OK) return _s; \
  } while (0)

// Records a launch and checks its configuration error.
#define QFG_LAUNCHED(ctx)                                      \
  do {                                                         \
    (ctx)->launches++;                                         \
    cudaError_t _e = cudaGetLastError();                       \
    if (_e != cudaSuccess) return ::qfg::cuda_error((ctx), _e, "kernel launch"); \
  } while (0)

// Device-wide exclusive scan of n uint32 values (in place allowed).  Returns
// the total through *total_dev (device, may be null).
int exclusive_scan_u32(Ctx* ctx, const uint32_t* in, uint32_t* out, int64_t n,
                       uint32_t* total_dev);
// Rows per label that qfg_extend_bindings(bindings, lit) produces (joins.cu).
int extension_counts(Ctx* ctx, const qfg_bindings* b, const qfg_literal* lit, int64_t* num_pos,
                     int64_t* num_neg);

// Stable radix partition into the reference layout (see qfg_radix_partition).
int radix_partition_ref(Ctx* ctx, const int32_t* values, int64_t n, int bits,
                        int32_t* out_tuples, int64_t* out_offsets);

// Stable LSD sort of n (key < 2^key_bits, payload) pairs; the first pass
// takes the row index as payload.  Buffers ping-pong; the result is returned
// through k_out / p_out.
int sort_pairs_u32(Ctx* ctx, uint32_t* k0, int32_t* p0, uint32_t* k1, int32_t* p1, int64_t n,
                   int key_bits, uint32_t** k_out, int32_t** p_out);

// Cached reference-layout partitions of a relation column.
int relation_partitions(Ctx* ctx, Relation* rel, int column, int bits,
                        PartitionedColumn** out);

// Cached deduplicated key table of a relation projection.
int relation_key_table(Ctx* ctx, Relation* rel, const std::vector<int>& positions,
                       KeyTable** out);

int find_relation(Ctx* ctx, int32_t id, Relation** out);

// BuildHashTableAfterSemiJoin in the reference's layout (after_semijoin.cu):
// nk key columns of n rows, readable past the end up to `readable` rows (a
// chain position beyond compares unequal), semi-join bits, chunk rows (<= 0:
// one chunk), FoilHashTable(num_build_tuples) arrays.
int after_semijoin_table(Ctx* ctx, const int32_t* const* cols, int nk, int64_t n, int64_t readable,
                         const uint64_t* d_bits, int64_t chunk_rows, int32_t num_build_tuples,
                         int32_t* d_buckets, int32_t* d_next, uint32_t* mask_out);

// Coverage as the reference computes it, through its chunk-relative
// projection tables (QFG_OPT_COVERAGE_COMPAT; after_semijoin.cu).  ex_cols[s]
// / ex_n[s]: the uncovered positives (s = 0) and the negatives (s = 1,
// ex_n 0 to skip); num_covered[2] and the positives' bits as qfg_coverage.
int coverage_compat(Ctx* ctx, const qfg_bindings* b, const qfg_literal* lit, int k,
                    const int32_t* const* ex_cols[2], const int64_t ex_n[2],
                    uint64_t* d_positive_bits, int64_t* num_covered);

}  // namespace qfg

struct qfg_ctx {
  qfg::Ctx impl;
};

struct qfg_bindings {
  int32_t num_columns = 0;
  int64_t num_positive = 0;
  int64_t num_negative = 0;
  bool borrowed = false;
  qfg::DevBuf storage;
  std::vector<const int32_t*> columns;  // device pointers, positives first
};
