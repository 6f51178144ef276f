/*
 * qfgpu.h -- C ABI of the GB300 candidate-literal engine (libqfgpu.so).
 *
 * Plain C: pointers, sizes and status codes, no C++ or CUDA types.  Every
 * call returns a status (QFG_OK == 0); none aborts.  qfg_status_string()
 * names a status and qfg_ctx_last_error() gives the detail of the last
 * failure on a context.
 *
 * Each entry point names the reference (jbalint/quickfoil) interface it
 * replaces.  The reference's operators are single-threaded C++ over host
 * int32 columns; this library keeps the same data model (int32 columns,
 * positives-first binding sets, four exact counts per candidate literal)
 * with columns resident in GPU memory.
 *
 * Threading: a context is used by one host thread at a time; different
 * contexts may be used concurrently.  Work is issued on the context's
 * stream (qfg_ctx_set_stream); calls that return host data synchronize it.
 */
#ifndef QFGPU_H_
#define QFGPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QFG_MAX_ARITY 8
#define QFG_MAX_RADIX_BITS 15

/* Status codes. */
enum {
  QFG_OK = 0,
  QFG_ERR_INVALID = 1,     /* bad argument or descriptor (rejected before any launch) */
  QFG_ERR_OOM = 2,         /* device allocation failed */
  QFG_ERR_BUDGET = 3,      /* allocation would exceed the context's HBM budget */
  QFG_ERR_CUDA = 4,        /* a CUDA call failed (message in qfg_ctx_last_error) */
  QFG_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  QFG_ERR_NOT_FOUND = 6,   /* unknown relation id */
  QFG_ERR_MISMATCH = 7     /* produced row counts differ from the announced ones */
};

/* Flags describing where caller columns live. */
enum {
  QFG_HOST = 0,            /* host memory: copied to the device */
  QFG_DEVICE_COPY = 1,     /* device memory: copied into engine-owned memory */
  QFG_DEVICE_BORROW = 2    /* device memory: used in place, caller keeps it alive */
};

/* Flags for the evaluation calls. */
enum {
  QFG_COUNTS_HOST = 0,     /* counts written to host memory, call synchronizes */
  QFG_COUNTS_DEVICE = 1    /* counts written to device memory, call is asynchronous */
};

/* Context options (qfg_ctx_set_option). */
enum {
  QFG_OPT_NUM_RADIX_BITS = 1,   /* FLAGS_num_radix_bits for qfg_radix_partition defaults (5) */
  QFG_OPT_EVAL_BITS = 2,        /* fixed partition bits of the batched path; 0 = automatic */
  QFG_OPT_WAIT_LIMIT = 3,       /* iteration limit of bounded device-side waits */
  QFG_OPT_USE_GRAPHS = 4,       /* 1 = qfg_evaluate_step replays cached CUDA graphs (see below) */
  QFG_OPT_STAGE_TIMING = 5,     /* 1 = time each evaluation stage with CUDA events */
  QFG_OPT_SHARD_INDEX = 6,      /* this context's shard of the partition space (default 0) */
  QFG_OPT_SHARD_COUNT = 7,      /* number of shards (default 1); see qfg_evaluate_step */
  QFG_OPT_AUTOTUNE = 8,         /* 1 = use the partition bits qfg_autotune_step chose per size class */
  QFG_OPT_PASS1_BITS = 9,       /* pass-1 bits of a two-pass partition (0 = automatic, else 1..8) */
  QFG_OPT_SERVER_DEPTH = 10,    /* requests a server slot holds at once, 1..8 (default 1); read by
                                   qfg_server_create (see the serving loop below) */
  QFG_OPT_TEST_WITHHOLD_COPIES = 11, /* tests of the bounded wait only: 1 = the batched evaluation
                                   kernel arms its tile barrier without issuing the tile copies,
                                   so its bounded wait runs out (QFG_OPT_WAIT_LIMIT polls) and
                                   the call returns QFG_ERR_TIMEOUT; nothing is in flight when
                                   the CTAs stop.  Default 0 */
  QFG_OPT_COVERAGE_COMPAT = 12, /* 1 = qfg_coverage / qfg_coverage_examples compute coverage as
                                   the reference does, through its chunk-relative projection
                                   tables (see qfg_coverage); 0 (default) = set membership */
  QFG_OPT_EVAL_MODE = 13        /* batched evaluation: 1 = tiled (binding-row tiles in shared
                                   memory, relation entries probing them), 2 = streamed
                                   (relation entries in shared memory, binding rows streamed
                                   past them), 0 (default) = automatic (the autotuner's choice
                                   for the size class, else tiled) */
};

/* Evaluation stages timed under QFG_OPT_STAGE_TIMING (the GPU counterpart of
 * the reference's QuickFoilTimer stages, learner/QuickFoilTimer.hpp:25-38). */
enum {
  QFG_STAGE_KEY_TABLES = 0,     /* relation partitions / key tables (first touch only) */
  QFG_STAGE_BIND_PARTITION = 1, /* binding-set partitioning */
  QFG_STAGE_EVALUATE = 2,       /* the persistent build + probe + count kernel */
  QFG_STAGE_PER_LITERAL = 3,    /* plain per-literal join-count kernels */
  QFG_STAGE_UNIT_PLAN = 4,      /* work units and entry records of the batched step */
  QFG_STAGE_COVERAGE_SCAN = 5,  /* coverage: the pass over the binding rows */
  QFG_STAGE_COVERAGE_EXAMPLES = 6, /* coverage: example key sets and bit vectors */
  QFG_NUM_STAGES = 7
};

typedef struct qfg_ctx qfg_ctx;
typedef struct qfg_bindings qfg_bindings;

/* A candidate literal (reference schema/FoilLiteral.hpp:21-164).
 * vars[i] >= 0: argument i is bound to clause variable vars[i], i.e. to
 * binding-set column vars[i]; vars[i] == -1: unbound (a new variable).
 * join_pos is FoilLiteral::join_key() (schema/FoilLiteral.hpp:133-144): the
 * bound argument with the largest variable type id, the first on ties. */
typedef struct {
  int32_t relation_id;
  int32_t num_args;
  int32_t join_pos;
  int32_t vars[QFG_MAX_ARITY];
} qfg_literal;

/* ---- library / context ------------------------------------------------ */
int qfg_version(void);
const char* qfg_status_string(int status);

/* Creates a context on CUDA device `device`.  hbm_budget_bytes bounds the
 * device memory the context may hold (0 = 90% of the free memory).  No
 * reference counterpart: the reference allocates with malloc and an
 * optional byte quota (memory/MemoryUsage.hpp:33-66). */
int qfg_ctx_create(int device, int64_t hbm_budget_bytes, qfg_ctx** out);
int qfg_ctx_destroy(qfg_ctx* ctx);
const char* qfg_ctx_last_error(const qfg_ctx* ctx);
/* stream is a cudaStream_t passed as void*; NULL selects the legacy stream. */
int qfg_ctx_set_stream(qfg_ctx* ctx, void* stream);
int qfg_ctx_synchronize(qfg_ctx* ctx);
int qfg_ctx_set_option(qfg_ctx* ctx, int option, int64_t value);
/* Bytes held and budget. */
int qfg_ctx_memory(const qfg_ctx* ctx, int64_t* used_bytes, int64_t* budget_bytes);
/* Number of kernels this context has launched (for launch accounting). */
int qfg_ctx_kernel_launches(const qfg_ctx* ctx, int64_t* launches);
/* Accumulated milliseconds and call counts per stage (QFG_NUM_STAGES
 * entries each; synchronizes the stream); reset_after != 0 clears them. */
int qfg_ctx_stage_times(qfg_ctx* ctx, double* ms, int64_t* calls, int reset_after);

/* ---- background relations --------------------------------------------- */
/* Replaces FoilPredicate's fact table (schema/FoilPredicate.hpp:21-68):
 * num_columns int32 columns of num_tuples rows, registered once per run.
 * Everything derived from the tuples is cached on the device until the
 * relation is registered again under its id or released, as TableView
 * caches partitions (storage/TableView.hpp:62-80): per-column partitions,
 * key tables, coverage key sets and filters, extension build sides.  A
 * relation registered with QFG_DEVICE_BORROW must therefore not change in
 * place; register it again after changing it. */
int qfg_relation_register(qfg_ctx* ctx, int32_t relation_id, int32_t num_columns,
                          const int32_t* const* columns, int64_t num_tuples, int flags);
int qfg_relation_release(qfg_ctx* ctx, int32_t relation_id);

/* ---- binding sets ------------------------------------------------------ */
/* Replaces FoilClause's binding blocks (schema/FoilClause.hpp:72-109):
 * consecutive layout, rows [0, num_positive) positive then num_negative
 * negative rows (integral_blocks). */
int qfg_bindings_create(qfg_ctx* ctx, int32_t num_columns, const int32_t* const* columns,
                        int64_t num_positive, int64_t num_negative, int flags,
                        qfg_bindings** out);
/* Split layout (positive_blocks / negative_blocks, schema/FoilClause.hpp:
 * 152-161); stored consecutively on the device. */
int qfg_bindings_create_split(qfg_ctx* ctx, int32_t num_columns,
                              const int32_t* const* positive_columns, int64_t num_positive,
                              const int32_t* const* negative_columns, int64_t num_negative,
                              int flags, qfg_bindings** out);
int qfg_bindings_destroy(qfg_ctx* ctx, qfg_bindings* bindings);
int qfg_bindings_info(const qfg_bindings* bindings, int32_t* num_columns,
                      int64_t* num_positive, int64_t* num_negative);
/* Device pointer of one column (rows positives first). */
int qfg_bindings_column(const qfg_bindings* bindings, int32_t column, const int32_t** device_ptr);
/* Copies all columns to host arrays of num_positive + num_negative rows. */
int qfg_bindings_download(qfg_ctx* ctx, const qfg_bindings* bindings,
                          int32_t* const* host_columns);

/* ---- candidate-literal evaluation (the hot path) ----------------------- */
/* counts receives 4 int64 per literal in CandidateLiteralInfo field order
 * (learner/CandidateLiteralInfo.hpp:15-26): num_covered_positive,
 * num_covered_negative, num_binding_positive, num_binding_negative.
 * covered = distinct binding rows of the label with at least one matching
 * relation tuple; binding = matching (relation tuple, binding row) pairs. */

/* CandidateLiteralEvaluator::Evaluate (learner/CandidateLiteralEvaluator.hpp:
 * 28-31, .cpp:264-406): every literal joins on clause variable
 * clause_join_key_id (vars[join_pos] == clause_join_key_id). */
int qfg_evaluate_group(qfg_ctx* ctx, const qfg_bindings* bindings, int32_t clause_join_key_id,
                       int32_t num_literals, const qfg_literal* literals, int64_t* counts,
                       int flags);

/* All candidate literals of one refinement step at once, any join variable
 * (the loop of QuickFoil::EvaluateAllCandidateLiterals,
 * learner/QuickFoil.cpp:418-440, in one batched evaluation).
 * With QFG_OPT_SHARD_COUNT = S > 1 the context evaluates only shard
 * QFG_OPT_SHARD_INDEX of the join-key hash partitions; every binding row
 * belongs to exactly one shard per literal, so the element-wise sum of the S
 * shards' counts is the full result (one int64 sum of 4 * n counters). */
int qfg_evaluate_step(qfg_ctx* ctx, const qfg_bindings* bindings, int32_t num_literals,
                      const qfg_literal* literals, int64_t* counts, int flags);

/* The plain per-literal GPU path: one RadixPartition -> BuildHashTable ->
 * HashJoin -> Filter -> CountAggregator chain per literal, as the
 * reference runs it (the operations/ sources).  As in the reference, the
 * binding side is partitioned once per join variable (once per Evaluate
 * call, learner/CandidateLiteralEvaluator.cpp:316-323) and each literal then
 * builds, probes and counts over that partition; relation partitions are
 * cached per (relation, column). */
int qfg_evaluate_per_literal(qfg_ctx* ctx, const qfg_bindings* bindings, int32_t num_literals,
                             const qfg_literal* literals, int64_t* counts, int flags);

/* Algorithmic bytes per stage (QFG_NUM_STAGES entries) that a batched step
 * over these literals moves: what each stage must read and write at least
 * once, the numerator of its HBM roofline.  Builds the relation key tables
 * when they are not cached yet.  No reference counterpart. */
int qfg_step_traffic(qfg_ctx* ctx, const qfg_bindings* bindings, int32_t num_literals,
                     const qfg_literal* literals, int64_t* bytes);

/* Device scratch (bytes) a batched step of these literals over this binding
 * set needs beyond the relations' cached key tables -- the figure the
 * serving loop admits requests by.  No reference counterpart. */
int qfg_step_scratch_bytes(qfg_ctx* ctx, const qfg_bindings* bindings, int32_t num_literals,
                           const qfg_literal* literals, int64_t* bytes);

/* Autotuner.  No reference counterpart (the reference reads FLAGS_num_radix_bits).
 * Times the batched step over `bindings` in both evaluation modes (see
 * QFG_OPT_EVAL_MODE): the tiled path at a few partition-bit settings around
 * its automatic choice -- the bits fix the partition pass count (one pass up
 * to 8 bits, two above) and the rows per shared-memory tile -- with both
 * splits of the bits between two passes (7 or 8 pass-1 bits), and the
 * streamed path with its per-group partition bits (chosen from each
 * literal group's relation entries, so that a partition's entries fit the
 * shared-memory table) offset by -1 .. +2; records the fastest for the
 * binding set's size class (floor(log2(rows))).  Under QFG_OPT_AUTOTUNE = 1
 * every batched step of that size class uses the recorded setting
 * (QFG_OPT_EVAL_MODE and QFG_OPT_EVAL_BITS still override).  Counts do not
 * depend on it.  best_bits / best_pass1_bits receive the tiled path's
 * partition and pass-1 bits (0 = one pass), or 0 and the bits offset when
 * the streamed path won; best_ms the time per step.  qfg_autotune_choice
 * reads the recorded setting of a size class back. */
int qfg_autotune_step(qfg_ctx* ctx, const qfg_bindings* bindings, int32_t num_literals,
                      const qfg_literal* literals, int32_t* best_bits, int32_t* best_pass1_bits,
                      double* best_ms);
/* The autotuner's setting for binding sets of num_rows rows: *mode (1 tiled,
 * 2 streamed, 0 = none recorded), *bits and *pass1_bits (tiled), *bias
 * (streamed: offset of the per-group partition bits). */
int qfg_autotune_choice(const qfg_ctx* ctx, int64_t num_rows, int32_t* mode, int32_t* bits,
                        int32_t* pass1_bits, int32_t* bias);

/* ---- batched steps replayed from CUDA graphs ---------------------------- */
/* No reference counterpart.  Captures the batched evaluation of `literals`
 * over `bindings` (as qfg_evaluate_step) into a CUDA graph with its own
 * scratch: planning, relation key tables, scratch sizing and the descriptor
 * upload happen here once; qfg_step_graph_launch replays the device work
 * with one launch on the context's stream and writes 4 int64 per literal to
 * counts_dev (device memory).  The graph reads the binding set's columns at
 * replay time, so binding data refilled in place (same binding set, same
 * sizes) is evaluated by a replay.  The binding set, the relations and
 * counts_dev must outlive the graph.
 * Under QFG_OPT_USE_GRAPHS = 1, qfg_evaluate_step itself keeps such graphs in
 * a per-context cache keyed by the binding set's shape (handle, column
 * pointers, sizes), the literal list and the partition options, and replays
 * the cached graph when a step repeats; registering or releasing a relation
 * empties the cache.  Stage timing does not apply to replayed steps. */
typedef struct qfg_step_graph qfg_step_graph;
int qfg_step_graph_create(qfg_ctx* ctx, const qfg_bindings* bindings, int32_t num_literals,
                          const qfg_literal* literals, int64_t* counts_dev,
                          qfg_step_graph** out);
int qfg_step_graph_launch(qfg_ctx* ctx, qfg_step_graph* graph);
int qfg_step_graph_destroy(qfg_ctx* ctx, qfg_step_graph* graph);

/* ---- serving loop -------------------------------------------------------- */
/* No reference counterpart (the reference runs one search at a time).  A
 * server scores candidate-literal batches of many concurrent rule searches:
 * each request is a device-resident binding set plus literals; requests are
 * admitted in arrival order when one of `slots` workspaces (own stream and
 * scratch) is free and the scratch they need fits hbm_budget_bytes (0 = half
 * the context budget) next to the requests in flight, run concurrently, and
 * are admitted as others finish.  qfg_server_submit returns at once;
 * qfg_server_poll retires finished requests (their counts land in the host
 * arrays given at submission), returns up to max_ids ids retired and not yet
 * returned, and admits queued ones; qfg_server_wait blocks
 * for one request; qfg_server_drain for all.  qfg_server_stats reports
 * latency percentiles (submission to completion).  A request is ordered
 * after the work queued on the context's stream when it was submitted, so a
 * binding set uploaded with qfg_bindings_create just before its submission
 * is complete when the request starts (and the next upload can overlap the
 * request).  With QFG_OPT_SERVER_DEPTH = d > 1 at creation a slot holds up
 * to d requests: the ones after the first are queued on the slot's stream
 * behind it (no host turnaround between them on the GPU) and the slot's
 * requests run one after another; qfg_server_wait then waits for its
 * request alone.  While a server is alive the context runs no other
 * evaluation. */
typedef struct qfg_server qfg_server;
int qfg_server_create(qfg_ctx* ctx, int32_t slots, int64_t hbm_budget_bytes, qfg_server** out);
int qfg_server_submit(qfg_server* server, const qfg_bindings* bindings, int32_t num_literals,
                      const qfg_literal* literals, int64_t* host_counts, int64_t* request_id);
int qfg_server_poll(qfg_server* server, int64_t* done_ids, int32_t max_ids, int32_t* num_done);
int qfg_server_wait(qfg_server* server, int64_t request_id);
int qfg_server_drain(qfg_server* server);
int qfg_server_stats(qfg_server* server, double* p50_ms, double* p99_ms, int64_t* completed,
                     int64_t* peak_in_flight);
/* Starts the statistics afresh (latencies, completed count, peak in flight),
 * e.g. after a warm-up that allocated the slots' scratch. */
int qfg_server_reset_stats(qfg_server* server);
int qfg_server_destroy(qfg_server* server);

/* ---- API-kept operators (device pointers, context stream) -------------- */
/* RadixPartition (operations/RadixPartition.hpp:13-14, .cpp:56-186):
 * stable partition of n int32 values by ((uint32)v) & (2^bits - 1) into
 * PartitionTuple{int32 value, int32 tuple_id} (storage/PartitionTuple.hpp:
 * 20-42).  d_out_tuples holds 2*n int32 and is 8-byte aligned (a tuple is
 * stored as one 8-byte word; cudaMalloc memory qualifies), else the call
 * returns QFG_ERR_INVALID; d_offsets 2^bits + 1 int64 (partition p = tuples
 * [offsets[p], offsets[p+1])).  1 <= bits <= 15. */
int qfg_radix_partition(qfg_ctx* ctx, const int32_t* d_values, int64_t n, int bits,
                        int32_t* d_out_tuples, int64_t* d_offsets);

/* No counterpart in the reference.  The radix partition of
 * qfg_radix_partition (same inputs, same output) for callers that must not
 * have device memory allocated on their behalf: a host process that owns all
 * GPU memory through its own allocator, or a loop that cannot take the
 * device-wide synchronization cudaMalloc / cudaFree bring.  It needs no
 * context and allocates nothing: its working memory is a fixed 4 MiB array
 * in the library's device image (held by every GPU that loads the library
 * until the process exits).  That bounds the input: about 32 Mi values at 5
 * radix bits, 8 Mi values at 12 or more bits; larger inputs return
 * QFG_ERR_INVALID with the reason in `error` (error_len bytes, may be NULL).
 * The first call on a device looks the array's device address up with that
 * device current; make that first call before any stream capture.  The
 * address is kept for the life of the process, so do not use this entry
 * point across a cudaDeviceReset.  All calls on a device share the array,
 * so calls whose work overlaps on the GPU race.  A CUDA error already
 * pending when the call starts is reported (QFG_ERR_CUDA) and left pending.
 * Work is queued on `stream` (a cudaStream_t, NULL = legacy stream). */
int qfg_radix_partition_static(void* stream, const int32_t* d_values, int64_t n, int bits,
                               int32_t* d_out_tuples, int64_t* d_offsets, char* error,
                               int error_len);

/* BuildHashTableOnPartitions (operations/BuildHashTable.cpp:54-93) with the
 * FoilHashTable layout (storage/FoilHashTable.cpp:34-49): for each non-empty
 * partition p, buckets[next_pow2(n_p)] of 1-based chain heads and next[n_p]
 * links, chains in descending position order, byte-identical to the
 * reference's.  Input is qfg_radix_partition's output (8-byte aligned,
 * else QFG_ERR_INVALID).  d_bucket_offsets
 * (2^bits + 1 int64) receives where partition p's buckets start inside
 * d_buckets, which must hold at least 2*n + 2^bits int32; d_masks (2^bits
 * uint32) receives FoilHashTable::mask(); d_next holds n int32. */
int qfg_build_hash_table_on_partitions(qfg_ctx* ctx, const int32_t* d_tuples,
                                       const int64_t* d_offsets, int64_t n, int bits,
                                       int32_t* d_buckets, int64_t* d_bucket_offsets,
                                       uint32_t* d_masks, int32_t* d_next);

/* BuildHashTableOnTable (operations/BuildHashTable.cpp:97-125,193-210):
 * whole-table chained table over num_keys key columns, hash = the
 * reference's Hash<k> HashCombine chain (utility/Hash.hpp:35-55).
 * d_buckets holds next_pow2(n) int32, d_next n int32; *mask_out receives
 * the mask.  Byte-identical to the reference's. */
int qfg_build_hash_table_on_table(qfg_ctx* ctx, const int32_t* const* d_keys, int32_t num_keys,
                                  int64_t n, int32_t* d_buckets, int32_t* d_next,
                                  uint32_t* mask_out);

/* BuildHashTableAfterSemiJoin (operations/BuildHashTable.cpp:127-189,
 * 212-236): the chained table the reference builds from a semi-join's
 * output, byte-identical.  d_keys are the semi-join's projected columns
 * (num_keys device columns of num_rows rows), d_bits its bit vector
 * (64-bit little-endian blocks, one bit per row).  The semi-join's chunks
 * are rows [c*chunk_rows, (c+1)*chunk_rows): a LeftSemiJoin cuts its probe
 * side into FLAGS_semijoin_chunck_size (32768) rows, a RightSemiJoin yields
 * one chunk (chunk_rows <= 0).  Within a chunk the set positions are taken
 * in order and, as in the reference, are chunk-relative: the id inserted is
 * the position within the chunk and keys are read at the chunk's rows, also
 * for positions already in a chain (operations/LeftSemiJoin.hpp:55-83).  A
 * position is inserted at the head of its bucket (Hash<k>, utility/Hash.hpp:
 * 35-55) unless its chain reaches a position with equal keys; a chain
 * position past the end of a short last chunk compares unequal (there the
 * reference reads past the end of its columns).  The table is
 * FoilHashTable(num_build_tuples, 0): d_buckets holds next_pow2(
 * num_build_tuples) 1-based heads, d_next num_build_tuples links (0 for
 * positions never inserted; the reference leaves those uninitialised), and
 * *mask_out the mask.  num_build_tuples must exceed every chunk-relative
 * position.  The first chunk is built in parallel; later chunks change
 * chains in an order-dependent way and are replayed in order by one GPU
 * thread (slow for many chunks; the learner's projected sides are label
 * sides of a binding set). */
int qfg_build_hash_table_after_semijoin(qfg_ctx* ctx, const int32_t* const* d_keys,
                                        int32_t num_keys, int64_t num_rows, const uint64_t* d_bits,
                                        int64_t chunk_rows, int32_t num_build_tuples,
                                        int32_t* d_buckets, int32_t* d_next, uint32_t* mask_out);

/* LeftSemiJoin<k> (operations/LeftSemiJoin.hpp:55-141): bit i of d_bits
 * (64-bit little-endian blocks, the BitVector layout of utility/BitVector.hpp)
 * is set when probe row i matches some build row on all num_keys keys.
 * *num_ones receives the set-bit count (SemiJoinChunk::num_ones). */
int qfg_left_semijoin(qfg_ctx* ctx, const int32_t* const* d_probe_keys, int64_t num_probe,
                      const int32_t* const* d_build_keys, int64_t num_build, int32_t num_keys,
                      uint64_t* d_bits, int64_t* num_ones);

/* RightSemiJoin<k> (operations/RightSemiJoin.hpp:44-82): bit j set when
 * build row j is matched by some probe row. */
int qfg_right_semijoin(qfg_ctx* ctx, const int32_t* const* d_probe_keys, int64_t num_probe,
                       const int32_t* const* d_build_keys, int64_t num_build, int32_t num_keys,
                       uint64_t* d_bits, int64_t* num_ones);

/* CreateLabelAwareBindingTables (operations/MultiColumnHashJoin.cpp:117-256):
 * the binding set extended by `literal`: every (binding row, relation
 * tuple) pair matching on the literal's bound arguments, projecting the
 * binding columns then one column per unbound argument, positives first,
 * in the reference's row order.  num_out_positive / num_out_negative are
 * the literal's binding counts; a different produced count returns
 * QFG_ERR_MISMATCH.  The new binding set stays on the device. */
int qfg_extend_bindings(qfg_ctx* ctx, const qfg_bindings* bindings, const qfg_literal* literal,
                        int64_t num_out_positive, int64_t num_out_negative,
                        qfg_bindings** out);

/* ---- facts from text --------------------------------------------------- */
/* LoadData (main/main.cpp:49-109), parsed on the device: lines end at '\n';
 * an empty line or one starting with '#' is skipped; fields split at every
 * '|' (empty fields kept) must number num_arguments (1..64); every argument
 * whose skipped[] flag is zero (skipped may be NULL) is converted as
 * std::stoi does (types/FromString.hpp:23-30: leading white space, an
 * optional sign, at least one digit, the value within int32, anything after
 * the digits ignored).  text is host memory (flags QFG_HOST, copied) or
 * device memory (QFG_DEVICE_BORROW).  The kept columns are written to
 * d_out_columns (capacity rows each); *num_rows receives the row count,
 * also when it exceeds capacity (QFG_ERR_INVALID, nothing written).  The
 * reference aborts on a bad line; here the first one is named in
 * *error_line (1-based, may be NULL) and the call returns QFG_ERR_INVALID. */
int qfg_parse_text(qfg_ctx* ctx, const char* text, int64_t num_bytes, int flags,
                   int32_t num_arguments, const int32_t* skipped, int32_t* const* d_out_columns,
                   int64_t capacity, int64_t* num_rows, int64_t* error_line);

/* CreateBackgroundPredicate (main/main.cpp:113-132): parses a predicate's
 * facts as qfg_parse_text does and registers them as relation relation_id
 * (engine-owned memory).  *num_tuples receives the fact count. */
int qfg_relation_register_text(qfg_ctx* ctx, int32_t relation_id, const char* text,
                               int64_t num_bytes, int flags, int32_t num_arguments,
                               const int32_t* skipped, int64_t* num_tuples, int64_t* error_line);

/* ---- coverage of a literal appended to the building clause ------------- */
/* QuickFoil::ComputeCoverageOnUncoveredData (learner/QuickFoil.cpp:471-573)
 * and LiteralSelector::ComputeCoveredPositives (learner/LiteralSelector.cpp:
 * 150-210).  `bindings` is the building clause's binding set, its first
 * num_target_columns columns the target's variables (the clause head).
 * A label side's binding rows whose bound arguments match some tuple of the
 * literal's relation project onto those columns; an example is covered when
 * its tuple is among that side's projections.  The examples are the
 * uncovered positives (num_uncovered_positive rows of num_target_columns
 * device columns) against the positive side and the original negatives
 * against the negative side (d_negative NULL with num_negative 0 skips them:
 * ComputeCoveredPositives).  num_covered[0] / [1] receive the covered
 * positive / negative counts.  d_positive_bits (may be NULL) receives one bit
 * per uncovered positive, set when covered, in 64-bit little-endian blocks
 * (ceil(n/64) of them, bits past the last row zero): the concatenated
 * SemiJoinChunk bit vectors of the reference (operations/SemiJoin.hpp:25-37).
 * The reference keys its projection tables by row ids that are relative to
 * each 32768-row chunk when a label side is split into chunks (a left
 * semi-join over a side of more than 32768 rows that is not smaller than
 * the relation, operations/BuildHashTable.cpp:152-189 with
 * operations/LeftSemiJoin.hpp:55-83); there its counts are not set
 * membership.  These are set membership for every size, which equals the
 * reference wherever its row ids are whole-table.  Under
 * QFG_OPT_COVERAGE_COMPAT = 1 the reference's own procedure is followed
 * instead, chunk-relative ids included: per label side the bit vector of the
 * first semi-join, the table qfg_build_hash_table_after_semijoin builds from
 * it (32768-row chunks when the side is not smaller than the relation, as
 * SelectAndCreateSemiJoin chooses, operations/SemiJoinFactory.cpp:45-82),
 * and the examples probed through that table against the side's rows.  The
 * positive side reads past its end into the negative rows, as the
 * reference's positive view of a consecutive binding set does; past the
 * negative side's end a position compares unequal (the reference reads past
 * its columns there).  1 <= num_target_columns <= 8; the literal needs at
 * least one bound argument. */
int qfg_coverage(qfg_ctx* ctx, const qfg_bindings* bindings, const qfg_literal* literal,
                 int32_t num_target_columns, const int32_t* const* d_uncovered_positive,
                 int64_t num_uncovered_positive, const int32_t* const* d_negative,
                 int64_t num_negative, uint64_t* d_positive_bits, int64_t* num_covered);

/* No counterpart in the reference: an example table prepared once for many
 * coverage calls -- the original negatives for a whole run, the uncovered
 * positives for one clause.  num_columns (1..8) device columns of num_rows
 * rows are borrowed, not copied, and must stay unchanged while the handle
 * lives; their key set is built here.  Calls that use one handle are
 * ordered on the context stream. */
typedef struct qfg_examples qfg_examples;
int qfg_examples_create(qfg_ctx* ctx, int32_t num_columns, const int32_t* const* d_columns,
                        int64_t num_rows, qfg_examples** out);
int qfg_examples_destroy(qfg_ctx* ctx, qfg_examples* examples);

/* qfg_coverage on prepared example tables: the target columns are the
 * examples' columns (num_columns of uncovered_positive; negative, which may
 * be NULL, has the same count).  Same results as qfg_coverage. */
int qfg_coverage_examples(qfg_ctx* ctx, const qfg_bindings* bindings, const qfg_literal* literal,
                          const qfg_examples* uncovered_positive, const qfg_examples* negative,
                          uint64_t* d_positive_bits, int64_t* num_covered);

/* QuickFoilTestRunner::RunTest (learner/QuickFoilTestRunner.cpp:128-161) on
 * device tables: the test rows (num_target_columns device columns of
 * num_rows rows) that none of the learnt clauses covers.  Clause i has
 * clause_lengths[i] >= 1 body literals, stored one clause after another in
 * body_literals; a literal's vars[] names binding columns (the target's
 * columns first, then one column per unbound argument of each earlier body
 * literal, in order) and -1 for an argument that introduces a new variable.
 * For every clause the full test table is extended by all body literals but
 * the last (CreateBindingTable, operations/MultiColumnHashJoin.cpp:26-115);
 * the test rows still uncovered whose tuple the last literal's coverage
 * holds are removed (ComputeUnCoveredData, QuickFoilTestRunner.cpp:40-126).
 * *num_uncovered receives the rows left; d_uncovered_out (may be NULL)
 * receives them in order (num_target_columns device columns with room for
 * num_rows rows).  Coverage is set membership (see qfg_coverage). */
int qfg_run_test(qfg_ctx* ctx, int32_t num_clauses, const int32_t* clause_lengths,
                 const qfg_literal* body_literals, int32_t num_target_columns,
                 const int32_t* const* d_test_columns, int64_t num_rows, int64_t* num_uncovered,
                 int32_t* const* d_uncovered_out);

/* The uncovered-example compaction of learner/QuickFoil.cpp:612-708 (and of
 * QuickFoilTestRunner::ComputeUnCoveredData, learner/QuickFoilTestRunner.cpp:99-116):
 * the rows of num_columns device columns whose bit in d_bits (the layout of
 * qfg_coverage's d_positive_bits) is clear (keep_set 0: the still uncovered
 * examples) or set (keep_set 1), in row order, written to d_out_columns.
 * *num_out receives the kept row count; more than out_capacity returns
 * QFG_ERR_INVALID before anything is written. */
int qfg_compact_rows(qfg_ctx* ctx, int32_t num_columns, const int32_t* const* d_columns,
                     int64_t num_rows, const uint64_t* d_bits, int32_t keep_set,
                     int32_t* const* d_out_columns, int64_t out_capacity, int64_t* num_out);

#ifdef __cplusplus
}
#endif

#endif /* QFGPU_H_ */
