// eval_common.cuh -- declarations shared by the evaluation paths.
#pragma once

#include "qfg_common.cuh"

namespace qfg {

// Checks every literal against the registered relations and the binding
// set (arity, bound join key, variable range) before anything is launched.
int validate_literals(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits);

// Zeroes the 4*n count words; for QFG_COUNTS_HOST they live in scratch.
int counts_begin(Ctx* ctx, int32_t n, int64_t* counts, int flags, unsigned long long** dev);
// Copies counts back (QFG_COUNTS_HOST, synchronizing) and reports a device
// wait that gave up.
int counts_end(Ctx* ctx, int32_t n, int64_t* counts, int flags, unsigned long long* dev);

// The plain per-literal chain: the binding join column partitioned in the
// reference layout (once per join column), then one literal's build / probe
// / count over it (counts[0..3] accumulate).
int plain_partition_bindings(Ctx* ctx, const qfg_bindings* b, int column, int* bits);
int plain_join_count(Ctx* ctx, const qfg_bindings* b, const qfg_literal& l, int bits,
                     unsigned long long* counts);

// All literals through the batched engine; counts[4*i..] accumulate.
int evaluate_batched(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                     unsigned long long* counts);

// A batched step split into its host part (planning, key tables, scratch,
// descriptors) and its device part (stream work only).
struct PreparedStep;
PreparedStep* prepared_step_new();
void prepared_step_free(PreparedStep* ps);
int prepare_step(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                 unsigned long long* counts, PreparedStep* ps);
// Copies the descriptors to the device: through pinned staging on the stream
// (sync = false) or with a blocking copy (sync = true, before a capture).
int upload_prepared(Ctx* ctx, const PreparedStep* ps, bool sync);
int enqueue_step(Ctx* ctx, const PreparedStep* ps);
bool prepared_is_empty(const PreparedStep* ps);
// Partition bits a batched step over nb binding rows uses (option, tuned
// table or the automatic rule).
int step_partition_bits(Ctx* ctx, int64_t nb);
// qfg_evaluate_step under QFG_OPT_USE_GRAPHS: replays (building on first use)
// the cached graph of this step, then copies its counts to `counts`.
int evaluate_step_cached(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                         unsigned long long* counts);
void graph_cache_clear(Ctx* ctx);
// Device scratch bytes a batched step over these literals needs.
int step_scratch_bytes(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                       int64_t* bytes);

}  // namespace qfg
