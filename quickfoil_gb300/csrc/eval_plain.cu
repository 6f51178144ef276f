// eval_plain.cu -- the plain per-literal GPU path and shared evaluation
// plumbing (literal validation, count buffers).
//
// One literal = one run of the reference chain over the binding join column
// partitioned once per join variable, as the reference partitions it once
// per Evaluate call (operations/RadixPartition.cpp:179-186,
// learner/CandidateLiteralEvaluator.cpp:316-323); the cached
// RadixPartition of the relation join column
// (learner/CandidateLiteralEvaluator.cpp:296-299), then per partition a
// chained hash table on the binding side probed by every relation tuple
// (BuildHashTableOnPartitions + HashJoin, operations/BuildHashTable.cpp:54-93,
// operations/HashJoin.cpp:23-86), the atom filter
// (operations/Filter.cpp:17-38) and the count aggregation with a semi bit
// vector over the binding partition (operations/CountAggregator.cpp:111-243).
// On the GPU the last three run fused in one kernel: a CTA loads a tile of a
// binding partition into shared memory, links it into chains with
// atomicExch on the bucket heads, streams the relation partition through
// it, checks atoms by gathering the two columns, and marks covered rows in a
// shared-memory bit vector (atomicOr; a row counts when its bit was clear).
// Binding partitions larger than a tile are processed tile by tile; a
// binding row belongs to exactly one tile, so covered counts add up.
#include <algorithm>
#include <map>
#include <vector>

#include "eval_common.cuh"

namespace qfg {

namespace {

constexpr int kPlainTile = 2048;
constexpr int kPlainSlots = 4096;
constexpr int kPlainThreads = 512;

struct PlainArgs {
  const int2* btuples;
  const int64_t* boffsets;
  const int2* rtuples;
  const int64_t* roffsets;
  int num_partitions;
  int num_atoms;
  const int32_t* atom_rel[QFG_MAX_ARITY];
  const int32_t* atom_bind[QFG_MAX_ARITY];
  int64_t num_positive;
  unsigned long long* counts;
};

__global__ void __launch_bounds__(kPlainThreads)
plain_join_count_kernel(PlainArgs a) {
  __shared__ int32_t s_val[kPlainTile];
  __shared__ int32_t s_tid[kPlainTile];
  __shared__ int32_t s_next[kPlainTile];
  __shared__ int32_t s_head[kPlainSlots];
  __shared__ uint32_t s_semi[kPlainTile / 32];
  __shared__ long long s_red[kPlainThreads / 32][4];

  long long c0 = 0, c1 = 0, c2 = 0, c3 = 0;
  for (int p = blockIdx.x; p < a.num_partitions; p += gridDim.x) {
    const int64_t b0 = a.boffsets[p], b1 = a.boffsets[p + 1];
    const int64_t r0 = a.roffsets[p], r1 = a.roffsets[p + 1];
    if (b0 == b1 || r0 == r1) continue;
    for (int64_t t0 = b0; t0 < b1; t0 += kPlainTile) {
      const int nt = (int)(b1 - t0 < kPlainTile ? b1 - t0 : kPlainTile);
      __syncthreads();
      for (int i = threadIdx.x; i < kPlainSlots; i += blockDim.x) s_head[i] = -1;
      for (int i = threadIdx.x; i < kPlainTile / 32; i += blockDim.x) s_semi[i] = 0u;
      __syncthreads();
      for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        const int2 t = a.btuples[t0 + i];
        s_val[i] = t.x;
        s_tid[i] = t.y;
        const uint32_t slot = mix32((uint32_t)t.x) & (kPlainSlots - 1);
        s_next[i] = atomicExch(&s_head[slot], i);
      }
      __syncthreads();
      for (int64_t k = r0 + threadIdx.x; k < r1; k += blockDim.x) {
        const int2 rt = a.rtuples[k];
        const uint32_t slot = mix32((uint32_t)rt.x) & (kPlainSlots - 1);
        for (int e = s_head[slot]; e >= 0; e = s_next[e]) {
          if (s_val[e] != rt.x) continue;
          const int32_t b = s_tid[e];
          bool pass = true;
          for (int q = 0; q < a.num_atoms; ++q) {
            if (__ldg(a.atom_rel[q] + rt.y) != __ldg(a.atom_bind[q] + b)) {
              pass = false;
              break;
            }
          }
          if (!pass) continue;
          const bool neg = b >= a.num_positive;
          const uint32_t bit = 1u << (e & 31);
          const bool fresh = !(atomicOr(&s_semi[e >> 5], bit) & bit);
          if (neg) {
            c3 += 1;
            c1 += fresh;
          } else {
            c2 += 1;
            c0 += fresh;
          }
        }
      }
    }
  }
  c0 = warp_sum(c0);
  c1 = warp_sum(c1);
  c2 = warp_sum(c2);
  c3 = warp_sum(c3);
  if (lane_id() == 0) {
    s_red[warp_id()][0] = c0;
    s_red[warp_id()][1] = c1;
    s_red[warp_id()][2] = c2;
    s_red[warp_id()][3] = c3;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    long long s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += s_red[w][threadIdx.x];
    if (s != 0) atomicAdd(&a.counts[threadIdx.x], as_ull(s));
  }
}

int auto_plain_bits(Ctx* ctx, int64_t n) {
  if (ctx->eval_bits > 0) return ctx->eval_bits;
  int bits = 1;
  while (bits < QFG_MAX_RADIX_BITS && (n >> bits) > kPlainTile / 2) ++bits;
  return bits;
}

}  // namespace

int validate_literals(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits) {
  if (n < 0 || (n > 0 && lits == nullptr))
    return set_error(ctx, QFG_ERR_INVALID, "invalid literal array");
  for (int32_t i = 0; i < n; ++i) {
    const qfg_literal& l = lits[i];
    Relation* rel = nullptr;
    QFG_TRY(find_relation(ctx, l.relation_id, &rel));
    if (l.num_args < 1 || l.num_args > QFG_MAX_ARITY || l.num_args != rel->num_columns)
      return set_error(ctx, QFG_ERR_INVALID,
                       "literal " + std::to_string(i) + ": argument count differs from the relation arity");
    if (l.join_pos < 0 || l.join_pos >= l.num_args || l.vars[l.join_pos] < 0)
      return set_error(ctx, QFG_ERR_INVALID,
                       "literal " + std::to_string(i) + ": join key argument is not bound");
    for (int k = 0; k < l.num_args; ++k)
      if (l.vars[k] < -1 || l.vars[k] >= b->num_columns)
        return set_error(ctx, QFG_ERR_INVALID,
                         "literal " + std::to_string(i) + ": variable out of the binding-set range");
  }
  return QFG_OK;
}

int counts_begin(Ctx* ctx, int32_t n, int64_t* counts, int flags, unsigned long long** dev) {
  if (counts == nullptr && n > 0) return set_error(ctx, QFG_ERR_INVALID, "null counts");
  if (flags != QFG_COUNTS_HOST && flags != QFG_COUNTS_DEVICE)
    return set_error(ctx, QFG_ERR_INVALID, "invalid counts flag");
  if (flags == QFG_COUNTS_DEVICE) {
    *dev = reinterpret_cast<unsigned long long*>(counts);
  } else {
    QFG_TRY(ctx->scratch[kScrCounts].reserve(ctx, sizeof(int64_t) * 4 * (size_t)std::max(n, 1)));
    *dev = ctx->scratch[kScrCounts].as<unsigned long long>();
  }
  if (n > 0)
    QFG_CUDA(ctx, cudaMemsetAsync(*dev, 0, sizeof(int64_t) * 4 * (size_t)n, ctx->stream));
  return QFG_OK;
}

int counts_end(Ctx* ctx, int32_t n, int64_t* counts, int flags, unsigned long long* dev) {
  if (flags == QFG_COUNTS_HOST) {
    if (n > 0)
      QFG_CUDA(ctx, cudaMemcpyAsync(counts, dev, sizeof(int64_t) * 4 * (size_t)n,
                                    cudaMemcpyDeviceToHost, ctx->stream));
    QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int flag = 0;
    QFG_CUDA(ctx, cudaMemcpy(&flag, ctx->error_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag != 0) {
      cudaMemset(ctx->error_flag, 0, sizeof(int));
      return set_error(ctx, QFG_ERR_TIMEOUT, "a bounded device-side wait gave up");
    }
  }
  return QFG_OK;
}

// Binding join column `column` in the reference partition layout, into the
// context's binding-partition scratch (the reference's once-per-Evaluate
// RadixPartition of the binding set, learner/CandidateLiteralEvaluator.cpp:
// 316-323).  *bits receives the partition bits.
int plain_partition_bindings(Ctx* ctx, const qfg_bindings* b, int column, int* bits) {
  const int64_t nb = b->num_positive + b->num_negative;
  *bits = auto_plain_bits(ctx, nb);
  const int P = 1 << *bits;
  QFG_TRY(ctx->scratch[kScrBindPart].reserve(ctx, sizeof(int32_t) * 2 * (size_t)std::max<int64_t>(nb, 1)));
  QFG_TRY(ctx->scratch[kScrBindOffsets].reserve(ctx, sizeof(int64_t) * (size_t)(P + 1)));
  QFG_TRY(stage_begin(ctx, QFG_STAGE_BIND_PARTITION));
  QFG_TRY(radix_partition_ref(ctx, b->columns[column], nb, *bits,
                              ctx->scratch[kScrBindPart].as<int32_t>(),
                              ctx->scratch[kScrBindOffsets].as<int64_t>()));
  QFG_TRY(stage_end(ctx, QFG_STAGE_BIND_PARTITION));
  return QFG_OK;
}

// One literal's build / probe / filter / count chain over the binding
// partition left by plain_partition_bindings (same join column and bits).
int plain_join_count(Ctx* ctx, const qfg_bindings* b, const qfg_literal& l, int bits,
                     unsigned long long* counts) {
  Relation* rel = nullptr;
  QFG_TRY(find_relation(ctx, l.relation_id, &rel));
  const int64_t nb = b->num_positive + b->num_negative;
  if (nb == 0 || rel->num_tuples == 0) return QFG_OK;
  const int P = 1 << bits;
  // Relation side: cached for the run.
  PartitionedColumn* rp = nullptr;
  QFG_TRY(relation_partitions(ctx, rel, l.join_pos, bits, &rp));
  PlainArgs a;
  a.btuples = ctx->scratch[kScrBindPart].as<int2>();
  a.boffsets = ctx->scratch[kScrBindOffsets].as<int64_t>();
  a.rtuples = rp->tuples.as<int2>();
  a.roffsets = rp->offsets.as<int64_t>();
  a.num_partitions = P;
  a.num_atoms = 0;
  for (int k = 0; k < l.num_args; ++k) {
    if (k == l.join_pos || l.vars[k] < 0) continue;
    a.atom_rel[a.num_atoms] = rel->columns[k];
    a.atom_bind[a.num_atoms] = b->columns[l.vars[k]];
    ++a.num_atoms;
  }
  a.num_positive = b->num_positive;
  a.counts = counts;
  const unsigned grid = (unsigned)std::min(P, ctx->num_sms * 4);
  QFG_TRY(stage_begin(ctx, QFG_STAGE_PER_LITERAL));
  plain_join_count_kernel<<<grid, kPlainThreads, 0, ctx->stream>>>(a);
  QFG_LAUNCHED(ctx);
  QFG_TRY(stage_end(ctx, QFG_STAGE_PER_LITERAL));
  return QFG_OK;
}

}  // namespace qfg

using namespace qfg;

extern "C" int qfg_evaluate_per_literal(qfg_ctx* c, const qfg_bindings* b, int32_t n,
                                        const qfg_literal* lits, int64_t* counts, int flags) {
  if (c == nullptr || b == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  QFG_TRY(validate_literals(ctx, b, n, lits));
  unsigned long long* dev = nullptr;
  QFG_TRY(counts_begin(ctx, n, counts, flags, &dev));
  const int64_t nb = b->num_positive + b->num_negative;
  if (nb > 0) {
    // As the reference: the binding set partitioned once per clause join
    // variable (once per Evaluate call), then one chain per literal.
    std::map<int, std::vector<int32_t>> by_column;
    for (int32_t i = 0; i < n; ++i) by_column[lits[i].vars[lits[i].join_pos]].push_back(i);
    for (const auto& kv : by_column) {
      int bits = 0;
      QFG_TRY(plain_partition_bindings(ctx, b, kv.first, &bits));
      for (int32_t i : kv.second) QFG_TRY(plain_join_count(ctx, b, lits[i], bits, dev + 4 * i));
    }
  }
  return counts_end(ctx, n, counts, flags, dev);
}
