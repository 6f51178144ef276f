// eval_batched.cu -- batched evaluation of all candidate literals of a
// refinement step.
//
// Counting identity.  For a literal with bound arguments (a, k1, k2, ...) on
// relation R, a binding row b joins relation tuple r when every bound
// argument matches: R[a][r] == B[var(a)][b], R[k][r] == B[var(k)][b].  So r
// matters only through its projected key tuple K(r) = (R[a], R[k1], ...), and
// b matches exactly the relation tuples whose K equals b's projection.  With
// the relation deduplicated to distinct key tuples t and multiplicities m(t):
//   num_binding_{pos,neg} = sum over (t, b matching t) of m(t)
//   num_covered_{pos,neg} = number of (t, b matching t) pairs
// because each binding row matches at most one distinct tuple.  These are
// exactly the reference's counts (operations/CountAggregator.cpp:111-243:
// one binding count per passing join pair, one covered count per binding row
// with at least one passing pair), computed without per-pair bit vectors.
//
// Data movement.  Relation key tables are built once per (relation,
// argument list) and cached for the run (the reference caches relation
// partitions the same way, learner/CandidateLiteralEvaluator.cpp:296-299).
// The binding set is partitioned once per join column (per group of
// literals sharing that column): each row goes to partition
// top_bits(mix32(B[j])) and label (positives first), carrying the join
// column and the atom columns the group's literals test.  The evaluation
// kernel is persistent: each CTA repeatedly takes a (group, partition) work
// item, loads that binding partition into shared memory, builds a
// shared-memory table of its distinct join keys (atomicCAS on slot owners)
// with per-label row counts and per-key row lists, and then streams, for
// every literal of the group, the relation key tuples of the same partition
// range through it.  Counts are reduced with warp shuffles into per-CTA
// int64 accumulators and flushed to global memory once per CTA.
#include <algorithm>
#include <unordered_map>

#include "eval_common.cuh"

namespace qfg {

namespace {

constexpr int kTile = 2560;            // binding rows per shared-memory tile
constexpr int kSlots = 4096;           // key-table slots (power of two > kTile)
constexpr int kEvalThreads = 1024;
constexpr int kGroupCols = QFG_MAX_ARITY;  // join column + up to 7 atom columns
constexpr int kMaxLitsPerLaunch = 512;
constexpr int kMaxPartitionBits = 14;

// ----------------------------------------------------------------------------
// Relation key tables.

struct ProjArgs {
  const int32_t* cols[QFG_MAX_ARITY];
  int nk;
  int64_t n;
};

__device__ __forceinline__ uint32_t tuple_hash(const ProjArgs& a, int64_t r) {
  uint32_t h = mix32((uint32_t)a.cols[0][r]);
  for (int k = 1; k < a.nk; ++k) h = mix32(h + 0x9e3779b9u + (uint32_t)a.cols[k][r]);
  return h;
}

__device__ __forceinline__ bool tuple_equal(const ProjArgs& a, int64_t x, int64_t y) {
  for (int k = 0; k < a.nk; ++k)
    if (a.cols[k][x] != a.cols[k][y]) return false;
  return true;
}

// Open addressing over `cap_mask + 1` slots (at least twice the tuple
// count, so a free slot always exists); the first tuple of each distinct key
// tuple owns a slot and collects the multiplicity.
__global__ void dedup_insert_kernel(ProjArgs a, int32_t* __restrict__ owner, uint32_t cap_mask,
                                    int32_t* __restrict__ mult) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n;
       r += (int64_t)gridDim.x * blockDim.x) {
    uint32_t slot = tuple_hash(a, r) & cap_mask;
    for (uint32_t probe = 0; probe <= cap_mask; ++probe) {
      const int32_t o = atomicCAS(&owner[slot], -1, (int32_t)r);
      if (o == -1) {
        atomicAdd(&mult[r], 1);
        break;
      }
      if (tuple_equal(a, o, r)) {
        atomicAdd(&mult[o], 1);
        break;
      }
      slot = (slot + 1) & cap_mask;
    }
  }
}

__global__ void keytable_hist_kernel(ProjArgs a, const int32_t* __restrict__ mult,
                                     uint32_t* __restrict__ hist) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n;
       r += (int64_t)gridDim.x * blockDim.x) {
    if (mult[r] > 0) atomicAdd(&hist[mix32((uint32_t)a.cols[0][r]) >> (32 - kRelPartitionBits)], 1u);
  }
}

__global__ void keytable_scatter_kernel(ProjArgs a, const int32_t* __restrict__ mult,
                                        uint32_t* __restrict__ cursor, int32_t* __restrict__ keys,
                                        int64_t stride, int32_t* __restrict__ out_mult) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t m = mult[r];
    if (m <= 0) continue;
    const uint32_t bin = mix32((uint32_t)a.cols[0][r]) >> (32 - kRelPartitionBits);
    const uint32_t pos = atomicAdd(&cursor[bin], 1u);
    for (int k = 0; k < a.nk; ++k) keys[k * stride + pos] = a.cols[k][r];
    out_mult[pos] = m;
  }
}

unsigned grid_for_rows(Ctx* ctx, int64_t n, int threads) {
  const int64_t blocks = (n + threads - 1) / threads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)ctx->num_sms * 8));
}

// ----------------------------------------------------------------------------
// Binding-set partitioning per group.

struct BPartArgs {
  const int32_t* cols[kGroupCols];  // cols[0] = join column
  int ncols;
  int64_t n, npos;
  int bits;
  uint32_t* tot;   // 2 << bits bin totals (zeroed)
  uint32_t* base;  // gridDim.x * (2 << bits) per-CTA bases
  int32_t* out;    // ncols SoA columns of n rows
};

__device__ __forceinline__ void cta_range(int64_t n, int64_t* r0, int64_t* r1) {
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  *r0 = min(n, (int64_t)blockIdx.x * per);
  *r1 = min(n, *r0 + per);
}

__device__ __forceinline__ uint32_t bind_bin(int32_t key, int bits, bool neg) {
  return ((mix32((uint32_t)key) >> (32 - bits)) << 1) | (neg ? 1u : 0u);
}

__global__ void __launch_bounds__(1024) bpart_hist_kernel(BPartArgs a) {
  extern __shared__ uint32_t sh_bins[];
  const int nbins = 2 << a.bits;
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) sh_bins[i] = 0;
  __syncthreads();
  int64_t r0, r1;
  cta_range(a.n, &r0, &r1);
  const int32_t* __restrict__ key = a.cols[0];
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x)
    atomicAdd(&sh_bins[bind_bin(key[r], a.bits, r >= a.npos)], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) {
    const uint32_t c = sh_bins[i];
    a.base[(int64_t)blockIdx.x * nbins + i] = c ? atomicAdd(&a.tot[i], c) : 0u;
  }
}

__global__ void __launch_bounds__(1024)
bpart_scatter_kernel(BPartArgs a, const uint32_t* __restrict__ start) {
  extern __shared__ uint32_t sh_cur[];
  const int nbins = 2 << a.bits;
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    sh_cur[i] = start[i] + a.base[(int64_t)blockIdx.x * nbins + i];
  __syncthreads();
  int64_t r0, r1;
  cta_range(a.n, &r0, &r1);
  const int32_t* __restrict__ key = a.cols[0];
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const int32_t k = key[r];
    const uint32_t pos = atomicAdd(&sh_cur[bind_bin(k, a.bits, r >= a.npos)], 1u);
    a.out[pos] = k;
    for (int c = 1; c < a.ncols; ++c) a.out[(int64_t)c * a.n + pos] = a.cols[c][r];
  }
}

// ----------------------------------------------------------------------------
// Persistent evaluation kernel.

struct GroupDesc {
  const int32_t* cols;    // ncols SoA columns of n rows, partitioned
  int64_t n;
  const uint32_t* start;  // (2 << bits) + 1 bin offsets
  int bits, ncols;
  int lit_begin, lit_end;
  int has_atoms;
  int64_t item_begin;
};

struct LitDesc {
  const int32_t* keys;       // nk SoA columns of `stride` entries
  int64_t stride;
  const int32_t* mult;
  const uint32_t* offsets;   // (1 << kRelPartitionBits) + 1
  int nk;
  int atom_col[QFG_MAX_ARITY];  // key q >= 1 is compared with group column atom_col[q]
  int out;                   // literal index in the caller's array
};

struct EvalArgs {
  const GroupDesc* groups;
  int num_groups;
  const LitDesc* lits;
  int num_lits;
  int64_t total_items;
  unsigned int* work_counter;
  unsigned long long* counts;
};

size_t eval_smem_bytes(int num_lits) {
  return sizeof(long long) * 4 * (size_t)num_lits + sizeof(int32_t) * kGroupCols * kTile +
         sizeof(int32_t) * kSlots * 4 + sizeof(uint16_t) * 2 * kTile;
}

__global__ void __launch_bounds__(kEvalThreads, 1) eval_batched_kernel(EvalArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(smem);
  int32_t* scol = reinterpret_cast<int32_t*>(acc + 4 * a.num_lits);
  int32_t* owner = scol + kGroupCols * kTile;
  uint32_t* cntp = reinterpret_cast<uint32_t*>(owner + kSlots);
  uint32_t* cntn = cntp + kSlots;
  uint32_t* lend = cntn + kSlots;
  uint16_t* rows = reinterpret_cast<uint16_t*>(lend + kSlots);
  uint16_t* rslot = rows + kTile;
  __shared__ long long s_item;
  __shared__ uint32_t s_warp[32];

  for (int i = threadIdx.x; i < 4 * a.num_lits; i += blockDim.x) acc[i] = 0ull;
  __syncthreads();

  for (;;) {
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(a.work_counter, 1u);
    __syncthreads();
    const long long item = s_item;
    if (item >= a.total_items) break;
    int g = 0;
    while (g + 1 < a.num_groups && a.groups[g + 1].item_begin <= item) ++g;
    const GroupDesc G = a.groups[g];
    const int p = (int)(item - G.item_begin);
    const uint32_t b0 = G.start[2 * p], bm = G.start[2 * p + 1], b1 = G.start[2 * p + 2];
    const int shift = kRelPartitionBits - G.bits;
    const uint32_t q0 = (uint32_t)p << shift, q1 = (uint32_t)(p + 1) << shift;

    for (uint32_t t0 = b0; t0 < b1; t0 += kTile) {
      const int nt = (int)umin((uint32_t)kTile, b1 - t0);
      const int npos = (int)umin((uint32_t)nt, bm > t0 ? bm - t0 : 0u);
      for (int c = 0; c < G.ncols; ++c)
        for (int i = threadIdx.x; i < nt; i += blockDim.x)
          scol[c * kTile + i] = G.cols[(int64_t)c * G.n + t0 + i];
      for (int i = threadIdx.x; i < kSlots; i += blockDim.x) {
        owner[i] = -1;
        cntp[i] = 0u;
        cntn[i] = 0u;
      }
      __syncthreads();
      // Distinct join keys of the tile with per-label row counts.
      for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        const int32_t key = scol[i];
        uint32_t slot = mix32((uint32_t)key) & (kSlots - 1);
        for (int probe = 0; probe < kSlots; ++probe) {
          const int32_t o = atomicCAS(&owner[slot], -1, i);
          if (o == -1 || scol[o] == key) break;
          slot = (slot + 1) & (kSlots - 1);
        }
        rslot[i] = (uint16_t)slot;
        atomicAdd(i < npos ? &cntp[slot] : &cntn[slot], 1u);
      }
      __syncthreads();
      if (G.has_atoms) {
        // Row lists per key: exclusive scan of row counts, then fill; after
        // the fill lend[s] is the end of slot s's list.
        constexpr int kPer = kSlots / kEvalThreads;
        uint32_t v[kPer];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
          const int s = threadIdx.x * kPer + k;
          v[k] = cntp[s] + cntn[s];
          sum += v[k];
        }
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(kFullMask, x, o);
          if (lane_id() >= o) x += y;
        }
        if (lane_id() == 31) s_warp[warp_id()] = x;
        __syncthreads();
        if (warp_id() == 0) {
          const uint32_t t = s_warp[lane_id()];
          uint32_t s = t;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFullMask, s, o);
            if (lane_id() >= o) s += y;
          }
          s_warp[lane_id()] = s - t;
        }
        __syncthreads();
        uint32_t run = x - sum + s_warp[warp_id()];
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
          lend[threadIdx.x * kPer + k] = run;
          run += v[k];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nt; i += blockDim.x) {
          const uint32_t pos = atomicAdd(&lend[rslot[i]], 1u);
          rows[pos] = (uint16_t)i;
        }
        __syncthreads();
      }
      // Stream each literal's relation key tuples of this partition range.
      for (int L = G.lit_begin; L < G.lit_end; ++L) {
        const LitDesc d = a.lits[L];
        const uint32_t e0 = d.offsets[q0], e1 = d.offsets[q1];
        long long bp = 0, bn = 0, cp = 0, cn = 0;
        for (uint32_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
          const int32_t k0 = __ldg(d.keys + e);
          uint32_t slot = mix32((uint32_t)k0) & (kSlots - 1);
          int32_t o = -1;
          for (int probe = 0; probe < kSlots; ++probe) {
            o = owner[slot];
            if (o < 0 || scol[o] == k0) break;
            slot = (slot + 1) & (kSlots - 1);
          }
          if (o < 0 || scol[o] != k0) continue;
          const long long m = __ldg(d.mult + e);
          if (d.nk == 1) {
            const uint32_t P = cntp[slot], N = cntn[slot];
            bp += m * P;
            bn += m * N;
            cp += P;
            cn += N;
          } else {
            int32_t kq[QFG_MAX_ARITY];
            for (int q = 1; q < d.nk; ++q) kq[q] = __ldg(d.keys + q * d.stride + e);
            const uint32_t end = lend[slot];
            const uint32_t beg = end - (cntp[slot] + cntn[slot]);
            for (uint32_t x = beg; x < end; ++x) {
              const int row = rows[x];
              bool pass = true;
              for (int q = 1; q < d.nk; ++q) {
                if (scol[d.atom_col[q] * kTile + row] != kq[q]) {
                  pass = false;
                  break;
                }
              }
              if (!pass) continue;
              if (row < npos) {
                bp += m;
                cp += 1;
              } else {
                bn += m;
                cn += 1;
              }
            }
          }
        }
        bp = warp_sum(bp);
        bn = warp_sum(bn);
        cp = warp_sum(cp);
        cn = warp_sum(cn);
        if (lane_id() == 0 && (bp | bn | cp | cn) != 0) {
          unsigned long long* dst = acc + 4 * L;
          atomicAdd(dst + 0, as_ull(cp));
          atomicAdd(dst + 1, as_ull(cn));
          atomicAdd(dst + 2, as_ull(bp));
          atomicAdd(dst + 3, as_ull(bn));
        }
      }
      __syncthreads();
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 4 * a.num_lits; i += blockDim.x) {
    const unsigned long long v = acc[i];
    if (v != 0ull) atomicAdd(&a.counts[4 * a.lits[i >> 2].out + (i & 3)], v);
  }
}

int auto_group_bits(Ctx* ctx, int64_t n) {
  if (ctx->eval_bits > 0) return std::min(ctx->eval_bits, kMaxPartitionBits);
  int bits = 1;
  while (bits < kMaxPartitionBits && (n >> bits) > kTile / 2) ++bits;
  return bits;
}

struct HostGroup {
  int join_col;
  std::vector<int> cols;  // cols[0] = join column
  std::vector<int> lits;  // literal indices
  bool has_atoms = false;
};

}  // namespace

int relation_key_table(Ctx* ctx, Relation* rel, const std::vector<int>& positions,
                       KeyTable** out) {
  auto it = rel->key_tables.find(positions);
  if (it != rel->key_tables.end()) {
    *out = it->second.get();
    return QFG_OK;
  }
  auto kt = std::make_unique<KeyTable>();
  kt->num_keys = (int)positions.size();
  const int64_t n = rel->num_tuples;
  const int nbins = 1 << kRelPartitionBits;
  QFG_TRY(kt->offsets.reserve(ctx, sizeof(uint32_t) * (size_t)(nbins + 1)));
  uint32_t* offsets = kt->offsets.as<uint32_t>();
  QFG_CUDA(ctx, cudaMemsetAsync(offsets, 0, sizeof(uint32_t) * (nbins + 1), ctx->stream));
  if (n > 0) {
    ProjArgs pa;
    pa.nk = kt->num_keys;
    pa.n = n;
    for (int k = 0; k < pa.nk; ++k) pa.cols[k] = rel->columns[positions[k]];
    uint32_t cap = 1;
    while (cap < (uint32_t)(2 * n)) cap <<= 1;
    QFG_TRY(ctx->scratch[kScrDedup].reserve(ctx, sizeof(int32_t) * ((size_t)cap + (size_t)n)));
    int32_t* owner = ctx->scratch[kScrDedup].as<int32_t>();
    int32_t* mult = owner + cap;
    QFG_CUDA(ctx, cudaMemsetAsync(owner, 0xff, sizeof(int32_t) * cap, ctx->stream));
    QFG_CUDA(ctx, cudaMemsetAsync(mult, 0, sizeof(int32_t) * (size_t)n, ctx->stream));
    const unsigned grid = grid_for_rows(ctx, n, 256);
    dedup_insert_kernel<<<grid, 256, 0, ctx->stream>>>(pa, owner, cap - 1, mult);
    QFG_LAUNCHED(ctx);
    QFG_TRY(ctx->scratch[kScrMisc].reserve(ctx, sizeof(uint32_t) * (size_t)(2 * nbins + 2)));
    uint32_t* hist = ctx->scratch[kScrMisc].as<uint32_t>();
    uint32_t* total = hist + nbins;
    QFG_CUDA(ctx, cudaMemsetAsync(hist, 0, sizeof(uint32_t) * nbins, ctx->stream));
    keytable_hist_kernel<<<grid, 256, 0, ctx->stream>>>(pa, mult, hist);
    QFG_LAUNCHED(ctx);
    QFG_TRY(exclusive_scan_u32(ctx, hist, offsets, nbins, total));
    QFG_CUDA(ctx, cudaMemcpyAsync(offsets + nbins, total, sizeof(uint32_t),
                                  cudaMemcpyDeviceToDevice, ctx->stream));
    uint32_t distinct = 0;
    QFG_CUDA(ctx, cudaMemcpyAsync(&distinct, total, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    kt->num_entries = distinct;
    QFG_TRY(kt->keys.reserve(ctx, sizeof(int32_t) * (size_t)kt->num_keys * std::max<int64_t>(distinct, 1)));
    QFG_TRY(kt->mult.reserve(ctx, sizeof(int32_t) * (size_t)std::max<int64_t>(distinct, 1)));
    QFG_CUDA(ctx, cudaMemcpyAsync(hist, offsets, sizeof(uint32_t) * nbins, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    keytable_scatter_kernel<<<grid, 256, 0, ctx->stream>>>(pa, mult, hist, kt->keys.as<int32_t>(),
                                                           std::max<int64_t>(distinct, 1),
                                                           kt->mult.as<int32_t>());
    QFG_LAUNCHED(ctx);
  } else {
    QFG_TRY(kt->keys.reserve(ctx, sizeof(int32_t) * (size_t)kt->num_keys));
    QFG_TRY(kt->mult.reserve(ctx, sizeof(int32_t)));
  }
  *out = kt.get();
  rel->key_tables[positions] = std::move(kt);
  return QFG_OK;
}

// Host plan of a batched step: the key table of every literal and the
// literal groups (shared join column, at most kGroupCols binding columns).
struct StepPlan {
  std::vector<KeyTable*> tables;
  std::vector<std::vector<int>> bind_cols;  // [join column, atom columns...]
  std::vector<HostGroup> groups;
};

static int plan_step(Ctx* ctx, int32_t n, const qfg_literal* lits, StepPlan* plan) {
  plan->tables.assign(n, nullptr);
  plan->bind_cols.assign(n, {});
  for (int i = 0; i < n; ++i) {
    const qfg_literal& l = lits[i];
    Relation* rel = nullptr;
    QFG_TRY(find_relation(ctx, l.relation_id, &rel));
    std::vector<int> positions{l.join_pos};
    plan->bind_cols[i].push_back(l.vars[l.join_pos]);
    for (int k = 0; k < l.num_args; ++k) {
      if (k == l.join_pos || l.vars[k] < 0) continue;
      positions.push_back(k);
      plan->bind_cols[i].push_back(l.vars[k]);
    }
    QFG_TRY(relation_key_table(ctx, rel, positions, &plan->tables[i]));
  }
  const auto& bind_cols = plan->bind_cols;
  auto& groups = plan->groups;
  groups.clear();
  std::map<int, std::vector<int>> by_col;
  for (int i = 0; i < n; ++i) by_col[bind_cols[i][0]].push_back(i);
  auto missing_cols = [&](const HostGroup& g, int i) {
    std::vector<int> add;
    for (size_t q = 1; q < bind_cols[i].size(); ++q) {
      const int c = bind_cols[i][q];
      if (std::find(g.cols.begin(), g.cols.end(), c) == g.cols.end() &&
          std::find(add.begin(), add.end(), c) == add.end())
        add.push_back(c);
    }
    return add;
  };
  for (auto& kv : by_col) {
    HostGroup cur;
    cur.join_col = kv.first;
    cur.cols = {kv.first};
    for (int i : kv.second) {
      std::vector<int> add = missing_cols(cur, i);
      if ((int)(cur.cols.size() + add.size()) > kGroupCols ||
          (int)cur.lits.size() >= kMaxLitsPerLaunch) {
        groups.push_back(cur);
        cur = HostGroup();
        cur.join_col = kv.first;
        cur.cols = {kv.first};
        add = missing_cols(cur, i);
      }
      cur.cols.insert(cur.cols.end(), add.begin(), add.end());
      cur.lits.push_back(i);
      if (bind_cols[i].size() > 1) cur.has_atoms = true;
    }
    groups.push_back(cur);
  }
  return QFG_OK;
}

int evaluate_batched(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                     unsigned long long* counts) {
  const int64_t nb = b->num_positive + b->num_negative;
  if (n == 0 || nb == 0) return QFG_OK;

  QFG_TRY(stage_begin(ctx, QFG_STAGE_KEY_TABLES));
  StepPlan plan;
  QFG_TRY(plan_step(ctx, n, lits, &plan));
  QFG_TRY(stage_end(ctx, QFG_STAGE_KEY_TABLES));
  const auto& tables = plan.tables;
  const auto& bind_cols = plan.bind_cols;
  const auto& groups = plan.groups;

  // Partition the binding set once per group.
  const int bits = auto_group_bits(ctx, nb);
  const int nbins = 2 << bits;
  const unsigned pgrid = (unsigned)ctx->num_sms;
  size_t part_words = 0;
  for (auto& g : groups) part_words += g.cols.size() * (size_t)nb;
  const size_t bins_words = (size_t)nbins + 1 + (size_t)pgrid * nbins;
  QFG_TRY(ctx->scratch[kScrBindPart].reserve(ctx, sizeof(int32_t) * part_words));
  QFG_TRY(ctx->scratch[kScrBindOffsets].reserve(ctx, sizeof(uint32_t) * (groups.size() * ((size_t)nbins + 1) + bins_words)));
  int32_t* part_base = ctx->scratch[kScrBindPart].as<int32_t>();
  uint32_t* starts = ctx->scratch[kScrBindOffsets].as<uint32_t>();
  uint32_t* tot = starts + groups.size() * ((size_t)nbins + 1);
  uint32_t* cta_base = tot + nbins + 1;
  const size_t hist_smem = sizeof(uint32_t) * nbins;
  QFG_CUDA(ctx, cudaFuncSetAttribute(bpart_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)hist_smem));
  QFG_CUDA(ctx, cudaFuncSetAttribute(bpart_scatter_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hist_smem));
  std::vector<GroupDesc> gdesc(groups.size());
  std::vector<LitDesc> ldesc;
  QFG_TRY(stage_begin(ctx, QFG_STAGE_BIND_PARTITION));
  size_t off = 0;
  int64_t items = 0;
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const HostGroup& g = groups[gi];
    BPartArgs pa;
    pa.ncols = (int)g.cols.size();
    for (int c = 0; c < pa.ncols; ++c) pa.cols[c] = b->columns[g.cols[c]];
    pa.n = nb;
    pa.npos = b->num_positive;
    pa.bits = bits;
    pa.tot = tot;
    pa.base = cta_base;
    pa.out = part_base + off;
    uint32_t* start = starts + gi * ((size_t)nbins + 1);
    QFG_CUDA(ctx, cudaMemsetAsync(tot, 0, sizeof(uint32_t) * nbins, ctx->stream));
    bpart_hist_kernel<<<pgrid, 1024, hist_smem, ctx->stream>>>(pa);
    QFG_LAUNCHED(ctx);
    QFG_TRY(exclusive_scan_u32(ctx, tot, start, nbins, start + nbins));
    bpart_scatter_kernel<<<pgrid, 1024, hist_smem, ctx->stream>>>(pa, start);
    QFG_LAUNCHED(ctx);

    GroupDesc& d = gdesc[gi];
    d.cols = pa.out;
    d.n = nb;
    d.start = start;
    d.bits = bits;
    d.ncols = pa.ncols;
    d.lit_begin = (int)ldesc.size();
    d.has_atoms = g.has_atoms ? 1 : 0;
    d.item_begin = items;
    items += (int64_t)1 << bits;
    for (int i : g.lits) {
      LitDesc ld;
      memset(&ld, 0, sizeof(ld));
      KeyTable* kt = tables[i];
      ld.keys = kt->keys.as<int32_t>();
      ld.stride = std::max<int64_t>(kt->num_entries, 1);
      ld.mult = kt->mult.as<int32_t>();
      ld.offsets = kt->offsets.as<uint32_t>();
      ld.nk = kt->num_keys;
      for (int q = 1; q < ld.nk; ++q)
        ld.atom_col[q] = (int)(std::find(g.cols.begin(), g.cols.end(), bind_cols[i][q]) - g.cols.begin());
      ld.out = i;
      ldesc.push_back(ld);
    }
    d.lit_end = (int)ldesc.size();
    off += g.cols.size() * (size_t)nb;
  }

  QFG_TRY(stage_end(ctx, QFG_STAGE_BIND_PARTITION));

  // Descriptors, then launches of at most kMaxLitsPerLaunch literals (groups
  // never straddle a launch: they are capped at that size).  Each launch
  // gets its own rebased copy of its groups; everything goes up in one copy.
  struct Launch {
    size_t gbeg, gend;
    int lit0, nl;
  };
  std::vector<Launch> launches;
  std::vector<GroupDesc> sub_all;
  for (size_t gbeg = 0; gbeg < gdesc.size();) {
    size_t gend = gbeg;
    int nl = 0;
    while (gend < gdesc.size() &&
           nl + (gdesc[gend].lit_end - gdesc[gend].lit_begin) <= kMaxLitsPerLaunch) {
      nl += gdesc[gend].lit_end - gdesc[gend].lit_begin;
      ++gend;
    }
    const int lit0 = gdesc[gbeg].lit_begin;
    const int64_t item0 = gdesc[gbeg].item_begin;
    for (size_t g = gbeg; g < gend; ++g) {
      GroupDesc s = gdesc[g];
      s.lit_begin -= lit0;
      s.lit_end -= lit0;
      s.item_begin -= item0;
      sub_all.push_back(s);
    }
    launches.push_back({gbeg, gend, lit0, nl});
    gbeg = gend;
  }
  const size_t gbytes = sizeof(GroupDesc) * sub_all.size();
  const size_t lbytes = sizeof(LitDesc) * ldesc.size();
  std::vector<unsigned char> blob(gbytes + lbytes);
  memcpy(blob.data(), sub_all.data(), gbytes);
  memcpy(blob.data() + gbytes, ldesc.data(), lbytes);
  QFG_TRY(ctx->scratch[kScrLits].reserve(ctx, blob.size() + 64));
  GroupDesc* gdev = ctx->scratch[kScrLits].as<GroupDesc>();
  LitDesc* ldev = reinterpret_cast<LitDesc*>(gdev + sub_all.size());
  unsigned int* counter = reinterpret_cast<unsigned int*>(ldev + ldesc.size());
  QFG_TRY(upload_small(ctx, gdev, blob.data(), blob.size()));
  QFG_TRY(stage_begin(ctx, QFG_STAGE_EVALUATE));
  for (const Launch& L : launches) {
    QFG_CUDA(ctx, cudaMemsetAsync(counter, 0, sizeof(unsigned int), ctx->stream));
    EvalArgs ea;
    ea.groups = gdev + L.gbeg;
    ea.num_groups = (int)(L.gend - L.gbeg);
    ea.lits = ldev + L.lit0;
    ea.num_lits = L.nl;
    ea.total_items = (int64_t)(L.gend - L.gbeg) << bits;
    ea.work_counter = counter;
    ea.counts = counts;
    const size_t smem = eval_smem_bytes(L.nl);
    QFG_CUDA(ctx, cudaFuncSetAttribute(eval_batched_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    eval_batched_kernel<<<ctx->num_sms, kEvalThreads, smem, ctx->stream>>>(ea);
    QFG_LAUNCHED(ctx);
  }
  QFG_TRY(stage_end(ctx, QFG_STAGE_EVALUATE));
  return QFG_OK;
}

}  // namespace qfg

using namespace qfg;

extern "C" int qfg_evaluate_step(qfg_ctx* c, const qfg_bindings* b, int32_t n,
                                 const qfg_literal* lits, int64_t* counts, int flags) {
  if (c == nullptr || b == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  QFG_TRY(validate_literals(ctx, b, n, lits));
  unsigned long long* dev = nullptr;
  QFG_TRY(counts_begin(ctx, n, counts, flags, &dev));
  QFG_TRY(evaluate_batched(ctx, b, n, lits, dev));
  return counts_end(ctx, n, counts, flags, dev);
}

extern "C" int qfg_step_traffic(qfg_ctx* c, const qfg_bindings* b, int32_t n,
                                const qfg_literal* lits, int64_t* bytes) {
  if (c == nullptr || b == nullptr || bytes == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  QFG_TRY(validate_literals(ctx, b, n, lits));
  for (int s = 0; s < QFG_NUM_STAGES; ++s) bytes[s] = 0;
  const int64_t nb = b->num_positive + b->num_negative;
  if (n == 0) return QFG_OK;
  StepPlan plan;
  QFG_TRY(plan_step(ctx, n, lits, &plan));
  // Key tables: read the projected relation columns once, write the table.
  std::map<const KeyTable*, int> seen;
  for (int i = 0; i < n; ++i) {
    const KeyTable* kt = plan.tables[i];
    if (seen.count(kt)) continue;
    seen[kt] = 1;
    Relation* rel = nullptr;
    QFG_TRY(find_relation(ctx, lits[i].relation_id, &rel));
    bytes[QFG_STAGE_KEY_TABLES] += 4 * rel->num_tuples * kt->num_keys +
                                   4 * kt->num_entries * (kt->num_keys + 1);
  }
  for (const HostGroup& g : plan.groups) {
    // Partition: each carried column read once and written once.
    bytes[QFG_STAGE_BIND_PARTITION] += 8 * nb * (int64_t)g.cols.size();
    // Evaluate: partitioned columns read once, every literal's key tuples
    // and multiplicities read once, four int64 counts written.
    bytes[QFG_STAGE_EVALUATE] += 4 * nb * (int64_t)g.cols.size();
    for (int i : g.lits)
      bytes[QFG_STAGE_EVALUATE] += 4 * plan.tables[i]->num_entries * (plan.tables[i]->num_keys + 1) + 32;
  }
  // The plain path re-partitions the join column per literal (value +
  // tuple id, 12 bytes a row), reads the relation partition (8 bytes a
  // tuple) and the join pairs' atom columns are gathered.
  for (int i = 0; i < n; ++i) {
    Relation* rel = nullptr;
    QFG_TRY(find_relation(ctx, lits[i].relation_id, &rel));
    bytes[QFG_STAGE_PER_LITERAL] += 12 * nb + 8 * rel->num_tuples + 32;
  }
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return QFG_OK;
}

extern "C" int qfg_evaluate_group(qfg_ctx* c, const qfg_bindings* b, int32_t clause_join_key_id,
                                  int32_t n, const qfg_literal* lits, int64_t* counts, int flags) {
  if (c == nullptr || b == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  QFG_TRY(validate_literals(ctx, b, n, lits));
  for (int32_t i = 0; i < n; ++i)
    if (lits[i].vars[lits[i].join_pos] != clause_join_key_id)
      return set_error(ctx, QFG_ERR_INVALID,
                       "literal " + std::to_string(i) + " does not join on the clause variable");
  unsigned long long* dev = nullptr;
  QFG_TRY(counts_begin(ctx, n, counts, flags, &dev));
  QFG_TRY(evaluate_batched(ctx, b, n, lits, dev));
  return counts_end(ctx, n, counts, flags, dev);
}
