// joins.cu -- semi-joins and the label-aware binding-set extension.
//
// Both rest on a device key set: the distinct key tuples of one side in an
// open-addressing table whose slots hold the row that first claimed the
// tuple (atomicCAS), every row of that side mapping to that representative.
//
// LeftSemiJoin / RightSemiJoin (operations/LeftSemiJoin.hpp:55-141,
// operations/RightSemiJoin.hpp:44-82) only need membership: the rows of the
// other side check a bit filter of the set side's key tuples, look up the
// tuples that pass, and a warp turns 32 answers into one 32-bit word with
// __ballot_sync.  Two consecutive words form one 64-bit block of
// the reference's BitVector (dynamic_bitset<unsigned long>, little-endian
// bit order), so the output is byte-identical; bits past the last row stay
// zero as the reference requires (utility/BitVectorBuilder.hpp:46-54).
//
// CreateLabelAwareBindingTables (operations/MultiColumnHashJoin.cpp:117-256)
// must also reproduce the row order.  In the reference every probe row emits
// its matches in chain order, and a chain built by head insertion lists
// equal-key build rows in descending row order (MultiColumnHashJoin.cpp:
// 496-528, BuildHashTable.cpp:97-125).  Here the build rows are sorted
// stably by representative, each probe row counts its matches, an exclusive
// scan gives every probe row its output offset, and the probe row writes its
// matches walking its build segment from the end.  The side that is built on
// follows the reference: the binding set when both label sides are smaller
// than the relation (CollaborateJoin, :172-207), else the relation (:208-250).
// The relation's build side (key set, sorted rows, segments) depends only on
// the relation and the bound argument positions, so it is kept on the
// relation for later extensions; a binding-set build side is built per call.
#include <cstring>

#include "keysets.cuh"

namespace qfg {

namespace {

// Set side's filter: bit (hash >> (32 - fbits)) of every set row's key tuple
// (the key set's slots use the hash's low bits).  A probe row whose bit is
// clear has no match, so most misses never touch the key set.  Built only
// when the probed side is at least twice the set side: otherwise building it
// costs about what it saves.
__global__ void semijoin_filter_kernel(KeyCols set, int64_t n, uint32_t* __restrict__ filter,
                                       int fbits) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t b = keys_hash<0>(set, r) >> (32 - fbits);
    // Repeated keys find their bit set and spare the word's atomics.
    if (!((filter[b >> 5] >> (b & 31)) & 1u)) atomicOr(&filter[b >> 5], 1u << (b & 31));
  }
}

// Probes the key set of `build` with the rows of `probe`.  MARK false: the
// answers go to 32-row words (and their count to *ones).  MARK true: each
// matched representative row o gets flag[o] = 1.  The mode is a template
// argument so that the word form keeps its 32 registers (8 CTAs an SM).
template <int NK, bool MARK>
__global__ void semijoin_bits_kernel(KeyCols build, const int32_t* __restrict__ owner, uint32_t mask,
                                     const uint32_t* __restrict__ filter, int fbits,
                                     KeyCols probe, int64_t n, uint32_t* __restrict__ words,
                                     int64_t nwords, unsigned long long* __restrict__ ones,
                                     uint8_t* __restrict__ flag) {
  const int64_t warps_total = (int64_t)gridDim.x * blockDim.x / 32;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = lane_id();
  constexpr int W = 4;  // words a warp keeps in flight: the lookups are latency-bound
  unsigned long long c = 0;
  for (int64_t w0 = gw; w0 < nwords; w0 += warps_total * W) {
    uint32_t h[W];
    bool live[W];
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const int64_t i = (w0 + u * warps_total) * 32 + lane;
      live[u] = i < n;
      h[u] = live[u] ? keys_hash<NK>(probe, i) : 0u;
    }
    if (fbits > 0) {
#pragma unroll
      for (int u = 0; u < W; ++u) {
        const uint32_t b = h[u] >> (32 - fbits);
        if (live[u]) live[u] = (__ldg(filter + (b >> 5)) >> (b & 31)) & 1u;
      }
    }
    int32_t o[W];
#pragma unroll
    for (int u = 0; u < W; ++u) o[u] = live[u] ? owner[h[u] & mask] : -1;
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const int64_t i = (w0 + u * warps_total) * 32 + lane;
      bool hit = false;
      uint32_t slot = h[u] & mask;
      for (uint32_t p = 0; p <= mask && o[u] >= 0; ++p) {
        if (keys_eq<NK>(build, o[u], probe, i)) {
          hit = true;
          break;
        }
        slot = (slot + 1) & mask;
        o[u] = owner[slot];
      }
      if constexpr (MARK) {
        if (hit && flag[o[u]] == 0) flag[o[u]] = 1;
        continue;
      }
      const int64_t w = w0 + u * warps_total;
      const unsigned ball = __ballot_sync(kFullMask, hit);
      if (lane == 0 && w < nwords) {
        if (words != nullptr) words[w] = ball;
        c += (unsigned long long)__popc(ball);
      }
    }
  }
  // One count a warp: a count a word serialises a million atomics on one address.
  if (lane == 0 && c != 0) atomicAdd(ones, c);
}

// Bits of the rows of a key set's own table: row i is in when its
// representative was marked.
__global__ void semijoin_rep_bits_kernel(const int32_t* __restrict__ rep,
                                         const uint8_t* __restrict__ flag, int64_t n,
                                         uint32_t* __restrict__ words, int64_t nwords,
                                         unsigned long long* __restrict__ ones) {
  const int64_t warps_total = (int64_t)gridDim.x * blockDim.x / 32;
  const int lane = lane_id();
  unsigned long long c = 0;
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; w < nwords;
       w += warps_total) {
    const int64_t i = w * 32 + lane;
    const int32_t r = i < n ? rep[i] : -1;
    const unsigned ball = __ballot_sync(kFullMask, r >= 0 && flag[r] != 0);
    if (lane == 0) {
      words[w] = ball;
      c += (unsigned long long)__popc(ball);
    }
  }
  if (lane == 0 && c != 0) atomicAdd(ones, c);
}

// After a stable sort of build rows by representative: first and last
// sorted position of every representative's segment.
__global__ void segments_kernel(const uint32_t* __restrict__ skey, int64_t n,
                                int32_t* __restrict__ seg_first, int32_t* __restrict__ seg_last) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t r = skey[s];
    if (s == 0 || skey[s - 1] != r) seg_first[r] = (int32_t)s;
    if (s == n - 1 || skey[s + 1] != r) seg_last[r] = (int32_t)s;
  }
}

__global__ void match_count_kernel(KeyCols build, const int32_t* __restrict__ owner, uint32_t mask,
                                   KeyCols probe, int64_t n, const int32_t* __restrict__ seg_first,
                                   const int32_t* __restrict__ seg_last, int32_t* __restrict__ prep,
                                   uint32_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = keyset_find(build, owner, mask, probe, i);
    prep[i] = r;
    cnt[i] = r < 0 ? 0u : (uint32_t)(seg_last[r] - seg_first[r] + 1);
  }
}

struct ExtendArgs {
  const int32_t* const* bind_cols;  // nc device pointers (full binding set)
  int nc;
  const int32_t* unbound[QFG_MAX_ARITY];  // relation columns of the unbound arguments
  int nu;
  int64_t label_lo;        // first binding row of this label
  int relation_is_probe;   // probe rows are relation rows (else binding rows)
  int64_t out_rows;        // rows of every output column
  int64_t out_base;        // first output row of this label
  int32_t* out;            // (nc + nu) columns of out_rows
};

// One thread per output row (a probe row matching a key of many build rows
// would otherwise write them all alone): output row o belongs to the last
// probe row i with pos[i] <= o (pos is the exclusive scan of the match
// counts, so that row has a match left), and is its (o - pos[i])-th match.
__global__ void extend_write_kernel(ExtendArgs a, int64_t n_probe, int64_t produced,
                                    const int32_t* __restrict__ prep,
                                    const uint32_t* __restrict__ pos,
                                    const int32_t* __restrict__ seg_last,
                                    const int32_t* __restrict__ sorted_rows) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < produced;
       k += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = n_probe - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if ((int64_t)pos[mid] <= k) lo = mid; else hi = mid - 1;
    }
    const int64_t i = lo;
    // The build segment in descending row order = the reference's chain order.
    const int32_t brow = sorted_rows[seg_last[prep[i]] - (int32_t)(k - (int64_t)pos[i])];
    const int64_t b = a.label_lo + (a.relation_is_probe ? (int64_t)brow : i);
    const int64_t rr = a.relation_is_probe ? i : (int64_t)brow;
    const int64_t o = a.out_base + k;
    for (int c = 0; c < a.nc; ++c) a.out[(int64_t)c * a.out_rows + o] = a.bind_cols[c][b];
    for (int u = 0; u < a.nu; ++u) a.out[(int64_t)(a.nc + u) * a.out_rows + o] = a.unbound[u][rr];
  }
}

int make_keycols(Ctx* ctx, const int32_t* const* host_ptrs, int nk, KeyCols* out) {
  if (nk < 1 || nk > QFG_MAX_ARITY || host_ptrs == nullptr)
    return set_error(ctx, QFG_ERR_INVALID, "key column count must be in [1, 8]");
  out->nk = nk;
  for (int q = 0; q < nk; ++q) out->c[q] = host_ptrs[q];
  return QFG_OK;
}

// A grid of as many 256-thread CTAs as fit on the GPU at once (or fewer, 8
// words a CTA): the probe loop is grid-strided, so a second partial wave
// would only add a tail.
template <typename Kernel>
unsigned resident_grid(Ctx* ctx, Kernel k, int64_t words) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((words + 7) / 8, (int64_t)ctx->num_sms * per_sm));
}

template <bool MARK>
int launch_semijoin_probe(Ctx* ctx, int nk, const KeyCols& small, const int32_t* owner,
                          uint32_t mask, const uint32_t* filter, int fbits, const KeyCols& large,
                          int64_t n_large, uint32_t* pout, int64_t pwords,
                          unsigned long long* ones, uint8_t* flag) {
  auto k = nk == 1 ? semijoin_bits_kernel<1, MARK>
                   : nk == 2 ? semijoin_bits_kernel<2, MARK> : semijoin_bits_kernel<0, MARK>;
  k<<<resident_grid(ctx, k, pwords), 256, 0, ctx->stream>>>(small, owner, mask, filter, fbits,
                                                            large, n_large, pout, pwords, ones,
                                                            flag);
  QFG_LAUNCHED(ctx);
  return QFG_OK;
}

int semijoin(Ctx* ctx, const KeyCols& set_side, int64_t n_set, const KeyCols& bit_side,
             int64_t n_bits, uint64_t* d_bits, int64_t* num_ones) {
  const int64_t nwords = 2 * ((n_bits + 63) / 64);
  QFG_TRY(ctx->scratch[kScrTmpC].reserve(ctx, sizeof(unsigned long long)));
  unsigned long long* ones = ctx->scratch[kScrTmpC].as<unsigned long long>();
  QFG_CUDA(ctx, cudaMemsetAsync(ones, 0, sizeof(unsigned long long), ctx->stream));
  if (n_set == 0 || n_bits == 0) {
    if (nwords > 0)
      QFG_CUDA(ctx, cudaMemsetAsync(d_bits, 0, sizeof(uint32_t) * nwords, ctx->stream));
  } else {
    // The key set holds the smaller side and the larger side probes it.  When
    // the smaller side is the one that gets bits, the probes mark its
    // representatives and its rows read their bit through their representative.
    const bool mark = n_set > n_bits;
    const KeyCols& small = mark ? bit_side : set_side;
    const KeyCols& large = mark ? set_side : bit_side;
    const int64_t n_small = mark ? n_bits : n_set;
    const int64_t n_large = mark ? n_set : n_bits;
    const uint32_t mask = table_mask(n_small);
    QFG_TRY(ctx->scratch[kScrJoin].reserve(ctx, sizeof(int32_t) * ((size_t)mask + 1)));
    int32_t* owner = ctx->scratch[kScrJoin].as<int32_t>();
    int32_t* rep = nullptr;
    uint8_t* flag = nullptr;
    if (mark) {
      QFG_TRY(ctx->scratch[kScrJoin2].reserve(ctx, (sizeof(int32_t) + 1) * (size_t)n_small));
      rep = ctx->scratch[kScrJoin2].as<int32_t>();
      flag = reinterpret_cast<uint8_t*>(rep + n_small);
      QFG_CUDA(ctx, cudaMemsetAsync(flag, 0, (size_t)n_small, ctx->stream));
    }
    QFG_CUDA(ctx, cudaMemsetAsync(owner, 0xff, sizeof(int32_t) * ((size_t)mask + 1), ctx->stream));
    keyset_insert_kernel<0><<<rows_grid(ctx, n_small), 256, 0, ctx->stream>>>(small, n_small,
                                                                           owner, mask, rep);
    QFG_LAUNCHED(ctx);
    // About 8 filter bits a key-set row (2^16 to 2^28 bits); fbits 0 = no filter.
    int fbits = 0;
    const uint32_t* filter = nullptr;
    if (n_large >= 2 * n_small) {
      fbits = 16;
      while (fbits < 28 && ((int64_t)1 << fbits) < 8 * n_small) ++fbits;
      const size_t fwords = (size_t)1 << (fbits - 5);
      QFG_TRY(ctx->scratch[kScrTmpB].reserve(ctx, sizeof(uint32_t) * fwords));
      uint32_t* f = ctx->scratch[kScrTmpB].as<uint32_t>();
      QFG_CUDA(ctx, cudaMemsetAsync(f, 0, sizeof(uint32_t) * fwords, ctx->stream));
      semijoin_filter_kernel<<<rows_grid(ctx, n_small), 256, 0, ctx->stream>>>(small, n_small, f,
                                                                              fbits);
      QFG_LAUNCHED(ctx);
      filter = f;
    }
    // 32-row words of the probing side (the output's words when not marking).
    const int64_t pwords = mark ? (n_large + 31) / 32 : nwords;
    uint32_t* words = reinterpret_cast<uint32_t*>(d_bits);
    uint32_t* pout = mark ? nullptr : words;
    if (mark) {
      QFG_TRY(launch_semijoin_probe<true>(ctx, small.nk, small, owner, mask, filter, fbits, large,
                                          n_large, pout, pwords, ones, flag));
    } else {
      QFG_TRY(launch_semijoin_probe<false>(ctx, small.nk, small, owner, mask, filter, fbits, large,
                                           n_large, pout, pwords, ones, flag));
    }
    if (mark) {
      semijoin_rep_bits_kernel<<<resident_grid(ctx, semijoin_rep_bits_kernel, nwords), 256, 0,
                                 ctx->stream>>>(rep, flag, n_bits, words, nwords, ones);
      QFG_LAUNCHED(ctx);
    }
  }
  unsigned long long h = 0;
  QFG_CUDA(ctx, cudaMemcpyAsync(&h, ones, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (num_ones != nullptr) *num_ones = (int64_t)h;
  return QFG_OK;
}

// The build side of an extension: the key set of `build`, its rows sorted
// stably by representative, each representative's segment.
struct BuildView {
  const int32_t* owner;
  uint32_t mask;
  const int32_t* sorted;
  const int32_t* seg_first;
  const int32_t* seg_last;
};

// Builds the view for `build` (n_build > 0) into `owner_mem` (mask + 1) and
// `rows_mem` (3 * n_build: sorted rows, segment firsts, segment lasts).
int build_side(Ctx* ctx, const KeyCols& build, int64_t n_build, uint32_t mask, int32_t* owner,
               int32_t* rows_mem, BuildView* v) {
  const size_t cap = (size_t)mask + 1;
  QFG_TRY(ctx->scratch[kScrJoin].reserve(ctx, sizeof(int32_t) * (size_t)n_build));
  int32_t* rep = ctx->scratch[kScrJoin].as<int32_t>();
  QFG_CUDA(ctx, cudaMemsetAsync(owner, 0xff, sizeof(int32_t) * cap, ctx->stream));
  keyset_insert_kernel<0><<<rows_grid(ctx, n_build), 256, 0, ctx->stream>>>(build, n_build, owner,
                                                                            mask, rep);
  QFG_LAUNCHED(ctx);
  QFG_TRY(ctx->scratch[kScrSortA].reserve(ctx, 2 * sizeof(uint32_t) * (size_t)n_build));
  QFG_TRY(ctx->scratch[kScrSortB].reserve(ctx, 2 * sizeof(uint32_t) * (size_t)n_build));
  uint32_t* k0 = ctx->scratch[kScrSortA].as<uint32_t>();
  int32_t* p0 = reinterpret_cast<int32_t*>(k0 + n_build);
  uint32_t* k1 = ctx->scratch[kScrSortB].as<uint32_t>();
  int32_t* p1 = reinterpret_cast<int32_t*>(k1 + n_build);
  QFG_CUDA(ctx, cudaMemcpyAsync(k0, rep, sizeof(int32_t) * (size_t)n_build,
                                cudaMemcpyDeviceToDevice, ctx->stream));
  int bits = 1;
  while (bits < 31 && ((int64_t)1 << bits) < n_build) ++bits;
  uint32_t* skey;
  int32_t* srow;
  QFG_TRY(sort_pairs_u32(ctx, k0, p0, k1, p1, n_build, bits, &skey, &srow));
  int32_t* sorted = rows_mem;
  int32_t* seg_first = rows_mem + n_build;
  int32_t* seg_last = seg_first + n_build;
  QFG_CUDA(ctx, cudaMemcpyAsync(sorted, srow, sizeof(int32_t) * (size_t)n_build,
                                cudaMemcpyDeviceToDevice, ctx->stream));
  segments_kernel<<<rows_grid(ctx, n_build), 256, 0, ctx->stream>>>(skey, n_build, seg_first,
                                                                    seg_last);
  QFG_LAUNCHED(ctx);
  *v = BuildView{owner, mask, sorted, seg_first, seg_last};
  return QFG_OK;
}

// The relation's build side over the literal's bound argument positions,
// built on first use and kept on the relation (its rows never change while
// it is registered).
int relation_build_side(Ctx* ctx, Relation* rel, const std::vector<int>& args,
                        const KeyCols& keys, BuildView* v) {
  auto it = rel->ext_builds.find(args);
  if (it == rel->ext_builds.end()) {
    auto eb = std::make_unique<ExtensionBuild>();
    eb->mask = table_mask(rel->num_tuples);
    QFG_TRY(eb->owner.reserve(ctx, sizeof(int32_t) * ((size_t)eb->mask + 1)));
    QFG_TRY(eb->sorted.reserve(ctx, sizeof(int32_t) * 3 * (size_t)rel->num_tuples));
    BuildView tmp;
    QFG_TRY(build_side(ctx, keys, rel->num_tuples, eb->mask, eb->owner.as<int32_t>(),
                       eb->sorted.as<int32_t>(), &tmp));
    it = rel->ext_builds.emplace(args, std::move(eb)).first;
  }
  const ExtensionBuild& eb = *it->second;
  const int32_t* base = eb.sorted.as<int32_t>();
  *v = BuildView{eb.owner.as<int32_t>(), eb.mask, base, base + rel->num_tuples,
                 base + 2 * rel->num_tuples};
  return QFG_OK;
}

// One label of the extension: joins `probe` rows against the build side and
// writes the matches in the reference's order at output rows
// [out_base, out_base + expected).
int probe_side(Ctx* ctx, const KeyCols& build, const BuildView& v, const KeyCols& probe,
               int64_t n_probe, int64_t expected, ExtendArgs args,
               int64_t* produced_only = nullptr) {
  QFG_TRY(ctx->scratch[kScrJoin2].reserve(ctx, sizeof(int32_t) * (2 * (size_t)n_probe + 2)));
  int32_t* prep = ctx->scratch[kScrJoin2].as<int32_t>();
  uint32_t* cnt = reinterpret_cast<uint32_t*>(prep + n_probe);
  uint32_t* total = cnt + n_probe;
  match_count_kernel<<<rows_grid(ctx, n_probe), 256, 0, ctx->stream>>>(
      build, v.owner, v.mask, probe, n_probe, v.seg_first, v.seg_last, prep, cnt);
  QFG_LAUNCHED(ctx);
  QFG_TRY(exclusive_scan_u32(ctx, cnt, cnt, n_probe, total));
  uint32_t produced = 0;
  QFG_CUDA(ctx, cudaMemcpyAsync(&produced, total, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                ctx->stream));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (produced_only != nullptr) {  // counting only: the row count, nothing written
    *produced_only = produced;
    return QFG_OK;
  }
  if ((int64_t)produced != expected)
    return set_error(ctx, QFG_ERR_MISMATCH,
                     "extension produced " + std::to_string(produced) + " rows for a label, " +
                         std::to_string(expected) + " announced");
  extend_write_kernel<<<rows_grid(ctx, (int64_t)produced), 256, 0, ctx->stream>>>(
      args, n_probe, (int64_t)produced, prep, cnt, v.seg_last, v.sorted);
  QFG_LAUNCHED(ctx);
  // The next label reuses (and may regrow) the same scratch.
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return QFG_OK;
}

// One label of the extension with the binding rows as the build side (built
// for this call only).
int extend_label_binding_build(Ctx* ctx, const KeyCols& build, int64_t n_build,
                               const KeyCols& probe, int64_t n_probe, int64_t expected,
                               ExtendArgs args, int64_t* produced_only = nullptr) {
  if (n_build == 0 || n_probe == 0) {
    if (produced_only != nullptr) {
      *produced_only = 0;
      return QFG_OK;
    }
    return expected == 0 ? QFG_OK
                         : set_error(ctx, QFG_ERR_MISMATCH, "extension produced 0 rows for a label");
  }
  const uint32_t mask = table_mask(n_build);
  // Context scratch that nothing else of an extension uses (grow-only).
  DevBuf& owner = ctx->scratch[kScrDedup];
  DevBuf& rows = ctx->scratch[kScrMisc];
  QFG_TRY(owner.reserve(ctx, sizeof(int32_t) * ((size_t)mask + 1)));
  QFG_TRY(rows.reserve(ctx, sizeof(int32_t) * 3 * (size_t)n_build));
  BuildView v;
  QFG_TRY(build_side(ctx, build, n_build, mask, owner.as<int32_t>(), rows.as<int32_t>(), &v));
  return probe_side(ctx, build, v, probe, n_probe, expected, args, produced_only);
}

}  // namespace

// The rows an extension by `lit` produces per label (the binding counts of
// the literal), from the extension's own match counts.
int extension_counts(Ctx* ctx, const qfg_bindings* b, const qfg_literal* lit, int64_t* num_pos,
                     int64_t* num_neg) {
  Relation* rel = nullptr;
  QFG_TRY(find_relation(ctx, lit->relation_id, &rel));
  if (lit->num_args != rel->num_columns)
    return set_error(ctx, QFG_ERR_INVALID, "extension: literal arity differs from the relation");
  KeyCols rel_keys, pos_keys, neg_keys;
  rel_keys.nk = pos_keys.nk = neg_keys.nk = 0;
  std::vector<int> bound_args;
  const int64_t P = b->num_positive, N = b->num_negative, R = rel->num_tuples;
  for (int k = 0; k < lit->num_args; ++k) {
    const int v = lit->vars[k];
    if (v >= b->num_columns || v < -1)
      return set_error(ctx, QFG_ERR_INVALID, "extension: variable out of range");
    if (v < 0) continue;
    bound_args.push_back(k);
    rel_keys.c[rel_keys.nk++] = rel->columns[k];
    pos_keys.c[pos_keys.nk++] = b->columns[v];
    neg_keys.c[neg_keys.nk++] = b->columns[v] + P;
  }
  if (rel_keys.nk == 0)
    return set_error(ctx, QFG_ERR_INVALID, "extension: literal has no bound argument");
  ExtendArgs args;
  memset(&args, 0, sizeof(args));
  const bool relation_is_probe = P < R && N < R;
  int64_t got[2] = {0, 0};
  for (int label = 0; label < 2; ++label) {
    const KeyCols& bind_keys = label == 0 ? pos_keys : neg_keys;
    const int64_t n_label = label == 0 ? P : N;
    if (relation_is_probe) {
      QFG_TRY(extend_label_binding_build(ctx, bind_keys, n_label, rel_keys, R, 0, args,
                                         &got[label]));
    } else if (R > 0 && n_label > 0) {
      BuildView v;
      QFG_TRY(relation_build_side(ctx, rel, bound_args, rel_keys, &v));
      QFG_TRY(probe_side(ctx, rel_keys, v, bind_keys, n_label, 0, args, &got[label]));
    }
  }
  *num_pos = got[0];
  *num_neg = got[1];
  return QFG_OK;
}

}  // namespace qfg

using namespace qfg;

extern "C" int qfg_extend_bindings(qfg_ctx* c, const qfg_bindings* b, const qfg_literal* lit,
                                   int64_t num_out_positive, int64_t num_out_negative,
                                   qfg_bindings** out) {
  if (c == nullptr || b == nullptr || lit == nullptr || out == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  *out = nullptr;
  Relation* rel = nullptr;
  QFG_TRY(find_relation(ctx, lit->relation_id, &rel));
  if (lit->num_args != rel->num_columns || num_out_positive < 0 || num_out_negative < 0 ||
      num_out_positive + num_out_negative > INT32_MAX)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_extend_bindings: invalid literal or counts");
  KeyCols rel_keys, pos_keys, neg_keys;
  rel_keys.nk = pos_keys.nk = neg_keys.nk = 0;
  std::vector<int> bound_args;
  ExtendArgs args;
  memset(&args, 0, sizeof(args));
  const int64_t P = b->num_positive, N = b->num_negative, R = rel->num_tuples;
  for (int k = 0; k < lit->num_args; ++k) {
    const int v = lit->vars[k];
    if (v >= b->num_columns || v < -1)
      return set_error(ctx, QFG_ERR_INVALID, "qfg_extend_bindings: variable out of range");
    if (v >= 0) {
      bound_args.push_back(k);
      rel_keys.c[rel_keys.nk++] = rel->columns[k];
      pos_keys.c[pos_keys.nk++] = b->columns[v];
      neg_keys.c[neg_keys.nk++] = b->columns[v] + P;
    } else {
      args.unbound[args.nu++] = rel->columns[k];
    }
  }
  if (rel_keys.nk == 0)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_extend_bindings: literal has no bound argument");
  const int nc = b->num_columns;
  const int64_t total = num_out_positive + num_out_negative;
  auto nb = std::make_unique<qfg_bindings>();
  nb->num_columns = nc + args.nu;
  nb->num_positive = num_out_positive;
  nb->num_negative = num_out_negative;
  QFG_TRY(nb->storage.reserve(ctx, sizeof(int32_t) * (size_t)nb->num_columns *
                                       (size_t)std::max<int64_t>(total, 1)));
  nb->columns.resize(nb->num_columns);
  for (int i = 0; i < nb->num_columns; ++i) nb->columns[i] = nb->storage.as<int32_t>() + i * total;
  // Device copy of the binding column pointers (any number of columns).
  QFG_TRY(ctx->scratch[kScrTmpB].reserve(ctx, sizeof(const int32_t*) * (size_t)nc));
  const int32_t** dcols = ctx->scratch[kScrTmpB].as<const int32_t*>();
  QFG_TRY(upload_small(ctx, dcols, b->columns.data(), sizeof(const int32_t*) * (size_t)nc));
  args.bind_cols = dcols;
  args.nc = nc;
  args.out_rows = total;
  args.out = nb->storage.as<int32_t>();
  args.relation_is_probe = (P < R && N < R) ? 1 : 0;
  for (int label = 0; label < 2; ++label) {
    const KeyCols& bind_keys = label == 0 ? pos_keys : neg_keys;
    const int64_t n_label = label == 0 ? P : N;
    args.label_lo = label == 0 ? 0 : P;
    args.out_base = label == 0 ? 0 : num_out_positive;
    const int64_t expected = label == 0 ? num_out_positive : num_out_negative;
    if (args.relation_is_probe) {
      QFG_TRY(extend_label_binding_build(ctx, bind_keys, n_label, rel_keys, R, expected, args));
    } else if (R == 0 || n_label == 0) {
      if (expected != 0)
        return set_error(ctx, QFG_ERR_MISMATCH, "extension produced 0 rows for a label");
    } else {
      BuildView v;
      QFG_TRY(relation_build_side(ctx, rel, bound_args, rel_keys, &v));
      QFG_TRY(probe_side(ctx, rel_keys, v, bind_keys, n_label, expected, args));
    }
  }
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *out = nb.release();
  return QFG_OK;
}

extern "C" int qfg_left_semijoin(qfg_ctx* c, const int32_t* const* d_probe_keys, int64_t num_probe,
                                 const int32_t* const* d_build_keys, int64_t num_build,
                                 int32_t num_keys, uint64_t* d_bits, int64_t* num_ones) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_probe < 0 || num_build < 0 || num_probe > INT32_MAX || num_build > INT32_MAX ||
      (num_probe > 0 && d_bits == nullptr))
    return set_error(ctx, QFG_ERR_INVALID, "qfg_left_semijoin: invalid arguments");
  KeyCols probe, build;
  QFG_TRY(make_keycols(ctx, d_probe_keys, num_keys, &probe));
  QFG_TRY(make_keycols(ctx, d_build_keys, num_keys, &build));
  return semijoin(ctx, build, num_build, probe, num_probe, d_bits, num_ones);
}

extern "C" int qfg_right_semijoin(qfg_ctx* c, const int32_t* const* d_probe_keys, int64_t num_probe,
                                  const int32_t* const* d_build_keys, int64_t num_build,
                                  int32_t num_keys, uint64_t* d_bits, int64_t* num_ones) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_probe < 0 || num_build < 0 || num_probe > INT32_MAX || num_build > INT32_MAX ||
      (num_build > 0 && d_bits == nullptr))
    return set_error(ctx, QFG_ERR_INVALID, "qfg_right_semijoin: invalid arguments");
  KeyCols probe, build;
  QFG_TRY(make_keycols(ctx, d_probe_keys, num_keys, &probe));
  QFG_TRY(make_keycols(ctx, d_build_keys, num_keys, &build));
  return semijoin(ctx, probe, num_probe, build, num_build, d_bits, num_ones);
}
