// after_semijoin.cu -- BuildHashTableAfterSemiJoin in the reference's exact
// table layout, and the probe of such a table.
//
// The reference (operations/BuildHashTable.cpp:127-189, 212-236) visits the
// chunks a semi-join yields in order and, within a chunk, the positions whose
// bit is set in increasing order; each position is inserted at the head of
// its bucket's chain (FoilHashTable with radix bits 0, buckets[next_pow2(n)],
// 1-based links) unless the chain reaches a position with equal keys.
// Positions and key reads are relative to the chunk: LeftSemiJoin::Next
// (operations/LeftSemiJoin.hpp:55-83) cuts its probe side into
// FLAGS_semijoin_chunck_size-row chunks and offsets the chunk's output
// columns by the chunk start, while RightSemiJoin yields one chunk.
//
// First chunk, in parallel.  The table starts empty, so a position is
// inserted exactly when it is the first set position of its key tuple (an
// earlier equal one is in the same bucket's chain).  A key set keeps the
// smallest set position of every tuple (atomicCAS to claim a slot,
// atomicMin among equal tuples); the first positions are compacted in
// order, sorted stably by bucket, and each links to its predecessor in the
// bucket, the last one becoming the head -- the chains the reference's head
// insertion leaves.
//
// Later chunks, in order.  Their positions are compared through the current
// chunk's columns also against positions an earlier chunk inserted, and a
// position inserted again relinks its `next` word, which changes what other
// chains reach; the outcome depends on the exact insertion order.  One GPU
// thread therefore replays those chunks as the reference does, over the
// device-resident table (chains stay acyclic: a position a chain already
// reaches compares equal to itself and is never inserted again; the walk is
// still bounded by the table size and a longer one is reported).  A chain
// position past the end of a short last chunk compares unequal (the
// reference reads past the end of its columns there).
#include <algorithm>

#include "keysets.cuh"

namespace qfg {

namespace {

__device__ __forceinline__ bool bit_set(const uint64_t* __restrict__ bits, int64_t r) {
  return (bits[r >> 6] >> (r & 63)) & 1ull;
}

// Hash<k> of utility/Hash.hpp:35-55 (identity, HashCombine chain) at row r.
__device__ __forceinline__ uint32_t ref_keys_hash(const KeyCols& k, int64_t r) {
  uint32_t h = ref_hash(k.c[0][r]);
  for (int q = 1; q < k.nk; ++q) h = ref_hash_combine(h, k.c[q][r]);
  return h;
}

// Empty key-set slot: every row index is below it (rows are checked on entry).
constexpr int32_t kAsjEmpty = 0x7f7f7f7f;

// Smallest set position of every key tuple among rows [0, n): slot owners
// start at kAsjEmpty (a byte-wise memset value above every row index).
__global__ void asj_first_kernel(KeyCols k, int64_t n, const uint64_t* __restrict__ bits,
                                 int32_t* __restrict__ owner, uint32_t mask) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    if (!bit_set(bits, r)) continue;
    uint32_t slot = keys_hash(k, r) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
      const int32_t o = atomicCAS(&owner[slot], kAsjEmpty, (int32_t)r);
      if (o == kAsjEmpty) break;
      // Only rows with the slot's key tuple ever write it after its claim.
      if (keys_eq(k, o, k, r)) {
        atomicMin(&owner[slot], (int32_t)r);
        break;
      }
      slot = (slot + 1) & mask;
    }
  }
}

// flag[r] = 1 when row r is the first set position of its key tuple.
__global__ void asj_flag_kernel(KeyCols k, int64_t n, const uint64_t* __restrict__ bits,
                                const int32_t* __restrict__ owner, uint32_t mask,
                                uint32_t* __restrict__ flag) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    uint32_t f = 0;
    if (bit_set(bits, r)) {
      uint32_t slot = keys_hash(k, r) & mask;
      for (uint32_t probe = 0; probe <= mask; ++probe) {
        const int32_t o = owner[slot];
        if (o == kAsjEmpty) break;  // not reached: every set row is in the set
        if (keys_eq(k, o, k, r)) {
          f = o == (int32_t)r ? 1u : 0u;
          break;
        }
        slot = (slot + 1) & mask;
      }
    }
    flag[r] = f;
  }
}

// The first positions in row order with their buckets.
__global__ void asj_compact_kernel(KeyCols k, int64_t n, const uint32_t* __restrict__ flag,
                                   const uint32_t* __restrict__ pos, uint32_t table_mask,
                                   int32_t* __restrict__ rows, uint32_t* __restrict__ gid) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    if (!flag[r]) continue;
    const uint32_t j = pos[r];
    rows[j] = (int32_t)r;
    gid[j] = ref_keys_hash(k, r) & table_mask;
  }
}

// After a stable sort by bucket (payload = index into rows): each position
// links to its predecessor in its bucket; the last one is the head.
__global__ void asj_links_kernel(const uint32_t* __restrict__ sgid, const int32_t* __restrict__ sidx,
                                 const int32_t* __restrict__ rows, int64_t m,
                                 int32_t* __restrict__ buckets, int32_t* __restrict__ next) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < m;
       s += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t g = sgid[s];
    const int32_t r = rows[sidx[s]];
    next[r] = (s > 0 && sgid[s - 1] == g) ? rows[sidx[s - 1]] + 1 : 0;
    if (s == m - 1 || sgid[s + 1] != g) buckets[g] = r + 1;
  }
}

// Chunks from row `from` on, replayed in order by one thread as
// InsertIfNotPresent does (keys of both positions read in the current
// chunk).  status[0] = 1 when a chain walk exceeded `limit` steps.
__global__ void asj_replay_kernel(KeyCols k, int64_t n, int64_t readable, const uint64_t* __restrict__ bits,
                                  int64_t from, int64_t chunk, uint32_t table_mask,
                                  int32_t* __restrict__ buckets, int32_t* __restrict__ next,
                                  int64_t limit, int* __restrict__ status) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  KeyCols kc = k;
  for (int64_t c0 = from; c0 < n; c0 += chunk) {
    const int64_t len = min(chunk, n - c0);
    for (int q = 0; q < k.nk; ++q) kc.c[q] = k.c[q] + c0;
    for (int64_t tid = 0; tid < len; ++tid) {
      if (!bit_set(bits, c0 + tid)) continue;
      const uint32_t b = ref_keys_hash(kc, tid) & table_mask;
      bool exist = false;
      int64_t steps = 0;
      for (int32_t p = buckets[b] - 1; p >= 0; p = next[p] - 1) {
        // A position past the end of a short last chunk (inserted by an
        // earlier chunk) is read where the columns go on (`readable` rows
        // from the start) and compares unequal past them; the reference
        // reads past the end of its columns there.
        if (c0 + p < readable && keys_eq(kc, tid, kc, p)) {
          exist = true;
          break;
        }
        if (++steps > limit) {
          status[0] = 1;
          return;
        }
      }
      if (!exist) {
        next[tid] = buckets[b];
        buckets[b] = (int32_t)tid + 1;
      }
    }
  }
}

unsigned grid_rows(Ctx* ctx, int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
}

}  // namespace

int after_semijoin_table(Ctx* ctx, const int32_t* const* cols, int nk, int64_t n, int64_t readable,
                         const uint64_t* d_bits, int64_t chunk_rows, int32_t num_build_tuples,
                         int32_t* d_buckets, int32_t* d_next, uint32_t* mask_out) {
  if (nk < 1 || nk > QFG_MAX_ARITY || cols == nullptr || n < 0 || n >= kAsjEmpty || readable < n)
    return set_error(ctx, QFG_ERR_INVALID, "after-semijoin table: invalid key columns or row count");
  KeyCols keys;
  keys.nk = nk;
  for (int q = 0; q < nk; ++q) keys.c[q] = cols[q];
  const int64_t chunk = (chunk_rows <= 0 || chunk_rows >= n) ? n : chunk_rows;
  if (num_build_tuples < 1 || (int64_t)num_build_tuples < std::min(chunk, n))
    return set_error(ctx, QFG_ERR_INVALID,
                     "after-semijoin table: num_build_tuples must exceed every chunk position");
  uint32_t nb = (uint32_t)num_build_tuples - 1u;
  nb |= nb >> 1; nb |= nb >> 2; nb |= nb >> 4; nb |= nb >> 8; nb |= nb >> 16;
  nb += 1u;
  const uint32_t table_mask = nb - 1u;
  *mask_out = table_mask;
  QFG_CUDA(ctx, cudaMemsetAsync(d_buckets, 0, sizeof(int32_t) * nb, ctx->stream));
  QFG_CUDA(ctx, cudaMemsetAsync(d_next, 0, sizeof(int32_t) * (size_t)num_build_tuples, ctx->stream));
  if (n == 0) return QFG_OK;

  // First chunk.
  const int64_t m0 = chunk;
  uint32_t cap = 1;
  while (cap < (uint32_t)(2 * m0)) cap <<= 1;
  QFG_TRY(ctx->scratch[kScrJoin].reserve(ctx, sizeof(int32_t) * (size_t)cap));
  QFG_TRY(ctx->scratch[kScrJoin2].reserve(ctx, sizeof(uint32_t) * (4 * (size_t)m0 + 8)));
  int32_t* owner = ctx->scratch[kScrJoin].as<int32_t>();
  uint32_t* flag = ctx->scratch[kScrJoin2].as<uint32_t>();
  uint32_t* pos = flag + m0;
  int32_t* rows = reinterpret_cast<int32_t*>(pos + m0);
  uint32_t* total = reinterpret_cast<uint32_t*>(rows + m0);
  int* status = reinterpret_cast<int*>(total + 1);
  QFG_CUDA(ctx, cudaMemsetAsync(owner, 0x7f, sizeof(int32_t) * cap, ctx->stream));  // kAsjEmpty
  QFG_CUDA(ctx, cudaMemsetAsync(status, 0, sizeof(int), ctx->stream));
  const unsigned g0 = grid_rows(ctx, m0);
  asj_first_kernel<<<g0, 256, 0, ctx->stream>>>(keys, m0, d_bits, owner, cap - 1);
  QFG_LAUNCHED(ctx);
  asj_flag_kernel<<<g0, 256, 0, ctx->stream>>>(keys, m0, d_bits, owner, cap - 1, flag);
  QFG_LAUNCHED(ctx);
  QFG_TRY(exclusive_scan_u32(ctx, flag, pos, m0, total));
  uint32_t inserted = 0;
  QFG_CUDA(ctx, cudaMemcpyAsync(&inserted, total, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                ctx->stream));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (inserted > 0) {
    QFG_TRY(ctx->scratch[kScrSortA].reserve(ctx, 2 * sizeof(uint32_t) * (size_t)inserted));
    QFG_TRY(ctx->scratch[kScrSortB].reserve(ctx, 2 * sizeof(uint32_t) * (size_t)inserted));
    uint32_t* k0 = ctx->scratch[kScrSortA].as<uint32_t>();
    int32_t* p0 = reinterpret_cast<int32_t*>(k0 + inserted);
    uint32_t* k1 = ctx->scratch[kScrSortB].as<uint32_t>();
    int32_t* p1 = reinterpret_cast<int32_t*>(k1 + inserted);
    asj_compact_kernel<<<g0, 256, 0, ctx->stream>>>(keys, m0, flag, pos, table_mask, rows, k0);
    QFG_LAUNCHED(ctx);
    int key_bits = 1;
    while (key_bits < 32 && (1ull << key_bits) < (unsigned long long)nb) ++key_bits;
    uint32_t* sk;
    int32_t* sp;
    QFG_TRY(sort_pairs_u32(ctx, k0, p0, k1, p1, inserted, key_bits, &sk, &sp));
    asj_links_kernel<<<grid_rows(ctx, inserted), 256, 0, ctx->stream>>>(sk, sp, rows, inserted,
                                                                        d_buckets, d_next);
    QFG_LAUNCHED(ctx);
  }
  // Later chunks, replayed in order.
  if (chunk < n) {
    asj_replay_kernel<<<1, 1, 0, ctx->stream>>>(keys, n, readable, d_bits, chunk, chunk, table_mask,
                                                d_buckets, d_next, (int64_t)num_build_tuples + 1,
                                                status);
    QFG_LAUNCHED(ctx);
    int st = 0;
    QFG_CUDA(ctx, cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (st != 0)
      return set_error(ctx, QFG_ERR_INVALID, "after-semijoin table: a chain walk exceeded the table size");
  }
  return QFG_OK;
}

namespace {

// One bit per row of `rows` binding rows (columns `probe`, the literal's
// bound arguments): set when the tuple is in the relation's key set (the
// reference's first semi-join of a coverage, bit for bit).  32-bit words,
// two per 64-bit BitVector block.
__global__ void asj_member_bits_kernel(KeyCols rel, const int32_t* __restrict__ owner, uint32_t mask,
                                       KeyCols probe, int64_t rows, uint32_t* __restrict__ words) {
  const int64_t nw = (rows + 31) >> 5;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = warp; w < nw; w += nwarps) {
    const int64_t r = (w << 5) + lane_id();
    const bool hit = r < rows && keyset_find(rel, owner, mask, probe, r) >= 0;
    const unsigned word = __ballot_sync(kFullMask, hit);
    if (lane_id() == 0) words[w] = word;
  }
}

// The reference's second semi-join of a coverage (a LeftSemiJoin of the
// examples against the projected label side through the after-semijoin
// table): example e is covered when the chain of its bucket reaches a
// position whose projected row (read at the label side's row = position)
// equals its tuple.  Bits per example in 32-bit words; the count of covered
// examples is added to *count.  Walks are bounded by the table size.
__global__ void asj_probe_kernel(const int32_t* __restrict__ buckets, const int32_t* __restrict__ next,
                                 uint32_t table_mask, KeyCols side, KeyCols ex, int64_t n_ex,
                                 int64_t limit, uint32_t* __restrict__ words,
                                 unsigned long long* __restrict__ count) {
  const int64_t nw = (n_ex + 31) >> 5;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  unsigned long long c = 0;
  for (int64_t w = warp; w < nw; w += nwarps) {
    const int64_t e = (w << 5) + lane_id();
    bool hit = false;
    if (e < n_ex) {
      const uint32_t b = ref_keys_hash(ex, e) & table_mask;
      int64_t steps = 0;
      for (int32_t p = buckets[b] - 1; p >= 0 && steps <= limit; p = next[p] - 1, ++steps) {
        if (keys_eq(ex, e, side, p)) {
          hit = true;
          break;
        }
      }
    }
    const unsigned word = __ballot_sync(kFullMask, hit);
    if (lane_id() == 0) {
      if (words != nullptr) words[w] = word;
      c += (unsigned long long)__popc(word);
    }
  }
  // One count a warp, not one a word: the words' atomics would share one address.
  if (lane_id() == 0 && c != 0) atomicAdd(count, c);
}

}  // namespace

// The reference's chunk size of a left semi-join (FLAGS_semijoin_chunck_size,
// operations/LeftSemiJoin.cpp:12-14).
constexpr int64_t kRefSemiJoinChunk = 32768;

int coverage_compat(Ctx* ctx, const qfg_bindings* b, const qfg_literal* lit, int k,
                    const int32_t* const* ex_cols[2], const int64_t ex_n[2],
                    uint64_t* d_positive_bits, int64_t* num_covered) {
  Relation* rel = nullptr;
  QFG_TRY(find_relation(ctx, lit->relation_id, &rel));
  KeyCols rk, bk;
  rk.nk = bk.nk = 0;
  for (int a = 0; a < lit->num_args; ++a) {
    if (lit->vars[a] < 0) continue;
    rk.c[rk.nk++] = rel->columns[a];
    bk.c[bk.nk++] = b->columns[lit->vars[a]];
  }
  const int64_t P = b->num_positive, N = b->num_negative, nrel = rel->num_tuples;
  const int64_t side_start[2] = {0, P}, side_rows[2] = {P, N};
  num_covered[0] = num_covered[1] = 0;
  if (d_positive_bits != nullptr && ex_n[0] > 0)
    QFG_CUDA(ctx, cudaMemsetAsync(d_positive_bits, 0, sizeof(uint64_t) * (size_t)((ex_n[0] + 63) / 64),
                                  ctx->stream));
  // The relation's key set over the bound arguments.
  const uint32_t rmask = table_mask(std::max<int64_t>(nrel, 1));
  const int64_t nside_max = std::max(P, N);
  const size_t words_side = (size_t)((nside_max + 63) / 64) * 2;
  const int32_t nbt_max = (int32_t)std::max<int64_t>(nside_max, 1);
  uint32_t nb_max = 1;
  while (nb_max < (uint32_t)nbt_max) nb_max <<= 1;
  const size_t need = sizeof(int32_t) * ((size_t)rmask + 1) + sizeof(uint32_t) * words_side +
                      sizeof(int32_t) * ((size_t)nb_max + (size_t)nbt_max) + 64;
  QFG_TRY(ctx->scratch[kScrTmpB].reserve(ctx, need));
  int32_t* owner = ctx->scratch[kScrTmpB].as<int32_t>();
  uint32_t* member = reinterpret_cast<uint32_t*>(owner + rmask + 1);
  int32_t* buckets = reinterpret_cast<int32_t*>(member + words_side);
  int32_t* nxt = buckets + nb_max;
  QFG_TRY(ctx->scratch[kScrTmpC].reserve(ctx, 2 * sizeof(unsigned long long)));
  unsigned long long* cnt = ctx->scratch[kScrTmpC].as<unsigned long long>();
  QFG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), ctx->stream));
  QFG_CUDA(ctx, cudaMemsetAsync(owner, 0xff, sizeof(int32_t) * ((size_t)rmask + 1), ctx->stream));
  if (nrel > 0) {
    launch_keyset_insert(rows_grid(ctx, nrel), ctx->stream, rk, nrel, owner, rmask, nullptr);
    QFG_LAUNCHED(ctx);
  }
  for (int s = 0; s < 2; ++s) {
    const int64_t rows = side_rows[s];
    // The reference crashes on an empty label side; that side covers nothing here.
    if (rows == 0 || ex_n[s] == 0) continue;
    KeyCols probe = bk, target;
    target.nk = k;
    for (int q = 0; q < bk.nk; ++q) probe.c[q] = bk.c[q] + side_start[s];
    for (int q = 0; q < k; ++q) target.c[q] = b->columns[q] + side_start[s];
    QFG_CUDA(ctx, cudaMemsetAsync(member, 0, sizeof(uint32_t) * words_side, ctx->stream));
    asj_member_bits_kernel<<<rows_grid(ctx, rows), 256, 0, ctx->stream>>>(rk, owner, rmask, probe, rows,
                                                                         member);
    QFG_LAUNCHED(ctx);
    // SelectAndCreateSemiJoin (operations/SemiJoinFactory.cpp:45-82): a
    // right semi-join (one chunk) when the side is smaller than the
    // relation, else a left semi-join in 32768-row chunks.  The positive
    // side is a view of the binding set's consecutive columns, so reads
    // past its end land on the negative rows; past the negative side's end
    // they compare unequal.
    const int64_t chunk = rows < nrel ? 0 : kRefSemiJoinChunk;
    const int64_t readable = s == 0 ? P + N : N;
    uint32_t tmask = 0;
    QFG_TRY(after_semijoin_table(ctx, target.c, k, rows, readable,
                                 reinterpret_cast<const uint64_t*>(member), chunk, (int32_t)rows,
                                 buckets, nxt, &tmask));
    KeyCols ex;
    ex.nk = k;
    for (int q = 0; q < k; ++q) ex.c[q] = ex_cols[s][q];
    uint32_t* out_words = s == 0 ? reinterpret_cast<uint32_t*>(d_positive_bits) : nullptr;
    asj_probe_kernel<<<rows_grid(ctx, ex_n[s]), 256, 0, ctx->stream>>>(
        buckets, nxt, tmask, target, ex, ex_n[s], rows + 1, out_words, cnt + s);
    QFG_LAUNCHED(ctx);
  }
  unsigned long long host[2] = {0, 0};
  QFG_CUDA(ctx, cudaMemcpyAsync(host, cnt, sizeof(host), cudaMemcpyDeviceToHost, ctx->stream));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  num_covered[0] = (int64_t)host[0];
  num_covered[1] = (int64_t)host[1];
  return QFG_OK;
}

}  // namespace qfg

using namespace qfg;

extern "C" int qfg_build_hash_table_after_semijoin(qfg_ctx* c, const int32_t* const* d_keys,
                                                   int32_t num_keys, int64_t num_rows,
                                                   const uint64_t* d_bits, int64_t chunk_rows,
                                                   int32_t num_build_tuples, int32_t* d_buckets,
                                                   int32_t* d_next, uint32_t* mask_out) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_rows < 0 || num_rows > INT32_MAX || num_build_tuples < 1 || d_buckets == nullptr ||
      d_next == nullptr || mask_out == nullptr || (num_rows > 0 && d_bits == nullptr))
    return set_error(ctx, QFG_ERR_INVALID, "qfg_build_hash_table_after_semijoin: invalid arguments");
  QFG_TRY(after_semijoin_table(ctx, d_keys, num_keys, num_rows, num_rows, d_bits, chunk_rows,
                               num_build_tuples, d_buckets, d_next, mask_out));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return QFG_OK;
}
