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
// item, loads that binding partition into shared memory (a producer warp
// feeding TMA bulk copies), builds a shared-memory table of its distinct
// join keys (atomicCAS on slot owners) with per-label row counts and per-key
// row lists, and then streams, for every literal of the group, the relation
// key tuples of the same partition range through it.  Counts are reduced
// with warp shuffles into per-CTA int64 accumulators and flushed to global
// memory once per CTA.
#include <algorithm>
#include <cstring>
#include <set>
#include <unordered_map>

#include "bulk.cuh"
#include "eval_common.cuh"

namespace qfg {

namespace {

constexpr int kTile = 1280;            // binding rows per shared-memory tile
constexpr int kTargetRows = 1024;      // partition bits keep the mean partition below this
constexpr int kSlots = 2048;           // key-table slots (power of two > kTile)
constexpr int kEvalThreads = 288;     // evaluation block: eight consumer warps and one producer warp
constexpr int kConsumers = kEvalThreads - 32;
constexpr int kGroupCols = QFG_MAX_ARITY;  // join column + up to 7 atom columns
constexpr int kMaxLitsPerLaunch = 512;
constexpr int kChunk = 2 * kConsumers;       // relation entries per work unit: two per consumer
constexpr int kUnitEntries = 8 * kChunk;     // relation entries per evaluation unit (one key table)
constexpr int kMaxGroupLits = 256;  // literals of one group (one thread each in a per-item prefix)
constexpr int kPartThreads = 1024;
constexpr int kDefaultCoarseBits = 7;  // pass 1 fan-out: 2 << 7 = 256 bins (hash prefix, label)
constexpr int kMaxCoarseBits = 8;      // at most 512 pass-1 bins
constexpr int kMaxSubBits = 9;         // pass 2 fan-out: up to 512 sub-bins
constexpr int kMaxSinglePassBits = 8;  // one pass up to 2 << 8 = 512 bins
constexpr int kMaxPartitionBits = 16;
static_assert(kMaxPartitionBits <= kRelPartitionBits, "relation bins must refine binding bins");
static_assert(kMaxPartitionBits <= kMaxCoarseBits + kMaxSubBits, "two passes reach every bit count");
static_assert(kSlots > kTile, "slot table shape");

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

// Exclusive scan of one value per thread (blockDim.x <= 1024); every thread
// must call it.  *total receives the sum.
__device__ __forceinline__ uint32_t block_scan_excl(uint32_t v, uint32_t* s_warp, uint32_t* total) {
  const int lane = lane_id(), warp = warp_id();
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFullMask, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    const uint32_t t = lane < nw ? s_warp[lane] : 0u;
    uint32_t s = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFullMask, s, o);
      if (lane >= o) s += y;
    }
    s_warp[lane] = s - t;
    if (lane == 31) *total = s;
  }
  __syncthreads();
  const uint32_t r = x - v + s_warp[warp];
  __syncthreads();
  return r;
}

// ----------------------------------------------------------------------------
// Binding-set partitioning per group.
//
// Partition p of a group holds the binding rows whose join key has
// top_bits(mix32(key), bits) == p, positives and negatives in two separate
// segments.  A fan-out of 2^15 partitions is far too wide for coalesced
// stores, so the scatter runs in two passes of modest fan-out: pass 1 sends
// rows to (top cbits bits, label) coarse bins, pass 2 splits every coarse
// bin, inside its own range, into its 2^(bits - cbits) partitions.  Both
// passes stage rounds of rows in shared memory, counting-sort them by
// destination bin there and write each bin's run with consecutive threads on
// consecutive addresses.  A histogram pass counts the coarse bins per CTA
// (one atomicAdd per bin and CTA gives the CTA its cursor); pass 2 counts its
// own sub-bins, so no global fine histogram exists.  With bits <= 8 a single
// pass writes the partitions directly.

// One literal group's partition job.  Every partition kernel takes the
// array of all groups' jobs and serves group blockIdx.y, so one launch of
// each kernel covers the whole step (the groups' scratch is separate).
struct BPartArgs {
  const int32_t* cols[kGroupCols];  // cols[0] = join column
  int ncols;
  int64_t n, npos;
  int bits;                 // partition bits
  int cbits;                // pass-1 bits (== bits: single pass)
  int two_pass;
  int vec;                  // every source column 16-byte aligned
  uint32_t* p1_tot;         // 2 << cbits bin totals (zeroed)
  uint32_t* p1_base;        // gridDim.x * (2 << cbits) per-CTA bases
  uint32_t* p1_pad;         // (2 << cbits) + 1 padded bin starts (two passes)
  uint32_t* p1_unp;         // (2 << cbits) + 1 bin starts (one pass: the segment starts)
  uint32_t* chunk_start;    // (2 << cbits) + 1 first pass-2 chunk of every bin
  uint32_t* chunk_bin;      // coarse bin of every pass-2 chunk
  uint32_t* h2;             // pass-2 chunk sub-bin counts, then cursors
  int32_t* tmp;             // pass-1 output (two passes), column stride tmp_stride
  int64_t tmp_stride;
  int32_t* out;             // partitioned columns, column stride out_stride
  int64_t out_stride;
  uint32_t* fstart;         // (2 << bits) + 1 segment starts
  // Rows whose top cbits hash bits fall outside [keep_lo, keep_hi] belong to
  // other shards' partitions and are dropped in pass 1 (QFG_OPT_SHARD_*).
  uint32_t keep_lo, keep_hi;
};

// Rows [r0, r1) of this CTA; r0 is a multiple of 4 so that 16-byte loads
// stay aligned when the column base pointers are.
__device__ __forceinline__ void cta_range4(int64_t n, int64_t* r0, int64_t* r1) {
  int64_t per = (n + gridDim.x - 1) / gridDim.x;
  per = (per + 3) & ~int64_t(3);
  *r0 = min(n, (int64_t)blockIdx.x * per);
  *r1 = min(n, *r0 + per);
}

__device__ __forceinline__ uint32_t top_bits(int32_t key, int bits) {
  return mix32((uint32_t)key) >> (32 - bits);
}

__device__ __forceinline__ int lane_of(const int4& v, int k) {
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

constexpr int kHistCopies = 8;  // histogram copies of a CTA (warp w counts into copy w mod 8)

template <bool kVec>
__device__ __forceinline__ void bpart_hist_body(const BPartArgs& a, uint32_t (*hc)[2 << kMaxCoarseBits]) {
  const int np1 = 2 << a.cbits;
  for (int i = threadIdx.x; i < kHistCopies * np1; i += blockDim.x) hc[i / np1][i % np1] = 0;
  __syncthreads();
  uint32_t* p1 = hc[warp_id() % kHistCopies];
  int64_t r0, r1;
  cta_range4(a.n, &r0, &r1);
  const int32_t* __restrict__ key = a.cols[0];
  auto count = [&](int32_t k, int64_t r) {
    const uint32_t t = top_bits(k, a.cbits);
    if (t >= a.keep_lo && t <= a.keep_hi) atomicAdd(&p1[(t << 1) | (r >= a.npos ? 1u : 0u)], 1u);
  };
  int64_t rs = r0;
  if (kVec) {
    const int64_t nv = (r1 - r0) >> 2;
    const int4* __restrict__ kv = reinterpret_cast<const int4*>(key + r0);
    const int64_t step = blockDim.x;
    int64_t v = threadIdx.x;
    for (; v + 3 * step < nv; v += 4 * step) {
      int4 kk[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) kk[u] = __ldg(kv + v + u * step);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
#pragma unroll
        for (int k = 0; k < 4; ++k) count(lane_of(kk[u], k), r0 + 4 * (v + u * step) + k);
      }
    }
    for (; v + step < nv; v += 2 * step) {
      const int4 k0 = __ldg(kv + v), k1 = __ldg(kv + v + step);
#pragma unroll
      for (int k = 0; k < 4; ++k) count(lane_of(k0, k), r0 + 4 * v + k);
#pragma unroll
      for (int k = 0; k < 4; ++k) count(lane_of(k1, k), r0 + 4 * (v + step) + k);
    }
    if (v < nv) {
      const int4 k0 = __ldg(kv + v);
#pragma unroll
      for (int k = 0; k < 4; ++k) count(lane_of(k0, k), r0 + 4 * v + k);
    }
    rs = r0 + 4 * nv;
  }
  for (int64_t r = rs + threadIdx.x; r < r1; r += blockDim.x) count(key[r], r);
  __syncthreads();
  for (int i = threadIdx.x; i < np1; i += blockDim.x) {
    uint32_t c = 0;
#pragma unroll
    for (int h = 0; h < kHistCopies; ++h) c += hc[h][i];
    a.p1_base[(int64_t)blockIdx.x * np1 + i] = c ? atomicAdd(&a.p1_tot[i], c) : 0u;
  }
}

__global__ void __launch_bounds__(kPartThreads, 1) bpart_hist_kernel(const BPartArgs* __restrict__ A) {
  __shared__ uint32_t hc[kHistCopies][2 << kMaxCoarseBits];
  const BPartArgs& a = A[blockIdx.y];
  if (a.vec)
    bpart_hist_body<true>(a, hc);
  else
    bpart_hist_body<false>(a, hc);
}

// Round processing.  A round is up to kPassRows consecutive rows of one
// label.  Its join column is counting-sorted by destination bin in shared
// memory: each thread ranks 16 rows with shared atomics on the bin counters
// (ranks kept in registers), one block scan gives the bins' starts and their
// output positions, and the permutation records (row, bin) at each sorted
// position; every thread then keeps the output position and the source row
// of its 16 sorted positions in registers.  The carried columns stream
// through two shared-memory buffers one at a time: while column q of the
// round is written in sorted order (consecutive threads on consecutive
// addresses of a bin's run), column q + 1, or the next round's join column,
// arrives by cp.async (16-byte copies where the source is aligned).  Sorting
// once per round and holding one column at a time lets a round span 16K
// rows in 200 KB of shared memory whatever the column count, so each bin's
// run of a column averages 512 bytes at 128 bins.
constexpr int kPassThreads = 1024;
constexpr int kPassRows = 16384;                              // rows per round
constexpr int kPassRowsPerThread = kPassRows / kPassThreads;  // 16
constexpr int kPassPieces = kPassRows / (4 * kPassThreads);   // 4-row copy pieces per thread
static_assert(kPassRows <= 65536, "a round's row index packs into 16 bits");
static_assert((2 << kMaxCoarseBits) < kPassThreads && (1 << kMaxSubBits) < kPassThreads,
              "one thread per bin (and the drop bin) in the round scan");

// Bin arrays hold nbins + 1 entries: bin nbins collects the rows a shard
// drops; it sorts last, so a round writes only its first sorted positions.
struct PassSmem {
  int32_t* buf0;      // kPassRows: one column of a round
  int32_t* buf1;      // kPassRows: the column after it
  uint32_t* perm;     // kPassRows: row | bin << 16 at each sorted position
  uint32_t* lcount;   // nbins + 1
  uint32_t* lstart;   // nbins + 1
  uint32_t* gpos;     // nbins + 1: output position of sorted position 0 of bin b
  uint32_t* cursor;   // nbins + 1: output cursor of each bin (pass 1)
};

__device__ __forceinline__ PassSmem carve_pass(unsigned char* smem, int nbins) {
  PassSmem S;
  S.buf0 = reinterpret_cast<int32_t*>(smem);
  S.buf1 = S.buf0 + kPassRows;
  S.perm = reinterpret_cast<uint32_t*>(S.buf1 + kPassRows);
  S.lcount = S.perm + kPassRows;
  S.lstart = S.lcount + nbins + 1;
  S.gpos = S.lstart + nbins + 1;
  S.cursor = S.gpos + nbins + 1;
  return S;
}

size_t pass_smem_bytes(int nbins) {
  return sizeof(uint32_t) * (3 * (size_t)kPassRows + 4 * ((size_t)nbins + 1));
}

__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Starts the copies of rows [rr, rr + nt) of one column into dst: the
// thread copies the 4-row pieces t, t + T, t + 2T and t + 3T, each with one
// 16-byte copy when `vec` (the source piece is 16-byte aligned) and the
// piece is whole.
__device__ __forceinline__ void issue_column(const int32_t* __restrict__ src, uint32_t rr, int nt,
                                             int32_t* dst, bool vec) {
#pragma unroll
  for (int m = 0; m < kPassPieces; ++m) {
    const int i0 = 4 * ((int)threadIdx.x + m * kPassThreads);
    if (i0 < nt) {
      if (vec && i0 + 4 <= nt) {
        cp_async16(dst + i0, src + rr + i0);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (i0 + j < nt) cp_async4(dst + i0 + j, src + rr + i0 + j);
      }
    }
  }
  cp_async_commit();
}

// End of the round starting at rr: rounds are anchored at r0 and never
// straddle `split`.
__device__ __forceinline__ uint32_t round_end(uint32_t r0, uint32_t rr, uint32_t r1, uint32_t split,
                                              uint32_t R) {
  const uint32_t e = umin(r0 + ((rr - r0) / R + 1) * R, r1);
  return (rr < split && split < e) ? split : e;
}

// Rows [rr, re) of a round; `chunk` is its pass-2 chunk.
struct PassRound {
  uint32_t rr, re, chunk;
  bool valid;
};

// Streams the CTA's rounds, starting at `cur`.  next_of(round) gives the
// round after it (invalid at the end); it runs at the start of a round, so
// its global reads overlap the sort.  bin_of(key, row) gives a row's bin.
// A bin's output position in a round comes from the CTA's cursors (pass 1:
// h2 == nullptr) or from h2[chunk * nbins + bin] (pass 2, one round per
// chunk).  src and dst are the columns (shared-memory arrays of pointers).
template <typename NextFn, typename BinFn>
__device__ __forceinline__ void stream_pass(const PassSmem& S, const int32_t* const* src,
                                            int32_t* const* dst, int ncols, int nbins, bool aligned,
                                            PassRound cur, const uint32_t* __restrict__ h2,
                                            uint32_t* s_warp, uint32_t* s_total, NextFn next_of,
                                            BinFn bin_of) {
  constexpr int T = kPassThreads;
  constexpr int J = kPassRowsPerThread;
  const int t = threadIdx.x;
  if (!cur.valid) return;
  issue_column(src[0], cur.rr, (int)(cur.re - cur.rr), S.buf0, aligned && (cur.rr & 3u) == 0u);
  bool slot = false;
  uint32_t oidx[J];       // output position of sorted positions t + j T
  uint32_t rowp[J / 2];   // their rows in the round, two 16-bit rows a word
  while (true) {
    const PassRound nxt = next_of(cur);
    const int nt = (int)(cur.re - cur.rr);
    const bool vec = aligned && (cur.rr & 3u) == 0u;
    for (int q = 0; q < ncols; ++q) {
      cp_async_wait_all();
      __syncthreads();
      const int32_t* const cbuf = slot ? S.buf1 : S.buf0;
      int32_t* const obuf = slot ? S.buf0 : S.buf1;
      if (q + 1 < ncols)
        issue_column(src[q + 1], cur.rr, nt, obuf, vec);
      else if (nxt.valid)
        issue_column(src[0], nxt.rr, (int)(nxt.re - nxt.rr), obuf, aligned && (nxt.rr & 3u) == 0u);
      if (q == 0) {
        uint32_t hb = 0;
        if (h2 != nullptr && t < nbins) hb = __ldg(h2 + (size_t)cur.chunk * (size_t)nbins + t);
        uint32_t pk[J];   // rank | bin << 16
#pragma unroll
        for (int j = 0; j < J; ++j) {
          const int i = t + j * T;
          pk[j] = 0xffffffffu;
          if (i < nt) {
            const uint32_t b = bin_of(cbuf[i], cur.rr + (uint32_t)i);
            pk[j] = atomicAdd(&S.lcount[b], 1u) | (b << 16);
          }
        }
        __syncthreads();
        const uint32_t c = t <= nbins ? S.lcount[t] : 0u;
        const uint32_t ex = block_scan_excl(c, s_warp, s_total);
        if (t <= nbins) {
          S.lstart[t] = ex;
          if (t == nbins) {
            S.gpos[t] = 0u;  // dropped rows: never written
          } else if (h2 != nullptr) {
            S.gpos[t] = hb - ex;
          } else {
            S.gpos[t] = S.cursor[t] - ex;
            S.cursor[t] += c;
          }
          S.lcount[t] = 0u;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < J; ++j) {
          if (pk[j] != 0xffffffffu) {
            const uint32_t b = pk[j] >> 16;
            S.perm[S.lstart[b] + (pk[j] & 0xffffu)] = (uint32_t)(t + j * T) | (b << 16);
          }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < J; ++j) {
          const int kk = t + j * T;
          uint32_t w = 0;
          if (kk < nt) w = S.perm[kk];
          oidx[j] = S.gpos[w >> 16] + (uint32_t)kk;
          if (j & 1)
            rowp[j >> 1] |= (w & 0xffffu) << 16;
          else
            rowp[j >> 1] = w & 0xffffu;
        }
      }
      int32_t* __restrict__ out = dst[q];
      const int nkeep = (int)S.lstart[nbins];  // sorted positions before the drop bin
#pragma unroll
      for (int j = 0; j < J; ++j) {
        const int kk = t + j * T;
        if (kk < nkeep) out[oidx[j]] = cbuf[(rowp[j >> 1] >> (16 * (j & 1))) & 0xffffu];
      }
      slot = !slot;
    }
    if (!nxt.valid) break;
    cur = nxt;
  }
}

// Pass 1: the CTA's chunk of the original columns into pass-1 bins at
// p1_start[bin] + this CTA's base (out: column stride out_stride).
__global__ void __launch_bounds__(kPassThreads, 1) bpart_pass1_kernel(const BPartArgs* __restrict__ A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const BPartArgs& a = A[blockIdx.y];
  // Two passes: into the padded coarse bins of the scratch; one pass: into
  // the partitions themselves.
  const uint32_t* __restrict__ p1_start = a.two_pass ? a.p1_pad : a.p1_unp;
  int32_t* __restrict__ out = a.two_pass ? a.tmp : a.out;
  const int64_t out_stride = a.two_pass ? a.tmp_stride : a.out_stride;
  const int aligned = a.vec;
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  __shared__ const int32_t* s_src[kGroupCols];
  __shared__ int32_t* s_dst[kGroupCols];
  const int np1 = 2 << a.cbits;
  const PassSmem S = carve_pass(smem, np1);
  for (int i = threadIdx.x; i <= np1; i += blockDim.x) {
    S.cursor[i] = i < np1 ? p1_start[i] + a.p1_base[(int64_t)blockIdx.x * np1 + i] : 0u;
    S.lcount[i] = 0u;
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < kGroupCols; ++q) {
      if (q < a.ncols) {
        s_src[q] = a.cols[q];
        s_dst[q] = out + (int64_t)q * out_stride;
      }
    }
  }
  __syncthreads();
  int64_t r0l, r1l;
  cta_range4(a.n, &r0l, &r1l);
  const uint32_t r0 = (uint32_t)r0l, r1 = (uint32_t)r1l;
  const int cbits = a.cbits;
  const uint32_t npos = (uint32_t)a.npos;
  const uint32_t keep_lo = a.keep_lo, keep_hi = a.keep_hi;
  PassRound first;
  first.rr = r0;
  first.re = r0 < r1 ? round_end(r0, r0, r1, npos, kPassRows) : r0;
  first.chunk = 0;
  first.valid = r0 < r1;
  stream_pass(
      S, s_src, s_dst, a.ncols, np1, aligned != 0, first, nullptr, s_warp, &s_total,
      [=](const PassRound& r) {
        PassRound n;
        n.rr = r.re;
        n.valid = r.re < r1;
        n.re = n.valid ? round_end(r0, r.re, r1, npos, kPassRows) : r.re;
        n.chunk = 0;
        return n;
      },
      [=](int32_t key, uint32_t r) {
        const uint32_t tb = top_bits(key, cbits);
        return (tb >= keep_lo && tb <= keep_hi) ? (tb << 1) | (r >= npos ? 1u : 0u) : (uint32_t)np1;
      });
}

// Rows of a pass-2 work chunk: coarse bins (up to 9x apart in size, since
// negatives outnumber positives) are cut into chunks so the persistent pass
// 2 stays balanced.
constexpr uint32_t kP2Chunk = 16384;
static_assert(kP2Chunk <= (uint32_t)kPassRows, "a pass-2 chunk is one round");

// Bin starts of pass 1, twice: padded to multiples of 4 rows (where pass 1
// writes and pass 2 reads, so that pass 2's copies are 16-byte aligned) and
// unpadded (where pass 2 writes); the first pass-2 chunk of every bin
// (chunk_start[nbins] = number of chunks) and the bin of every chunk.  One
// block, nbins <= blockDim.x.
__global__ void pad_scan_kernel(const BPartArgs* __restrict__ A) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  const BPartArgs& a = A[blockIdx.x];
  const uint32_t* __restrict__ tot = a.p1_tot;
  const int nbins = 2 << a.cbits;
  uint32_t* __restrict__ pad = a.p1_pad;
  uint32_t* __restrict__ unp = a.p1_unp;
  uint32_t* __restrict__ chunk_start = a.chunk_start;
  uint32_t* __restrict__ chunk_bin = a.chunk_bin;
  const bool two = a.two_pass != 0;
  const uint32_t c = (int)threadIdx.x < nbins ? tot[threadIdx.x] : 0u;
  const uint32_t ex = block_scan_excl(c, s_warp, &s_total);
  const uint32_t total = s_total;
  const uint32_t exp = block_scan_excl((c + 3u) & ~3u, s_warp, &s_total);
  const uint32_t total_pad = s_total;
  const uint32_t exc = block_scan_excl((c + kP2Chunk - 1u) / kP2Chunk, s_warp, &s_total);
  if ((int)threadIdx.x < nbins) {
    unp[threadIdx.x] = ex;
    if (two) {
      pad[threadIdx.x] = exp;
      chunk_start[threadIdx.x] = exc;
      const uint32_t nch = (c + kP2Chunk - 1u) / kP2Chunk;
      for (uint32_t j = 0; j < nch; ++j) chunk_bin[exc + j] = threadIdx.x;
    }
  }
  if (threadIdx.x == 0) {
    unp[nbins] = total;
    if (two) {
      pad[nbins] = total_pad;
      chunk_start[nbins] = s_total;
    }
  }
}

// Pass-2 chunk c: its coarse bin (from the chunk -> bin table) and row
// range in the padded layout.
struct P2Chunk {
  int bin;
  uint32_t r0, r1;
};
__device__ __forceinline__ P2Chunk p2_chunk(const uint32_t* __restrict__ chunk_bin,
                                            const uint32_t* __restrict__ chunk_start,
                                            const uint32_t* __restrict__ pad,
                                            const uint32_t* __restrict__ unp, uint32_t c) {
  const int b = (int)chunk_bin[c];
  const uint32_t k = c - chunk_start[b];
  const uint32_t cnt = unp[b + 1] - unp[b];
  P2Chunk r;
  r.bin = b;
  r.r0 = pad[b] + k * kP2Chunk;
  r.r1 = pad[b] + umin(cnt, (k + 1) * kP2Chunk);
  return r;
}

// Sub-bin counts of every pass-2 chunk: h2[c * nsub + sub].
__global__ void __launch_bounds__(512) bpart_p2hist_kernel(const BPartArgs* __restrict__ A) {
  __shared__ uint32_t cntr[1 << kMaxSubBits];
  const BPartArgs& a = A[blockIdx.y];
  if (!a.two_pass) return;
  const uint32_t* __restrict__ pad = a.p1_pad;
  const uint32_t* __restrict__ unp = a.p1_unp;
  const uint32_t* __restrict__ chunk_start = a.chunk_start;
  const uint32_t* __restrict__ chunk_bin = a.chunk_bin;
  const int32_t* __restrict__ keys = a.tmp;  // the join column of the pass-1 output
  uint32_t* __restrict__ h2 = a.h2;
  const int np1 = 2 << a.cbits;
  const int bits = a.bits;
  const int nsub = 1 << (a.bits - a.cbits);
  const uint32_t mask = (uint32_t)(nsub - 1);
  const uint32_t nch = chunk_start[np1];
  for (uint32_t c = blockIdx.x; c < nch; c += gridDim.x) {
    const P2Chunk ch = p2_chunk(chunk_bin, chunk_start, pad, unp, c);
    for (int i = threadIdx.x; i < nsub; i += blockDim.x) cntr[i] = 0u;
    __syncthreads();
    uint32_t r = ch.r0 + threadIdx.x;
    for (; r + 7 * blockDim.x < ch.r1; r += 8 * blockDim.x) {
      int32_t k[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) k[j] = __ldg(keys + r + j * blockDim.x);
#pragma unroll
      for (int j = 0; j < 8; ++j) atomicAdd(&cntr[top_bits(k[j], bits) & mask], 1u);
    }
    for (; r < ch.r1; r += blockDim.x) atomicAdd(&cntr[top_bits(__ldg(keys + r), bits) & mask], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < nsub; i += blockDim.x) h2[(int64_t)c * nsub + i] = cntr[i];
    __syncthreads();
  }
}

// Per coarse bin b (one block, nsub <= blockDim.x): turns its chunks' sub-bin
// counts into output cursors (sub-bin start + the counts of the bin's earlier
// chunks) and records where each sub-bin starts: fine_start[(b << sbits) +
// sub] (the last block also writes the end, n).
__global__ void __launch_bounds__(512) bpart_p2scan_kernel(const BPartArgs* __restrict__ A) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  const BPartArgs& a = A[blockIdx.y];
  const int np1 = 2 << a.cbits;
  if (!a.two_pass || (int)blockIdx.x >= np1) return;  // block-uniform
  const uint32_t* __restrict__ unp = a.p1_unp;
  const uint32_t* __restrict__ chunk_start = a.chunk_start;
  uint32_t* __restrict__ h2 = a.h2;
  uint32_t* __restrict__ fine_start = a.fstart;
  const int sbits = a.bits - a.cbits;
  const int nsub = 1 << sbits;
  const int b = blockIdx.x;
  const uint32_t c0 = chunk_start[b], c1 = chunk_start[b + 1];
  const int sub = threadIdx.x;
  uint32_t run = 0;
  if (sub < nsub) {
    for (uint32_t c = c0; c < c1; ++c) {
      const uint32_t v = h2[(int64_t)c * nsub + sub];
      h2[(int64_t)c * nsub + sub] = run;
      run += v;
    }
  }
  const uint32_t ex = block_scan_excl(sub < nsub ? run : 0u, s_warp, &s_total);
  if (sub < nsub) {
    const uint32_t base = unp[b] + ex;
    fine_start[((int64_t)b << sbits) + sub] = base;
    for (uint32_t c = c0; c < c1; ++c) h2[(int64_t)c * nsub + sub] += base;
  }
  if (b == np1 - 1 && threadIdx.x == 0) fine_start[(int64_t)np1 << sbits] = unp[np1];
}

// Pass 2, persistent over chunks: each chunk of a coarse bin, read from the
// padded layout, is split into sub-bins 0 .. 2^sbits - 1 at its cursors.
__global__ void __launch_bounds__(kPassThreads, 1)
bpart_pass2_kernel(const BPartArgs* __restrict__ A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const BPartArgs& a = A[blockIdx.y];
  if (!a.two_pass) return;
  const uint32_t* __restrict__ pad = a.p1_pad;
  const uint32_t* __restrict__ unp = a.p1_unp;
  const uint32_t* __restrict__ chunk_start = a.chunk_start;
  const uint32_t* __restrict__ chunk_bin = a.chunk_bin;
  const uint32_t* __restrict__ h2 = a.h2;
  const int32_t* __restrict__ in = a.tmp;
  const int64_t in_stride = a.tmp_stride;
  int32_t* __restrict__ out = a.out;
  const int64_t out_stride = a.out_stride;
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  __shared__ const int32_t* s_src[kGroupCols];
  __shared__ int32_t* s_dst[kGroupCols];
  const int np1 = 2 << a.cbits;
  const int nsub = 1 << (a.bits - a.cbits);
  const PassSmem S = carve_pass(smem, nsub);
  const uint32_t mask = (uint32_t)(nsub - 1);
  const int bits = a.bits;
  for (int i = threadIdx.x; i <= nsub; i += blockDim.x) S.lcount[i] = 0u;
  if (threadIdx.x == 0) {
    for (int q = 0; q < a.ncols; ++q) {
      s_src[q] = in + (int64_t)q * in_stride;
      s_dst[q] = out + (int64_t)q * out_stride;
    }
  }
  __syncthreads();
  const uint32_t nch = chunk_start[np1];
  auto round_of = [=](uint32_t c) {
    PassRound r;
    r.chunk = c;
    r.valid = c < nch;
    r.rr = r.re = 0;
    if (r.valid) {
      const P2Chunk ch = p2_chunk(chunk_bin, chunk_start, pad, unp, c);
      r.rr = ch.r0;
      r.re = ch.r1;
    }
    return r;
  };
  const uint32_t stride = gridDim.x;
  stream_pass(
      S, s_src, s_dst, a.ncols, nsub, true, round_of(blockIdx.x), h2, s_warp, &s_total,
      [=](const PassRound& r) { return round_of(r.chunk + stride); },
      [=](int32_t key, uint32_t) { return top_bits(key, bits) & mask; });
}

// ----------------------------------------------------------------------------
// Persistent evaluation kernel.
//
// Work unit = a range of at most kChunk relation entries of one (group,
// partition) item; evaluation unit = up to kUnitEntries / kChunk consecutive
// units of one item.  Three launches per literal batch:
//   plan_units   lists the units: each item's segment bounds and the number
//                of relation entries its literals hold in the item's key
//                range; items without rows or entries are dropped, the
//                entries of an item are cut into units of kChunk (one gather
//                warp each) with a block of entry records apiece, and items
//                with more than kUnitEntries entries (hot join keys of skewed
//                relations) into several evaluation units, so no CTA is left
//                with a long tail;
//   gather       one warp per unit forms the item's literal-major entry
//                space and writes the unit's entry records (join key, up to
//                two further keys, multiplicity, literal and check columns)
//                into its block, so the evaluation loads them with one
//                coalesced round trip;
//   eval         a producer warp claims evaluation units, publishes each
//                record one unit ahead and feeds the tiles (the partition's
//                binding rows, one 16-byte aligned run per column and label)
//                by TMA bulk copies on full/empty mbarriers; eight consumer
//                warps load a unit's first entry records as soon as its
//                record is published, build a key table of the tile (one
//                32-bit atomicCAS per new key, whose count atomics also give
//                every row its rank within its key and label), give each key
//                a run of the row list by a warp-aggregated atomic and place
//                its rows there (positives first), then probe the table with
//                the unit's entries kChunk at a time and check each key's
//                rows against the entries' further keys; per-literal sums
//                are combined with a segmented warp scan into per-CTA int64
//                accumulators, flushed to global memory when the CTA retires.

struct GroupDesc {
  const int32_t* cols;      // ncols SoA partitioned columns, column stride n (a multiple of 4)
  int64_t n;
  const uint32_t* fstart;   // (2 << bits) + 1 segment starts
  int bits, sbits, ncols;
  int lit_begin, lit_end;
  int sig_begin, sig_end;   // streamed path: the group's key signatures
  int has_atoms;
  uint32_t p_lo;            // first partition of this context's shard
  int64_t item_begin;
};

// Streamed path: a key signature is the ascending list of group columns
// (besides the join column) that a literal's further bound arguments are
// compared with.  Literals with the same signature share one composite key
// (join key, the signature columns' values) in the entry table.
struct SigDesc {
  int32_t ncols;
  int32_t col[kGroupCols - 1];
};
static_assert(sizeof(SigDesc) == 32, "signature record");

struct LitDesc {
  const int32_t* keys;       // nk SoA columns of `stride` entries
  const int32_t* mult;
  const uint32_t* offsets;   // (1 << kRelPartitionBits) + 1
  int64_t stride;
  int nk;
  int out;                   // literal index in the caller's array
  int8_t atom_col[QFG_MAX_ARITY];  // key q >= 1 is compared with group column atom_col[q]
  int sig;                   // streamed path: signature (index into the launch's SigDesc array)
  int8_t spos[QFG_MAX_ARITY];  // key q >= 1: its position in the signature, -1: must equal key 0
};

struct WorkUnit {
  const int32_t* cols;       // the group's partitioned columns
  int64_t stride;            // their column stride (a multiple of 4 rows)
  uint32_t group, p;
  uint32_t ps, Pp, ns, Np;   // positive / negative segment of the partition
  uint32_t f0, ecnt;         // entries [f0, f0 + ecnt) of the item's literal-major space
  uint32_t eoff;             // first record of the unit's entry block (multiple of 4)
  uint32_t lit_begin;        // first literal of the group
  uint32_t flags;            // carried columns | has_atoms << 8
  uint32_t pad;
};
static_assert(sizeof(WorkUnit) == 64, "work unit record");

// Entry records, SoA over the launch's entry blocks.  meta packs the
// literal within its group (bits 0-7), the number of columns to check
// (bits 8-9; 3 = more than two, read the keys from the key table), "keys
// compared with the join column itself all equal the join key" (bit 10),
// and the group columns of the first two checks (bits 12-14, 16-18).  For
// an entry with more than two checks kA holds its key-table index.
struct EntryRecs {
  int32_t* k0;
  int32_t* kA;
  int32_t* kB;
  uint32_t* meta;
  int32_t* mult;
};

struct EvalArgs {
  const GroupDesc* groups;
  int num_groups;
  const LitDesc* lits;
  int num_lits;
  int max_cols;
  int64_t total_items;
  WorkUnit* units;
  WorkUnit* eunits;          // tiled path: evaluation units, up to kUnitEntries entries each
  uint32_t* unit_count;      // [units, entry records, evaluation units]
  uint32_t unit_cap;         // of units, and of evaluation units
  uint32_t entry_cap;
  EntryRecs rec;
  unsigned int* work_counter;
  unsigned long long* counts;
  int* error_flag;           // set when a bounded wait gave up
  int64_t wait_limit;        // iterations of a bounded wait
  int withhold_copies;       // tests: arm the tile barrier, issue no copy
  const SigDesc* sigs;       // streamed path: signatures of the launch's groups
  uint32_t piece;            // relation entries per work unit
  uint32_t row_chunk;        // streamed path: binding rows per work unit (0 = all)
  int records;               // tiled path: units reserve entry records
};

// Shared-memory stride of a tile column.  Each segment (positives,
// negatives) arrives as the 16-byte chunks of the aligned run of global rows
// that encloses it, so a segment's rows keep their global offset modulo
// 4 and the negatives' run starts on the next 16-byte boundary after the
// positives' run: at most 12 rows of padding per column.
constexpr int kTileStride = kTile + 16;

size_t eval_smem_bytes(int num_lits, int max_cols) {
  return sizeof(unsigned long long) * 4 * (size_t)num_lits + sizeof(uint32_t) * 2 * kSlots +
         sizeof(int32_t) * (size_t)max_cols * kTileStride + sizeof(uint16_t) * kSlots +
         sizeof(uint16_t) * 4 * kTile;
}

// Where one tile of a work unit lies: rows [t0, t0 + nt) of the unit's
// positives-then-negatives order, npos of them positive.  Global rows
// [gP, gP + npos) and [gN, gN + nt - npos) of every carried column; in shared
// memory a positive row i sits at shP + i and a negative row i at
// baseN + (i - npos).  bytesP / bytesN: the two aligned runs per column,
// landing at shared index 0 and aN.
struct TileGeo {
  uint32_t nt, npos, gP, gN, shP, aN, baseN, bytesP, bytesN;
};

__device__ __forceinline__ TileGeo tile_geo(const WorkUnit& U, uint32_t t0) {
  TileGeo g;
  const uint32_t total = U.Pp + U.Np;
  g.nt = umin((uint32_t)kTile, total - t0);
  g.npos = umin(g.nt, U.Pp > t0 ? U.Pp - t0 : 0u);
  const uint32_t cN = g.nt - g.npos;
  g.gP = U.ps + t0;
  g.gN = U.ns + (t0 > U.Pp ? t0 - U.Pp : 0u);
  g.shP = g.npos > 0u ? (g.gP & 3u) : 0u;
  g.bytesP = g.npos > 0u ? 4u * (((g.gP + g.npos + 3u) & ~3u) - (g.gP & ~3u)) : 0u;
  g.aN = g.npos > 0u ? ((g.shP + g.npos + 3u) & ~3u) : 0u;
  g.baseN = g.aN + (g.gN & 3u);
  g.bytesN = cN > 0u ? 4u * (((g.gN + cN + 3u) & ~3u) - (g.gN & ~3u)) : 0u;
  return g;
}

__global__ void __launch_bounds__(256) plan_units_kernel(EvalArgs a) {
  const int lane = lane_id();
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < a.total_items;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t item = base + threadIdx.x;
    uint32_t nch = 0, E = 0, espace = 0;
    WorkUnit u{};
    if (item < a.total_items) {
      int lo = 0, hi = a.num_groups - 1;  // largest g with item_begin <= item
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.groups[mid].item_begin <= item) lo = mid; else hi = mid - 1;
      }
      const GroupDesc& G = a.groups[lo];
      const uint32_t p = G.p_lo + (uint32_t)(item - G.item_begin);
      const int s = G.sbits;
      const uint32_t hc = p >> s, sub = p & ((1u << s) - 1u);
      const uint32_t ip = ((2u * hc) << s) + sub, in_ = ((2u * hc + 1u) << s) + sub;
      u.cols = G.cols;
      u.stride = G.n;
      u.lit_begin = (uint32_t)G.lit_begin;
      u.flags = (uint32_t)G.ncols | (G.has_atoms ? 0x100u : 0u);
      u.group = (uint32_t)lo;
      u.p = p;
      u.ps = G.fstart[ip];
      u.Pp = G.fstart[ip + 1] - u.ps;
      u.ns = G.fstart[in_];
      u.Np = G.fstart[in_ + 1] - u.ns;
      if (u.Pp + u.Np > 0) {
        const int rshift = kRelPartitionBits - G.bits;
        const uint32_t q0 = p << rshift, q1 = (p + 1) << rshift;
#pragma unroll 4
        for (int L = G.lit_begin; L < G.lit_end; ++L) {
          const uint32_t* off = a.lits[L].offsets;
          E += __ldg(off + q1) - __ldg(off + q0);
        }
        nch = (E + a.piece - 1) / a.piece;
        if (a.row_chunk > 0) nch *= 1u + (u.Pp + u.Np - 1u) / a.row_chunk;
        if (nch > 0 && a.records)
          espace = (nch - 1) * a.piece + ((E - (nch - 1) * a.piece + 3u) & ~3u);
      }
    }
    // Evaluation units (tiled path): runs of up to kUnitEntries / piece
    // consecutive units of the item, whose entry blocks are consecutive.
    const uint32_t per_eu = (uint32_t)kUnitEntries / a.piece;
    const uint32_t neu = a.eunits != nullptr ? (nch + per_eu - 1u) / per_eu : 0u;
    // Warp-aggregated reservation of unit slots, entry records and
    // evaluation units.
    uint32_t x = nch, y = espace, z = neu;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t xu = __shfl_up_sync(kFullMask, x, o), yu = __shfl_up_sync(kFullMask, y, o);
      const uint32_t zu = __shfl_up_sync(kFullMask, z, o);
      if (lane >= o) {
        x += xu;
        y += yu;
        z += zu;
      }
    }
    const uint32_t tu = __shfl_sync(kFullMask, x, 31), te = __shfl_sync(kFullMask, y, 31);
    const uint32_t tv = __shfl_sync(kFullMask, z, 31);
    uint32_t ub = 0, eb = 0, vb = 0;
    if (lane == 31 && tu > 0) {
      ub = atomicAdd(&a.unit_count[0], tu);
      eb = atomicAdd(&a.unit_count[1], te);
      if (tv > 0) vb = atomicAdd(&a.unit_count[2], tv);
    }
    ub = __shfl_sync(kFullMask, ub, 31) + x - nch;
    eb = __shfl_sync(kFullMask, eb, 31) + y - espace;
    vb = __shfl_sync(kFullMask, vb, 31) + z - neu;
    if (a.row_chunk > 0) {
      // Streamed path: (entry piece, row chunk) pairs; a unit's rows are
      // [pad, pad + ecnt2) of the item's positives-then-negatives order,
      // kept in eoff (first row) and pad (row count).
      const uint32_t rows = u.Pp + u.Np;
      const uint32_t nrc = rows == 0 ? 1u : 1u + (rows - 1u) / a.row_chunk;
      for (uint32_t k = 0; k < nch; ++k) {
        if (ub + k >= a.unit_cap) break;
        const uint32_t piece = k / nrc, rc = k % nrc;
        WorkUnit v = u;
        v.f0 = piece * a.piece;
        v.ecnt = umin(E - piece * a.piece, a.piece);
        v.eoff = rc * a.row_chunk;
        v.pad = umin(rows - rc * a.row_chunk, a.row_chunk);
        a.units[ub + k] = v;
      }
      continue;
    }
    for (uint32_t k = 0; k < nch; ++k) {
      if (ub + k >= a.unit_cap) break;  // never read: the evaluation stops at unit_cap
      u.f0 = k * a.piece;
      u.ecnt = umin(E - k * a.piece, a.piece);
      u.eoff = eb + k * a.piece;
      if ((uint64_t)u.eoff + ((u.ecnt + 3u) & ~3u) > a.entry_cap) {
        // Out of entry records (the capacity is an upper bound, so this does
        // not happen): an empty unit keeps the list well formed.
        u.ecnt = 0;
        u.Pp = u.Np = 0;
      }
      a.units[ub + k] = u;
    }
    for (uint32_t k = 0; k < neu; ++k) {
      if (vb + k >= a.unit_cap) break;  // never read: the evaluation stops at unit_cap
      WorkUnit v = u;
      v.f0 = k * (uint32_t)kUnitEntries;
      v.ecnt = umin(E - v.f0, (uint32_t)kUnitEntries);
      v.eoff = eb + v.f0;
      if ((uint64_t)v.eoff + ((v.ecnt + 3u) & ~3u) > a.entry_cap) {
        v.ecnt = 0;  // as above: never happens
        v.Pp = v.Np = 0;
      }
      a.eunits[vb + k] = v;
    }
  }
}

constexpr int kGatherWarps = 8;

// One warp per unit: the item's literal-major entry space (offsets pair per
// literal, warp scan), then the unit's entry records.
__global__ void __launch_bounds__(32 * kGatherWarps) gather_entries_kernel(EvalArgs a) {
  __shared__ uint32_t s_lstart[kGatherWarps][kMaxGroupLits + 1];
  __shared__ uint32_t s_le0[kGatherWarps][kMaxGroupLits];
  const int lane = lane_id(), w = warp_id();
  uint32_t* lstart = s_lstart[w];
  uint32_t* le0 = s_le0[w];
  const uint32_t nunits = umin(a.unit_count[0], a.unit_cap);
  for (uint32_t ui = blockIdx.x * kGatherWarps + w; ui < nunits; ui += gridDim.x * kGatherWarps) {
    const WorkUnit U = a.units[ui];
    if (U.eoff + U.ecnt > a.entry_cap) continue;
    const GroupDesc& G = a.groups[U.group];
    const int m = G.lit_end - G.lit_begin;
    const int rshift = kRelPartitionBits - G.bits;
    const uint32_t q0 = U.p << rshift, q1 = (U.p + 1) << rshift;
    uint32_t run = 0;
    for (int L0 = 0; L0 < m; L0 += 32) {
      const int L = L0 + lane;
      uint32_t c = 0;
      if (L < m) {
        const uint32_t* off = a.lits[G.lit_begin + L].offsets;
        const uint32_t e0 = __ldg(off + q0);
        c = __ldg(off + q1) - e0;
        le0[L] = e0;
      }
      uint32_t x = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFullMask, x, o);
        if (lane >= o) x += y;
      }
      if (L < m) lstart[L] = run + x - c;
      run += __shfl_sync(kFullMask, x, 31);
    }
    if (lane == 0) lstart[m] = run;
    __syncwarp();
    // Four entries a lane at a time, each step for all four together so
    // their round trips overlap: the literal (a branch-free binary search of
    // the literal starts), its descriptor, the key columns, the record.
    int top = 1;
    while (top * 2 <= m) top *= 2;
    for (uint32_t jb = 0; jb < U.ecnt; jb += 4 * 32) {
      uint32_t f[4], e[4];
      int lo[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        f[q] = U.f0 + jb + (uint32_t)(lane + 32 * q);
        lo[q] = 0;  // largest L with lstart[L] <= f
      }
      for (int step = top; step > 0; step >>= 1) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (lo[q] + step < m && lstart[lo[q] + step] <= f[q]) lo[q] += step;
      }
      const LitDesc* d[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        d[q] = a.lits + G.lit_begin + lo[q];
        e[q] = le0[lo[q]] + (f[q] - lstart[lo[q]]);
      }
      int32_t k[4][3];
      int nk[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const bool valid = jb + (uint32_t)(lane + 32 * q) < U.ecnt;
        nk[q] = valid ? d[q]->nk : 0;
        const int32_t* kp = d[q]->keys;
        const int64_t st = d[q]->stride;
        k[q][0] = nk[q] > 0 ? __ldg(kp + e[q]) : 0;
        k[q][1] = nk[q] > 1 ? __ldg(kp + st + e[q]) : 0;
        k[q][2] = nk[q] > 2 ? __ldg(kp + 2 * st + e[q]) : 0;
      }
      int32_t mlt[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) mlt[q] = nk[q] > 0 ? __ldg(d[q]->mult + e[q]) : 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (nk[q] == 0) continue;
        const LitDesc& dd = *d[q];
        const int32_t k0 = k[q][0];
        int32_t kA = 0, kB = 0;
        uint32_t nchk = 0, colA = 0, colB = 0, ok0 = 1;
        for (int c = 1; c < nk[q]; ++c) {
          const int ac = dd.atom_col[c];
          const int32_t kc = c == 1 ? k[q][1] : c == 2 ? k[q][2] : __ldg(dd.keys + c * dd.stride + e[q]);
          if (ac == 0) {
            ok0 &= kc == k0 ? 1u : 0u;
          } else {
            if (nchk == 0) { kA = kc; colA = (uint32_t)ac; }
            else if (nchk == 1) { kB = kc; colB = (uint32_t)ac; }
            ++nchk;
          }
        }
        if (nchk > 2) {
          nchk = 3;
          kA = (int32_t)e[q];
        }
        const uint32_t r = U.eoff + jb + (uint32_t)(lane + 32 * q);
        a.rec.k0[r] = k0;
        a.rec.kA[r] = kA;
        a.rec.kB[r] = kB;
        a.rec.mult[r] = mlt[q];
        a.rec.meta[r] = (uint32_t)lo[q] | (nchk << 8) | (ok0 << 10) | (colA << 12) | (colB << 16);
      }
    }
    __syncwarp();
  }
}

// Inclusive scan restricted to runs of equal `seg` across consecutive lanes.
__device__ __forceinline__ long long seg_scan(long long v, int seg) {
  const int lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(kFullMask, v, o);
    const int s = __shfl_up_sync(kFullMask, seg, o);
    if (lane >= o && s == seg) v += y;
  }
  return v;
}

// Per-CTA int64 accumulators updated as (low, high) 32-bit word pairs: the
// low word's atomic tells whether it wrapped, and the carry goes into the
// high word with the value's high half.  Concurrent adds each carry their
// own wrap, so the pair always sums exactly (shared-memory 32-bit atomics
// are native; 64-bit adds are not).
__device__ __forceinline__ void acc_add32(uint32_t* p, unsigned long long v) {
  const uint32_t lo = (uint32_t)v, hi = (uint32_t)(v >> 32);
  const uint32_t old = atomicAdd(p, lo);
  const uint32_t c = hi + ((old + lo < old) ? 1u : 0u);
  if (c != 0u) atomicAdd(p + 1, c);
}

__device__ __forceinline__ void flush_acc32(unsigned long long* dst, long long cp, long long cn,
                                            long long bp, long long bn) {
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  if (cp) acc_add32(d + 0, (unsigned long long)cp);
  if (cn) acc_add32(d + 2, (unsigned long long)cn);
  if (bp) acc_add32(d + 4, (unsigned long long)bp);
  if (bn) acc_add32(d + 6, (unsigned long long)bn);
}

__device__ __forceinline__ void flush_acc(unsigned long long* dst, long long cp, long long cn,
                                          long long bp, long long bn) {
  if (cp) atomicAdd(dst + 0, as_ull(cp));
  if (cn) atomicAdd(dst + 1, as_ull(cn));
  if (bp) atomicAdd(dst + 2, as_ull(bp));
  if (bn) atomicAdd(dst + 3, as_ull(bn));
}

constexpr int kRowsPerThread = kTile / kConsumers;
constexpr int kInsertBatch = 5;  // rows of a thread whose key-table inserts overlap
static_assert(kTile % kConsumers == 0, "a tile is whole rows per consumer thread");

// Barrier of the consumer warps only (the producer warp never joins it).
__device__ __forceinline__ void consumer_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
}

// Rows x = b, b + step, ... < e of a key's row list (its positive rows
// before mid) whose column value equals k: positive matches in the low 16
// bits, negative matches in the high 16 (four rows' loads in flight at a
// time).
__device__ __forceinline__ uint32_t count_matches1(const uint16_t* rows, const int32_t* c, int32_t k,
                                                   uint32_t b, uint32_t mid, uint32_t e,
                                                   uint32_t step) {
  uint32_t h = 0, x = b;
  for (; x + 3u * step < e; x += 4u * step) {
    const int r0 = rows[x], r1 = rows[x + step], r2 = rows[x + 2u * step], r3 = rows[x + 3u * step];
    h += (uint32_t)(c[r0] == k) << (x >= mid ? 16 : 0);
    h += (uint32_t)(c[r1] == k) << (x + step >= mid ? 16 : 0);
    h += (uint32_t)(c[r2] == k) << (x + 2u * step >= mid ? 16 : 0);
    h += (uint32_t)(c[r3] == k) << (x + 3u * step >= mid ? 16 : 0);
  }
  for (; x < e; x += step) h += (uint32_t)(c[rows[x]] == k) << (x >= mid ? 16 : 0);
  return h;
}

// The same with two columns, both of which must match.
__device__ __forceinline__ uint32_t count_matches2(const uint16_t* rows, const int32_t* ca,
                                                   const int32_t* cb, int32_t ka, int32_t kb,
                                                   uint32_t b, uint32_t mid, uint32_t e,
                                                   uint32_t step) {
  uint32_t h = 0, x = b;
  for (; x + 1u * step < e; x += 2u * step) {
    const int r0 = rows[x], r1 = rows[x + step];
    h += (uint32_t)((ca[r0] == ka) & (cb[r0] == kb)) << (x >= mid ? 16 : 0);
    h += (uint32_t)((ca[r1] == ka) & (cb[r1] == kb)) << (x + step >= mid ? 16 : 0);
  }
  for (; x < e; x += step) {
    const int r = rows[x];
    h += (uint32_t)((ca[r] == ka) & (cb[r] == kb)) << (x >= mid ? 16 : 0);
  }
  return h;
}

__global__ void __launch_bounds__(kEvalThreads, 3) eval_batched_kernel(EvalArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(smem);
  uint32_t* owner = reinterpret_cast<uint32_t*>(acc + 4 * a.num_lits);   // kSlots
  uint32_t* cnt = owner + kSlots;                                         // kSlots
  int32_t* raw = reinterpret_cast<int32_t*>(cnt + kSlots);                // max_cols * kTileStride
  uint16_t* sstart = reinterpret_cast<uint16_t*>(raw + a.max_cols * kTileStride);  // kSlots
  uint16_t* rslot = sstart + kSlots;                                      // kTile
  uint16_t* rrank = rslot + kTile;                                        // kTile
  uint16_t* rows = rrank + kTile;                                         // kTile: shared positions
  uint16_t* klist = rows + kTile;  // kTile: the slots of the tile's distinct keys, in claim order
  __shared__ __align__(8) uint64_t s_full;    // a tile (or the end mark) is in the buffer
  __shared__ __align__(8) uint64_t s_empty;   // the consumers are done with the buffer
  __shared__ __align__(8) uint64_t s_rec[3];  // a unit record (or the end mark) is published
  __shared__ __align__(16) WorkUnit s_unit[3];  // unit records, by unit index modulo 3
  __shared__ uint32_t s_uidx[3];
  __shared__ uint32_t s_count;
  __shared__ uint32_t s_nkeys[2];  // distinct keys of a tile (entries of klist), by tile parity
  __shared__ uint32_t s_alloc;     // row-list space handed out in the current tile
  __shared__ uint32_t s_abort;     // a bounded wait gave up: the CTA stops

  for (int i = threadIdx.x; i < 4 * a.num_lits; i += blockDim.x) acc[i] = 0ull;
  for (int i = threadIdx.x; i < kSlots; i += blockDim.x) {
    owner[i] = 0u;
    cnt[i] = 0u;
  }
  if (threadIdx.x == 0) {
    s_nkeys[0] = s_nkeys[1] = 0u;
    s_alloc = 0u;
    s_abort = 0u;
    s_count = umin(a.unit_count[2], a.unit_cap);
    mbar_init(&s_full, 1);
    mbar_init(&s_empty, 1);
    for (int k = 0; k < 3; ++k) mbar_init(&s_rec[k], 1);
    fence_mbar_init();
  }
  __syncthreads();  // the last barrier of the whole block: the roles split here

  if (threadIdx.x >= kConsumers) {
    // Producer: one thread claims the units and publishes each unit's
    // record one unit ahead (record slot u mod 3: its last reader finished
    // with unit u - 3 before this unit's predecessor released the buffer),
    // and puts every tile in flight (bulk copies of each column's positive
    // and negative runs) as soon as the consumers release the buffer.  After
    // the last unit it publishes an index past the end, as a record and as
    // an empty tile.
    if (threadIdx.x != kConsumers) return;
    const uint32_t count = s_count;
    auto claim = [&](uint32_t slot, WorkUnit& V) -> uint32_t {
      const uint32_t idx = atomicAdd(a.work_counter, 1u);
      if (idx < count) {
        V = a.eunits[idx];
        s_unit[slot] = V;
      }
      s_uidx[slot] = idx;
      mbar_arrive(&s_rec[slot]);
      return idx;
    };
    uint32_t ephase = 0, slot = 0;
    bool first = true;
    WorkUnit V{};
    uint32_t idx = claim(0u, V);
    for (;;) {
      const uint32_t total = idx < count ? V.Pp + V.Np : 0u;
      const uint32_t nslot = slot == 2u ? 0u : slot + 1u;
      WorkUnit NV{};
      uint32_t nidx = count;
      uint32_t t0 = 0;
      do {
        if (!first) {
          int64_t it = 0;
          while (!mbar_try_wait(&s_empty, ephase)) {
            if (++it > a.wait_limit) {
              atomicExch(a.error_flag, 1);  // the consumers' own bounded waits stop them
              return;
            }
          }
          ephase ^= 1u;
        }
        first = false;
        if (idx >= count) {
          mbar_arrive(&s_full);  // the end mark: no tile
          return;
        }
        const TileGeo g = tile_geo(V, t0);
        const int nc = (int)(V.flags & 0xffu);
        fence_proxy_async_smem();  // the copies come after the consumers' reads of the buffer
        const uint32_t tx = (uint32_t)nc * (g.bytesP + g.bytesN);
        if (a.withhold_copies) {
          mbar_arrive_expect_tx(&s_full, tx > 0u ? tx : 16u);  // tests: bytes that never arrive
        } else {
          mbar_arrive_expect_tx(&s_full, tx);
          for (int q = 0; q < nc; ++q) {
            const int32_t* col = V.cols + (int64_t)q * V.stride;
            if (g.bytesP) bulk_g2s(raw + q * kTileStride, col + (g.gP & ~3u), g.bytesP, &s_full);
            if (g.bytesN) bulk_g2s(raw + q * kTileStride + g.aN, col + (g.gN & ~3u), g.bytesN, &s_full);
          }
        }
        if (t0 == 0) nidx = claim(nslot, NV);  // the next unit, while this tile is in flight
        t0 += (uint32_t)kTile;
      } while (t0 < total);
      idx = nidx;
      V = NV;
      slot = nslot;
    }
  }

  // Consumers.  Bounded wait for the next tile: a wait that gives up flags
  // the context, waits once more (bounded) for copies still in flight, so
  // that none lands after the CTA has stopped, and stops the CTA: all
  // consumers leave the unit loop after the barrier that follows, nothing is
  // flushed, and the call reports QFG_ERR_TIMEOUT.  (Should the second wait
  // give up too, the CTA stops all the same.)
  uint32_t phase = 0, tp = 0, cur = 0;
  auto wait_tile = [&]() -> bool {
    int64_t it = 0;
    while (!mbar_try_wait(&s_full, phase)) {
      if (++it > a.wait_limit) {
        atomicExch(a.error_flag, 1);
        s_abort = 1u;
        for (int64_t k2 = 0; k2 < a.wait_limit && !mbar_try_wait(&s_full, phase); ++k2) {
        }
        break;
      }
    }
    phase ^= 1u;
    consumer_sync();
    return s_abort != 0u;
  };

  // This thread's entry records of a unit.  More entries than consumers:
  // a pair of consecutive records per thread.  At most half as many: `tpe`
  // (2 to 8) neighbouring threads share one entry and split its row checks
  // (thread `sub` takes rows sub, sub + tpe, ...).  Otherwise one each.
  // They are loaded as soon as the unit's record is published, so the loads
  // are in flight while the previous unit's sums are reduced.
  uint32_t tpe = 1, sub = 0;
  bool have = false, have1 = false;
  int2 e_k0 = make_int2(0, 0), e_kA = e_k0, e_kB = e_k0, e_mult = e_k0;
  uint2 e_meta = make_uint2(0u, 0u);
  uint32_t rphase = 0;  // bit k: parity of record slot k's next phase
  // Entries [c0, c0 + kChunk) of unit V into this thread's registers.
  auto setup_chunk = [&](const WorkUnit& V, uint32_t c0) {
    const uint32_t cnt = umin((uint32_t)kChunk, V.ecnt - c0);
    tpe = 1;
    sub = 0;
    const bool pairs = cnt > (uint32_t)kConsumers;
    if (!pairs && 2u * cnt <= (uint32_t)kConsumers) {
      const uint32_t q = (uint32_t)kConsumers / (cnt > 0u ? cnt : 1u);
      tpe = q >= 8u ? 8u : q >= 4u ? 4u : 2u;
      sub = threadIdx.x & (tpe - 1u);
    }
    const uint32_t j0 = pairs ? 2u * threadIdx.x : threadIdx.x / tpe;
    have = j0 < cnt && V.eoff + V.ecnt <= a.entry_cap;
    have1 = pairs && have && j0 + 1 < cnt;
    if (have) {
      // pairs: even (c0 and the block start are multiples of 4)
      const uint32_t r = V.eoff + c0 + j0;
      if (pairs) {
        e_k0 = __ldg(reinterpret_cast<const int2*>(a.rec.k0 + r));
        e_kA = __ldg(reinterpret_cast<const int2*>(a.rec.kA + r));
        e_kB = __ldg(reinterpret_cast<const int2*>(a.rec.kB + r));
        e_mult = __ldg(reinterpret_cast<const int2*>(a.rec.mult + r));
        e_meta = __ldg(reinterpret_cast<const uint2*>(a.rec.meta + r));
      } else {
        e_k0.x = __ldg(a.rec.k0 + r);
        e_kA.x = __ldg(a.rec.kA + r);
        e_kB.x = __ldg(a.rec.kB + r);
        e_mult.x = __ldg(a.rec.mult + r);
        e_meta.x = __ldg(a.rec.meta + r);
      }
    }
  };
  // The first chunk of the unit in record slot rslot_i, once published.
  auto load_entries = [&](uint32_t rslot_i) -> bool {
    int64_t it = 0;
    while (!mbar_try_wait(&s_rec[rslot_i], (rphase >> rslot_i) & 1u)) {
      if (++it > a.wait_limit) {
        atomicExch(a.error_flag, 1);
        s_abort = 1u;  // seen after the next wait's barrier
        return false;
      }
    }
    rphase ^= 1u << rslot_i;
    if (s_uidx[rslot_i] >= s_count) return false;
    setup_chunk(s_unit[rslot_i], 0u);
    return true;
  };

  // Per-literal sums of the warp's lanes into the CTA's accumulators.  A
  // thread's entries are contiguous and increasing within a chunk, so equal
  // literals sit on consecutive lanes (the segmented scan needs that); idle
  // lanes (Lrun = -1) trail.  A thread with no entry in a later chunk
  // flushes its sums on its own, so every lane's literal at the unit's end
  // comes from the unit's last chunk.
  long long bp = 0, bn = 0, cp = 0, cn = 0;
  int Lrun = -1;
  auto reduce_sums = [&](int lit_begin, bool small) {
    if (small) {
      // Fewer than 2^20 rows in the unit: a lane's covered counts stay below
      // 2^24 (at most 16 entries), their 32-lane sums below 2^29, so both
      // counts travel in one 64-bit scan.
      const long long c2 = seg_scan(cp | (cn << 32), Lrun);
      cp = c2 & 0xffffffffll;
      cn = (long long)((unsigned long long)c2 >> 32);
    } else {
      cp = seg_scan(cp, Lrun);
      cn = seg_scan(cn, Lrun);
    }
    bp = seg_scan(bp, Lrun);
    bn = seg_scan(bn, Lrun);
    const int next_L = __shfl_down_sync(kFullMask, Lrun, 1);
    const bool seg_end = lane_id() == 31 || next_L != Lrun;
    if (seg_end && Lrun >= 0 && (cp | cn | bp | bn) != 0)
      flush_acc32(acc + 4 * (lit_begin + Lrun), cp, cn, bp, bn);
    bp = bn = cp = cn = 0;
    Lrun = -1;
  };

  load_entries(0u);
  for (;;) {
    if (wait_tile()) break;
    if (s_uidx[cur] >= s_count) break;  // the producer's end mark
    const WorkUnit& U = s_unit[cur];
    const int lit_begin = (int)U.lit_begin;
    const bool has_atoms = (U.flags & 0x100u) != 0u;
    const uint32_t total = U.Pp + U.Np;

    for (uint32_t t0 = 0; t0 < total || t0 == 0; t0 += kTile) {  // an empty unit: one empty tile
      if (t0 > 0 && wait_tile()) break;
      const TileGeo g = tile_geo(U, t0);
      const int nt = (int)g.nt, npos = (int)g.npos;
      const uint32_t shP = g.shP, baseN = g.baseN;
      // The other parity's key count was last read before the wait's barrier.
      if (threadIdx.x == 0) s_nkeys[tp ^ 1u] = 0u;
      // Distinct join keys of the tile: owner = first row + 1, claimed by
      // CAS; the count atomics return each row's rank within its key and
      // label (positive count low half, negative count high half).  A
      // thread's rows go through each step in batches of kInsertBatch, so
      // their shared-memory round trips overlap: keys, the owners of their
      // home slots, the owners' keys; only a row whose home slot is free or
      // holds another key takes the probe loop with CAS.
      for (int k0 = 0; k0 < kRowsPerThread; k0 += kInsertBatch) {
        int32_t key[kInsertBatch];
        uint32_t slot[kInsertBatch], own[kInsertBatch];
#pragma unroll
        for (int k = 0; k < kInsertBatch; ++k) {
          const int i = (int)threadIdx.x + (k0 + k) * kConsumers;
          const uint32_t pos = i < npos ? (uint32_t)i + shP : baseN + (uint32_t)(i - npos);
          key[k] = i < nt ? raw[pos] : 0;
          slot[k] = mix32((uint32_t)key[k]) & (kSlots - 1);
        }
#pragma unroll
        for (int k = 0; k < kInsertBatch; ++k) own[k] = owner[slot[k]];
#pragma unroll
        for (int k = 0; k < kInsertBatch; ++k) {
          const int i = (int)threadIdx.x + (k0 + k) * kConsumers;
          if (i >= nt) continue;
          if (own[k] != 0u && raw[own[k] - 1u] == key[k]) continue;  // the key's home slot
          const uint32_t pos = i < npos ? (uint32_t)i + shP : baseN + (uint32_t)(i - npos);
          uint32_t sl = slot[k];
          for (int probe = 0; probe < kSlots; ++probe) {
            const uint32_t o = atomicCAS(&owner[sl], 0u, pos + 1u);
            if (o == 0u) {
              klist[atomicAdd(&s_nkeys[tp], 1u)] = (uint16_t)sl;
              break;
            }
            if (raw[o - 1u] == key[k]) break;
            sl = (sl + 1) & (kSlots - 1);
          }
          slot[k] = sl;
        }
        uint32_t old[kInsertBatch];
#pragma unroll
        for (int k = 0; k < kInsertBatch; ++k) {
          const int i = (int)threadIdx.x + (k0 + k) * kConsumers;
          old[k] = i < nt ? atomicAdd(&cnt[slot[k]], i < npos ? 1u : 0x10000u) : 0u;
        }
        if (has_atoms) {
#pragma unroll
          for (int k = 0; k < kInsertBatch; ++k) {
            const int i = (int)threadIdx.x + (k0 + k) * kConsumers;
            if (i < nt) {
              rslot[i] = (uint16_t)slot[k];
              rrank[i] = (uint16_t)(i < npos ? (old[k] & 0xffffu) : (old[k] >> 16));
            }
          }
        }
      }
      consumer_sync();
      const uint32_t nk = s_nkeys[tp];
      {
        // Owners become keys (probes compare keys directly).  With atom
        // literals each key also takes the run of the row list for its
        // rows by a warp-aggregated atomic (the runs' order is free).
        for (uint32_t d0 = 0; d0 < nk; d0 += kConsumers) {
          const uint32_t d = d0 + threadIdx.x;
          uint32_t c = 0, sl = 0;
          if (d < nk) {
            sl = klist[d];
            const uint32_t w = cnt[sl];
            c = (w & 0xffffu) + (w >> 16);
            owner[sl] = (uint32_t)raw[owner[sl] - 1u];
          }
          if (has_atoms) {
            uint32_t x = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const uint32_t y = __shfl_up_sync(kFullMask, x, o);
              if (lane_id() >= o) x += y;
            }
            uint32_t base = 0;
            if (lane_id() == 31 && x > 0u) base = atomicAdd(&s_alloc, x);
            base = __shfl_sync(kFullMask, base, 31);
            if (d < nk) sstart[sl] = (uint16_t)(base + x - c);
          }
        }
      }
      consumer_sync();
      if (has_atoms) {
        if (threadIdx.x == 0) s_alloc = 0u;  // last used above; next used after the next tile's wait
        // All of a thread's loads first, then its stores (the shared arrays
        // may alias as far as the compiler knows).
        uint32_t dst[kRowsPerThread];
#pragma unroll
        for (int k = 0; k < kRowsPerThread; ++k) {
          const int i = (int)threadIdx.x + k * kConsumers;
          dst[k] = 0u;
          if (i < nt) {
            const int sl = rslot[i];
            const uint32_t rk = rrank[i];
            dst[k] = (uint32_t)sstart[sl] + (i < npos ? rk : (cnt[sl] & 0xffffu) + rk);
          }
        }
#pragma unroll
        for (int k = 0; k < kRowsPerThread; ++k) {
          const int i = (int)threadIdx.x + k * kConsumers;
          if (i < nt) rows[dst[k]] = (uint16_t)(i < npos ? (uint32_t)i + shP : baseN + (uint32_t)(i - npos));
        }
        consumer_sync();
      }
      // This thread's entries against the tile, a chunk of the unit's
      // entries at a time (the first chunk's records were loaded when the
      // unit's record was published; a later tile reloads it).
      for (uint32_t c0 = 0; c0 < U.ecnt || c0 == 0; c0 += kChunk) {
        if (c0 > 0 || t0 > 0) {
          setup_chunk(U, c0);
          if (!have && Lrun >= 0) {
            // No entry in this chunk: the thread's sums go now, so at the
            // unit's end every lane's literal is from the last chunk.
            if ((cp | cn | bp | bn) != 0) flush_acc32(acc + 4 * (lit_begin + Lrun), cp, cn, bp, bn);
            bp = bn = cp = cn = 0;
            Lrun = -1;
          }
        }
        // Both entries' home slots first, so their shared-memory round trips
        // overlap; a key that is not in its home slot probes onwards.
        uint32_t hslot[2], hw[2], hown[2];
#pragma unroll
        for (int j = 0; j < 2; ++j)
          hslot[j] = mix32((uint32_t)(j == 0 ? e_k0.x : e_k0.y)) & (kSlots - 1);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          hw[j] = cnt[hslot[j]];
          hown[j] = owner[hslot[j]];
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          if (!(j == 0 ? have : have1)) continue;
          const int32_t k0 = j == 0 ? e_k0.x : e_k0.y;
          const uint32_t meta = j == 0 ? e_meta.x : e_meta.y;
          const int L = (int)(meta & 0xffu);
          if (L != Lrun) {
            if (Lrun >= 0 && (cp | cn | bp | bn) != 0)
              flush_acc32(acc + 4 * (lit_begin + Lrun), cp, cn, bp, bn);
            bp = bn = cp = cn = 0;
            Lrun = L;
          }
          if (!((meta >> 10) & 1u)) continue;
          uint32_t slot = hslot[j];
          uint32_t w = hw[j];
          if (w != 0u && (int32_t)hown[j] != k0) {
            for (int probe = 1; probe < kSlots; ++probe) {
              slot = (slot + 1) & (kSlots - 1);
              w = cnt[slot];
              if (w == 0u || (int32_t)owner[slot] == k0) break;
            }
          }
          if (w == 0u) continue;
          const uint32_t P = w & 0xffffu, N = w >> 16;
          const uint32_t nchk = (meta >> 8) & 3u;
          uint32_t hp = 0, hn = 0;
          if (nchk == 0) {
            if (sub == 0u) {
              hp = P;
              hn = N;
            }
          } else {
            const uint32_t beg = sstart[slot], mid = beg + P, end = mid + N;
            const int32_t kA = j == 0 ? e_kA.x : e_kA.y;
            if (nchk == 1) {
              const int32_t* ca = raw + ((meta >> 12) & 7u) * kTileStride;
              const uint32_t h = count_matches1(rows, ca, kA, beg + sub, mid, end, tpe);
              hp = h & 0xffffu;
              hn = h >> 16;
            } else if (nchk == 2) {
              const int32_t kB = j == 0 ? e_kB.x : e_kB.y;
              const int32_t* ca = raw + ((meta >> 12) & 7u) * kTileStride;
              const int32_t* cb = raw + ((meta >> 16) & 7u) * kTileStride;
              const uint32_t h = count_matches2(rows, ca, cb, kA, kB, beg + sub, mid, end, tpe);
              hp = h & 0xffffu;
              hn = h >> 16;
            } else {
              // More than two checked columns: keys from the key table.
              const LitDesc& d = a.lits[lit_begin + L];
              const uint32_t e = (uint32_t)kA;
              for (uint32_t x = beg + sub; x < end; x += tpe) {
                const int r = rows[x];
                bool pass = true;
                for (int q = 1; q < d.nk && pass; ++q) {
                  const int ac = d.atom_col[q];
                  if (ac != 0) pass = raw[ac * kTileStride + r] == __ldg(d.keys + q * d.stride + e);
                }
                if (pass) {
                  if (x < mid) ++hp; else ++hn;
                }
              }
            }
          }
          const long long mlt = j == 0 ? e_mult.x : e_mult.y;
          bp += mlt * hp;
          bn += mlt * hn;
          cp += hp;
          cn += hn;
        }
      }
      consumer_sync();
      // The tile's slots are cleared (the next key table is built after the
      // next wait's barrier) and the buffer goes back to the producer.
      for (uint32_t d = threadIdx.x; d < nk; d += kConsumers) {
        const uint32_t sl = klist[d];
        owner[sl] = 0u;
        cnt[sl] = 0u;
      }
      if (threadIdx.x == 0) mbar_arrive(&s_empty);
      tp ^= 1u;
    }
    if (s_abort != 0u) break;  // read after the barrier that follows the wait
    const uint32_t next = cur == 2u ? 0u : cur + 1u;
    load_entries(next);
    reduce_sums(lit_begin, total < (1u << 20));
    cur = next;
  }
  consumer_sync();
  if (s_abort != 0u) return;
  for (int i = threadIdx.x; i < 4 * a.num_lits; i += kConsumers) {
    const unsigned long long v = acc[i];
    if (v != 0ull) atomicAdd(&a.counts[4 * a.lits[i >> 2].out + (i & 3)], v);
  }
}

// ----------------------------------------------------------------------------
// Streamed evaluation.
//
// Work unit = (item, piece of at most kSEntries relation entries).  The CTA
// loads the piece's entries -- every literal's distinct key tuples in the
// item's key range -- and files each under its composite key (signature,
// join key, the signature columns' keys) in a shared-memory key table
// (open addressing; the first entry with a composite key claims its slot by
// atomicCAS, later ones with the same key -- other literals -- share it).
// Then its threads stream the item's binding rows straight from the
// partitioned columns (coalesced loads, no staging) and look each row's
// composite key up once per signature of the group; a hit adds 1 to the
// slot's positive or negative row counter, so a row costs one atomic per
// signature it matches, however many literals share that key.  Afterwards
// every entry takes its slot's counts: covered += count, binding +=
// multiplicity x count (a binding row matches at most one distinct key tuple
// of a literal).

constexpr int kSThreads = 512;
constexpr int kSEntries = 1536;        // relation entries per unit
constexpr int kSSlots = 4096;          // key-table slots (more than twice the entries)
constexpr int kSMaxSigs = 64;          // signatures of one group
constexpr uint32_t kSRowTarget = 32768;  // mean binding rows of an item (partition bits)
constexpr uint32_t kSEntryTarget = 1024;  // mean relation entries of an item
static_assert((kSSlots & (kSSlots - 1)) == 0 && kSSlots > 2 * kSEntries, "slot table shape");

size_t stream_smem_bytes(int num_lits) {
  return sizeof(unsigned long long) * 4 * (size_t)num_lits + sizeof(int32_t) * 3 * kSSlots +
         sizeof(int32_t) * 7 * (size_t)kSEntries;
}

// Hash of a composite key: the join key's mix, salted by the signature,
// folded with every signature column's key.  Entries and probing rows use
// the same function.
__device__ __forceinline__ uint32_t skey_start(uint32_t hk, int sig) {
  return hk + (uint32_t)sig * 0x61c88647u;
}
__device__ __forceinline__ uint32_t skey_fold(uint32_t h, int32_t v) {
  return (h ^ (uint32_t)v) * 0x85ebca6bu;
}
__device__ __forceinline__ uint32_t skey_slot(uint32_t h) { return (h ^ (h >> 15)) & (kSSlots - 1); }

__device__ __forceinline__ int32_t pick(const int32_t (&v)[kGroupCols], int c) {
  int32_t x = v[0];
#pragma unroll
  for (int q = 1; q < kGroupCols; ++q) x = c == q ? v[q] : x;
  return x;
}

// Key q >= 2 of a signature position of entry e (signatures of more than
// two columns keep those in the key table).
__device__ __forceinline__ int32_t sig_key_from_table(const LitDesc& d, int32_t gidx, int pos) {
  int32_t x = 0;
  for (int q = 1; q < d.nk; ++q)
    if (d.spos[q] == pos) x = __ldg(d.keys + q * d.stride + gidx);
  return x;
}

__global__ void __launch_bounds__(kSThreads, 2) stream_eval_kernel(EvalArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(smem);
  int32_t* owner = reinterpret_cast<int32_t*>(acc + 4 * a.num_lits);  // kSSlots: entry or -1
  uint32_t* kcp = reinterpret_cast<uint32_t*>(owner + kSSlots);       // kSSlots
  uint32_t* kcn = kcp + kSSlots;                                       // kSSlots
  int32_t* e_k0 = reinterpret_cast<int32_t*>(kcn + kSSlots);           // kSEntries each:
  int32_t* e_s1 = e_k0 + kSEntries;
  int32_t* e_s2 = e_s1 + kSEntries;
  uint32_t* e_meta = reinterpret_cast<uint32_t*>(e_s2 + kSEntries);    // literal | sig << 10 | valid << 31
  int32_t* e_mult = reinterpret_cast<int32_t*>(e_meta + kSEntries);
  int32_t* e_slot = e_mult + kSEntries;
  int32_t* e_gidx = e_slot + kSEntries;  // key-table index of the entry
  __shared__ uint32_t s_lstart[kMaxGroupLits + 1];
  __shared__ uint32_t s_le0[kMaxGroupLits];
  __shared__ SigDesc s_sig[kSMaxSigs];
  __shared__ WorkUnit s_unit;
  __shared__ uint32_t s_idx, s_count;
  __shared__ int s_group;  // group whose signatures s_sig holds

  for (int i = threadIdx.x; i < 4 * a.num_lits; i += blockDim.x) acc[i] = 0ull;
  for (int i = threadIdx.x; i < kSSlots; i += blockDim.x) {
    owner[i] = -1;
    kcp[i] = 0u;
    kcn[i] = 0u;
  }
  if (threadIdx.x == 0) {
    s_count = umin(a.unit_count[0], a.unit_cap);
    s_idx = atomicAdd(a.work_counter, 1u);
    if (s_idx < s_count) s_unit = a.units[s_idx];
    s_group = -1;
  }
  __syncthreads();
  const int lane = lane_id(), warp = warp_id();

  for (;;) {
    const uint32_t idx = s_idx;
    if (idx >= s_count) break;
    const WorkUnit U = s_unit;
    const GroupDesc& G = a.groups[U.group];
    const int m = G.lit_end - G.lit_begin;
    const int nsig = G.sig_end - G.sig_begin;
    uint32_t nidx = 0;
    if (threadIdx.x == 0) nidx = atomicAdd(a.work_counter, 1u);
    // The item's literal-major entry space (warp 0) and the group's
    // signatures (warp 1) in shared memory.
    if (warp == 0) {
      const int rshift = kRelPartitionBits - G.bits;
      const uint32_t q0 = U.p << rshift, q1 = (U.p + 1) << rshift;
      uint32_t run = 0;
      for (int L0 = 0; L0 < m; L0 += 32) {
        const int L = L0 + lane;
        uint32_t c = 0;
        if (L < m) {
          const uint32_t* off = a.lits[G.lit_begin + L].offsets;
          const uint32_t e0 = __ldg(off + q0);
          c = __ldg(off + q1) - e0;
          s_le0[L] = e0;
        }
        uint32_t x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(kFullMask, x, o);
          if (lane >= o) x += y;
        }
        if (L < m) s_lstart[L] = run + x - c;
        run += __shfl_sync(kFullMask, x, 31);
      }
      if (lane == 0) s_lstart[m] = run;
    } else if (warp == 1 && s_group != (int)U.group) {
      for (int q = lane; q < nsig; q += 32) s_sig[q] = a.sigs[G.sig_begin + q];
    }
    __syncthreads();
    if (threadIdx.x == 0) s_group = (int)U.group;
    // The unit's entries into the key table.
    for (uint32_t j = threadIdx.x; j < U.ecnt; j += blockDim.x) {
      const uint32_t f = U.f0 + j;
      int lo = 0, hi = m - 1;  // largest L with s_lstart[L] <= f
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_lstart[mid] <= f) lo = mid; else hi = mid - 1;
      }
      const LitDesc& d = a.lits[G.lit_begin + lo];
      const uint32_t e = s_le0[lo] + (f - s_lstart[lo]);
      const int32_t k0 = __ldg(d.keys + e);
      const int sg = d.sig - G.sig_begin;
      const int sn = s_sig[sg].ncols;
      int32_t sk[kGroupCols - 1];
#pragma unroll
      for (int i = 0; i < kGroupCols - 1; ++i) sk[i] = 0;
      uint32_t filled = 0;
      bool valid = true;
      for (int q = 1; q < d.nk; ++q) {
        const int32_t kq = __ldg(d.keys + q * d.stride + e);
        const int pq = d.spos[q];
        if (pq < 0) {
          valid &= kq == k0;  // compared with the join column itself
        } else {
#pragma unroll
          for (int i = 0; i < kGroupCols - 1; ++i) {
            if (i != pq) continue;
            if (filled & (1u << i)) valid &= sk[i] == kq;  // two arguments, one variable
            sk[i] = kq;
          }
          filled |= 1u << pq;
        }
      }
      uint32_t h = skey_start(mix32((uint32_t)k0), sg);
#pragma unroll
      for (int i = 0; i < kGroupCols - 1; ++i)
        if (i < sn) h = skey_fold(h, sk[i]);
      e_k0[j] = k0;
      e_s1[j] = sk[0];
      e_s2[j] = sk[1];
      e_mult[j] = __ldg(d.mult + e);
      e_gidx[j] = (int32_t)e;
      e_meta[j] = (uint32_t)lo | ((uint32_t)sg << 10) | (valid ? 0x80000000u : 0u);
      int32_t slot = -1;
      if (valid) {
        // The entry's keys are visible to the block before it may own a slot.
        __threadfence_block();
        uint32_t sl = skey_slot(h);
        for (int probe = 0; probe < kSSlots; ++probe) {
          const int32_t o = atomicCAS(&owner[sl], -1, (int32_t)j);
          if (o < 0) {
            slot = (int32_t)sl;
            break;
          }
          const uint32_t om = e_meta[o];
          bool same = (int)((om >> 10) & 0x3ffu) == sg && e_k0[o] == k0 && e_s1[o] == sk[0] &&
                      e_s2[o] == sk[1];
          if (same && sn > 2) {
            const LitDesc& od = a.lits[G.lit_begin + (om & 0x3ffu)];
            for (int i = 2; i < sn && same; ++i)
              same = sig_key_from_table(od, e_gidx[o], i) == sig_key_from_table(d, (int32_t)e, i);
          }
          if (same) {
            slot = (int32_t)sl;
            break;
          }
          sl = (sl + 1) & (kSSlots - 1);
        }
      }
      e_slot[j] = slot;
    }
    __syncthreads();
    // The item's binding rows, positives then negatives, against the table.
    {
      const int ncols = G.ncols;
      const int64_t stride = G.n;
      const uint32_t r0 = U.eoff, r1 = U.eoff + U.pad;  // rows of the item, positives first
      for (uint32_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const bool pos = r < U.Pp;
        const uint32_t row = pos ? U.ps + r : U.ns + (r - U.Pp);
        int32_t v[kGroupCols];
#pragma unroll
        for (int q = 0; q < kGroupCols; ++q) v[q] = q < ncols ? __ldg(G.cols + q * stride + row) : 0;
        uint32_t* cnt = pos ? kcp : kcn;
        const uint32_t hk = mix32((uint32_t)v[0]);
        for (int sg = 0; sg < nsig; ++sg) {
          const SigDesc& S = s_sig[sg];
          uint32_t h = skey_start(hk, sg);
          for (int i = 0; i < S.ncols; ++i) h = skey_fold(h, pick(v, S.col[i]));
          uint32_t sl = skey_slot(h);
          for (int probe = 0; probe < kSSlots; ++probe) {
            const int32_t o = owner[sl];
            if (o < 0) break;
            const uint32_t om = e_meta[o];
            if ((int)((om >> 10) & 0x3ffu) == sg && e_k0[o] == v[0] &&
                (S.ncols < 1 || e_s1[o] == pick(v, S.col[0])) &&
                (S.ncols < 2 || e_s2[o] == pick(v, S.col[1]))) {
              bool ok = true;
              if (S.ncols > 2) {
                const LitDesc& d = a.lits[G.lit_begin + (om & 0x3ffu)];
                for (int i = 2; i < S.ncols && ok; ++i)
                  ok = sig_key_from_table(d, e_gidx[o], i) == pick(v, S.col[i]);
              }
              if (ok) {
                atomicAdd(&cnt[sl], 1u);
                break;
              }
            }
            sl = (sl + 1) & (kSSlots - 1);
          }
        }
      }
    }
    if (threadIdx.x == 0 && nidx < s_count) s_unit = a.units[nidx];
    __syncthreads();
    // Entry counts into the literals' sums; entries are literal-major, so
    // equal literals sit on consecutive lanes (segmented warp scans).
    for (uint32_t j0 = 0; j0 < U.ecnt; j0 += blockDim.x) {
      const uint32_t j = j0 + threadIdx.x;
      int L = -1;
      long long cp = 0, cn = 0, bp = 0, bn = 0;
      if (j < U.ecnt) {
        L = (int)(e_meta[j] & 0x3ffu);
        const int32_t sl = e_slot[j];
        if (sl >= 0) {
          const uint32_t p = kcp[sl], q = kcn[sl];
          const long long mlt = e_mult[j];
          cp = p;
          cn = q;
          bp = mlt * p;
          bn = mlt * q;
        }
      }
      cp = seg_scan(cp, L);
      cn = seg_scan(cn, L);
      bp = seg_scan(bp, L);
      bn = seg_scan(bn, L);
      const int next_L = __shfl_down_sync(kFullMask, L, 1);
      if ((lane == 31 || next_L != L) && L >= 0 && (cp | cn | bp | bn) != 0)
        flush_acc(acc + 4 * (G.lit_begin + L), cp, cn, bp, bn);
    }
    __syncthreads();
    // The slots this unit used back to empty.
    for (uint32_t j = threadIdx.x; j < U.ecnt; j += blockDim.x) {
      const int32_t sl = e_slot[j];
      if (sl >= 0) {
        owner[sl] = -1;
        kcp[sl] = 0u;
        kcn[sl] = 0u;
      }
    }
    if (threadIdx.x == 0) s_idx = nidx;
    __syncthreads();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 4 * a.num_lits; i += blockDim.x) {
    const unsigned long long v = acc[i];
    if (v != 0ull) atomicAdd(&a.counts[4 * a.lits[i >> 2].out + (i & 3)], v);
  }
}

// Binding-size class of the autotuner: floor(log2(rows)).
int size_class(int64_t n) {
  int c = 0;
  while ((n >> (c + 1)) > 0) ++c;
  return c;
}

int auto_group_bits(Ctx* ctx, int64_t n) {
  if (ctx->eval_bits > 0) return std::min(ctx->eval_bits, kMaxPartitionBits);
  if (ctx->autotune) {
    auto it = ctx->tuned_bits.find(size_class(n));
    if (it != ctx->tuned_bits.end()) return it->second.first;
  }
  int bits = 1;
  while (bits < kMaxPartitionBits && (n >> bits) > kTargetRows) ++bits;
  return bits;
}

// Pass-1 bits of a two-pass partition into `bits` bits: an override, the
// autotuned choice of the size class, or the default; always leaving pass 2
// at most kMaxSubBits.
int coarse_bits(Ctx* ctx, int64_t n, int bits) {
  int cb = kDefaultCoarseBits;
  if (ctx->eval_cbits > 0) {
    cb = ctx->eval_cbits;
  } else if (ctx->autotune && ctx->eval_bits == 0) {
    auto it = ctx->tuned_bits.find(size_class(n));
    if (it != ctx->tuned_bits.end() && it->second.first == bits) cb = it->second.second;
  }
  cb = std::min(std::max(cb, bits - kMaxSubBits), std::min(kMaxCoarseBits, bits - 1));
  return std::max(cb, 1);
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
    // A cached table is read later from any stream (serving slots, graphs).
    QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
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

// max_sigs > 0 (streamed path): a group holds literals of at most max_sigs
// distinct key signatures (sets of further bound binding columns).
static int plan_step(Ctx* ctx, int32_t n, const qfg_literal* lits, StepPlan* plan,
                     int max_sigs = 0) {
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
  auto signature = [&](int i) {
    std::vector<int> sig;
    for (size_t q = 1; q < bind_cols[i].size(); ++q)
      if (bind_cols[i][q] != bind_cols[i][0]) sig.push_back(bind_cols[i][q]);
    std::sort(sig.begin(), sig.end());
    sig.erase(std::unique(sig.begin(), sig.end()), sig.end());
    return sig;
  };
  for (auto& kv : by_col) {
    HostGroup cur;
    std::set<std::vector<int>> sigs;
    cur.join_col = kv.first;
    cur.cols = {kv.first};
    for (int i : kv.second) {
      std::vector<int> add = missing_cols(cur, i);
      const std::vector<int> sig = signature(i);
      if ((int)(cur.cols.size() + add.size()) > kGroupCols ||
          (int)cur.lits.size() >= kMaxGroupLits ||
          (max_sigs > 0 && !sigs.count(sig) && (int)sigs.size() >= max_sigs)) {
        groups.push_back(cur);
        cur = HostGroup();
        sigs.clear();
        cur.join_col = kv.first;
        cur.cols = {kv.first};
        add = missing_cols(cur, i);
      }
      cur.cols.insert(cur.cols.end(), add.begin(), add.end());
      cur.lits.push_back(i);
      sigs.insert(sig);
      if (bind_cols[i].size() > 1) cur.has_atoms = true;
    }
    groups.push_back(cur);
  }
  return QFG_OK;
}

// A batched step decided on the host: scratch reserved, descriptors built,
// partition passes and evaluation launches listed.  enqueue_step() then
// issues only stream work (memsets and kernel launches, no host
// synchronization), so a prepared step can be enqueued directly or captured
// into a CUDA graph and replayed on new binding data of the same shape.
struct PartJob {
  BPartArgs pa;             // pa.bits / pa.cbits: this group's partition shape
  int np1, sbits;
};

struct LaunchJob {
  EvalArgs ea;
  size_t smem;
  int grid;
  int plan_grid;
  int gather_grid;
  bool streamed;
};

struct PreparedStep {
  int mode = 0;             // kModeTiled or kModeStreamed
  unsigned pgrid = 0;
  uint32_t* p1_tot = nullptr;     // every group's pass-1 bin totals, contiguous (zeroed per step)
  size_t p1_tot_words = 0;
  int np1_max = 0;                // widest pass-1 fan-out of the groups
  size_t p1_smem = 0, p2_smem = 0;
  bool any_two_pass = false;
  const BPartArgs* part_args_dev = nullptr;  // the groups' jobs in the descriptor blob
  int64_t col_stride = 0;   // column stride of the partitioned layout
  std::vector<PartJob> parts;
  std::vector<LaunchJob> launches;
  std::vector<unsigned char> blob;  // descriptors, to be copied to blob_dev
  void* blob_dev = nullptr;
  unsigned int* counter = nullptr;  // [work counter, unit count, entry-record count]
};

constexpr int kModeTiled = 1;
constexpr int kModeStreamed = 2;

// The evaluation mode of a batched step over nb binding rows: the option,
// else the autotuner's choice for the size class, else tiled (measured on
// the 32M x 6, 256-literal step: evaluation 4.1 ms tiled (+0.8 ms unit
// planning and entry gather) against 7.9 ms streamed (+0.05 ms)).
int step_mode(Ctx* ctx, int64_t nb) {
  if (ctx->eval_mode == kModeTiled || ctx->eval_mode == kModeStreamed) return ctx->eval_mode;
  if (ctx->autotune) {
    auto it = ctx->tuned_mode.find(size_class(nb));
    if (it != ctx->tuned_mode.end()) return it->second.first;
  }
  return kModeTiled;
}

// Offset of the streamed path's partition bits: a tuning trial's, else the
// autotuner's choice for the size class, else 0.
int stream_bias(Ctx* ctx, int64_t nb) {
  if (ctx->stream_bias != 0) return ctx->stream_bias;
  if (ctx->autotune) {
    auto it = ctx->tuned_mode.find(size_class(nb));
    if (it != ctx->tuned_mode.end() && it->second.first == kModeStreamed) return it->second.second;
  }
  return 0;
}

// Partition bits of one literal group.  Tiled: from the binding-set size
// (rows per shared-memory tile).  Streamed: enough partitions that the mean
// item holds at most kSEntryTarget of the group's relation entries (they
// must fit the shared-memory table) and at most kSRowTarget binding rows
// (work balance).  QFG_OPT_EVAL_BITS fixes the bits of every group.
int group_bits(Ctx* ctx, int mode, int64_t nb, int64_t entries) {
  if (mode == kModeTiled || ctx->eval_bits > 0) return auto_group_bits(ctx, nb);
  int bits = 1;
  while (bits < kMaxPartitionBits &&
         ((entries >> bits) > (int64_t)kSEntryTarget || (nb >> bits) > (int64_t)kSRowTarget))
    ++bits;
  return std::max(1, std::min(kMaxPartitionBits, bits + stream_bias(ctx, nb)));
}

// The key signatures of a group (streamed path) and, per literal, its
// signature and the signature position of every further key.
void group_signatures(const HostGroup& g, const std::vector<std::vector<int>>& bind_cols,
                      std::vector<SigDesc>* sigs, std::vector<int>* lit_sig,
                      std::vector<std::vector<int8_t>>* lit_spos) {
  std::vector<std::vector<int>> lists;
  lit_sig->clear();
  lit_spos->clear();
  for (int i : g.lits) {
    std::vector<int> cols;
    for (size_t q = 1; q < bind_cols[i].size(); ++q) {
      const int c = (int)(std::find(g.cols.begin(), g.cols.end(), bind_cols[i][q]) - g.cols.begin());
      if (c != 0 && std::find(cols.begin(), cols.end(), c) == cols.end()) cols.push_back(c);
    }
    std::sort(cols.begin(), cols.end());
    int sig = (int)(std::find(lists.begin(), lists.end(), cols) - lists.begin());
    if (sig == (int)lists.size()) lists.push_back(cols);
    std::vector<int8_t> spos(QFG_MAX_ARITY, -1);
    for (size_t q = 1; q < bind_cols[i].size(); ++q) {
      const int c = (int)(std::find(g.cols.begin(), g.cols.end(), bind_cols[i][q]) - g.cols.begin());
      spos[q] = c == 0 ? -1 : (int8_t)(std::find(cols.begin(), cols.end(), c) - cols.begin());
    }
    lit_sig->push_back(sig);
    lit_spos->push_back(spos);
  }
  sigs->clear();
  for (const auto& l : lists) {
    SigDesc d;
    memset(&d, 0, sizeof(d));
    d.ncols = (int32_t)l.size();
    for (size_t i = 0; i < l.size(); ++i) d.col[i] = l[i];
    sigs->push_back(d);
  }
}

int prepare_step(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                 unsigned long long* counts, PreparedStep* ps) {
  const int64_t nb = b->num_positive + b->num_negative;
  ps->parts.clear();
  ps->launches.clear();
  ps->blob.clear();
  if (n == 0 || nb == 0) return QFG_OK;
  const int mode = step_mode(ctx, nb);
  ps->mode = mode;

  QFG_TRY(stage_begin(ctx, QFG_STAGE_KEY_TABLES));
  StepPlan plan;
  QFG_TRY(plan_step(ctx, n, lits, &plan, mode == kModeStreamed ? kSMaxSigs : 0));
  QFG_TRY(stage_end(ctx, QFG_STAGE_KEY_TABLES));
  const auto& tables = plan.tables;
  const auto& bind_cols = plan.bind_cols;
  const auto& groups = plan.groups;
  if (ctx->shard_index >= ctx->shard_count)
    return set_error(ctx, QFG_ERR_INVALID, "shard index must be below the shard count");

  // Partition shape of every group.
  ps->pgrid = (unsigned)ctx->num_sms;
  // Partitioned columns: stride a multiple of 4 rows, so every column of a
  // group has the same 16-byte alignment (the evaluation's bulk copies).
  ps->col_stride = ((int64_t)nb + 3) & ~int64_t(3);
  const size_t G = groups.size();
  std::vector<int> gbits(G), gcbits(G);
  size_t part_words = 0, fs_words = 0, tot_words = 0, bins_words = 0, tmp_words = 0;
  ps->np1_max = 2;
  int sbits_max = 1;
  ps->any_two_pass = false;
  for (size_t gi = 0; gi < G; ++gi) {
    const HostGroup& g = groups[gi];
    int64_t entries = 0;
    for (int i : g.lits) entries += tables[i]->num_entries;
    gbits[gi] = group_bits(ctx, mode, nb, entries);
    const bool two = gbits[gi] > kMaxSinglePassBits;
    gcbits[gi] = two ? coarse_bits(ctx, nb, gbits[gi]) : gbits[gi];
    const int np1 = 2 << gcbits[gi];
    const size_t chunks = (size_t)nb / kP2Chunk + (size_t)np1 + 1;
    part_words += g.cols.size() * (size_t)ps->col_stride;
    fs_words += ((size_t)2 << gbits[gi]) + 1;
    tot_words += (size_t)np1 + 1;
    bins_words += (size_t)ps->pgrid * np1;  // per-CTA bases
    if (two) {
      bins_words += 3 * ((size_t)np1 + 1) + chunks + (chunks << (gbits[gi] - gcbits[gi]));
      tmp_words += g.cols.size() * (size_t)((((int64_t)nb + 3) & ~int64_t(3)) + 4 * (int64_t)np1);
      sbits_max = std::max(sbits_max, gbits[gi] - gcbits[gi]);
      ps->any_two_pass = true;
    }
    ps->np1_max = std::max(ps->np1_max, np1);
  }
  const size_t tmp_off = (part_words + 63) & ~size_t(63);
  QFG_TRY(ctx->scratch[kScrBindPart].reserve(ctx, sizeof(int32_t) * (tmp_off + tmp_words + 64)));
  QFG_TRY(ctx->scratch[kScrBindOffsets].reserve(
      ctx, sizeof(uint32_t) * (fs_words + tot_words + bins_words + 64)));
  int32_t* part_base = ctx->scratch[kScrBindPart].as<int32_t>();
  uint32_t* fstarts = ctx->scratch[kScrBindOffsets].as<uint32_t>();
  ps->p1_tot = fstarts + fs_words;
  ps->p1_tot_words = tot_words;
  ps->p1_smem = pass_smem_bytes(ps->np1_max);
  ps->p2_smem = pass_smem_bytes(1 << sbits_max);
  QFG_CUDA(ctx, cudaFuncSetAttribute(bpart_pass1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)ps->p1_smem));
  QFG_CUDA(ctx, cudaFuncSetAttribute(bpart_pass2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)ps->p2_smem));
  // Carving cursors: bin arrays after the totals, pass-1 outputs after the
  // partitioned columns (each two-pass group's own, 16-byte aligned).
  uint32_t* bins_cur = ps->p1_tot + tot_words;
  uint32_t* tot_cur = ps->p1_tot;
  int32_t* tmp_cur = part_base + tmp_off;

  std::vector<GroupDesc> gdesc(groups.size());
  std::vector<LitDesc> ldesc;
  std::vector<SigDesc> sdesc;
  size_t off = 0, fs_off = 0;
  int64_t items = 0;
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const HostGroup& g = groups[gi];
    const int bits = gbits[gi];
    // Shard s owns partitions [s * 2^bits / S, (s + 1) * 2^bits / S).
    const uint32_t shard_lo = (uint32_t)(((int64_t)ctx->shard_index << bits) / ctx->shard_count);
    const uint32_t shard_hi = (uint32_t)(((int64_t)(ctx->shard_index + 1) << bits) / ctx->shard_count);
    PartJob job;
    BPartArgs& pa = job.pa;
    memset(&pa, 0, sizeof(pa));
    pa.two_pass = bits > kMaxSinglePassBits ? 1 : 0;
    const int cbits = gcbits[gi];
    job.sbits = bits - cbits;
    job.np1 = 2 << cbits;
    pa.ncols = (int)g.cols.size();
    for (int c = 0; c < pa.ncols; ++c) pa.cols[c] = b->columns[g.cols[c]];
    pa.n = nb;
    pa.npos = b->num_positive;
    pa.bits = bits;
    pa.cbits = cbits;
    pa.vec = 1;
    for (int c = 0; c < pa.ncols; ++c)
      if (reinterpret_cast<uintptr_t>(pa.cols[c]) % 16 != 0) pa.vec = 0;
    // The shard's partitions [shard_lo, shard_hi) cover these pass-1 hash
    // ranges; rows of other ranges are dropped before their columns move.
    pa.keep_lo = shard_lo >> job.sbits;
    pa.keep_hi = shard_hi > shard_lo ? (shard_hi - 1) >> job.sbits : 0u;
    if (shard_hi <= shard_lo) pa.keep_lo = 1u;  // an empty shard keeps nothing
    pa.out = part_base + off;
    pa.out_stride = ps->col_stride;
    pa.fstart = fstarts + fs_off;
    pa.p1_tot = tot_cur;
    tot_cur += job.np1 + 1;
    pa.p1_base = bins_cur;
    bins_cur += (size_t)ps->pgrid * job.np1;
    if (pa.two_pass) {
      const size_t chunks = (size_t)nb / kP2Chunk + (size_t)job.np1 + 1;
      pa.p1_pad = bins_cur;
      pa.p1_unp = pa.p1_pad + job.np1 + 1;
      pa.chunk_start = pa.p1_unp + job.np1 + 1;
      pa.chunk_bin = pa.chunk_start + job.np1 + 1;
      pa.h2 = pa.chunk_bin + chunks;
      bins_cur = pa.h2 + (chunks << job.sbits);
      pa.tmp_stride = ((((int64_t)nb + 3) & ~int64_t(3)) + 4 * (int64_t)job.np1);
      pa.tmp = tmp_cur;
      tmp_cur += (size_t)pa.ncols * (size_t)pa.tmp_stride;
    } else {
      pa.p1_unp = pa.fstart;  // one pass: the bin starts are the segment starts
    }
    ps->parts.push_back(job);

    GroupDesc& d = gdesc[gi];
    d.cols = pa.out;
    d.n = ps->col_stride;
    d.fstart = pa.fstart;
    d.bits = bits;
    d.sbits = job.sbits;
    d.ncols = pa.ncols;
    d.lit_begin = (int)ldesc.size();
    d.has_atoms = g.has_atoms ? 1 : 0;
    d.p_lo = shard_lo;
    d.item_begin = items;
    items += (int64_t)(shard_hi - shard_lo);
    std::vector<SigDesc> gsig;
    std::vector<int> lit_sig;
    std::vector<std::vector<int8_t>> lit_spos;
    if (mode == kModeStreamed) group_signatures(g, bind_cols, &gsig, &lit_sig, &lit_spos);
    d.sig_begin = (int)sdesc.size();
    sdesc.insert(sdesc.end(), gsig.begin(), gsig.end());
    d.sig_end = (int)sdesc.size();
    for (size_t li = 0; li < g.lits.size(); ++li) {
      const int i = g.lits[li];
      LitDesc ld;
      memset(&ld, 0, sizeof(ld));
      KeyTable* kt = tables[i];
      ld.keys = kt->keys.as<int32_t>();
      ld.stride = std::max<int64_t>(kt->num_entries, 1);
      ld.mult = kt->mult.as<int32_t>();
      ld.offsets = kt->offsets.as<uint32_t>();
      ld.nk = kt->num_keys;
      for (int q = 1; q < ld.nk; ++q)
        ld.atom_col[q] = (int8_t)(std::find(g.cols.begin(), g.cols.end(), bind_cols[i][q]) - g.cols.begin());
      ld.out = i;
      if (mode == kModeStreamed) {
        ld.sig = d.sig_begin + lit_sig[li];
        for (int q = 0; q < QFG_MAX_ARITY; ++q) ld.spos[q] = lit_spos[li][q];
      }
      ldesc.push_back(ld);
    }
    d.lit_end = (int)ldesc.size();
    off += g.cols.size() * (size_t)ps->col_stride;
    fs_off += ((size_t)2 << bits) + 1;
  }

  // Launches of at most kMaxLitsPerLaunch literals (groups never straddle a
  // launch: they are capped below that size); each launch gets a rebased copy
  // of its groups (literal and signature indices relative to the launch),
  // and all descriptors go up in one copy.
  struct Span {
    size_t gbeg, gend;
    int lit0, nl, sig0;
  };
  std::vector<Span> spans;
  std::vector<GroupDesc> sub_all;
  std::vector<LitDesc> lit_all;
  std::vector<SigDesc> sig_all;
  for (size_t gbeg = 0; gbeg < gdesc.size();) {
    size_t gend = gbeg;
    int nl = 0;
    while (gend < gdesc.size() &&
           nl + (gdesc[gend].lit_end - gdesc[gend].lit_begin) <= kMaxLitsPerLaunch) {
      nl += gdesc[gend].lit_end - gdesc[gend].lit_begin;
      ++gend;
    }
    const int lit0 = gdesc[gbeg].lit_begin;
    const int sig0 = gdesc[gbeg].sig_begin;
    const int64_t item0 = gdesc[gbeg].item_begin;
    for (size_t g = gbeg; g < gend; ++g) {
      GroupDesc sd = gdesc[g];
      sd.lit_begin -= lit0;
      sd.lit_end -= lit0;
      sd.sig_begin -= sig0;
      sd.sig_end -= sig0;
      sd.item_begin -= item0;
      sub_all.push_back(sd);
    }
    for (int l = lit0; l < lit0 + nl; ++l) {
      LitDesc ld = ldesc[l];
      ld.sig -= sig0;
      lit_all.push_back(ld);
    }
    spans.push_back({gbeg, gend, lit0, nl, sig0});
    gbeg = gend;
  }
  for (const SigDesc& sd : sdesc) sig_all.push_back(sd);
  std::vector<BPartArgs> part_all;
  for (const PartJob& j : ps->parts) part_all.push_back(j.pa);
  const size_t gbytes = sizeof(GroupDesc) * sub_all.size();
  const size_t lbytes = sizeof(LitDesc) * lit_all.size();
  const size_t sbytes = sizeof(SigDesc) * sig_all.size();
  const size_t pbytes = sizeof(BPartArgs) * part_all.size();
  ps->blob.resize(gbytes + lbytes + sbytes + pbytes);
  memcpy(ps->blob.data(), sub_all.data(), gbytes);
  memcpy(ps->blob.data() + gbytes, lit_all.data(), lbytes);
  if (sbytes) memcpy(ps->blob.data() + gbytes + lbytes, sig_all.data(), sbytes);
  memcpy(ps->blob.data() + gbytes + lbytes + sbytes, part_all.data(), pbytes);
  QFG_TRY(ctx->scratch[kScrLits].reserve(ctx, ps->blob.size() + 64));
  // Work units: at most one per item plus one per `piece` entries; entry
  // records (tiled path): every entry once, each unit's block padded to 4.
  const uint32_t piece = mode == kModeStreamed ? (uint32_t)kSEntries : (uint32_t)kChunk;
  std::vector<int64_t> caps, ecaps;
  int64_t max_cap = 1, max_ecap = 4;
  for (const Span& S : spans) {
    int64_t cap = 1, ecap = 4;
    for (size_t g = S.gbeg; g < S.gend; ++g) {
      const int bits = gbits[g];
      cap += (int64_t)((((int64_t)(ctx->shard_index + 1) << bits) / ctx->shard_count) -
                       (((int64_t)ctx->shard_index << bits) / ctx->shard_count));
    }
    for (int l = S.lit0; l < S.lit0 + S.nl; ++l) {
      cap += ldesc[l].stride / piece + 1;
      ecap += ldesc[l].stride;
    }
    ecap += 4 * cap;
    ecap = (ecap + 3) & ~int64_t(3);
    if (mode == kModeStreamed) ecap = 4;  // no entry records
    if (cap > (int64_t)UINT32_MAX || ecap > (int64_t)UINT32_MAX)
      return set_error(ctx, QFG_ERR_INVALID, "too many work units");
    caps.push_back(cap);
    ecaps.push_back(ecap);
    max_cap = std::max(max_cap, cap);
    max_ecap = std::max(max_ecap, ecap);
  }
  // Units, then (tiled path) as many evaluation units at most.
  QFG_TRY(ctx->scratch[kScrWork].reserve(ctx, sizeof(WorkUnit) * 2 * (size_t)max_cap));
  QFG_TRY(ctx->scratch[kScrEntries].reserve(ctx, sizeof(int32_t) * 5 * (size_t)max_ecap));
  EntryRecs recs;
  {
    int32_t* eb = ctx->scratch[kScrEntries].as<int32_t>();
    recs.k0 = eb;
    recs.kA = eb + max_ecap;
    recs.kB = eb + 2 * max_ecap;
    recs.meta = reinterpret_cast<uint32_t*>(eb + 3 * max_ecap);
    recs.mult = eb + 4 * max_ecap;
  }
  GroupDesc* gdev = ctx->scratch[kScrLits].as<GroupDesc>();
  LitDesc* ldev = reinterpret_cast<LitDesc*>(gdev + sub_all.size());
  SigDesc* sdev = reinterpret_cast<SigDesc*>(ldev + lit_all.size());
  BPartArgs* pdev = reinterpret_cast<BPartArgs*>(sdev + sig_all.size());
  ps->blob_dev = gdev;
  ps->part_args_dev = pdev;
  ps->counter = reinterpret_cast<unsigned int*>(pdev + part_all.size());
  for (size_t si = 0; si < spans.size(); ++si) {
    const Span& S = spans[si];
    LaunchJob L;
    L.streamed = mode == kModeStreamed;
    EvalArgs& ea = L.ea;
    memset(&ea, 0, sizeof(ea));
    ea.groups = gdev + S.gbeg;
    ea.num_groups = (int)(S.gend - S.gbeg);
    ea.lits = ldev + S.lit0;
    ea.num_lits = S.nl;
    ea.sigs = sdev + S.sig0;
    int64_t total = 0;
    for (size_t g = S.gbeg; g < S.gend; ++g) {
      const int bits = gbits[g];
      total += (int64_t)((((int64_t)(ctx->shard_index + 1) << bits) / ctx->shard_count) -
                         (((int64_t)ctx->shard_index << bits) / ctx->shard_count));
    }
    ea.total_items = total;
    ea.work_counter = ps->counter;
    ea.units = ctx->scratch[kScrWork].as<WorkUnit>();
    ea.eunits = L.streamed ? nullptr : ea.units + max_cap;
    ea.unit_count = ps->counter + 1;
    ea.unit_cap = (uint32_t)caps[si];
    ea.entry_cap = (uint32_t)ecaps[si];
    ea.rec = recs;
    ea.error_flag = ctx->error_flag;
    ea.wait_limit = ctx->wait_limit;
    ea.withhold_copies = ctx->withhold_copies ? 1 : 0;
    ea.counts = counts;
    ea.piece = piece;
    ea.row_chunk = L.streamed ? 0xffffffffu : 0u;  // streamed: a unit streams all its item's rows
    // Tiled path: the evaluation kernel reads the entry records the gather
    // kernel writes (coalesced, one round trip per unit).
    ea.records = L.streamed ? 0 : 1;
    ea.max_cols = 1;
    for (size_t g = S.gbeg; g < S.gend; ++g) ea.max_cols = std::max(ea.max_cols, gdesc[g].ncols);
    int per_sm = 0;
    if (L.streamed) {
      L.smem = stream_smem_bytes(S.nl);
      QFG_CUDA(ctx, cudaFuncSetAttribute(stream_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)L.smem));
      QFG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stream_eval_kernel,
                                                                 kSThreads, L.smem));
    } else {
      L.smem = eval_smem_bytes(S.nl, ea.max_cols);
      QFG_CUDA(ctx, cudaFuncSetAttribute(eval_batched_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
      QFG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, eval_batched_kernel,
                                                                 kEvalThreads, L.smem));
    }
    L.grid = ctx->num_sms * std::max(per_sm, 1);
    // One wave of resident gather blocks: each block strides over the units,
    // so blocks beyond what the SMs hold at once would run as a second wave.
    int gather_per_sm = 0;
    QFG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gather_per_sm, gather_entries_kernel,
                                                                32 * kGatherWarps, 0));
    L.gather_grid = ctx->num_sms * std::max(gather_per_sm, 1);
    L.plan_grid = (int)std::max<int64_t>(
        1, std::min<int64_t>((ea.total_items + 255) / 256, (int64_t)ctx->num_sms * 8));
    ps->launches.push_back(L);
  }
  return QFG_OK;
}

int enqueue_step(Ctx* ctx, const PreparedStep* pps) {
  const PreparedStep& ps = *pps;
  if (ps.parts.empty()) return QFG_OK;
  QFG_TRY(stage_begin(ctx, QFG_STAGE_BIND_PARTITION));
  // One launch of each partition kernel covers every literal group
  // (blockIdx.y = group); groups with one pass skip the pass-2 kernels.
  const unsigned G = (unsigned)ps.parts.size();
  const BPartArgs* A = ps.part_args_dev;
  QFG_CUDA(ctx, cudaMemsetAsync(ps.p1_tot, 0, sizeof(uint32_t) * ps.p1_tot_words, ctx->stream));
  bpart_hist_kernel<<<dim3(ps.pgrid, G), kPartThreads, 0, ctx->stream>>>(A);
  QFG_LAUNCHED(ctx);
  pad_scan_kernel<<<G, 512, 0, ctx->stream>>>(A);
  QFG_LAUNCHED(ctx);
  bpart_pass1_kernel<<<dim3(ps.pgrid, G), kPassThreads, ps.p1_smem, ctx->stream>>>(A);
  QFG_LAUNCHED(ctx);
  if (ps.any_two_pass) {
    bpart_p2hist_kernel<<<dim3(ps.pgrid * 2, G), 512, 0, ctx->stream>>>(A);
    QFG_LAUNCHED(ctx);
    bpart_p2scan_kernel<<<dim3((unsigned)ps.np1_max, G), 512, 0, ctx->stream>>>(A);
    QFG_LAUNCHED(ctx);
    bpart_pass2_kernel<<<dim3(ps.pgrid, G), kPassThreads, ps.p2_smem, ctx->stream>>>(A);
    QFG_LAUNCHED(ctx);
  }
  QFG_TRY(stage_end(ctx, QFG_STAGE_BIND_PARTITION));
  for (const LaunchJob& L : ps.launches) {
    QFG_TRY(stage_begin(ctx, QFG_STAGE_UNIT_PLAN));
    QFG_CUDA(ctx, cudaMemsetAsync(ps.counter, 0, 4 * sizeof(unsigned int), ctx->stream));
    plan_units_kernel<<<L.plan_grid, 256, 0, ctx->stream>>>(L.ea);
    QFG_LAUNCHED(ctx);
    if (L.ea.records) {
      gather_entries_kernel<<<L.gather_grid, 32 * kGatherWarps, 0, ctx->stream>>>(L.ea);
      QFG_LAUNCHED(ctx);
    }
    QFG_TRY(stage_end(ctx, QFG_STAGE_UNIT_PLAN));
    QFG_TRY(stage_begin(ctx, QFG_STAGE_EVALUATE));
    if (L.streamed)
      stream_eval_kernel<<<L.grid, kSThreads, L.smem, ctx->stream>>>(L.ea);
    else
      eval_batched_kernel<<<L.grid, kEvalThreads, L.smem, ctx->stream>>>(L.ea);
    QFG_LAUNCHED(ctx);
    QFG_TRY(stage_end(ctx, QFG_STAGE_EVALUATE));
  }
  return QFG_OK;
}

PreparedStep* prepared_step_new() { return new PreparedStep(); }
void prepared_step_free(PreparedStep* ps) { delete ps; }
bool prepared_is_empty(const PreparedStep* ps) { return ps->parts.empty(); }

int upload_prepared(Ctx* ctx, const PreparedStep* ps, bool sync) {
  if (ps->blob.empty()) return QFG_OK;
  if (!sync) return upload_small(ctx, ps->blob_dev, ps->blob.data(), ps->blob.size());
  QFG_CUDA(ctx, cudaMemcpy(ps->blob_dev, ps->blob.data(), ps->blob.size(), cudaMemcpyHostToDevice));
  return QFG_OK;
}

int step_scratch_bytes(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                       int64_t* bytes) {
  *bytes = 0;
  const int64_t nb = b->num_positive + b->num_negative;
  if (n == 0 || nb == 0) return QFG_OK;
  const int mode = step_mode(ctx, nb);
  StepPlan plan;
  QFG_TRY(plan_step(ctx, n, lits, &plan, mode == kModeStreamed ? kSMaxSigs : 0));
  int64_t words = 256, units = 0, entries = 0;
  for (auto& g : plan.groups) {
    int64_t ge = 0;
    for (int i : g.lits) ge += plan.tables[i]->num_entries;
    const int bits = group_bits(ctx, mode, nb, ge);
    words += (int64_t)g.cols.size() * (nb + 4) + (2 << bits) + 1;
    const bool two = bits > kMaxSinglePassBits;
    const int cb = two ? coarse_bits(ctx, nb, bits) : bits;
    const int64_t np1 = 2 << cb;
    words += np1 + 1 + np1 * ctx->num_sms;
    if (two) {
      // each two-pass group keeps its own pass-1 output and bin arrays
      const int64_t chunks = nb / kP2Chunk + np1 + 1;
      words += (int64_t)g.cols.size() * (nb + 4 + 4 * np1) + 3 * (np1 + 1) + chunks +
               (chunks << (bits - cb));
    }
    units += (int64_t)1 << bits;
  }
  const int64_t piece = mode == kModeStreamed ? kSEntries : kChunk;
  for (KeyTable* kt : plan.tables) {
    units += kt->num_entries / piece + 1;
    entries += std::max<int64_t>(kt->num_entries, 1);
  }
  words += (mode == kModeStreamed ? 1 : 2) * units * (int64_t)(sizeof(WorkUnit) / 4) +
           (mode == kModeStreamed ? 20 : 5 * (entries + 4 * units + 8));
  *bytes = 4 * words + (int64_t)(sizeof(GroupDesc) + sizeof(LitDesc) + sizeof(SigDesc)) * n +
           32 * (int64_t)n;
  return QFG_OK;
}

int evaluate_batched(Ctx* ctx, const qfg_bindings* b, int32_t n, const qfg_literal* lits,
                     unsigned long long* counts) {
  PreparedStep ps;
  QFG_TRY(prepare_step(ctx, b, n, lits, counts, &ps));
  if (ps.parts.empty()) return QFG_OK;
  QFG_TRY(upload_prepared(ctx, &ps, false));
  return enqueue_step(ctx, &ps);
}

int step_partition_bits(Ctx* ctx, int64_t nb) {
  // The graph cache key: the tiled path's bits, the evaluation mode and the
  // streamed path's bits offset.
  return auto_group_bits(ctx, nb) | (step_mode(ctx, nb) << 8) | ((stream_bias(ctx, nb) + 16) << 12);
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
  if (ctx->use_graphs)
    QFG_TRY(evaluate_step_cached(ctx, b, n, lits, dev));
  else
    QFG_TRY(evaluate_batched(ctx, b, n, lits, dev));
  return counts_end(ctx, n, counts, flags, dev);
}

extern "C" int qfg_autotune_step(qfg_ctx* c, const qfg_bindings* b, int32_t n,
                                 const qfg_literal* lits, int32_t* best_bits, int32_t* best_pass1_bits,
                                 double* best_ms) {
  if (c == nullptr || b == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  QFG_TRY(validate_literals(ctx, b, n, lits));
  const int64_t nb = b->num_positive + b->num_negative;
  const int saved_bits = ctx->eval_bits, saved_cbits = ctx->eval_cbits, saved_mode = ctx->eval_mode;
  const bool saved_tune = ctx->autotune, saved_timing = ctx->stage_timing;
  ctx->eval_bits = 0;
  ctx->autotune = false;
  const int base = auto_group_bits(ctx, nb);
  // Trials: the tiled path at partition bits around its automatic choice,
  // with both splits of the bits between two passes; the streamed path with
  // its per-group bits offset by -1 .. +2.
  struct Trial {
    int mode, bits, cbits, bias;
  };
  std::vector<Trial> trials;
  for (int cand = std::max(1, base - 2); cand <= std::min(kMaxPartitionBits, base + 1); ++cand) {
    const int cb_lo = cand > kMaxSinglePassBits ? kDefaultCoarseBits : 0;
    const int cb_hi = cand > kMaxSinglePassBits ? kMaxCoarseBits : 0;
    for (int cb = cb_lo; cb <= cb_hi; ++cb)
      if (cb == 0 || cand - cb <= kMaxSubBits) trials.push_back({kModeTiled, cand, cb, 0});
  }
  for (int bias = -1; bias <= 2; ++bias) trials.push_back({kModeStreamed, 0, 0, bias});
  QFG_TRY(ctx->scratch[kScrCounts].reserve(ctx, sizeof(int64_t) * 4 * (size_t)std::max(n, 1)));
  unsigned long long* dev = ctx->scratch[kScrCounts].as<unsigned long long>();
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = QFG_OK;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    st = cuda_error(ctx, cudaGetLastError(), "cudaEventCreate");
  Trial best{kModeTiled, base, 0, 0};
  float best_t = -1.0f;
  ctx->stage_timing = false;
  for (const Trial& t : trials) {
    if (st != QFG_OK) break;
    ctx->eval_mode = t.mode;
    ctx->eval_bits = t.bits;
    ctx->eval_cbits = t.cbits;
    ctx->stream_bias = t.bias;
    st = evaluate_batched(ctx, b, n, lits, dev);  // sizes the scratch of this setting
    if (st != QFG_OK) break;
    if (cudaEventRecord(e0, ctx->stream) != cudaSuccess) {
      st = cuda_error(ctx, cudaGetLastError(), "cudaEventRecord");
      break;
    }
    for (int rep = 0; rep < 2 && st == QFG_OK; ++rep) st = evaluate_batched(ctx, b, n, lits, dev);
    if (st != QFG_OK) break;
    float ms = 0.0f;
    if (cudaEventRecord(e1, ctx->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      st = cuda_error(ctx, cudaGetLastError(), "timing");
      break;
    }
    ms *= 0.5f;
    if (best_t < 0.0f || ms < best_t) {
      best_t = ms;
      best = t;
    }
  }
  ctx->eval_cbits = saved_cbits;
  ctx->eval_mode = saved_mode;
  ctx->stream_bias = 0;
  if (e0 != nullptr) cudaEventDestroy(e0);
  if (e1 != nullptr) cudaEventDestroy(e1);
  ctx->eval_bits = saved_bits;
  ctx->autotune = saved_tune;
  ctx->stage_timing = saved_timing;
  if (st != QFG_OK) return st;
  if (best.mode == kModeTiled) ctx->tuned_bits[size_class(nb)] = std::make_pair(best.bits, best.cbits);
  ctx->tuned_mode[size_class(nb)] = std::make_pair(best.mode, best.bias);
  graph_cache_clear(ctx);
  if (best_bits != nullptr) *best_bits = best.mode == kModeTiled ? best.bits : 0;
  if (best_pass1_bits != nullptr) *best_pass1_bits = best.mode == kModeTiled ? best.cbits : best.bias;
  if (best_ms != nullptr) *best_ms = best_t;
  return QFG_OK;
}

extern "C" int qfg_autotune_choice(const qfg_ctx* c, int64_t num_rows, int32_t* mode, int32_t* bits,
                                   int32_t* pass1_bits, int32_t* bias) {
  if (c == nullptr || mode == nullptr || bits == nullptr || pass1_bits == nullptr || bias == nullptr)
    return QFG_ERR_INVALID;
  const Ctx* ctx = &c->impl;
  const int cls = size_class(num_rows);
  *mode = *bits = *pass1_bits = *bias = 0;
  auto m = ctx->tuned_mode.find(cls);
  if (m == ctx->tuned_mode.end()) return QFG_OK;
  *mode = m->second.first;
  if (*mode == kModeStreamed) {
    *bias = m->second.second;
  } else {
    auto t = ctx->tuned_bits.find(cls);
    if (t != ctx->tuned_bits.end()) {
      *bits = t->second.first;
      *pass1_bits = t->second.second;
    }
  }
  return QFG_OK;
}

extern "C" int qfg_step_traffic(qfg_ctx* c, const qfg_bindings* b, int32_t n,
                                const qfg_literal* lits, int64_t* bytes) {
  if (c == nullptr || b == nullptr || bytes == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  QFG_TRY(validate_literals(ctx, b, n, lits));
  for (int s = 0; s < QFG_NUM_STAGES; ++s) bytes[s] = 0;
  const int64_t nb = b->num_positive + b->num_negative;
  if (n == 0) return QFG_OK;
  const int mode = step_mode(ctx, nb);
  StepPlan plan;
  QFG_TRY(plan_step(ctx, n, lits, &plan, mode == kModeStreamed ? kSMaxSigs : 0));
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
    int64_t ge = 0;
    for (int i : g.lits) ge += plan.tables[i]->num_entries;
    const int bits = group_bits(ctx, mode, nb, ge);
    // Partition: each carried column read once and written once.
    bytes[QFG_STAGE_BIND_PARTITION] += 8 * nb * (int64_t)g.cols.size();
    // Evaluation: the partitioned columns read once, four int64 counts
    // written per literal.  Work units: each literal's offsets pair per
    // partition read.  Tiled path: entry records written once (join key, two
    // further keys, meta, multiplicity) after the key tables' keys and
    // multiplicities were read, and read once by the evaluation kernel.
    // Streamed path: the evaluation kernel reads the key tables' keys and
    // multiplicities itself.
    bytes[QFG_STAGE_EVALUATE] += 4 * nb * (int64_t)g.cols.size();
    for (int i : g.lits) {
      const int64_t ne = plan.tables[i]->num_entries;
      const int64_t tab = 4 * ne * (plan.tables[i]->num_keys + 1);
      bytes[QFG_STAGE_UNIT_PLAN] += 8 * ((int64_t)1 << bits);
      if (mode == kModeStreamed) {
        bytes[QFG_STAGE_EVALUATE] += tab + 32;
      } else {
        bytes[QFG_STAGE_UNIT_PLAN] += tab + 20 * ne;
        bytes[QFG_STAGE_EVALUATE] += 20 * ne + 32;
      }
    }
  }
  // The plain path partitions each distinct join column once (value +
  // tuple id, 12 bytes a row); per literal it reads the binding partition
  // (8 bytes a row) and the relation partition (8 bytes a tuple), and the
  // join pairs' atom columns are gathered.
  std::map<int, int> join_cols;
  for (int i = 0; i < n; ++i) join_cols[lits[i].vars[lits[i].join_pos]] = 1;
  bytes[QFG_STAGE_PER_LITERAL] += 12 * nb * (int64_t)join_cols.size();
  for (int i = 0; i < n; ++i) {
    Relation* rel = nullptr;
    QFG_TRY(find_relation(ctx, lits[i].relation_id, &rel));
    bytes[QFG_STAGE_PER_LITERAL] += 8 * nb + 8 * rel->num_tuples + 32;
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
