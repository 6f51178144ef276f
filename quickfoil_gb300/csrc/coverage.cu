// coverage.cu -- coverage of a literal appended to the building clause, and
// the uncovered-example compaction.
//
// Coverage (QuickFoil::ComputeCoverageOnUncoveredData, learner/QuickFoil.cpp:
// 471-573; LiteralSelector::ComputeCoveredPositives, learner/LiteralSelector.
// cpp:150-210) chains two semi-joins per label side: binding rows whose bound
// arguments occur in the relation, projected onto the target variables
// (binding columns 0..k-1), against the examples (uncovered positives, or the
// original negatives).  The reference takes both through hash tables of tuple
// ids (operations/BuildHashTable.cpp:152-189); here only membership is kept.
//
// The relation side is a key set over the bound argument positions, built
// once and kept on the relation.  For one or two bound arguments its slots
// hold the key tuple itself (64 bits), so a binding row's test is one load
// from a table that stays in L2; each thread tests several rows at a time
// with their loads in flight together.  Three or more bound arguments use the
// row-owner form of keysets.cuh.  A relation with at most 2^18 distinct key
// tuples also gets a 2^20-bit filter (a bit per hashed tuple, 128 KiB) that
// every block keeps in shared memory: most binding rows fail it and never
// touch L2, so the pass streams the binding columns at HBM speed.  Larger
// relations, and the example tables, get filters of about 8 bits a tuple in
// global memory, small enough to stay in L2: a row then costs one random L2
// read instead of a DRAM miss in a key set of tens of megabytes.
//
// The second semi-join is built on the smaller of its two sides:
//  * examples (usually: a few million examples against tens of millions of
//    binding rows): the examples go into a key set (inline tuples for one or
//    two target columns, row owners beyond); one pass over the binding rows
//    flags the slot (or representative example) of every passing row's
//    target tuple; each example then reads its flag.  A prepared example
//    table (qfg_examples) keeps that key set between calls: the original
//    negatives for a whole run, the uncovered positives for a clause.
//  * binding rows: passing rows insert their target tuple into a key set and
//    the examples look theirs up.
// Either gives a bit per example (the reference's SemiJoinChunk bit vectors,
// operations/SemiJoin.hpp:25-37, concatenated) and the covered count.
//
// The uncovered-example compaction (learner/QuickFoil.cpp:612-708) keeps the
// rows whose coverage bit is clear, in order: per 2048-row tile a kept count,
// an exclusive scan of the tile counts, then each tile writes its rows at its
// offset, a warp ballot ranking the rows of every 32-row word.
#include <cstring>

#include "keysets.cuh"

struct qfg_examples {
  int32_t num_columns = 0;
  int64_t num_rows = 0;
  std::vector<const int32_t*> columns;  // borrowed device columns
  uint32_t mask = 0;                    // key-set slots - 1
  qfg::DevBuf storage;                  // the example key set (coverage.cu: ExSet)
};

namespace qfg {

namespace {

constexpr unsigned long long kEmpty64 = ~0ull;
constexpr int kRowsPerThread = 8;  // rows a thread keeps in flight (key-set path)

// Inline key of one or two int32 keys; (-1, -1) encodes as kEmpty64 and is
// recorded in the extra slot mask + 1 instead.
template <int NB>
__device__ __forceinline__ unsigned long long inline_key(const KeyCols& k, int64_t r) {
  if constexpr (NB == 1) {
    return (unsigned long long)(uint32_t)k.c[0][r];
  } else {
    return ((unsigned long long)(uint32_t)k.c[0][r] << 32) | (uint32_t)k.c[1][r];
  }
}

// The same key read with an evict-first hint: the binding columns stream
// through once and should not push the relation's key set out of L2.
template <int NB>
__device__ __forceinline__ unsigned long long inline_key_streamed(const KeyCols& k, int64_t r) {
  if constexpr (NB == 1) {
    return (unsigned long long)(uint32_t)__ldcs(k.c[0] + r);
  } else {
    return ((unsigned long long)(uint32_t)__ldcs(k.c[0] + r) << 32) | (uint32_t)__ldcs(k.c[1] + r);
  }
}

__device__ __forceinline__ uint32_t hash64(unsigned long long v) {
  return mix32((uint32_t)v ^ mix32((uint32_t)(v >> 32) + 0x9e3779b9u));
}

// Inline key set: slots[mask + 1], then the (-1, -1) marker, then the
// count of distinct tuples.
template <int NB>
__global__ void inline_keyset_insert_kernel(KeyCols keys, int64_t n,
                                            unsigned long long* __restrict__ table, uint32_t mask) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long v = inline_key<NB>(keys, r);
    if (v == kEmpty64) {
      table[(size_t)mask + 1] = 1ull;
      continue;
    }
    uint32_t slot = hash64(v) & mask;
    for (uint32_t p = 0; p <= mask; ++p) {
      unsigned long long o = table[slot];  // an occupied slot never changes
      if (o == v) break;
      if (o == kEmpty64) o = atomicCAS(&table[slot], kEmpty64, v);
      if (o == kEmpty64) atomicAdd(&table[(size_t)mask + 2], 1ull);
      if (o == kEmpty64 || o == v) break;
      slot = (slot + 1) & mask;
    }
  }
}

constexpr int kFilterBits = 20;                         // 2^20-bit filter, 128 KiB
constexpr int kFilterWords = (1 << kFilterBits) / 32;
constexpr int64_t kFilterMaxKeys = int64_t(1) << 18;    // false positives below 23%

// Filter bit of a key tuple among 2^bits: a multiplicative hash (two
// multiplies), cheap enough for every binding row; independent of the key
// set's slot hash.
__device__ __forceinline__ uint32_t filter_bit(unsigned long long v, int bits = kFilterBits) {
  return (((uint32_t)v * 0x9e3779b1u) ^ ((uint32_t)(v >> 32) * 0x85ebca77u)) >> (32 - bits);
}

// A relation with more distinct tuples than the shared-memory filter takes
// gets a filter of about 8 bits per tuple in global memory (at most 2^28
// bits): small enough to stay in L2, so most binding rows whose key is not
// in the relation skip the key set's (larger, DRAM-resident) slots.
constexpr int kMaxGlobalFilterBits = 28;

__global__ void filter_build_kernel(const unsigned long long* __restrict__ table, uint32_t mask,
                                    uint32_t* __restrict__ filter, int bits) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s <= (int64_t)mask;
       s += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long t = table[s];
    if (t == kEmpty64) continue;
    const uint32_t b = filter_bit(t, bits);
    atomicOr(&filter[b >> 5], 1u << (b & 31));
  }
}

// Continues a lookup of v (not kEmpty64) from `slot`.
__device__ __forceinline__ bool inline_keyset_probe(const unsigned long long* __restrict__ table,
                                                    uint32_t mask, unsigned long long v,
                                                    uint32_t slot) {
  for (uint32_t p = 0; p <= mask; ++p) {
    const unsigned long long t = table[slot];
    if (t == v) return true;
    if (t == kEmpty64) return false;
    slot = (slot + 1) & mask;
  }
  return false;
}

// The relation side of a coverage: inline keys (1-2 bound arguments) or row
// owners (3 or more).
struct RelSet {
  const unsigned long long* table;  // inline form
  const int32_t* owner;             // owner form
  uint32_t mask;
  KeyCols keys;                     // the relation's bound-argument columns
  const uint32_t* filter;           // hashed-bit filter for shared memory (inline form), or null
  const uint32_t* gfilter;          // larger filter read from global memory, or null
  int gbits;
};

// The global filter's verdict on a key tuple (true when there is none).
__device__ __forceinline__ bool gfilter_pass(const RelSet& rs, unsigned long long v) {
  if (rs.gfilter == nullptr) return true;
  const uint32_t b = filter_bit(v, rs.gbits);
  return (__ldg(rs.gfilter + (b >> 5)) >> (b & 31)) & 1u;
}

// NB: bound-argument count, 1-3 fixed, 0 = 4 or more (run time).
template <int NB>
__device__ __forceinline__ bool rel_has(const RelSet& rs, const KeyCols& bound, int64_t r) {
  if constexpr (NB == 1 || NB == 2) {
    const unsigned long long v = inline_key<NB>(bound, r);
    if (v == kEmpty64) return rs.table[(size_t)rs.mask + 1] != 0ull;
    return inline_keyset_probe(rs.table, rs.mask, v, hash64(v) & rs.mask);
  } else {
    return keyset_find<NB>(rs.keys, rs.owner, rs.mask, bound, r) >= 0;
  }
}

// Finds v (not kEmpty64) in an inline key set; returns its slot or -1.
__device__ __forceinline__ int64_t inline_keyset_slot(const unsigned long long* __restrict__ table,
                                                      uint32_t mask, unsigned long long v) {
  uint32_t slot = hash64(v) & mask;
  for (uint32_t p = 0; p <= mask; ++p) {
    const unsigned long long t = table[slot];
    if (t == v) return slot;
    if (t == kEmpty64) return -1;
    slot = (slot + 1) & mask;
  }
  return -1;
}

// The example side of a coverage as the kernels see it.  Inline form (one
// or two target columns): slots hold the tuple, flag[slot] marks it covered,
// flag[mask + 1] stands for the tuple (-1, -1); rep[i] is example i's slot.
// Owner form: slots hold the representative example row, flag[row] marks
// it, rep[i] is example i's representative.
struct ExSet {
  KeyCols keys;
  const unsigned long long* table;
  const int32_t* owner;
  uint32_t mask;
  const int32_t* rep;
  uint8_t* flag;
  // Inline form: a filter of the example tuples (about 8 bits each, in
  // global memory small enough for L2), so most passing binding rows whose
  // tuple is no example skip the table's slots.
  const uint32_t* efilter;
  int ebits;
};

// Marks the example tuple of binding row r (target columns) as covered.
template <int K>
__device__ __forceinline__ void ex_mark(const ExSet& e, const KeyCols& target, int64_t r) {
  if constexpr (K == 1 || K == 2) {
    const unsigned long long v = inline_key<K>(target, r);
    if (v != kEmpty64) {
      const uint32_t b = filter_bit(v, e.ebits);
      if (!((__ldg(e.efilter + (b >> 5)) >> (b & 31)) & 1u)) return;
    }
    const int64_t s = v == kEmpty64 ? (int64_t)e.mask + 1 : inline_keyset_slot(e.table, e.mask, v);
    if (s >= 0 && e.flag[s] == 0) e.flag[s] = 1;
  } else {
    const int32_t o = keyset_find<K>(e.keys, e.owner, e.mask, target, r);
    if (o >= 0 && e.flag[o] == 0) e.flag[o] = 1;
  }
}

// The example tuples' filter bits (the (-1, -1) tuple has its own flag and
// is never filtered).
template <int K>
__global__ void example_filter_kernel(KeyCols keys, int64_t n, uint32_t* __restrict__ filter,
                                      int bits) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long v = inline_key<K>(keys, i);
    if (v == kEmpty64) continue;
    const uint32_t b = filter_bit(v, bits);
    atomicOr(&filter[b >> 5], 1u << (b & 31));
  }
}

template <int K>
__global__ void inline_example_insert_kernel(KeyCols keys, int64_t n,
                                             unsigned long long* __restrict__ table, uint32_t mask,
                                             int32_t* __restrict__ rep) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long v = inline_key<K>(keys, i);
    if (v == kEmpty64) {
      rep[i] = (int32_t)(mask + 1);
      continue;
    }
    uint32_t slot = hash64(v) & mask;
    for (uint32_t p = 0; p <= mask; ++p) {
      unsigned long long o = table[slot];  // an occupied slot never changes
      if (o == kEmpty64) o = atomicCAS(&table[slot], kEmpty64, v);
      if (o == kEmpty64 || o == v) break;
      slot = (slot + 1) & mask;
    }
    rep[i] = (int32_t)slot;
  }
}

// The pass over the binding rows for three or more bound arguments (the
// relation's key set in row-owner form): passing rows flag their target
// tuple; kRowsPerThread rows a thread.
template <int NB, int K>
__global__ void coverage_flag_kernel(RelSet rs, KeyCols bound, KeyCols target, int64_t n,
                                     ExSet ex) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; base < n;
       base += stride * kRowsPerThread) {
    bool pass[kRowsPerThread];
#pragma unroll
    for (int u = 0; u < kRowsPerThread; ++u) {
      const int64_t r = base + u * stride;
      pass[u] = r < n && rel_has<NB>(rs, bound, r);
    }
#pragma unroll
    for (int u = 0; u < kRowsPerThread; ++u)
      if (pass[u]) ex_mark<K>(ex, target, base + u * stride);
  }
}

// The pass for one or two bound arguments (inline key set).  Filtered: one
// block of kFilterThreads a SM keeps the relation's filter in shared memory
// and only rows whose bit is set probe the key set.  Unfiltered: every row
// probes.  Each thread keeps ROWS rows in flight: their key loads, then
// their first key-set loads, go out together.
constexpr int kFilterThreads = 1024;
constexpr int kFilterRows = 8;

template <int NB, int K, bool FILTERED, int ROWS>
__global__ void __launch_bounds__(FILTERED ? kFilterThreads : 256)
coverage_scan_kernel(RelSet rs, KeyCols bound, KeyCols target, int64_t n, ExSet ex) {
  extern __shared__ uint4 filter_smem4[];
  uint32_t* sfilter = reinterpret_cast<uint32_t*>(filter_smem4);
  if constexpr (FILTERED) {
    const uint4* f4 = reinterpret_cast<const uint4*>(rs.filter);
    for (int i = threadIdx.x; i < kFilterWords / 4; i += blockDim.x) filter_smem4[i] = f4[i];
    __syncthreads();
  }
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; base < n;
       base += stride * ROWS) {
    unsigned long long v[ROWS], t[ROWS];
    bool maybe[ROWS];
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      const int64_t r = base + u * stride;
      v[u] = r < n ? inline_key_streamed<NB>(bound, r) : 0ull;
    }
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      maybe[u] = base + u * stride < n;
      if constexpr (FILTERED) {
        if (maybe[u] && v[u] != kEmpty64) {
          const uint32_t b = filter_bit(v[u]);
          maybe[u] = (sfilter[b >> 5] >> (b & 31)) & 1u;
        }
      } else {
        if (maybe[u] && v[u] != kEmpty64) maybe[u] = gfilter_pass(rs, v[u]);
      }
      t[u] = maybe[u] && v[u] != kEmpty64 ? rs.table[hash64(v[u]) & rs.mask] : kEmpty64;
    }
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      if (!maybe[u]) continue;
      bool pass;
      if (v[u] == kEmpty64) {
        pass = rs.table[(size_t)rs.mask + 1] != 0ull;
      } else if (t[u] == v[u] || t[u] == kEmpty64) {
        pass = t[u] == v[u];
      } else {
        pass = inline_keyset_probe(rs.table, rs.mask, v[u], (hash64(v[u]) + 1) & rs.mask);
      }
      if (pass) ex_mark<K>(ex, target, base + u * stride);
    }
  }
}

// One bound argument: the key column is read four rows at a time by 16-byte
// loads (rows [h, h + 4 nq) with h the first 16-byte aligned row); the at
// most 3 rows before h and after the last quad are taken by the first
// threads of the grid.  QUADS quads a thread are in flight together.
template <bool FILTERED>
__device__ __forceinline__ bool scan1_test(const RelSet& rs, const uint32_t* sfilter,
                                           uint32_t key) {
  const unsigned long long v = key;
  if constexpr (FILTERED) {
    const uint32_t b = filter_bit(v);
    if (!((sfilter[b >> 5] >> (b & 31)) & 1u)) return false;
  } else {
    if (!gfilter_pass(rs, v)) return false;
  }
  return inline_keyset_probe(rs.table, rs.mask, v, hash64(v) & rs.mask);
}

template <int K, bool FILTERED, int QUADS>
__global__ void __launch_bounds__(FILTERED ? kFilterThreads : 256)
coverage_scan1_kernel(RelSet rs, KeyCols bound, KeyCols target, int64_t n, ExSet ex) {
  extern __shared__ uint4 filter_smem4[];
  uint32_t* sfilter = reinterpret_cast<uint32_t*>(filter_smem4);
  if constexpr (FILTERED) {
    const uint4* f4 = reinterpret_cast<const uint4*>(rs.filter);
    for (int i = threadIdx.x; i < kFilterWords / 4; i += blockDim.x) filter_smem4[i] = f4[i];
    __syncthreads();
  }
  const int32_t* col = bound.c[0];
  const int64_t h = min(n, (int64_t)((4 - (((uintptr_t)col >> 2) & 3)) & 3));
  const int64_t nq = (n - h) / 4;
  const int4* q4 = reinterpret_cast<const int4*>(col + h);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (int64_t base = gtid; base < nq; base += stride * QUADS) {
    int4 x[QUADS];
#pragma unroll
    for (int u = 0; u < QUADS; ++u) {
      const int64_t qi = base + u * stride;
      x[u] = qi < nq ? __ldcs(q4 + qi) : make_int4(0, 0, 0, 0);
    }
#pragma unroll
    for (int u = 0; u < QUADS; ++u) {
      const int64_t qi = base + u * stride;
      if (qi >= nq) continue;
      const int64_t r = h + 4 * qi;
      if (scan1_test<FILTERED>(rs, sfilter, (uint32_t)x[u].x)) ex_mark<K>(ex, target, r);
      if (scan1_test<FILTERED>(rs, sfilter, (uint32_t)x[u].y)) ex_mark<K>(ex, target, r + 1);
      if (scan1_test<FILTERED>(rs, sfilter, (uint32_t)x[u].z)) ex_mark<K>(ex, target, r + 2);
      if (scan1_test<FILTERED>(rs, sfilter, (uint32_t)x[u].w)) ex_mark<K>(ex, target, r + 3);
    }
  }
  // the head rows [0, h) and the tail rows [h + 4 nq, n)
  const int64_t tail = n - h - 4 * nq;
  if (gtid < h + tail) {
    const int64_t r = gtid < h ? gtid : h + 4 * nq + (gtid - h);
    if (scan1_test<FILTERED>(rs, sfilter, (uint32_t)col[r])) ex_mark<K>(ex, target, r);
  }
}

// Key set on the binding rows: passing rows insert their target tuple.
template <int NB, int K>
__global__ void coverage_target_set_kernel(RelSet rs, KeyCols bound, KeyCols target, int64_t n,
                                           int32_t* __restrict__ owner, uint32_t mask) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    if (rel_has<NB>(rs, bound, r)) keyset_insert<K>(target, owner, mask, r);
  }
}

// Bit per example (32 a warp, one ballot) and the covered count (one atomic
// a warp).  With a representative array the bit is its representative's
// flag; without, the example looks its tuple up in the binding-side set.
template <int K>
__global__ void coverage_bits_kernel(const int32_t* __restrict__ rep, const uint8_t* __restrict__ flag,
                                     KeyCols target, const int32_t* __restrict__ owner,
                                     uint32_t mask, KeyCols ex, int64_t n,
                                     uint32_t* __restrict__ words, int64_t nwords,
                                     unsigned long long* __restrict__ ones) {
  const int64_t warps_total = (int64_t)gridDim.x * blockDim.x / 32;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = lane_id();
  constexpr int W = 4;  // words a warp keeps in flight
  unsigned long long c = 0;
  for (int64_t w0 = gw; w0 < nwords; w0 += warps_total * W) {
    int32_t rp[W];
    bool hit[W];
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const int64_t i = (w0 + u * warps_total) * 32 + lane;
      rp[u] = rep != nullptr && i < n ? rep[i] : -1;
    }
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const int64_t i = (w0 + u * warps_total) * 32 + lane;
      if (rep != nullptr) hit[u] = rp[u] >= 0 && flag[rp[u]] != 0;
      else hit[u] = i < n && keyset_find<K>(target, owner, mask, ex, i) >= 0;
    }
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const int64_t w = w0 + u * warps_total;
      const unsigned ball = __ballot_sync(kFullMask, hit[u]);
      if (lane == 0 && w < nwords) {
        if (words != nullptr) words[w] = ball;
        c += (unsigned long long)__popc(ball);
      }
    }
  }
  if (lane == 0 && c != 0) atomicAdd(ones, c);
}

constexpr int kCompactTileWords = 64;  // 32-bit words per compaction tile
constexpr int kCompactTile = kCompactTileWords * 32;
constexpr int kCompactThreads = 256;

// Kept rows of a 32-row word: bits past the last row never count.
__device__ __forceinline__ uint32_t kept_mask(const uint32_t* __restrict__ words, int64_t w,
                                              int64_t n, int keep_set) {
  uint32_t m = keep_set ? words[w] : ~words[w];
  const int64_t rows = n - w * 32;
  if (rows < 32) m &= rows <= 0 ? 0u : ((1u << rows) - 1u);
  return m;
}

// One warp per tile: kept rows of the tile's 64 words.
__global__ void compact_count_kernel(const uint32_t* __restrict__ words, int64_t n, int keep_set,
                                     uint32_t* __restrict__ tile_count, int64_t ntiles) {
  const int64_t warps_total = (int64_t)gridDim.x * blockDim.x / 32;
  const int lane = lane_id();
  const int64_t nwords = (n + 31) / 32;
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; t < ntiles;
       t += warps_total) {
    const int64_t w0 = t * kCompactTileWords;
    uint32_t c = 0;
    for (int j = lane; j < kCompactTileWords; j += 32)
      if (w0 + j < nwords) c += __popc(kept_mask(words, w0 + j, n, keep_set));
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(kFullMask, c, o);
    if (lane == 0) tile_count[t] = c;
  }
}

struct CompactCols {
  const int32_t* in[QFG_MAX_ARITY];
  int32_t* out[QFG_MAX_ARITY];
  int nc;
};

// One block per tile (grid-stride): a scan of the 64 word counts in shared
// memory, then every warp writes the kept rows of its words.
__global__ void __launch_bounds__(kCompactThreads)
compact_write_kernel(CompactCols cols, const uint32_t* __restrict__ words, int64_t n,
                     int keep_set, const uint32_t* __restrict__ tile_offset, int64_t ntiles) {
  __shared__ uint32_t word_off[kCompactTileWords];
  const int lane = lane_id();
  const int warp = threadIdx.x / 32;
  const int64_t nwords = (n + 31) / 32;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t w0 = t * kCompactTileWords;
    if (warp == 0) {
      // lane owns words 2*lane and 2*lane + 1
      uint32_t a = 0, b = 0;
      if (w0 + 2 * lane < nwords) a = __popc(kept_mask(words, w0 + 2 * lane, n, keep_set));
      if (w0 + 2 * lane + 1 < nwords) b = __popc(kept_mask(words, w0 + 2 * lane + 1, n, keep_set));
      uint32_t incl = a + b;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl += v;
      }
      word_off[2 * lane] = incl - a - b;
      word_off[2 * lane + 1] = incl - b;
    }
    __syncthreads();
    const uint64_t base = tile_offset[t];
    for (int j = warp; j < kCompactTileWords; j += kCompactThreads / 32) {
      const int64_t w = w0 + j;
      if (w >= nwords) break;
      const uint32_t m = kept_mask(words, w, n, keep_set);
      if ((m >> lane) & 1u) {
        const int64_t row = w * 32 + lane;
        const int64_t o = (int64_t)base + word_off[j] + __popc(m & ((1u << lane) - 1u));
        for (int c = 0; c < cols.nc; ++c) cols.out[c][o] = cols.in[c][row];
      }
    }
    __syncthreads();
  }
}

// ---- host -------------------------------------------------------------

// Dispatches F<NB, K> over bound-argument counts 1-3 (else 0) and target
// column counts 1-3 (else 0).
template <template <int, int> class F, typename... A>
void dispatch_nb_k(int nb, int k, A&&... a) {
  const int NBc = nb <= 3 ? nb : 0, Kc = k <= 3 ? k : 0;
#define QFG_K(NB)                                     \
  switch (Kc) {                                       \
    case 1: F<NB, 1>::run(std::forward<A>(a)...); break; \
    case 2: F<NB, 2>::run(std::forward<A>(a)...); break; \
    case 3: F<NB, 3>::run(std::forward<A>(a)...); break; \
    default: F<NB, 0>::run(std::forward<A>(a)...); break; \
  }
  switch (NBc) {
    case 1: QFG_K(1) break;
    case 2: QFG_K(2) break;
    case 3: QFG_K(3) break;
    default: QFG_K(0) break;
  }
#undef QFG_K
}

struct FlagLaunch {
  unsigned grid;      // 256-thread blocks
  unsigned sms;       // filtered pass: one block a SM
  cudaStream_t st;
  RelSet rs;
  KeyCols bound, target;
  int64_t n;
  ExSet ex;
  cudaError_t* status;
};
template <int NB, int K>
struct RunFlag {
  static void run(const FlagLaunch& a) {
    if constexpr (NB == 1) {
      if (a.rs.filter != nullptr) {
        constexpr size_t smem = sizeof(uint32_t) * kFilterWords;
        auto kern = coverage_scan1_kernel<K, true, 4>;
        *a.status = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
        if (*a.status != cudaSuccess) return;
        const unsigned grid = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>(a.sms, (a.n / 4 + kFilterThreads - 1) / kFilterThreads));
        kern<<<grid, kFilterThreads, smem, a.st>>>(a.rs, a.bound, a.target, a.n, a.ex);
      } else {
        const unsigned grid = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>(a.grid, (a.n / 4 + 255) / 256));
        coverage_scan1_kernel<K, false, 2><<<grid, 256, 0, a.st>>>(a.rs, a.bound, a.target,
                                                                   a.n, a.ex);
      }
    } else if constexpr (NB == 2) {
      if (a.rs.filter != nullptr) {
        constexpr size_t smem = sizeof(uint32_t) * kFilterWords;
        auto kern = coverage_scan_kernel<NB, K, true, kFilterRows>;
        *a.status = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
        if (*a.status != cudaSuccess) return;
        const unsigned grid = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>(a.sms, (a.n + kFilterThreads - 1) / kFilterThreads));
        kern<<<grid, kFilterThreads, smem, a.st>>>(a.rs, a.bound, a.target, a.n, a.ex);
      } else {
        coverage_scan_kernel<NB, K, false, kRowsPerThread><<<a.grid, 256, 0, a.st>>>(
            a.rs, a.bound, a.target, a.n, a.ex);
      }
    } else {
      coverage_flag_kernel<NB, K><<<a.grid, 256, 0, a.st>>>(a.rs, a.bound, a.target, a.n, a.ex);
    }
  }
};

struct TargetSetLaunch {
  unsigned grid;
  cudaStream_t st;
  RelSet rs;
  KeyCols bound, target;
  int64_t n;
  int32_t* owner;
  uint32_t mask;
};
template <int NB, int K>
struct RunTargetSet {
  static void run(const TargetSetLaunch& a) {
    coverage_target_set_kernel<NB, K><<<a.grid, 256, 0, a.st>>>(a.rs, a.bound, a.target, a.n,
                                                                a.owner, a.mask);
  }
};

void launch_bits(Ctx* ctx, int k, const int32_t* rep, const uint8_t* flag, const KeyCols& target,
                 const int32_t* owner, uint32_t mask, const KeyCols& ex, int64_t n, uint32_t* words,
                 unsigned long long* ones) {
  const int64_t nwords = 2 * ((n + 63) / 64);
  const unsigned grid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((nwords + 7) / 8, (int64_t)ctx->num_sms * 8));
  switch (rep != nullptr ? 1 : (k <= 3 ? k : 0)) {
    case 1: coverage_bits_kernel<1><<<grid, 256, 0, ctx->stream>>>(rep, flag, target, owner, mask, ex, n, words, nwords, ones); break;
    case 2: coverage_bits_kernel<2><<<grid, 256, 0, ctx->stream>>>(rep, flag, target, owner, mask, ex, n, words, nwords, ones); break;
    case 3: coverage_bits_kernel<3><<<grid, 256, 0, ctx->stream>>>(rep, flag, target, owner, mask, ex, n, words, nwords, ones); break;
    default: coverage_bits_kernel<0><<<grid, 256, 0, ctx->stream>>>(rep, flag, target, owner, mask, ex, n, words, nwords, ones); break;
  }
}

// The relation's key set over argument positions `args` (columns `keys`),
// built on first use and kept until the relation is replaced or released.
int relation_key_set(Ctx* ctx, Relation* rel, const std::vector<int>& args, const KeyCols& keys,
                     RelSet* out) {
  auto it = rel->key_sets.find(args);
  KeySet* ks = nullptr;
  const bool inline_form = keys.nk <= 2;
  if (it != rel->key_sets.end()) {
    ks = it->second.get();
  } else {
    auto fresh = std::make_unique<KeySet>();
    fresh->mask = table_mask(rel->num_tuples);
    const size_t slots = (size_t)fresh->mask + 1;
    const unsigned grid = rows_grid(ctx, rel->num_tuples);
    if (inline_form) {
      QFG_TRY(fresh->owner.reserve(ctx, sizeof(unsigned long long) * (slots + 2)));
      unsigned long long* t = fresh->owner.as<unsigned long long>();
      QFG_CUDA(ctx, cudaMemsetAsync(t, 0xff, sizeof(unsigned long long) * slots, ctx->stream));
      QFG_CUDA(ctx, cudaMemsetAsync(t + slots, 0, 2 * sizeof(unsigned long long), ctx->stream));
      if (keys.nk == 1)
        inline_keyset_insert_kernel<1><<<grid, 256, 0, ctx->stream>>>(keys, rel->num_tuples, t,
                                                                      fresh->mask);
      else
        inline_keyset_insert_kernel<2><<<grid, 256, 0, ctx->stream>>>(keys, rel->num_tuples, t,
                                                                      fresh->mask);
      QFG_LAUNCHED(ctx);
      unsigned long long distinct = 0;
      QFG_CUDA(ctx, cudaMemcpyAsync(&distinct, t + slots + 1, sizeof(distinct),
                                    cudaMemcpyDeviceToHost, ctx->stream));
      QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      fresh->distinct = (int64_t)distinct;
      if (fresh->distinct <= kFilterMaxKeys) {
        QFG_TRY(fresh->filter.reserve(ctx, sizeof(uint32_t) * kFilterWords));
        QFG_CUDA(ctx, cudaMemsetAsync(fresh->filter.ptr(), 0, sizeof(uint32_t) * kFilterWords,
                                      ctx->stream));
        filter_build_kernel<<<rows_grid(ctx, (int64_t)slots), 256, 0, ctx->stream>>>(
            t, fresh->mask, fresh->filter.as<uint32_t>(), kFilterBits);
        QFG_LAUNCHED(ctx);
      } else {
        int gb = kFilterBits + 1;
        while (gb < kMaxGlobalFilterBits && ((int64_t)1 << gb) < 8 * fresh->distinct) ++gb;
        const size_t words = ((size_t)1 << gb) / 32;
        QFG_TRY(fresh->gfilter.reserve(ctx, sizeof(uint32_t) * words));
        QFG_CUDA(ctx, cudaMemsetAsync(fresh->gfilter.ptr(), 0, sizeof(uint32_t) * words,
                                      ctx->stream));
        filter_build_kernel<<<rows_grid(ctx, (int64_t)slots), 256, 0, ctx->stream>>>(
            t, fresh->mask, fresh->gfilter.as<uint32_t>(), gb);
        QFG_LAUNCHED(ctx);
        fresh->gbits = gb;
      }
    } else {
      QFG_TRY(fresh->owner.reserve(ctx, sizeof(int32_t) * slots));
      QFG_CUDA(ctx, cudaMemsetAsync(fresh->owner.ptr(), 0xff, sizeof(int32_t) * slots, ctx->stream));
      launch_keyset_insert(grid, ctx->stream, keys, rel->num_tuples, fresh->owner.as<int32_t>(),
                           fresh->mask, nullptr);
      QFG_LAUNCHED(ctx);
    }
    ks = fresh.get();
    rel->key_sets.emplace(args, std::move(fresh));
  }
  out->mask = ks->mask;
  out->keys = keys;
  out->filter = ks->filter.bytes() > 0 ? ks->filter.as<uint32_t>() : nullptr;
  out->gfilter = ks->gbits > 0 ? ks->gfilter.as<uint32_t>() : nullptr;
  out->gbits = ks->gbits;
  out->table = inline_form ? ks->owner.as<unsigned long long>() : nullptr;
  out->owner = inline_form ? nullptr : ks->owner.as<int32_t>();
  return QFG_OK;
}

// An example table with (or, for the binding-side strategy, without) its
// key set; the layout at `mem` depends on the column count (see ExSet).
struct Examples {
  KeyCols keys;
  int64_t n = 0;
  uint32_t mask = 0;
  char* mem = nullptr;  // key set, or null (binding-side strategy)
};

bool inline_examples(int k) { return k <= 2; }

size_t example_flag_bytes(int k, int64_t n, uint32_t mask) {
  return inline_examples(k) ? (size_t)mask + 2 : (size_t)n;
}

// Bits (log2) of an inline example table's filter: about 8 a tuple.
int example_filter_bits(int64_t n) {
  int b = kFilterBits;
  while (b < kMaxGlobalFilterBits && ((int64_t)1 << b) < 8 * n) ++b;
  return b;
}

// Layout at `mem`: slots, representative per example, flags, then (inline
// form) the filter at the next 16-byte boundary.
size_t example_filter_offset(int k, int64_t n, uint32_t mask) {
  const size_t slot = inline_examples(k) ? sizeof(unsigned long long) : sizeof(int32_t);
  return (slot * ((size_t)mask + 1) + sizeof(int32_t) * (size_t)n + example_flag_bytes(k, n, mask) +
          15) & ~(size_t)15;
}

size_t example_set_bytes(int k, int64_t n, uint32_t mask) {
  const size_t filter = inline_examples(k) ? ((size_t)1 << example_filter_bits(n)) / 8 : 0;
  return (example_filter_offset(k, n, mask) + filter + 255) & ~(size_t)255;
}

ExSet example_view(const Examples& e) {
  ExSet v;
  v.keys = e.keys;
  v.mask = e.mask;
  const bool in = inline_examples(e.keys.nk);
  v.table = in ? reinterpret_cast<const unsigned long long*>(e.mem) : nullptr;
  v.owner = in ? nullptr : reinterpret_cast<const int32_t*>(e.mem);
  int32_t* rep = reinterpret_cast<int32_t*>(
      e.mem + (in ? sizeof(unsigned long long) : sizeof(int32_t)) * ((size_t)e.mask + 1));
  v.rep = rep;
  v.flag = reinterpret_cast<uint8_t*>(rep + e.n);
  v.efilter = in ? reinterpret_cast<const uint32_t*>(
                       e.mem + example_filter_offset(e.keys.nk, e.n, e.mask))
                 : nullptr;
  v.ebits = in ? example_filter_bits(e.n) : 0;
  return v;
}

// Queues the build of an example key set at e->mem.
int build_example_set(Ctx* ctx, Examples* e) {
  const ExSet v = example_view(*e);
  const unsigned grid = rows_grid(ctx, e->n);
  int32_t* rep = const_cast<int32_t*>(v.rep);
  if (inline_examples(e->keys.nk)) {
    unsigned long long* table = const_cast<unsigned long long*>(v.table);
    QFG_CUDA(ctx, cudaMemsetAsync(table, 0xff, sizeof(unsigned long long) * ((size_t)e->mask + 1),
                                  ctx->stream));
    uint32_t* filter = const_cast<uint32_t*>(v.efilter);
    QFG_CUDA(ctx, cudaMemsetAsync(filter, 0, ((size_t)1 << v.ebits) / 8, ctx->stream));
    if (e->keys.nk == 1) {
      inline_example_insert_kernel<1><<<grid, 256, 0, ctx->stream>>>(e->keys, e->n, table,
                                                                      e->mask, rep);
      example_filter_kernel<1><<<grid, 256, 0, ctx->stream>>>(e->keys, e->n, filter, v.ebits);
    } else {
      inline_example_insert_kernel<2><<<grid, 256, 0, ctx->stream>>>(e->keys, e->n, table,
                                                                      e->mask, rep);
      example_filter_kernel<2><<<grid, 256, 0, ctx->stream>>>(e->keys, e->n, filter, v.ebits);
    }
  } else {
    int32_t* owner = const_cast<int32_t*>(v.owner);
    QFG_CUDA(ctx, cudaMemsetAsync(owner, 0xff, sizeof(int32_t) * ((size_t)e->mask + 1),
                                  ctx->stream));
    launch_keyset_insert(grid, ctx->stream, e->keys, e->n, owner, e->mask, rep);
  }
  QFG_LAUNCHED(ctx);
  return QFG_OK;
}

struct CoverageArgs {
  const qfg_bindings* b;
  Relation* rel;
  KeyCols rel_keys, bound[2], target[2];
  std::vector<int> bound_args;
  int k;
};

int coverage_args(Ctx* ctx, const qfg_bindings* b, const qfg_literal* lit, int k,
                  CoverageArgs* a) {
  if (b == nullptr || lit == nullptr)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_coverage: null argument");
  QFG_TRY(find_relation(ctx, lit->relation_id, &a->rel));
  if (lit->num_args != a->rel->num_columns || k < 1 || k > QFG_MAX_ARITY || k > b->num_columns)
    return set_error(ctx, QFG_ERR_INVALID,
                     "qfg_coverage: literal arity or target column count out of range");
  a->b = b;
  a->k = k;
  a->rel_keys.nk = a->bound[0].nk = a->bound[1].nk = 0;
  for (int i = 0; i < lit->num_args; ++i) {
    const int v = lit->vars[i];
    if (v >= b->num_columns || v < -1)
      return set_error(ctx, QFG_ERR_INVALID, "qfg_coverage: variable out of range");
    if (v < 0) continue;
    a->bound_args.push_back(i);
    a->rel_keys.c[a->rel_keys.nk++] = a->rel->columns[i];
    a->bound[0].c[a->bound[0].nk++] = b->columns[v];
    a->bound[1].c[a->bound[1].nk++] = b->columns[v] + b->num_positive;
  }
  if (a->rel_keys.nk == 0)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_coverage: literal has no bound argument");
  a->target[0].nk = a->target[1].nk = k;
  for (int q = 0; q < k; ++q) {
    a->target[0].c[q] = b->columns[q];
    a->target[1].c[q] = b->columns[q] + b->num_positive;
  }
  return QFG_OK;
}

// Runs both label sides.  ex[s].mem set: the key set on the examples is
// built (flags are cleared here); null: the binding-side set goes into
// `side_mem` (slots for the larger side).
int coverage_run(Ctx* ctx, const CoverageArgs& a, Examples ex[2], uint64_t* d_positive_bits,
                 int32_t* side_mem, int64_t* num_covered) {
  QFG_TRY(ctx->scratch[kScrTmpC].reserve(ctx, 2 * sizeof(unsigned long long)));
  unsigned long long* ones = ctx->scratch[kScrTmpC].as<unsigned long long>();
  QFG_CUDA(ctx, cudaMemsetAsync(ones, 0, 2 * sizeof(unsigned long long), ctx->stream));
  if (d_positive_bits != nullptr && ex[0].n > 0)
    QFG_CUDA(ctx, cudaMemsetAsync(d_positive_bits, 0, sizeof(uint64_t) * ((ex[0].n + 63) / 64),
                                  ctx->stream));
  const int64_t n_side[2] = {a.b->num_positive, a.b->num_negative};
  const bool work[2] = {n_side[0] > 0 && ex[0].n > 0, n_side[1] > 0 && ex[1].n > 0};
  if (a.rel->num_tuples > 0 && (work[0] || work[1])) {
    RelSet rs;
    QFG_TRY(relation_key_set(ctx, a.rel, a.bound_args, a.rel_keys, &rs));
    for (int s = 0; s < 2; ++s) {
      if (!work[s]) continue;
      uint32_t* words = s == 0 ? reinterpret_cast<uint32_t*>(d_positive_bits) : nullptr;
      // 256-thread blocks of up to 64 registers: four resident a SM
      const unsigned grid = (unsigned)std::max<int64_t>(
          1, std::min<int64_t>((n_side[s] + 255) / 256, (int64_t)ctx->num_sms * 4));
      if (ex[s].mem != nullptr) {
        const ExSet v = example_view(ex[s]);
        QFG_CUDA(ctx, cudaMemsetAsync(v.flag, 0, example_flag_bytes(a.k, ex[s].n, ex[s].mask),
                                      ctx->stream));
        cudaError_t status = cudaSuccess;
        const FlagLaunch fl{grid, (unsigned)ctx->num_sms, ctx->stream, rs, a.bound[s],
                            a.target[s], n_side[s], v, &status};
        QFG_TRY(stage_begin(ctx, QFG_STAGE_COVERAGE_SCAN));
        dispatch_nb_k<RunFlag>(a.rel_keys.nk, a.k, fl);
        QFG_CUDA(ctx, status);
        QFG_LAUNCHED(ctx);
        QFG_TRY(stage_end(ctx, QFG_STAGE_COVERAGE_SCAN));
        QFG_TRY(stage_begin(ctx, QFG_STAGE_COVERAGE_EXAMPLES));
        launch_bits(ctx, a.k, v.rep, v.flag, a.target[s], nullptr, 0, ex[s].keys, ex[s].n, words,
                    ones + s);
        QFG_LAUNCHED(ctx);
        QFG_TRY(stage_end(ctx, QFG_STAGE_COVERAGE_EXAMPLES));
      } else {
        const uint32_t mask = table_mask(n_side[s]);
        QFG_CUDA(ctx, cudaMemsetAsync(side_mem, 0xff, sizeof(int32_t) * ((size_t)mask + 1),
                                      ctx->stream));
        const TargetSetLaunch tl{grid, ctx->stream, rs, a.bound[s], a.target[s], n_side[s],
                                 side_mem, mask};
        QFG_TRY(stage_begin(ctx, QFG_STAGE_COVERAGE_SCAN));
        dispatch_nb_k<RunTargetSet>(a.rel_keys.nk, a.k, tl);
        QFG_LAUNCHED(ctx);
        QFG_TRY(stage_end(ctx, QFG_STAGE_COVERAGE_SCAN));
        QFG_TRY(stage_begin(ctx, QFG_STAGE_COVERAGE_EXAMPLES));
        launch_bits(ctx, a.k, nullptr, nullptr, a.target[s], side_mem, mask, ex[s].keys, ex[s].n,
                    words, ones + s);
        QFG_LAUNCHED(ctx);
        QFG_TRY(stage_end(ctx, QFG_STAGE_COVERAGE_EXAMPLES));
      }
    }
  }
  unsigned long long h[2] = {0, 0};
  QFG_CUDA(ctx, cudaMemcpyAsync(h, ones, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  num_covered[0] = (int64_t)h[0];
  num_covered[1] = (int64_t)h[1];
  return QFG_OK;
}

// Keeps the rows of `cols` whose bit is set (keep_set) or clear, in order.
int compact_rows(Ctx* ctx, int nc, const int32_t* const* in, int64_t n, const uint32_t* words,
                 int keep_set, int32_t* const* out, int64_t capacity, int64_t* num_out) {
  const int64_t ntiles = (n + kCompactTile - 1) / kCompactTile;
  QFG_TRY(ctx->scratch[kScrTmpA].reserve(ctx, sizeof(uint32_t) * (size_t)(2 * ntiles + 1)));
  uint32_t* count = ctx->scratch[kScrTmpA].as<uint32_t>();
  uint32_t* total = count + 2 * ntiles;
  const unsigned cgrid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((ntiles + 7) / 8, (int64_t)ctx->num_sms * 8));
  compact_count_kernel<<<cgrid, 256, 0, ctx->stream>>>(words, n, keep_set, count, ntiles);
  QFG_LAUNCHED(ctx);
  QFG_TRY(exclusive_scan_u32(ctx, count, count + ntiles, ntiles, total));
  uint32_t kept = 0;
  QFG_CUDA(ctx, cudaMemcpyAsync(&kept, total, sizeof(kept), cudaMemcpyDeviceToHost, ctx->stream));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *num_out = kept;
  if ((int64_t)kept > capacity)
    return set_error(ctx, QFG_ERR_INVALID,
                     "qfg_compact_rows: " + std::to_string(kept) + " rows kept, capacity " +
                         std::to_string(capacity));
  const unsigned wgrid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(ntiles, (int64_t)ctx->num_sms * 8));
  for (int c0 = 0; c0 < nc; c0 += QFG_MAX_ARITY) {
    CompactCols cc;
    cc.nc = std::min(nc - c0, QFG_MAX_ARITY);
    for (int c = 0; c < cc.nc; ++c) {
      cc.in[c] = in[c0 + c];
      cc.out[c] = out[c0 + c];
    }
    compact_write_kernel<<<wgrid, kCompactThreads, 0, ctx->stream>>>(cc, words, n, keep_set,
                                                                      count + ntiles, ntiles);
    QFG_LAUNCHED(ctx);
  }
  return QFG_OK;
}

int check_examples(Ctx* ctx, int k, const int32_t* const* cols, int64_t n, const char* what) {
  if (n < 0 || n > INT32_MAX || (n > 0 && cols == nullptr))
    return set_error(ctx, QFG_ERR_INVALID, std::string("qfg_coverage: invalid ") + what);
  for (int q = 0; q < k && n > 0; ++q)
    if (cols[q] == nullptr)
      return set_error(ctx, QFG_ERR_INVALID, std::string("qfg_coverage: null column in ") + what);
  return QFG_OK;
}

}  // namespace

}  // namespace qfg

using namespace qfg;

extern "C" int qfg_coverage(qfg_ctx* c, const qfg_bindings* b, const qfg_literal* lit,
                            int32_t num_target_columns, const int32_t* const* d_uncovered_positive,
                            int64_t num_uncovered_positive, const int32_t* const* d_negative,
                            int64_t num_negative, uint64_t* d_positive_bits,
                            int64_t* num_covered) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_covered == nullptr) return set_error(ctx, QFG_ERR_INVALID, "qfg_coverage: null argument");
  CoverageArgs a;
  QFG_TRY(coverage_args(ctx, b, lit, num_target_columns, &a));
  const int k = num_target_columns;
  QFG_TRY(check_examples(ctx, k, d_uncovered_positive, num_uncovered_positive,
                         "uncovered positives"));
  QFG_TRY(check_examples(ctx, k, d_negative, num_negative, "negatives"));
  if (ctx->coverage_compat) {
    const int32_t* const* cols[2] = {d_uncovered_positive, d_negative};
    const int64_t ns[2] = {num_uncovered_positive, d_negative != nullptr ? num_negative : 0};
    return coverage_compat(ctx, b, lit, k, cols, ns, d_positive_bits, num_covered);
  }
  Examples ex[2];
  const int64_t n_side[2] = {b->num_positive, b->num_negative};
  ex[0].n = num_uncovered_positive;
  ex[1].n = num_negative;
  for (int s = 0; s < 2; ++s) {
    ex[s].keys.nk = k;
    const int32_t* const* cols = s == 0 ? d_uncovered_positive : d_negative;
    for (int q = 0; q < k; ++q) ex[s].keys.c[q] = ex[s].n > 0 ? cols[q] : nullptr;
  }
  // Scratch of both sides, sized before the first launch so that no later
  // reserve moves memory a queued kernel still uses.
  size_t off[2], need = 0, side_need = 0;
  bool on_examples[2];
  for (int s = 0; s < 2; ++s) {
    const bool work = n_side[s] > 0 && ex[s].n > 0;
    on_examples[s] = work && ex[s].n <= n_side[s];
    off[s] = need;
    if (on_examples[s]) {
      ex[s].mask = table_mask(ex[s].n);
      need += example_set_bytes(k, ex[s].n, ex[s].mask);
    } else if (work) {
      side_need = std::max(side_need, sizeof(int32_t) * ((size_t)table_mask(n_side[s]) + 1));
    }
  }
  if (need + side_need > 0) QFG_TRY(ctx->scratch[kScrJoin2].reserve(ctx, need + side_need));
  char* base = ctx->scratch[kScrJoin2].as<char>();
  QFG_TRY(stage_begin(ctx, QFG_STAGE_COVERAGE_EXAMPLES));
  for (int s = 0; s < 2; ++s) {
    if (!on_examples[s]) continue;
    ex[s].mem = base + off[s];
    QFG_TRY(build_example_set(ctx, &ex[s]));
  }
  QFG_TRY(stage_end(ctx, QFG_STAGE_COVERAGE_EXAMPLES));
  return coverage_run(ctx, a, ex, d_positive_bits,
                      side_need > 0 ? reinterpret_cast<int32_t*>(base + need) : nullptr,
                      num_covered);
}

extern "C" int qfg_examples_create(qfg_ctx* c, int32_t num_columns, const int32_t* const* d_columns,
                                   int64_t num_rows, qfg_examples** out) {
  if (c == nullptr || out == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  *out = nullptr;
  if (num_columns < 1 || num_columns > QFG_MAX_ARITY)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_examples_create: 1 to 8 columns");
  QFG_TRY(check_examples(ctx, num_columns, d_columns, num_rows, "examples"));
  auto e = std::make_unique<qfg_examples>();
  e->num_columns = num_columns;
  e->num_rows = num_rows;
  e->columns.assign(d_columns, d_columns + (num_rows > 0 ? num_columns : 0));
  if (num_rows > 0) {
    e->mask = table_mask(num_rows);
    QFG_TRY(e->storage.reserve(ctx, example_set_bytes(num_columns, num_rows, e->mask)));
    Examples v;
    v.keys.nk = num_columns;
    for (int q = 0; q < num_columns; ++q) v.keys.c[q] = d_columns[q];
    v.n = num_rows;
    v.mask = e->mask;
    v.mem = e->storage.as<char>();
    QFG_TRY(build_example_set(ctx, &v));
    QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  *out = e.release();
  return QFG_OK;
}

extern "C" int qfg_examples_destroy(qfg_ctx* c, qfg_examples* e) {
  if (c == nullptr) return QFG_ERR_INVALID;
  if (e == nullptr) return QFG_OK;
  // Kernels queued on the examples' key set finish before its memory goes.
  QFG_CUDA(&c->impl, cudaStreamSynchronize(c->impl.stream));
  delete e;
  return QFG_OK;
}

extern "C" int qfg_coverage_examples(qfg_ctx* c, const qfg_bindings* b, const qfg_literal* lit,
                                     const qfg_examples* uncovered_positive,
                                     const qfg_examples* negative, uint64_t* d_positive_bits,
                                     int64_t* num_covered) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_covered == nullptr || uncovered_positive == nullptr)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_coverage_examples: null argument");
  const int k = uncovered_positive->num_columns;
  if (negative != nullptr && negative->num_columns != k)
    return set_error(ctx, QFG_ERR_INVALID,
                     "qfg_coverage_examples: positive and negative column counts differ");
  CoverageArgs a;
  QFG_TRY(coverage_args(ctx, b, lit, k, &a));
  if (ctx->coverage_compat) {
    const int32_t* const* cols[2] = {uncovered_positive->columns.data(),
                                     negative != nullptr ? negative->columns.data() : nullptr};
    const int64_t ns[2] = {uncovered_positive->num_rows, negative != nullptr ? negative->num_rows : 0};
    return coverage_compat(ctx, b, lit, k, cols, ns, d_positive_bits, num_covered);
  }
  Examples ex[2];
  const qfg_examples* src[2] = {uncovered_positive, negative};
  for (int s = 0; s < 2; ++s) {
    ex[s].keys.nk = k;
    if (src[s] == nullptr || src[s]->num_rows == 0) continue;
    ex[s].n = src[s]->num_rows;
    for (int q = 0; q < k; ++q) ex[s].keys.c[q] = src[s]->columns[q];
    ex[s].mask = src[s]->mask;
    ex[s].mem = src[s]->storage.as<char>();
  }
  return coverage_run(ctx, a, ex, d_positive_bits, nullptr, num_covered);
}

extern "C" int qfg_compact_rows(qfg_ctx* c, int32_t num_columns, const int32_t* const* d_columns,
                                int64_t num_rows, const uint64_t* d_bits, int32_t keep_set,
                                int32_t* const* d_out_columns, int64_t out_capacity,
                                int64_t* num_out) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_out == nullptr || num_columns < 0 || num_rows < 0 || num_rows > INT32_MAX ||
      out_capacity < 0 || (num_rows > 0 && d_bits == nullptr) ||
      (num_columns > 0 && (d_columns == nullptr || d_out_columns == nullptr)))
    return set_error(ctx, QFG_ERR_INVALID, "qfg_compact_rows: invalid arguments");
  *num_out = 0;
  if (num_rows == 0) return QFG_OK;
  return compact_rows(ctx, num_columns, d_columns, num_rows,
                      reinterpret_cast<const uint32_t*>(d_bits), keep_set != 0, d_out_columns,
                      out_capacity, num_out);
}
