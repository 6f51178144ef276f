// partition.cu -- stable radix partitioning and chained hash-table builds in
// the reference's exact layouts.
//
// RadixPartition (operations/RadixPartition.cpp:56-155) produces, per radix
// partition of the identity hash's low bits, the (value, tuple_id) pairs in
// input order.  Here a warp owns a contiguous chunk of rows; a histogram pass
// counts digits per (digit, warp chunk) with warp-aggregated updates
// (__match_any_sync: one shared-memory add per distinct digit per 32 rows),
// an exclusive scan in digit-major order turns the counts into output
// cursors, and a scatter pass re-reads the chunk and writes each row at its
// cursor plus its rank among same-digit lanes below it.  Chunks are disjoint
// and scanned in row order, so the result is stable.  Up to 8 radix bits one
// such pass writes the tuples; wider digits take two stable LSD passes of at
// most 8 bits each (low digit into (value, row) scratch, then high digit into
// the tuples), so the per-warp count table stays small and the grid fills
// the GPU at every bit count.
//
// The same stable pass, applied LSD-style to bucket ids, rebuilds the
// reference's chained FoilHashTable byte for byte: a chain lists the
// partition positions of one bucket in descending order, so after a stable
// sort by (partition, bucket) each element's `next` is its predecessor in the
// sorted order and the bucket head is the last one.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "qfg_common.cuh"

namespace qfg {

namespace {

constexpr int kMaxSmemPerBlock = 200 * 1024;

// RadixPartition API input/output: digit source = the value, payload = the
// row index, output = PartitionTuple{value, tuple_id} (8 bytes).
struct RefTupleIO {
  const int32_t* values;
  int2* out;
  __device__ __forceinline__ uint32_t key(int64_t i) const { return (uint32_t)values[i]; }
  __device__ __forceinline__ void write(int64_t pos, int64_t i, uint32_t k) const {
    out[pos] = make_int2((int32_t)k, (int32_t)i);
  }
};

// Second LSD pass of a wide RadixPartition: (value, row) pairs in
// structure-of-arrays form, written as PartitionTuple{value, tuple_id}.
struct SoAToRefIO {
  const uint32_t* keys_in;
  const int32_t* payload_in;
  int2* out;
  __device__ __forceinline__ uint32_t key(int64_t i) const { return keys_in[i]; }
  __device__ __forceinline__ void write(int64_t pos, int64_t i, uint32_t k) const {
    out[pos] = make_int2((int32_t)k, payload_in[i]);
  }
};

// One LSD pass over (u32 key, int32 payload) in structure-of-arrays form.
struct SortIO {
  const uint32_t* keys_in;
  const int32_t* payload_in;  // null: payload is the row index
  uint32_t* keys_out;
  int32_t* payload_out;
  __device__ __forceinline__ uint32_t key(int64_t i) const { return keys_in[i]; }
  __device__ __forceinline__ void write(int64_t pos, int64_t i, uint32_t k) const {
    keys_out[pos] = k;
    payload_out[pos] = payload_in != nullptr ? payload_in[i] : (int32_t)i;
  }
};

template <class IO>
__global__ void stable_hist_kernel(IO io, int64_t n, int shift, int bits, int64_t chunk,
                                   int64_t num_chunks, uint32_t* __restrict__ hist) {
  extern __shared__ uint32_t sh_hist[];
  const uint32_t P = 1u << bits, mask = P - 1u;
  const int warps = blockDim.x >> 5, lane = lane_id();
  uint32_t* h = sh_hist + (size_t)warp_id() * P;
  for (uint32_t d = lane; d < P; d += 32) h[d] = 0;
  __syncwarp();
  const int64_t wc = (int64_t)blockIdx.x * warps + warp_id();
  if (wc >= num_chunks) return;
  const int64_t start = wc * chunk, end = min(n, start + chunk);
  for (int64_t base = start; base < end; base += 32) {
    const int64_t i = base + lane;
    const bool valid = i < end;
    const uint32_t d = valid ? (io.key(i) >> shift) & mask : 0u;
    const unsigned act = __ballot_sync(kFullMask, valid);
    if (valid) {
      const unsigned peers = __match_any_sync(act, d);
      if (lane == __ffs(peers) - 1) h[d] += __popc(peers);
    }
    __syncwarp();
  }
  for (uint32_t d = lane; d < P; d += 32) hist[(int64_t)d * num_chunks + wc] = h[d];
}

template <class IO>
__global__ void stable_scatter_kernel(IO io, int64_t n, int shift, int bits, int64_t chunk,
                                      int64_t num_chunks, const uint32_t* __restrict__ cursors) {
  extern __shared__ uint32_t sh_cur[];
  const uint32_t P = 1u << bits, mask = P - 1u;
  const int warps = blockDim.x >> 5, lane = lane_id();
  uint32_t* cur = sh_cur + (size_t)warp_id() * P;
  const int64_t wc = (int64_t)blockIdx.x * warps + warp_id();
  if (wc >= num_chunks) return;
  for (uint32_t d = lane; d < P; d += 32) cur[d] = cursors[(int64_t)d * num_chunks + wc];
  __syncwarp();
  const int64_t start = wc * chunk, end = min(n, start + chunk);
  const unsigned lt = lanemask_lt();
  for (int64_t base = start; base < end; base += 32) {
    const int64_t i = base + lane;
    const bool valid = i < end;
    const uint32_t k = valid ? io.key(i) : 0u;
    const uint32_t d = (k >> shift) & mask;
    const unsigned act = __ballot_sync(kFullMask, valid);
    unsigned peers = 0;
    uint32_t pos = 0;
    if (valid) {
      peers = __match_any_sync(act, d);
      pos = cur[d] + __popc(peers & lt);
    }
    __syncwarp();
    if (valid) {
      io.write(pos, i, k);
      if (lane == __ffs(peers) - 1) cur[d] += __popc(peers);
    }
    __syncwarp();
  }
}

// Shared-memory staged stable pass (qfg_radix_partition).  A CTA owns a
// contiguous row range and takes it in rounds of kRTRound rows.  In a round
// warp w owns rows [w * kRTPerWarp, (w + 1) * kRTPerWarp) and walks them 32
// at a time: a row's rank among the warp's rows of its digit is the warp's
// running count of the digit plus its rank among the equal-digit lanes below
// it (one ballot per digit bit), with no block barrier between the steps.  One scan
// over the warps of every digit then turns the warps' counts into offsets,
// so each row's rank within the round is stable; the round's keys, staged in
// shared memory, are written in digit order, consecutive threads on
// consecutive output positions of a digit's run.  The CTA's cursors come
// from a digit-major scan of per-CTA digit counts, so the whole pass is
// stable.
constexpr int kRTThreads = 512;
constexpr int kRTWarps = kRTThreads / 32;
constexpr int kRTSteps = 8;                       // 32-row steps of a warp per round
constexpr int kRTPerWarp = 32 * kRTSteps;         // 256 rows
constexpr int kRTRound = kRTWarps * kRTPerWarp;   // 4096 rows a round
constexpr int kRTMaxBits = 8;
static_assert(kRTRound <= 65536, "a round's row packs into 16 bits");

size_t round_smem_bytes(int bits) {
  const size_t P = size_t(1) << bits;
  return sizeof(uint32_t) * (2 * (size_t)kRTRound + (size_t)kRTWarps * P + 4 * P);
}

template <class IO>
__global__ void __launch_bounds__(kRTThreads) round_hist_kernel(IO io, int64_t n, int shift, int bits,
                                                                int64_t per,
                                                                uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[1 << kRTMaxBits];
  const uint32_t P = 1u << bits, mask = P - 1u;
  for (uint32_t d = threadIdx.x; d < P; d += blockDim.x) h[d] = 0u;
  __syncthreads();
  const int64_t r0 = (int64_t)blockIdx.x * per, r1 = min(n, r0 + per);
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) atomicAdd(&h[(io.key(r) >> shift) & mask], 1u);
  __syncthreads();
  for (uint32_t d = threadIdx.x; d < P; d += blockDim.x) hist[(int64_t)d * gridDim.x + blockIdx.x] = h[d];
}

template <class IO>
__global__ void __launch_bounds__(kRTThreads) round_scatter_kernel(IO io, int64_t n, int shift, int bits,
                                                                   int64_t per,
                                                                   const uint32_t* __restrict__ cursors) {
  extern __shared__ uint32_t rs[];
  const uint32_t P = 1u << bits, mask = P - 1u;
  uint32_t* keys = rs;                   // kRTRound
  uint32_t* perm = keys + kRTRound;      // kRTRound: row | digit << 16 by sorted position
  uint32_t* wrun = perm + kRTRound;      // kRTWarps * P: a warp's count of each digit, then offset
  uint32_t* dcnt = wrun + kRTWarps * P;  // P: the round's count of each digit
  uint32_t* dstart = dcnt + P;           // P
  uint32_t* gpos = dstart + P;           // P
  uint32_t* cur = gpos + P;              // P: the CTA's output cursors
  __shared__ uint32_t s_warp[kRTWarps];
  const int t = threadIdx.x, lane = lane_id(), warp = warp_id();
  const unsigned lt = lanemask_lt();
  for (uint32_t d = t; d < P; d += blockDim.x) cur[d] = cursors[(int64_t)d * gridDim.x + blockIdx.x];
  for (uint32_t i = t; i < (uint32_t)kRTWarps * P; i += blockDim.x) wrun[i] = 0u;
  __syncthreads();
  uint32_t* my = wrun + warp * P;
  const int64_t r0 = (int64_t)blockIdx.x * per, r1 = min(n, r0 + per);
  for (int64_t rr = r0; rr < r1; rr += kRTRound) {
    const int nt = (int)min((int64_t)kRTRound, r1 - rr);
    uint32_t dj[kRTSteps], rk[kRTSteps];
#pragma unroll
    for (int j = 0; j < kRTSteps; ++j) {
      const int i = warp * kRTPerWarp + j * 32 + lane;
      const bool valid = i < nt;
      uint32_t k = 0;
      if (valid) {
        k = io.key(rr + i);
        keys[i] = k;
      }
      const uint32_t d = (k >> shift) & mask;
      const unsigned act = __ballot_sync(kFullMask, valid);
      // The lanes holding the same digit: one ballot per digit bit.
      unsigned peers = act;
#pragma unroll
      for (int b = 0; b < kRTMaxBits; ++b) {
        if (b < bits) {
          const bool bit = ((d >> b) & 1u) != 0u;
          const unsigned bb = __ballot_sync(kFullMask, bit);
          peers &= bit ? bb : ~bb;
        }
      }
      dj[j] = d;
      rk[j] = 0;
      if (valid) {
        rk[j] = my[d] + __popc(peers & lt);
        __syncwarp(act);
        if (lane == __ffs(peers) - 1) my[d] += __popc(peers);
      }
      __syncwarp();
    }
    __syncthreads();
    // Offsets of the warps' rows of every digit (warp order is row order).
    for (uint32_t d = t; d < P; d += blockDim.x) {
      uint32_t run = 0;
      for (int w = 0; w < kRTWarps; ++w) {
        const uint32_t c = wrun[w * P + d];
        wrun[w * P + d] = run;
        run += c;
      }
      dcnt[d] = run;
    }
    __syncthreads();
    // Digit starts within the round (block scan of the P counts) and output
    // positions: sorted position k of digit d goes to gpos[d] + k.
    {
      const uint32_t c = (uint32_t)t < P ? dcnt[t] : 0u;
      uint32_t x = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFullMask, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) s_warp[warp] = x;
      __syncthreads();
      if (warp == 0) {
        const uint32_t v = lane < kRTWarps ? s_warp[lane] : 0u;
        uint32_t sc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(kFullMask, sc, o);
          if (lane >= o) sc += y;
        }
        if (lane < kRTWarps) s_warp[lane] = sc - v;
      }
      __syncthreads();
      if ((uint32_t)t < P) {
        const uint32_t ex = x - c + s_warp[warp];
        dstart[t] = ex;
        gpos[t] = cur[t] - ex;
        cur[t] += c;
      }
      __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < kRTSteps; ++j) {
      const int i = warp * kRTPerWarp + j * 32 + lane;
      if (i < nt) perm[dstart[dj[j]] + my[dj[j]] + rk[j]] = (uint32_t)i | (dj[j] << 16);
    }
    __syncthreads();
    for (uint32_t i = t; i < (uint32_t)kRTWarps * P; i += blockDim.x) wrun[i] = 0u;
#pragma unroll
    for (int j = 0; j < kRTSteps; ++j) {
      const int k = j * kRTThreads + t;
      if (k < nt) {
        const uint32_t v = perm[k];
        const uint32_t row = v & 0xffffu;
        io.write((int64_t)gpos[v >> 16] + k, rr + row, keys[row]);
      }
    }
    __syncthreads();
  }
}

// offsets[d] = cursor of digit d in chunk 0; offsets[P] = n.
__global__ void digit_offsets_kernel(const uint32_t* __restrict__ scanned, int64_t num_chunks,
                                     int bits, int64_t n, int64_t* __restrict__ offsets) {
  const uint32_t P = 1u << bits;
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d <= P; d += gridDim.x * blockDim.x)
    offsets[d] = d == P ? n : (int64_t)scanned[(int64_t)d * num_chunks];
}

struct PassShape {
  int64_t chunk, num_chunks;
  int warps;
  size_t smem;
  unsigned grid;
};

PassShape pass_shape(int64_t n, int bits) {
  PassShape s;
  const int64_t P = int64_t(1) << bits;
  // Rows per warp chunk: large enough that the (digit, chunk) count table
  // stays at most n/8 entries, and a multiple of 32.
  s.chunk = std::max<int64_t>(1024, 8 * P);
  s.num_chunks = std::max<int64_t>(1, (n + s.chunk - 1) / s.chunk);
  const int64_t per_warp = 4 * P;
  s.warps = (int)std::min<int64_t>(8, std::max<int64_t>(1, kMaxSmemPerBlock / per_warp));
  s.smem = (size_t)(per_warp * s.warps);
  s.grid = (unsigned)((s.num_chunks + s.warps - 1) / s.warps);
  return s;
}

// One stable partition pass with the round kernels (bits <= kRTMaxBits):
// per-CTA digit counts, a digit-major scan, the staged scatter.
template <class IO>
int round_pass(Ctx* ctx, IO io, int64_t n, int shift, int bits, int64_t* digit_offsets) {
  const size_t smem = round_smem_bytes(bits);
  int per_sm = 0;
  QFG_CUDA(ctx, cudaFuncSetAttribute(round_scatter_kernel<IO>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  QFG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, round_scatter_kernel<IO>,
                                                              kRTThreads, smem));
  // One resident wave of CTAs, each a contiguous range of whole rounds.
  const int64_t rounds = (n + kRTRound - 1) / kRTRound;
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(rounds, (int64_t)ctx->num_sms *
                                                                          std::max(per_sm, 1)));
  const int64_t per = ((rounds + grid - 1) / grid) * kRTRound;
  const unsigned g = (unsigned)((n + per - 1) / per);
  const int64_t entries = (int64_t)g << bits;
  QFG_TRY(ctx->scratch[kScrHist].reserve(ctx, sizeof(uint32_t) * (size_t)entries));
  uint32_t* hist = ctx->scratch[kScrHist].as<uint32_t>();
  round_hist_kernel<IO><<<g, kRTThreads, 0, ctx->stream>>>(io, n, shift, bits, per, hist);
  QFG_LAUNCHED(ctx);
  QFG_TRY(exclusive_scan_u32(ctx, hist, hist, entries, nullptr));
  if (digit_offsets != nullptr) {
    const uint32_t P = 1u << bits;
    digit_offsets_kernel<<<(P + 256) / 256, 256, 0, ctx->stream>>>(hist, g, bits, n, digit_offsets);
    QFG_LAUNCHED(ctx);
  }
  round_scatter_kernel<IO><<<g, kRTThreads, smem, ctx->stream>>>(io, n, shift, bits, per, hist);
  QFG_LAUNCHED(ctx);
  return QFG_OK;
}

// Stable LSD sort of n (u32 key < 2^key_bits, int32 payload) pairs.  The
// first pass reads keys from k0 and takes the row index as payload; passes
// then ping-pong between (k0, p0) and (k1, p1).  The result ends in
// (*k_out, *p_out).
int stable_sort_pairs(Ctx* ctx, uint32_t* k0, int32_t* p0, uint32_t* k1, int32_t* p1, int64_t n,
                      int key_bits, uint32_t** k_out, int32_t** p_out) {
  uint32_t* kin = k0;
  int32_t* pin = p0;
  uint32_t* kout = k1;
  int32_t* pout = p1;
  if (n <= 0) {
    *k_out = kin;
    *p_out = pin;
    return QFG_OK;
  }
  // Passes of at most kRTMaxBits bits through the staged round kernels.
  const int passes = std::max(1, (key_bits + kRTMaxBits - 1) / kRTMaxBits);
  const int step = (key_bits + passes - 1) / passes;
  int shift = 0;
  for (int pass = 0; pass < passes; ++pass) {
    const int bits = std::max(1, std::min(step, key_bits - shift));
    SortIO io{kin, pass == 0 ? nullptr : pin, kout, pout};
    QFG_TRY(round_pass(ctx, io, n, shift, bits, nullptr));
    shift += bits;
    std::swap(kin, kout);
    std::swap(pin, pout);
  }
  *k_out = kin;
  *p_out = pin;
  return QFG_OK;
}

__device__ __forceinline__ int64_t find_partition(const int64_t* __restrict__ offsets, int P,
                                                  int64_t i) {
  int lo = 0, hi = P - 1;  // largest p with offsets[p] <= i
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void bucket_counts_kernel(const int64_t* __restrict__ offsets, int P,
                                     uint32_t* __restrict__ nb) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const int64_t c = offsets[p + 1] - offsets[p];
    uint32_t v = 0;
    if (c > 0) {  // NEXT_POW_2 (storage/FoilHashTable.cpp:17-31)
      v = (uint32_t)c - 1u;
      v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16;
      v += 1u;
    }
    nb[p] = v;
  }
}

__global__ void bucket_meta_kernel(const uint32_t* __restrict__ nb, const uint32_t* __restrict__ nb_scan,
                                   const uint32_t* __restrict__ total, int P, int bits,
                                   int64_t* __restrict__ bucket_offsets, uint32_t* __restrict__ masks) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= P; p += gridDim.x * blockDim.x) {
    if (p == P) {
      bucket_offsets[P] = *total;
    } else {
      bucket_offsets[p] = nb_scan[p];
      masks[p] = nb[p] > 0 ? ((nb[p] - 1u) << bits) : 0u;
    }
  }
}

// Global bucket id of every partition position: bucket_offsets[p] +
// ((uint32)v & mask_p) >> bits (operations/BuildHashTable.cpp:81-84).
__global__ void partition_bucket_ids_kernel(const int2* __restrict__ tuples, int64_t n,
                                            const int64_t* __restrict__ offsets, int P, int bits,
                                            const int64_t* __restrict__ bucket_offsets,
                                            const uint32_t* __restrict__ masks,
                                            uint32_t* __restrict__ gid) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = find_partition(offsets, P, i);
    const uint32_t b = (ref_hash(tuples[i].x) & masks[p]) >> bits;
    gid[i] = (uint32_t)bucket_offsets[p] + b;
  }
}

// After a stable sort by global bucket id: link each position to its
// predecessor in the same bucket and make the last one the bucket head.
// Positions are relative to the segment that row i belongs to.
__global__ void chain_links_kernel(const uint32_t* __restrict__ sorted_gid,
                                   const int32_t* __restrict__ sorted_row, int64_t n,
                                   const int64_t* __restrict__ offsets, int P,
                                   int32_t* __restrict__ buckets, int32_t* __restrict__ next) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t g = sorted_gid[s];
    const int64_t i = sorted_row[s];
    const int64_t base = offsets != nullptr ? offsets[find_partition(offsets, P, i)] : 0;
    int32_t link = 0;
    if (s > 0 && sorted_gid[s - 1] == g) link = (int32_t)(sorted_row[s - 1] - base + 1);
    next[i] = link;
    if (s == n - 1 || sorted_gid[s + 1] != g) buckets[g] = (int32_t)(i - base + 1);
  }
}

// Hash<k> (utility/Hash.hpp:35-55) bucket of every row, mask = nb - 1.
__global__ void table_bucket_ids_kernel(const int32_t* const* __restrict__ keys, int num_keys,
                                        int64_t n, uint32_t mask, uint32_t* __restrict__ gid) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h = ref_hash(keys[0][i]);
    for (int k = 1; k < num_keys; ++k) h = ref_hash_combine(h, keys[k][i]);
    gid[i] = h & mask;
  }
}

// Count of every full radix digit (value & (P - 1)), privatised per block in
// shared memory (P <= 2^15 words), added to hist (zeroed) once per block.
__global__ void digit_hist_kernel(const int32_t* __restrict__ values, int64_t n, uint32_t P,
                                  uint32_t* __restrict__ hist) {
  extern __shared__ uint32_t sh[];
  for (uint32_t d = threadIdx.x; d < P; d += blockDim.x) sh[d] = 0u;
  __syncthreads();
  const uint32_t mask = P - 1u;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&sh[(uint32_t)__ldg(values + i) & mask], 1u);
  __syncthreads();
  for (uint32_t d = threadIdx.x; d < P; d += blockDim.x)
    if (sh[d] != 0u) atomicAdd(&hist[d], sh[d]);
}

__global__ void offsets_to_i64_kernel(const uint32_t* __restrict__ scanned, uint32_t P, int64_t n,
                                      int64_t* __restrict__ offsets) {
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d <= P; d += gridDim.x * blockDim.x)
    offsets[d] = d == P ? n : (int64_t)scanned[d];
}

int bits_for(uint64_t x) {  // smallest b with 2^b > x - 1, at least 1
  int b = 1;
  while (b < 32 && (uint64_t(1) << b) < x) ++b;
  return b;
}

unsigned grid_for(Ctx* ctx, int64_t n, int threads) {
  int64_t blocks = (n + threads - 1) / threads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)ctx->num_sms * 16));
}

}  // namespace

int sort_pairs_u32(Ctx* ctx, uint32_t* k0, int32_t* p0, uint32_t* k1, int32_t* p1, int64_t n,
                   int key_bits, uint32_t** k_out, int32_t** p_out) {
  return stable_sort_pairs(ctx, k0, p0, k1, p1, n, key_bits, k_out, p_out);
}

// Widest digit one staged pass takes (its per-warp digit counts stay small
// and a round's runs average 16 or more rows a digit); wider partitions take
// two passes.
constexpr int kMaxOnePassRefBits = kRTMaxBits;

int radix_partition_ref(Ctx* ctx, const int32_t* values, int64_t n, int bits, int32_t* out_tuples,
                        int64_t* out_offsets) {
  const uint32_t P = 1u << bits;
  if (n == 0) {
    QFG_CUDA(ctx, cudaMemsetAsync(out_offsets, 0, sizeof(int64_t) * (P + 1), ctx->stream));
    return QFG_OK;
  }
  if (bits <= kMaxOnePassRefBits) {
    RefTupleIO io{values, reinterpret_cast<int2*>(out_tuples)};
    return round_pass(ctx, io, n, 0, bits, out_offsets);
  }
  // Two stable LSD passes: the low digit (value, row index into SoA
  // scratch), then the high digit, writing the tuples.  Both are stable, so
  // the result is ordered by the full digit and, within it, by row: the
  // reference's partition order.  The offsets come from a count of the full
  // digit.
  const int lo = bits / 2, hi = bits - lo;
  QFG_TRY(ctx->scratch[kScrSortA].reserve(ctx, 2 * sizeof(uint32_t) * (size_t)n));
  uint32_t* mid_keys = ctx->scratch[kScrSortA].as<uint32_t>();
  int32_t* mid_rows = reinterpret_cast<int32_t*>(mid_keys + n);
  SortIO a{reinterpret_cast<const uint32_t*>(values), nullptr, mid_keys, mid_rows};
  QFG_TRY(round_pass(ctx, a, n, 0, lo, nullptr));
  SoAToRefIO b{mid_keys, mid_rows, reinterpret_cast<int2*>(out_tuples)};
  QFG_TRY(round_pass(ctx, b, n, lo, hi, nullptr));
  QFG_TRY(ctx->scratch[kScrTmpA].reserve(ctx, sizeof(uint32_t) * (size_t)(P + 1)));
  uint32_t* hist = ctx->scratch[kScrTmpA].as<uint32_t>();
  QFG_CUDA(ctx, cudaMemsetAsync(hist, 0, sizeof(uint32_t) * P, ctx->stream));
  const size_t smem = sizeof(uint32_t) * P;
  if (smem > 48 * 1024)
    QFG_CUDA(ctx, cudaFuncSetAttribute(digit_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
  int per_sm = 0;
  QFG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, digit_hist_kernel, 512, smem));
  const int64_t want = (n + 512 * 16 - 1) / (512 * 16);
  const unsigned grid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(want, (int64_t)ctx->num_sms * std::max(per_sm, 1)));
  digit_hist_kernel<<<grid, 512, smem, ctx->stream>>>(values, n, P, hist);
  QFG_LAUNCHED(ctx);
  QFG_TRY(exclusive_scan_u32(ctx, hist, hist, P, nullptr));
  offsets_to_i64_kernel<<<(P + 256) / 256, 256, 0, ctx->stream>>>(hist, P, n, out_offsets);
  QFG_LAUNCHED(ctx);
  return QFG_OK;
}

int relation_partitions(Ctx* ctx, Relation* rel, int column, int bits, PartitionedColumn** out) {
  auto key = std::make_pair(column, bits);
  auto it = rel->partitions.find(key);
  if (it != rel->partitions.end()) {
    *out = it->second.get();
    return QFG_OK;
  }
  auto pc = std::make_unique<PartitionedColumn>();
  pc->bits = bits;
  pc->n = rel->num_tuples;
  QFG_TRY(pc->tuples.reserve(ctx, sizeof(int32_t) * 2 * (size_t)std::max<int64_t>(pc->n, 1)));
  QFG_TRY(pc->offsets.reserve(ctx, sizeof(int64_t) * ((size_t(1) << bits) + 1)));
  QFG_TRY(radix_partition_ref(ctx, rel->columns[column], pc->n, bits, pc->tuples.as<int32_t>(),
                              pc->offsets.as<int64_t>()));
  *out = pc.get();
  rel->partitions[key] = std::move(pc);
  return QFG_OK;
}

}  // namespace qfg

using namespace qfg;

extern "C" int qfg_radix_partition(qfg_ctx* c, const int32_t* d_values, int64_t n, int bits,
                                   int32_t* d_out_tuples, int64_t* d_offsets) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (bits < 1 || bits > QFG_MAX_RADIX_BITS || n < 0 || n > INT32_MAX || d_offsets == nullptr ||
      (n > 0 && (d_values == nullptr || d_out_tuples == nullptr)))
    return set_error(ctx, QFG_ERR_INVALID, "qfg_radix_partition: invalid arguments");
  if (reinterpret_cast<uintptr_t>(d_out_tuples) % 8 != 0)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_radix_partition: d_out_tuples must be 8-byte aligned");
  return radix_partition_ref(ctx, d_values, n, bits, d_out_tuples, d_offsets);
}

extern "C" int qfg_build_hash_table_on_partitions(qfg_ctx* c, const int32_t* d_tuples,
                                                  const int64_t* d_offsets, int64_t n, int bits,
                                                  int32_t* d_buckets, int64_t* d_bucket_offsets,
                                                  uint32_t* d_masks, int32_t* d_next) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (bits < 1 || bits > QFG_MAX_RADIX_BITS || n < 0 || n > INT32_MAX / 2 ||
      d_offsets == nullptr || d_bucket_offsets == nullptr || d_masks == nullptr ||
      (n > 0 && (d_tuples == nullptr || d_buckets == nullptr || d_next == nullptr)))
    return set_error(ctx, QFG_ERR_INVALID, "qfg_build_hash_table_on_partitions: invalid arguments");
  if (reinterpret_cast<uintptr_t>(d_tuples) % 8 != 0)
    return set_error(ctx, QFG_ERR_INVALID,
                     "qfg_build_hash_table_on_partitions: d_tuples must be 8-byte aligned");
  const int P = 1 << bits;
  QFG_TRY(ctx->scratch[kScrTmpA].reserve(ctx, sizeof(uint32_t) * (size_t)(2 * P + 2)));
  uint32_t* nb = ctx->scratch[kScrTmpA].as<uint32_t>();
  uint32_t* nb_scan = nb + P;
  uint32_t* total = nb + 2 * P;
  bucket_counts_kernel<<<(P + 255) / 256, 256, 0, ctx->stream>>>(d_offsets, P, nb);
  QFG_LAUNCHED(ctx);
  QFG_TRY(exclusive_scan_u32(ctx, nb, nb_scan, P, total));
  bucket_meta_kernel<<<(P + 256) / 256, 256, 0, ctx->stream>>>(nb, nb_scan, total, P, bits,
                                                              d_bucket_offsets, d_masks);
  QFG_LAUNCHED(ctx);
  if (n == 0) return QFG_OK;
  // Buckets start empty (calloc in storage/FoilHashTable.cpp:44).
  QFG_CUDA(ctx, cudaMemsetAsync(d_buckets, 0, sizeof(int32_t) * (size_t)(2 * n), ctx->stream));
  QFG_TRY(ctx->scratch[kScrSortA].reserve(ctx, 2 * sizeof(uint32_t) * (size_t)n));
  QFG_TRY(ctx->scratch[kScrSortB].reserve(ctx, 2 * sizeof(uint32_t) * (size_t)n));
  uint32_t* k0 = ctx->scratch[kScrSortA].as<uint32_t>();
  int32_t* p0 = reinterpret_cast<int32_t*>(k0 + n);
  uint32_t* k1 = ctx->scratch[kScrSortB].as<uint32_t>();
  int32_t* p1 = reinterpret_cast<int32_t*>(k1 + n);
  partition_bucket_ids_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
      reinterpret_cast<const int2*>(d_tuples), n, d_offsets, P, bits, d_bucket_offsets, d_masks, k0);
  QFG_LAUNCHED(ctx);
  uint32_t* ks;
  int32_t* ps;
  QFG_TRY(stable_sort_pairs(ctx, k0, p0, k1, p1, n, bits_for((uint64_t)(2 * n + 1)), &ks, &ps));
  chain_links_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(ks, ps, n, d_offsets, P,
                                                                     d_buckets, d_next);
  QFG_LAUNCHED(ctx);
  return QFG_OK;
}

extern "C" int qfg_build_hash_table_on_table(qfg_ctx* c, const int32_t* const* d_keys,
                                             int32_t num_keys, int64_t n, int32_t* d_buckets,
                                             int32_t* d_next, uint32_t* mask_out) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_keys < 1 || num_keys > QFG_MAX_ARITY || n < 1 || n > INT32_MAX / 2 ||
      d_keys == nullptr || d_buckets == nullptr || d_next == nullptr || mask_out == nullptr)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_build_hash_table_on_table: invalid arguments");
  uint32_t nb = (uint32_t)n - 1u;
  nb |= nb >> 1; nb |= nb >> 2; nb |= nb >> 4; nb |= nb >> 8; nb |= nb >> 16;
  nb += 1u;
  const uint32_t mask = nb - 1u;
  *mask_out = mask;
  QFG_TRY(ctx->scratch[kScrTmpB].reserve(ctx, sizeof(const int32_t*) * QFG_MAX_ARITY));
  const int32_t** keys_dev = ctx->scratch[kScrTmpB].as<const int32_t*>();
  QFG_CUDA(ctx, cudaMemcpyAsync(keys_dev, d_keys, sizeof(const int32_t*) * num_keys,
                                cudaMemcpyHostToDevice, ctx->stream));
  QFG_CUDA(ctx, cudaMemsetAsync(d_buckets, 0, sizeof(int32_t) * nb, ctx->stream));
  QFG_TRY(ctx->scratch[kScrSortA].reserve(ctx, 2 * sizeof(uint32_t) * (size_t)n));
  QFG_TRY(ctx->scratch[kScrSortB].reserve(ctx, 2 * sizeof(uint32_t) * (size_t)n));
  uint32_t* k0 = ctx->scratch[kScrSortA].as<uint32_t>();
  int32_t* p0 = reinterpret_cast<int32_t*>(k0 + n);
  uint32_t* k1 = ctx->scratch[kScrSortB].as<uint32_t>();
  int32_t* p1 = reinterpret_cast<int32_t*>(k1 + n);
  table_bucket_ids_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(keys_dev, num_keys, n,
                                                                          mask, k0);
  QFG_LAUNCHED(ctx);
  uint32_t* ks;
  int32_t* ps;
  QFG_TRY(stable_sort_pairs(ctx, k0, p0, k1, p1, n, bits_for((uint64_t)nb), &ks, &ps));
  chain_links_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(ks, ps, n, nullptr, 1,
                                                                     d_buckets, d_next);
  QFG_LAUNCHED(ctx);
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return QFG_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free radix partition.
//
// Some callers cannot let a library allocate device memory: a host process
// that reserves all GPU memory for its own allocator and forbids cudaMalloc
// from plug-ins, or a latency-critical loop that cannot afford the device-wide
// synchronization that cudaMalloc / cudaFree imply.  qfg_radix_partition_static
// serves them: it computes the same stable partition as qfg_radix_partition,
// but its only working memory (the per-chunk digit counts and the scan of
// those counts) is the fixed array below, which every GPU that loads this
// library keeps for the life of the process.  Nothing is allocated per call.
//
// The array is shared by all calls on a device and keeps what the last call
// left in it; every word a call reads is written earlier in the same call,
// so nothing has to be cleared first.  Two calls whose work overlaps on the
// GPU (different streams, or different host threads) race on the array.

namespace qfg {
namespace {

constexpr int64_t kStaticScratchWords = int64_t(1) << 20;  // 4 MiB of uint32
constexpr int kStaticScanThreads = 512;
constexpr int kStaticScanItems = 8;
constexpr int64_t kStaticScanTile = kStaticScanThreads * kStaticScanItems;

static __device__ __align__(256) uint32_t g_static_scratch[kStaticScratchWords];

// Device address of g_static_scratch per device ordinal, looked up once with
// that device current (a host-side name of a __device__ array is not a device
// address).  The cache lives as long as the process: after cudaDeviceReset
// the module is loaded again and the cached address is stale, so the entry
// point must not be used across a device reset.
std::mutex g_static_mutex;
std::map<int, uint32_t*> g_static_ptr;

int static_scratch_for_current_device(uint32_t** out, std::string* err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return QFG_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_static_mutex);
  auto it = g_static_ptr.find(dev);
  if (it == g_static_ptr.end()) {
    uint32_t* ptr = nullptr;
    e = cudaGetSymbolAddress(reinterpret_cast<void**>(&ptr), g_static_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
      *err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return QFG_ERR_CUDA;
    }
    it = g_static_ptr.emplace(dev, ptr).first;
  }
  *out = it->second;
  return QFG_OK;
}

// In-place exclusive scan of up to kStaticScratchWords - tiles words: tile
// scans with tile sums, one CTA scanning the sums, then the offsets added.
__global__ void static_scan_tiles_kernel(uint32_t* __restrict__ data, int64_t n,
                                         uint32_t* __restrict__ tile_sums) {
  __shared__ uint32_t warp_tot[32];
  const int64_t base = (int64_t)blockIdx.x * kStaticScanTile + (int64_t)threadIdx.x * kStaticScanItems;
  uint32_t v[kStaticScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kStaticScanItems; ++k) {
    v[k] = base + k < n ? data[base + k] : 0u;
    sum += v[k];
  }
  uint32_t x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFullMask, x, o);
    if (lane_id() >= o) x += y;
  }
  if (lane_id() == 31) warp_tot[warp_id()] = x;
  __syncthreads();
  if (warp_id() == 0) {
    const int nw = blockDim.x >> 5;
    const uint32_t t = lane_id() < nw ? warp_tot[lane_id()] : 0u;
    uint32_t s = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFullMask, s, o);
      if (lane_id() >= o) s += y;
    }
    warp_tot[lane_id()] = s - t;
    if (lane_id() == 31) tile_sums[blockIdx.x] = s;
  }
  __syncthreads();
  uint32_t run = x - sum + warp_tot[warp_id()];
#pragma unroll
  for (int k = 0; k < kStaticScanItems; ++k) {
    if (base + k < n) data[base + k] = run;
    run += v[k];
  }
}

__global__ void static_scan_sums_kernel(uint32_t* __restrict__ sums, int ntiles) {
  if (threadIdx.x != 0) return;
  uint32_t run = 0;
  for (int i = 0; i < ntiles; ++i) {
    const uint32_t v = sums[i];
    sums[i] = run;
    run += v;
  }
}

__global__ void static_scan_add_kernel(uint32_t* __restrict__ data, int64_t n,
                                       const uint32_t* __restrict__ tile_offsets) {
  const uint32_t add = tile_offsets[blockIdx.x];
  const int64_t base = (int64_t)blockIdx.x * kStaticScanTile;
  for (int k = threadIdx.x; k < kStaticScanTile; k += blockDim.x)
    if (base + k < n) data[base + k] += add;
}

}  // namespace
}  // namespace qfg

extern "C" int qfg_radix_partition_static(void* stream, const int32_t* d_values, int64_t n,
                                          int bits, int32_t* d_out_tuples, int64_t* d_offsets,
                                          char* error, int error_len) {
  std::string err;
  auto fail = [&](int status, const std::string& msg) {
    if (error != nullptr && error_len > 0) {
      strncpy(error, msg.c_str(), (size_t)error_len - 1);
      error[error_len - 1] = '\0';
    }
    return status;
  };
  if (bits < 1 || bits > QFG_MAX_RADIX_BITS || n < 0 || n > INT32_MAX || d_offsets == nullptr ||
      (n > 0 && (d_values == nullptr || d_out_tuples == nullptr)))
    return fail(QFG_ERR_INVALID, "qfg_radix_partition_static: invalid arguments");
  if (reinterpret_cast<uintptr_t>(d_out_tuples) % 8 != 0)
    return fail(QFG_ERR_INVALID, "qfg_radix_partition_static: d_out_tuples must be 8-byte aligned");
  const PassShape s = pass_shape(std::max<int64_t>(n, 1), bits);
  const int64_t entries = s.num_chunks * (int64_t(1) << bits);
  const int64_t tiles = (entries + kStaticScanTile - 1) / kStaticScanTile;
  if (entries + tiles > kStaticScratchWords)
    return fail(QFG_ERR_INVALID,
                "qfg_radix_partition_static: " + std::to_string(n) + " values at " +
                    std::to_string(bits) + " radix bits need " + std::to_string(entries + tiles) +
                    " scratch words, more than the " + std::to_string(kStaticScratchWords) +
                    " of the static scratch array");
  // An error left pending by the caller's own earlier CUDA work would be
  // returned by the launch checks below as if a launch of this call had
  // failed; report it as what it is and leave it pending.
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess)
    return fail(QFG_ERR_CUDA, std::string("qfg_radix_partition_static: a CUDA error was pending "
                                          "before the call: ") + cudaGetErrorString(e));
  uint32_t* scratch = nullptr;
  int st = static_scratch_for_current_device(&scratch, &err);
  if (st != QFG_OK) return fail(st, err);
  cudaStream_t strm = static_cast<cudaStream_t>(stream);
  const uint32_t P = 1u << bits;
  if (n == 0) {
    e = cudaMemsetAsync(d_offsets, 0, sizeof(int64_t) * (P + 1), strm);
    return e == cudaSuccess ? QFG_OK : fail(QFG_ERR_CUDA, cudaGetErrorString(e));
  }
  uint32_t* hist = scratch;
  uint32_t* tile_sums = scratch + entries;
  RefTupleIO io{d_values, reinterpret_cast<int2*>(d_out_tuples)};
  if (s.smem > 48 * 1024) {
    e = cudaFuncSetAttribute(stable_hist_kernel<RefTupleIO>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(stable_scatter_kernel<RefTupleIO>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e != cudaSuccess) return fail(QFG_ERR_CUDA, cudaGetErrorString(e));
  }
  // Each launch is checked on its own, so a failure names its kernel.
  auto launched = [&](const char* kernel) -> int {
    const cudaError_t le = cudaGetLastError();
    if (le == cudaSuccess) return QFG_OK;
    return fail(QFG_ERR_CUDA, std::string("qfg_radix_partition_static: launch of ") + kernel +
                                  " failed: " + cudaGetErrorString(le));
  };
  stable_hist_kernel<RefTupleIO><<<s.grid, 32 * s.warps, s.smem, strm>>>(io, n, 0, bits, s.chunk,
                                                                          s.num_chunks, hist);
  QFG_TRY(launched("stable_hist_kernel"));
  static_scan_tiles_kernel<<<(unsigned)tiles, kStaticScanThreads, 0, strm>>>(hist, entries, tile_sums);
  QFG_TRY(launched("static_scan_tiles_kernel"));
  static_scan_sums_kernel<<<1, 32, 0, strm>>>(tile_sums, (int)tiles);
  QFG_TRY(launched("static_scan_sums_kernel"));
  static_scan_add_kernel<<<(unsigned)tiles, kStaticScanThreads, 0, strm>>>(hist, entries, tile_sums);
  QFG_TRY(launched("static_scan_add_kernel"));
  digit_offsets_kernel<<<(P + 256) / 256, 256, 0, strm>>>(hist, s.num_chunks, bits, n, d_offsets);
  QFG_TRY(launched("digit_offsets_kernel"));
  stable_scatter_kernel<RefTupleIO><<<s.grid, 32 * s.warps, s.smem, strm>>>(io, n, 0, bits, s.chunk,
                                                                             s.num_chunks, hist);
  QFG_TRY(launched("stable_scatter_kernel"));
  return QFG_OK;
}
