// keysets.cuh -- device key sets shared by the join and coverage operators.
//
// A key set holds the distinct key tuples of one table in an open-addressing
// table (linear probing, at least twice as many slots as rows) whose slots
// hold the row that first claimed the tuple (atomicCAS); every row of the
// table maps to that representative.  Key columns are int32 device columns.
#ifndef QFG_KEYSETS_CUH_
#define QFG_KEYSETS_CUH_

#include "qfg_common.cuh"

namespace qfg {

namespace {

struct KeyCols {
  const int32_t* c[QFG_MAX_ARITY];
  int nk;
};

// NK > 0: the key count is NK, known at compile time (loops unrolled, the
// column pointers stay in parameter space); NK == 0: k.nk at run time.
template <int NK = 0>
__device__ __forceinline__ uint32_t keys_hash(const KeyCols& k, int64_t r) {
  uint32_t h = mix32((uint32_t)k.c[0][r]);
  if constexpr (NK > 0) {
#pragma unroll
    for (int q = 1; q < NK; ++q) h = mix32(h + 0x9e3779b9u + (uint32_t)k.c[q][r]);
  } else {
    for (int q = 1; q < k.nk; ++q) h = mix32(h + 0x9e3779b9u + (uint32_t)k.c[q][r]);
  }
  return h;
}

template <int NK = 0>
__device__ __forceinline__ bool keys_eq(const KeyCols& a, int64_t x, const KeyCols& b, int64_t y) {
  if constexpr (NK > 0) {
    bool eq = true;
#pragma unroll
    for (int q = 0; q < NK; ++q) eq &= a.c[q][x] == b.c[q][y];
    return eq;
  } else {
    for (int q = 0; q < a.nk; ++q)
      if (a.c[q][x] != b.c[q][y]) return false;
    return true;
  }
}

// Inserts row r; returns the row that represents its key tuple.  The table
// holds at least twice as many slots as rows, so a free slot always exists.
template <int NK = 0>
__device__ __forceinline__ int32_t keyset_insert(const KeyCols& build, int32_t* __restrict__ owner,
                                                 uint32_t mask, int64_t r) {
  uint32_t slot = keys_hash<NK>(build, r) & mask;
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    // A slot only ever goes from free to owned: a plain read that sees an
    // owner is final, and repeated keys then spare the slot's atomics.
    int32_t o = owner[slot];
    if (o == -1) o = atomicCAS(&owner[slot], -1, (int32_t)r);
    if (o == -1) return (int32_t)r;
    if (keys_eq<NK>(build, o, build, r)) return o;
    slot = (slot + 1) & mask;
  }
  return -1;
}

template <int NK = 0>
__global__ void keyset_insert_kernel(KeyCols build, int64_t n, int32_t* __restrict__ owner,
                                     uint32_t mask, int32_t* __restrict__ rep) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t o = keyset_insert<NK>(build, owner, mask, r);
    if (rep != nullptr) rep[r] = o;
  }
}

template <int NK = 0>
__device__ __forceinline__ int32_t keyset_find(const KeyCols& build, const int32_t* __restrict__ owner,
                                               uint32_t mask, const KeyCols& probe, int64_t i) {
  uint32_t slot = keys_hash<NK>(probe, i) & mask;
  for (uint32_t p = 0; p <= mask; ++p) {
    const int32_t o = owner[slot];
    if (o < 0) return -1;
    if (keys_eq<NK>(build, o, probe, i)) return o;
    slot = (slot + 1) & mask;
  }
  return -1;
}

// keyset_insert_kernel with the key count fixed for 1-3 keys.
void launch_keyset_insert(unsigned grid, cudaStream_t st, const KeyCols& keys, int64_t n,
                          int32_t* owner, uint32_t mask, int32_t* rep) {
  switch (keys.nk) {
    case 1: keyset_insert_kernel<1><<<grid, 256, 0, st>>>(keys, n, owner, mask, rep); break;
    case 2: keyset_insert_kernel<2><<<grid, 256, 0, st>>>(keys, n, owner, mask, rep); break;
    case 3: keyset_insert_kernel<3><<<grid, 256, 0, st>>>(keys, n, owner, mask, rep); break;
    default: keyset_insert_kernel<0><<<grid, 256, 0, st>>>(keys, n, owner, mask, rep); break;
  }
}

unsigned rows_grid(Ctx* ctx, int64_t n) {
  const int64_t blocks = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)ctx->num_sms * 8));
}

uint32_t table_mask(int64_t n) {
  uint32_t cap = 64;
  while (cap < (uint64_t)(2 * n)) cap <<= 1;
  return cap - 1;
}

}  // namespace

}  // namespace qfg

#endif  // QFG_KEYSETS_CUH_
