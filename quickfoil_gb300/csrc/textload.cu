// textload.cu -- '|'-delimited text to device columns.
//
// LoadData (main/main.cpp:49-109) reads a predicate's facts from text: one
// fact a line (std::getline, '\n'), lines that are empty or start with '#'
// skipped, fields split at every '|' (boost::split, empty fields kept), the
// field count checked against the predicate's arguments, every argument the
// configuration does not skip converted by std::stoi (FromString<kInt32>,
// types/FromString.hpp:23-30: leading white space, an optional sign, at
// least one digit, the value within int32, anything after the digits
// ignored).  The reference aborts on a bad line; here the call returns an
// error naming the first bad line.
//
// On the device: the text is cut into 4 KiB tiles; a first pass counts the
// newlines of every tile (256 threads read the tile's bytes coalesced, one
// ballot per 256 bytes), an exclusive scan of the tile counts gives each
// tile its first line, a second pass writes the position of every newline.
// Then one thread per line parses its fields into line-indexed columns in
// one pass (32-bit offsets; the kernel is issue-bound, so the pass count and
// the index width are what cost) and a ballot per 32 lines marks the data
// lines; the row compaction of coverage.cu keeps those, in order.
#include <cstring>
#include <vector>

#include "qfg_common.cuh"

// Row compaction of the coverage operators (coverage.cu).
extern "C" int qfg_compact_rows(qfg_ctx* ctx, int32_t num_columns, const int32_t* const* d_columns,
                                int64_t num_rows, const uint64_t* d_bits, int32_t keep_set,
                                int32_t* const* d_out_columns, int64_t out_capacity,
                                int64_t* num_out);

namespace qfg {

namespace {

constexpr int kTextThreads = 256;
constexpr int kTextTileBytes = 16 * kTextThreads;
constexpr int kMaxTextArgs = 64;

enum : unsigned long long {
  kTextBadFieldCount = 1,
  kTextNoDigits = 2,
  kTextOutOfRange = 3,
};

// Newline bytes of a 32-bit word: bit 7 of each byte set where it is '\n'
// (the classic zero-byte test on word ^ 0x0a0a0a0a, exact for every byte).
__device__ __forceinline__ uint32_t newline_bytes(uint32_t w) {
  const uint32_t x = w ^ 0x0a0a0a0au;
  return ~(((x & 0x7f7f7f7fu) + 0x7f7f7f7fu) | x | 0x7f7f7f7fu);
}

// The same two passes with one 16-byte load a thread (the text's start
// 16-byte aligned): thread t owns bytes [16 t, 16 t + 16) of the tile, a
// block scan of the threads' newline counts orders the positions.
template <int PASS>
__global__ void __launch_bounds__(kTextThreads)
text_newlines16_kernel(const uint8_t* __restrict__ text, int64_t n, int64_t ntiles,
                       uint32_t* __restrict__ tile_count, const uint32_t* __restrict__ tile_first,
                       int64_t* __restrict__ nl_pos) {
  __shared__ uint32_t warp_nl[kTextThreads / 32];
  const int lane = lane_id(), warp = threadIdx.x / 32;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t p0 = tile * kTextTileBytes + 16 * (int64_t)threadIdx.x;
    uint32_t m[4] = {0u, 0u, 0u, 0u};
    if (p0 + 16 <= n) {
      const uint4 v = *reinterpret_cast<const uint4*>(text + p0);
      m[0] = newline_bytes(v.x);
      m[1] = newline_bytes(v.y);
      m[2] = newline_bytes(v.z);
      m[3] = newline_bytes(v.w);
    } else {
      for (int b = 0; b < 16 && p0 + b < n; ++b)
        if (text[p0 + b] == '\n') m[b >> 2] |= 0x80u << (8 * (b & 3));
    }
    const uint32_t mine = __popc(m[0]) + __popc(m[1]) + __popc(m[2]) + __popc(m[3]);
    uint32_t incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(kFullMask, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) warp_nl[warp] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < kTextThreads / 32; ++w) {
      if (w < warp) before += warp_nl[w];
      total += warp_nl[w];
    }
    if (PASS == 1 && mine != 0) {
      uint32_t idx = tile_first[tile] + before + incl - mine;
      for (int q = 0; q < 4; ++q)
        for (uint32_t b = m[q]; b != 0; b &= b - 1) nl_pos[idx++] = p0 + 4 * q + ((__ffs(b) - 1) >> 3);
    }
    if (PASS == 0 && threadIdx.x == 0) tile_count[tile] = total;
    __syncthreads();
  }
}

// pass 0: newlines per tile -> tile_count; pass 1: newline positions, the
// tile's first newline index read from tile_first.
template <int PASS>
__global__ void __launch_bounds__(kTextThreads)
text_newlines_kernel(const uint8_t* __restrict__ text, int64_t n, int64_t ntiles,
                     uint32_t* __restrict__ tile_count, const uint32_t* __restrict__ tile_first,
                     int64_t* __restrict__ nl_pos) {
  __shared__ uint32_t warp_nl[kTextThreads / 32];
  const int lane = lane_id(), warp = threadIdx.x / 32;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t base = tile * kTextTileBytes;
    uint32_t running = PASS == 1 ? tile_first[tile] : 0u;
    for (int j = 0; j < kTextTileBytes / kTextThreads; ++j) {
      const int64_t p = base + (int64_t)j * kTextThreads + threadIdx.x;
      const bool nl = p < n && text[p] == '\n';
      const unsigned ball = __ballot_sync(kFullMask, nl);
      if (lane == 0) warp_nl[warp] = __popc(ball);
      __syncthreads();
      uint32_t before = 0, total = 0;
      for (int w = 0; w < kTextThreads / 32; ++w) {
        if (w < warp) before += warp_nl[w];
        total += warp_nl[w];
      }
      if (PASS == 1 && nl)
        nl_pos[running + before + __popc(ball & ((1u << lane) - 1u))] = p;
      running += total;
      __syncthreads();
    }
    if (PASS == 0 && threadIdx.x == 0) tile_count[tile] = running;
  }
}

__device__ __forceinline__ bool c_space(uint8_t c) {
  return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

struct ParseArgs {
  const uint8_t* text;
  int64_t n;
  const int64_t* nl_pos;
  int64_t num_nl;
  int64_t num_lines;
  int num_args;
  unsigned long long skipped;  // bit i: argument i skipped
  int32_t* cols;               // kept columns, line-indexed (stride num_lines)
  uint32_t* keep_words;        // bit per line: a data line
  unsigned long long* error;   // (line << 2 | code), atomicMin
};

// One thread per line (whole warps per 32 lines, for the ballot), one pass
// over the line with 32-bit offsets: each kept field is converted where it
// starts, every separator is counted, and a field count that differs wins
// over a conversion error (the reference checks the count first).
__global__ void __launch_bounds__(kTextThreads) text_parse_kernel(ParseArgs a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int lane = lane_id();
  for (int64_t li = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; li - lane < a.num_lines;
       li += stride) {
    bool keep = false;
    if (li < a.num_lines) {
      const int64_t s = li == 0 ? 0 : a.nl_pos[li - 1] + 1;
      const int64_t e = li < a.num_nl ? a.nl_pos[li] : a.n;
      const uint8_t* __restrict__ lp = a.text + s;
      const int len = (int)(e - s);
      if (len > 0 && __ldg(lp) != '#') {
        keep = true;
        unsigned long long err = 0;
        int field = 0, col = 0, i = 0;
        for (;;) {
          if (field < a.num_args && !((a.skipped >> field) & 1ull)) {
            if (err == 0) {
              // std::stoi on the field starting at i
              int j = i;
              uint8_t c = j < len ? __ldg(lp + j) : 0;
              while (j < len && c_space(c)) c = ++j < len ? __ldg(lp + j) : 0;
              bool neg = false;
              if (j < len && (c == '+' || c == '-')) {
                neg = c == '-';
                c = ++j < len ? __ldg(lp + j) : 0;
              }
              if (j >= len || c < '0' || c > '9') {
                err = kTextNoDigits;
              } else {
                unsigned long long v = 0;
                bool over = false;
                while (j < len && c >= '0' && c <= '9') {
                  if (!over) {
                    v = v * 10 + (c - '0');
                    over = v > 2147483648ull;
                  }
                  c = ++j < len ? __ldg(lp + j) : 0;
                }
                if (over || (!neg && v > 2147483647ull)) err = kTextOutOfRange;
                else a.cols[(int64_t)col * a.num_lines + li] = neg ? (int32_t)(-(long long)v) : (int32_t)v;
              }
              i = j;
            }
            ++col;
          }
          while (i < len && __ldg(lp + i) != '|') ++i;
          ++field;
          if (i >= len) break;
          ++i;
        }
        if (field != a.num_args) err = kTextBadFieldCount;
        if (err != 0) atomicMin(a.error, ((unsigned long long)li << 2) | err);
      }
    }
    const unsigned ball = __ballot_sync(kFullMask, keep);
    if (lane == 0 && li < a.num_lines + 32) a.keep_words[li >> 5] = ball;
  }
}

}  // namespace

// Parses text already on the device into out columns (capacity rows each).
int parse_text_device(Ctx* ctx, qfg_ctx* c, const uint8_t* text, int64_t n, int num_args,
                      const int32_t* skipped, int32_t* const* out, int64_t capacity,
                      int64_t* num_rows, int64_t* error_line) {
  *num_rows = 0;
  if (error_line != nullptr) *error_line = 0;
  if (n == 0) return QFG_OK;
  unsigned long long skip_mask = 0;
  int kept = 0;
  for (int i = 0; i < num_args; ++i) {
    if (skipped != nullptr && skipped[i] != 0) skip_mask |= 1ull << i;
    else ++kept;
  }
  // Working memory in the context's grow-only scratch (nothing is allocated
  // once a text of this size has been parsed): tile counts, newline
  // positions, line-indexed columns, line bits; a host text is staged in
  // TmpB.  The row compaction uses TmpA and the scan its own slot.
  const int64_t ntiles = (n + kTextTileBytes - 1) / kTextTileBytes;
  DevBuf& tiles = ctx->scratch[kScrSortA];
  QFG_TRY(tiles.reserve(ctx, sizeof(uint32_t) * (size_t)(2 * ntiles + 1)));
  uint32_t* tile_count = tiles.as<uint32_t>();
  uint32_t* tile_first = tile_count + ntiles;
  uint32_t* total = tile_first + ntiles;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)ctx->num_sms * 8));
  const bool aligned16 = ((uintptr_t)text & 15) == 0;
  if (aligned16)
    text_newlines16_kernel<0><<<grid, kTextThreads, 0, ctx->stream>>>(text, n, ntiles, tile_count,
                                                                      nullptr, nullptr);
  else
    text_newlines_kernel<0><<<grid, kTextThreads, 0, ctx->stream>>>(text, n, ntiles, tile_count,
                                                                    nullptr, nullptr);
  QFG_LAUNCHED(ctx);
  QFG_TRY(exclusive_scan_u32(ctx, tile_count, tile_first, ntiles, total));
  uint32_t num_nl = 0;
  uint8_t last = 0;
  QFG_CUDA(ctx, cudaMemcpyAsync(&num_nl, total, sizeof(num_nl), cudaMemcpyDeviceToHost, ctx->stream));
  QFG_CUDA(ctx, cudaMemcpyAsync(&last, text + n - 1, 1, cudaMemcpyDeviceToHost, ctx->stream));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const int64_t num_lines = (int64_t)num_nl + (last != '\n' ? 1 : 0);
  if (num_lines > INT32_MAX)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_parse_text: more than 2^31 - 1 lines");
  DevBuf& pos = ctx->scratch[kScrSortB];
  DevBuf& colbuf = ctx->scratch[kScrJoin];
  DevBuf& keep = ctx->scratch[kScrJoin2];
  QFG_TRY(pos.reserve(ctx, sizeof(int64_t) * (size_t)std::max<uint32_t>(num_nl, 1)));
  QFG_TRY(colbuf.reserve(ctx, sizeof(int32_t) * (size_t)std::max(kept, 1) * (size_t)num_lines));
  const int64_t nwords = (num_lines + 31) / 32 + 2;  // 64-bit blocks for the compaction
  // line bits, then the error word (8-byte aligned)
  const size_t err_off = ((sizeof(uint32_t) * (size_t)(nwords + 1)) + 7) & ~(size_t)7;
  QFG_TRY(keep.reserve(ctx, err_off + sizeof(unsigned long long)));
  unsigned long long* err_word = reinterpret_cast<unsigned long long*>(keep.as<char>() + err_off);
  QFG_CUDA(ctx, cudaMemsetAsync(keep.ptr(), 0, sizeof(uint32_t) * (size_t)(nwords + 1), ctx->stream));
  QFG_CUDA(ctx, cudaMemsetAsync(err_word, 0xff, sizeof(unsigned long long), ctx->stream));
  if (num_nl > 0) {
    if (aligned16)
      text_newlines16_kernel<1><<<grid, kTextThreads, 0, ctx->stream>>>(
          text, n, ntiles, nullptr, tile_first, pos.as<int64_t>());
    else
      text_newlines_kernel<1><<<grid, kTextThreads, 0, ctx->stream>>>(
          text, n, ntiles, nullptr, tile_first, pos.as<int64_t>());
    QFG_LAUNCHED(ctx);
  }
  ParseArgs pa;
  pa.text = text;
  pa.n = n;
  pa.nl_pos = pos.as<int64_t>();
  pa.num_nl = num_nl;
  pa.num_lines = num_lines;
  pa.num_args = num_args;
  pa.skipped = skip_mask;
  pa.cols = colbuf.as<int32_t>();
  pa.keep_words = keep.as<uint32_t>();
  pa.error = err_word;
  const unsigned pgrid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((num_lines + kTextThreads - 1) / kTextThreads, (int64_t)ctx->num_sms * 8));
  text_parse_kernel<<<pgrid, kTextThreads, 0, ctx->stream>>>(pa);
  QFG_LAUNCHED(ctx);
  unsigned long long e = 0;
  QFG_CUDA(ctx, cudaMemcpyAsync(&e, err_word, sizeof(e), cudaMemcpyDeviceToHost, ctx->stream));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (e != ~0ull) {
    const int64_t line = (int64_t)(e >> 2) + 1;
    if (error_line != nullptr) *error_line = line;
    const char* why = (e & 3) == kTextBadFieldCount ? "field count differs from the arguments"
                      : (e & 3) == kTextNoDigits    ? "a field is not a number"
                                                    : "a number is out of the int32 range";
    return set_error(ctx, QFG_ERR_INVALID,
                     "qfg_parse_text: line " + std::to_string(line) + ": " + why);
  }
  std::vector<const int32_t*> in((size_t)std::max(kept, 1));
  for (int q = 0; q < kept; ++q) in[q] = colbuf.as<int32_t>() + (size_t)q * num_lines;
  if (kept == 0) {
    // nothing to keep but the row count
    int64_t rows = 0;
    QFG_TRY(qfg_compact_rows(c, 0, in.data(), num_lines,
                             reinterpret_cast<const uint64_t*>(keep.ptr()), 1, nullptr, INT64_MAX,
                             &rows));
    *num_rows = rows;
    return QFG_OK;
  }
  int64_t rows = 0;
  const int rc = qfg_compact_rows(c, kept, in.data(), num_lines,
                                  reinterpret_cast<const uint64_t*>(keep.ptr()), 1, out, capacity,
                                  &rows);
  *num_rows = rows;
  if (rc != QFG_OK) return rc;
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return QFG_OK;
}

}  // namespace qfg

using namespace qfg;

extern "C" int qfg_parse_text(qfg_ctx* c, const char* text, int64_t num_bytes, int flags,
                              int32_t num_arguments, const int32_t* skipped,
                              int32_t* const* d_out_columns, int64_t capacity, int64_t* num_rows,
                              int64_t* error_line) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_rows == nullptr || num_bytes < 0 || (num_bytes > 0 && text == nullptr) ||
      num_arguments < 1 || num_arguments > kMaxTextArgs || capacity < 0 ||
      (flags != QFG_HOST && flags != QFG_DEVICE_BORROW))
    return set_error(ctx, QFG_ERR_INVALID, "qfg_parse_text: invalid arguments");
  int kept = 0;
  for (int i = 0; i < num_arguments; ++i) kept += skipped == nullptr || skipped[i] == 0;
  if (kept > 0 && capacity > 0 && d_out_columns == nullptr)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_parse_text: no output columns");
  const uint8_t* dtext = reinterpret_cast<const uint8_t*>(text);
  if (flags == QFG_HOST && num_bytes > 0) {
    DevBuf& staged = ctx->scratch[kScrTmpB];
    QFG_TRY(staged.reserve(ctx, (size_t)num_bytes));
    QFG_CUDA(ctx, cudaMemcpyAsync(staged.ptr(), text, (size_t)num_bytes, cudaMemcpyHostToDevice,
                                  ctx->stream));
    dtext = staged.as<uint8_t>();
  }
  return parse_text_device(ctx, c, dtext, num_bytes, num_arguments, skipped, d_out_columns,
                           capacity, num_rows, error_line);
}

extern "C" int qfg_relation_register_text(qfg_ctx* c, int32_t relation_id, const char* text,
                                          int64_t num_bytes, int flags, int32_t num_arguments,
                                          const int32_t* skipped, int64_t* num_tuples,
                                          int64_t* error_line) {
  if (c == nullptr) return QFG_ERR_INVALID;
  Ctx* ctx = &c->impl;
  if (num_tuples == nullptr)
    return set_error(ctx, QFG_ERR_INVALID, "qfg_relation_register_text: null argument");
  int kept = 0;
  for (int i = 0; i < num_arguments && i < kMaxTextArgs; ++i)
    kept += skipped == nullptr || skipped[i] == 0;
  if (kept < 1 || kept > QFG_MAX_ARITY)
    return set_error(ctx, QFG_ERR_INVALID,
                     "qfg_relation_register_text: 1 to 8 arguments must be kept");
  // Lines bound the rows: count them on the host side of the text when it
  // is there, else take one row per byte pair (a row needs a digit and a
  // newline).
  int64_t cap = num_bytes / 2 + 1;
  if (flags == QFG_HOST) {
    cap = 1;
    for (int64_t i = 0; i < num_bytes; ++i) cap += text[i] == '\n';
  }
  DevBuf out;
  QFG_TRY(out.reserve(ctx, sizeof(int32_t) * (size_t)kept * (size_t)cap));
  std::vector<int32_t*> cols(kept);
  for (int q = 0; q < kept; ++q) cols[q] = out.as<int32_t>() + (size_t)q * cap;
  int64_t rows = 0;
  QFG_TRY(qfg_parse_text(c, text, num_bytes, flags, num_arguments, skipped, cols.data(), cap,
                         &rows, error_line));
  std::vector<const int32_t*> ccols(cols.begin(), cols.end());
  QFG_TRY(qfg_relation_register(c, relation_id, kept, ccols.data(), rows, QFG_DEVICE_COPY));
  QFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *num_tuples = rows;
  return QFG_OK;
}
