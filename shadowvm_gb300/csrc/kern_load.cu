// The reference's text Loader (core/operator.cpp:24-48, conversions
// com/cpp/com.cu:33-44) as data-parallel passes over a text buffer in device
// memory, one warp per 4 KB span:
//
//   1. every span is summarised: row delimiters in it, column delimiters
//      after its last row delimiter, whether it has one;
//   2. an exclusive scan of the summaries (rows add; columns restart at a
//      row delimiter) gives each span's starting row and column;
//   3. every span converts the fields that END in it (a column delimiter).
//      A field that began in an earlier span is found by looking back at
//      most 4096 bytes.
//
// Spans are laid on the 16-byte grid of the text's address ("virtual"
// positions: v = real position + (text & 15)), so every full 16-byte
// granule is one aligned vector load; the few partial granules at the two
// ends are read byte by byte and masked.
//
// Within a span the warp walks 512-byte sub-tiles, lane l owning granule l:
// 16-bit masks of its column and row delimiters (SWAR byte compares), one
// packed warp scan for the row and column at the granule's start, a ballot
// for where its first field began; the lane then lists the fields that end in
// its granule (start, end, row, column) in a per-warp list in text order.
// Once 64 or more fields wait, the warp converts them 32 at a time, so every
// lane has a field in every round but the last.  Field bytes are read from
// the span staged in shared memory (plus a 64-byte halo before it).
//
// Items convert as strtol(s, NULL, 10) on LP64 -- leading isspace, optional
// sign, decimal digits, clamp to the 64-bit range on overflow -- then Int32
// columns keep the low 32 bits (atoi), Int64 columns the value (atol).
#include <atomic>

#include "kern_common.cuh"
#include "kernels.h"

namespace svm {
namespace {

constexpr int kSpan = 4096;       // bytes per warp work unit
constexpr int kSub = 512;         // bytes per sub-tile (16 per lane)
constexpr int kHalo = 64;         // staged bytes before the span
constexpr int kStage = kHalo + kSpan;
constexpr int kMaxItem = 4095;    // longest item (the reference's item buffer holds 4096 chars)
constexpr int kScanBlock = 1024;  // summaries per scan block
constexpr int kWarps = 8;         // warps per block (summary and parse)

__device__ __forceinline__ LoadPos combine(const LoadPos& a, const LoadPos& b) {
  LoadPos r;
  r.rows = a.rows + b.rows;
  r.cols = b.has ? b.cols : a.cols + b.cols;
  r.has = a.has | b.has;
  return r;
}

// 0x80 in exactly the bytes of t that are zero.
__device__ __forceinline__ uint32_t zero_bytes(uint32_t t) {
  return ~(((t & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | t | 0x7F7F7F7Fu);
}

// 4-bit mask (bit k = byte k) from 0x80-per-byte flags: the four flag bits
// (7, 15, 23, 31) move to bits 28..31 under one multiply whose partial
// products never overlap.
__device__ __forceinline__ uint32_t pack_flags(uint32_t f) { return (f * 0x00204081u) >> 28; }

// 16-bit mask of the bytes of w equal to the byte replicated in rep.
__device__ __forceinline__ uint32_t eq_mask16(const uint4& w, uint32_t rep) {
  return pack_flags(zero_bytes(w.x ^ rep)) | (pack_flags(zero_bytes(w.y ^ rep)) << 4) |
         (pack_flags(zero_bytes(w.z ^ rep)) << 8) | (pack_flags(zero_bytes(w.w ^ rep)) << 12);
}

__device__ __forceinline__ uint32_t rep4(char c) { return 0x01010101u * (uint32_t)(uint8_t)c; }

struct Text {
  const uint8_t* p;  // real byte 0
  const uint4* g;    // the 16-byte granule holding real byte 0
  long long mis;     // virtual position of real byte 0 (0..15)
  long long vend;    // virtual end: mis + bytes

  __device__ __forceinline__ Text(const uint8_t* text, unsigned long long bytes) {
    p = text;
    mis = (long long)(reinterpret_cast<uintptr_t>(text) & 15);
    g = reinterpret_cast<const uint4*>(text - mis);
    vend = mis + (long long)bytes;
  }
  // Mask of the real bytes in the granule at virtual position gb (a multiple of 16).
  __device__ __forceinline__ uint32_t valid16(long long gb) const {
    if (gb >= mis && gb + 16 <= vend) return 0xFFFFu;
    const long long lo = mis - gb > 0 ? mis - gb : 0;
    const long long hi = vend - gb < 16 ? vend - gb : 16;
    if (hi <= lo) return 0u;
    return ((1u << hi) - 1u) & ~((1u << lo) - 1u);
  }
  // Granule gi (virtual bytes [16 gi, 16 gi + 16)); bytes outside the text are zero.
  __device__ __forceinline__ uint4 granule(long long gi) const {
    const long long v0 = gi * 16;
    if (v0 >= mis && v0 + 16 <= vend) return g[gi];
    uint32_t b[4] = {0u, 0u, 0u, 0u};
    for (int k = 0; k < 16; k++) {
      const long long v = v0 + k;
      if (v >= mis && v < vend) b[k >> 2] |= (uint32_t)p[v - mis] << (8 * (k & 3));
    }
    return make_uint4(b[0], b[1], b[2], b[3]);
  }
  __device__ __forceinline__ uint8_t byte(long long v) const { return p[v - mis]; }
};

// Summary of one sub-tile from each lane's delimiter masks (warp-uniform result).
__device__ __forceinline__ LoadPos subtile_summary(uint32_t cd16, uint32_t rd16, int lane) {
  const uint32_t rbal = __ballot_sync(0xffffffffu, rd16 != 0);
  const int last = rbal ? 31 - __clz(rbal) : -1;  // last lane holding a row delimiter
  // column delimiters after the lane's last row delimiter (all of them without one)
  const uint32_t after = __popc(cd16 >> (32 - __clz(rd16)));
  const uint32_t mine = lane > last ? (uint32_t)__popc(cd16) : lane == last ? after : 0u;
  LoadPos t;
  t.rows = __reduce_add_sync(0xffffffffu, (uint32_t)__popc(rd16));
  t.cols = __reduce_add_sync(0xffffffffu, mine);
  t.has = rbal != 0;
  return t;
}

__global__ void __launch_bounds__(kWarps * 32) load_summary_kernel(const uint8_t* text, unsigned long long bytes,
                                                                  char cd, char rd, unsigned long long nspans,
                                                                  LoadPos* sum) {
  const Text tx(text, bytes);
  const int lane = threadIdx.x & 31;
  const uint32_t cdx = rep4(cd), rdx = rep4(rd);
  for (unsigned long long s = blockIdx.x * (unsigned long long)kWarps + (threadIdx.x >> 5); s < nspans;
       s += (unsigned long long)gridDim.x * kWarps) {
    const long long g0 = (long long)(s * (kSpan / 16)) + lane;
    uint4 w[kSpan / kSub];
#pragma unroll
    for (int q = 0; q < kSpan / kSub; q++) w[q] = tx.granule(g0 + q * (kSub / 16));
    LoadPos acc{0ull, 0u, 0u};
#pragma unroll
    for (int q = 0; q < kSpan / kSub; q++) {
      const uint32_t valid = tx.valid16((g0 + q * (kSub / 16)) * 16);
      const uint32_t cd16 = eq_mask16(w[q], cdx) & valid;
      const uint32_t rd16 = eq_mask16(w[q], rdx) & valid;
      acc = combine(acc, subtile_summary(cd16, rd16, lane));
    }
    if (lane == 0) sum[s] = acc;
  }
}

// Exclusive scan, pass 1: per block of kScanBlock summaries (one per thread).
__global__ void load_scan_block_kernel(const LoadPos* sum, unsigned long long n, LoadPos* pre, LoadPos* block_tot) {
  __shared__ LoadPos warp_tot[kScanBlock / 32];
  const unsigned long long i = blockIdx.x * (unsigned long long)kScanBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  LoadPos v = i < n ? sum[i] : LoadPos{0ull, 0u, 0u};
  LoadPos x = v;  // inclusive warp scan
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    LoadPos y;
    y.rows = __shfl_up_sync(0xffffffffu, x.rows, o);
    y.cols = __shfl_up_sync(0xffffffffu, x.cols, o);
    y.has = __shfl_up_sync(0xffffffffu, x.has, o);
    if (lane >= o) x = combine(y, x);
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    LoadPos t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      LoadPos y;
      y.rows = __shfl_up_sync(0xffffffffu, t.rows, o);
      y.cols = __shfl_up_sync(0xffffffffu, t.cols, o);
      y.has = __shfl_up_sync(0xffffffffu, t.has, o);
      if (lane >= o) t = combine(y, t);
    }
    warp_tot[lane] = t;  // inclusive over warps
  }
  __syncthreads();
  LoadPos before = warp > 0 ? warp_tot[warp - 1] : LoadPos{0ull, 0u, 0u};
  LoadPos prev;  // exclusive within the warp: the previous lane's inclusive value
  prev.rows = __shfl_up_sync(0xffffffffu, x.rows, 1);
  prev.cols = __shfl_up_sync(0xffffffffu, x.cols, 1);
  prev.has = __shfl_up_sync(0xffffffffu, x.has, 1);
  const LoadPos ex = lane > 0 ? combine(before, prev) : before;
  if (i < n) pre[i] = ex;
  if (threadIdx.x == kScanBlock - 1) block_tot[blockIdx.x] = combine(before, x);
}

// Pass 2: the block totals, exclusive-scanned in place by one block (each
// thread a contiguous segment); block_tot[nblocks] gets the grand total.
__global__ void load_scan_totals_kernel(LoadPos* block_tot, unsigned long long nblocks) {
  __shared__ LoadPos seg_tot[kScanBlock];
  const int t = threadIdx.x;
  const unsigned long long seg = (nblocks + kScanBlock - 1) / kScanBlock;
  const unsigned long long b0 = t * seg, b1 = b0 + seg < nblocks ? b0 + seg : nblocks;
  LoadPos run{0ull, 0u, 0u};
  for (unsigned long long b = b0; b < b1; b++) run = combine(run, block_tot[b]);
  seg_tot[t] = run;
  __syncthreads();
  if (t == 0) {
    const unsigned long long nseg = (nblocks + seg - 1) / seg;  // segments in use
    LoadPos acc{0ull, 0u, 0u};
    for (unsigned long long k = 0; k < nseg; k++) {
      const LoadPos v = seg_tot[k];
      seg_tot[k] = acc;
      acc = combine(acc, v);
    }
    block_tot[nblocks] = acc;
  }
  __syncthreads();
  LoadPos acc = seg_tot[t];
  for (unsigned long long b = b0; b < b1; b++) {
    const LoadPos v = block_tot[b];
    block_tot[b] = acc;  // exclusive
    acc = combine(acc, v);
  }
}

__device__ __forceinline__ bool is_space(uint32_t c) { return c == ' ' || c - '\t' < 5u; }

// strtol(s, NULL, 10) over the virtual bytes [s, e), read from global memory
// (any length; exact overflow clamp).
__device__ __noinline__ long long convert_global(const Text& tx, long long s, long long e) {
  while (s < e && is_space(tx.byte(s))) s++;
  bool neg = false;
  if (s < e && (tx.byte(s) == '+' || tx.byte(s) == '-')) {
    neg = tx.byte(s) == '-';
    s++;
  }
  const unsigned long long lim = neg ? 9223372036854775808ull : 9223372036854775807ull;
  unsigned long long acc = 0;
  bool over = false;
  for (; s < e; s++) {
    const uint32_t d = (uint32_t)tx.byte(s) - '0';
    if (d > 9) break;
    if (over) continue;
    if (acc > (lim - d) / 10) {
      over = true;
      continue;
    }
    acc = acc * 10 + d;
  }
  if (over) return neg ? (long long)0x8000000000000000ull : 0x7FFFFFFFFFFFFFFFll;
  return neg ? (long long)(0ull - acc) : (long long)acc;
}

// Where the item pending at virtual position b0 began, relative to b0: one
// past the last delimiter in the 4096 bytes before b0 (stage halo first, then
// global), the text's first byte when the search reaches it, else kUnknown
// (the item is longer than any allowed).
constexpr int kUnknown = -(1 << 30);

__device__ __forceinline__ int pending_start(const Text& tx, const uint8_t* st, long long b0, uint8_t cd, uint8_t rd,
                                             int lane) {
  if (b0 <= tx.mis) return (int)(tx.mis - b0);
  const long long lo = b0 - (kMaxItem + 1) > tx.mis ? b0 - (kMaxItem + 1) : tx.mis;
  for (long long hi = b0; hi > lo; hi -= 32) {
    const long long v = hi - 1 - lane;
    bool hit = false;
    if (v >= lo) {
      const uint8_t c = v >= b0 - kHalo ? st[v - (b0 - kHalo)] : tx.byte(v);
      hit = c == cd || c == rd;
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, hit);
    if (bal) return (int)(hi - (__ffs(bal) - 1) - b0);  // one past the delimiter nearest b0
  }
  return lo == tx.mis ? (int)(tx.mis - b0) : kUnknown;
}

// strtol over staged bytes [p, e) for an item of at most 18 digits (false:
// more digits, convert exactly from global memory).  kFree: neither delimiter
// can be part of a number, so the delimiter at *e ends every walk by itself.
template <bool kFree>
__device__ __forceinline__ bool convert_staged(const uint8_t* p, const uint8_t* e, bool wide, long long& val) {
  while ((kFree || p < e) && is_space(*p)) p++;
  bool neg = false;
  if ((kFree || p < e) && (*p == '-' || *p == '+')) {
    neg = *p == '-';
    p++;
  }
  const uint8_t* d0 = p;
  if (wide) {
    unsigned long long acc = 0;
    for (; kFree || p < e; p++) {
      const uint32_t d = (uint32_t)*p - '0';
      if (d > 9) break;
      acc = acc * 10 + d;
    }
    val = neg ? (long long)(0ull - acc) : (long long)acc;
  } else {  // the low 32 bits are all an Int32 column keeps
    uint32_t acc = 0;
    for (; kFree || p < e; p++) {
      const uint32_t d = (uint32_t)*p - '0';
      if (d > 9) break;
      acc = acc * 10 + d;
    }
    val = (int32_t)(neg ? 0u - acc : acc);
  }
  return p - d0 <= 18;  // 10^18 - 1 < 2^63: no clamp
}

// A field waiting for conversion: start + 4096 (13 bits), end (12 bits) and
// column (bits 25..31) relative to the span, and its row relative to the
// span's first row.  kNoField fills the slot of a field that is not stored.
constexpr int kListFlush = 64;                  // convert once this many wait
constexpr int kListCap = kListFlush - 1 + kSub;  // plus one sub-tile's worth
constexpr uint32_t kNoField = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t pack_field(int fs, int fe, uint32_t c) {
  return (uint32_t)(fs + kSpan) | ((uint32_t)fe << 13) | (c << 25);
}

template <bool kFree>
__global__ void __launch_bounds__(kWarps * 32) load_parse_kernel(const uint8_t* text, unsigned long long bytes,
                                                                char cd, char rd, unsigned long long nspans,
                                                                const LoadPos* pre, const LoadPos* block_tot,
                                                                LoadOut out, int* error) {
  __shared__ __align__(16) uint8_t stage[kWarps][kStage];
  __shared__ uint32_t list_f[kWarps][kListCap];
  __shared__ uint32_t list_r[kWarps][kListCap];
  __shared__ void* colp[kLoadMaxCols];
  __shared__ uint8_t wide[kLoadMaxCols];
  if (threadIdx.x < kLoadMaxCols) {
    colp[threadIdx.x] = out.col[threadIdx.x];
    wide[threadIdx.x] = out.wide[threadIdx.x];
  }
  __syncthreads();
  const Text tx(text, bytes);
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;  // lanes below this one
  uint8_t* st = stage[threadIdx.x >> 5];
  uint32_t* lf = list_f[threadIdx.x >> 5];
  uint32_t* lr = list_r[threadIdx.x >> 5];
  const uint32_t cdx = rep4(cd), rdx = rep4(rd);
  const uint32_t ncols = (uint32_t)out.ncols;
  const unsigned long long nrows = out.nrows;
  for (unsigned long long s = blockIdx.x * (unsigned long long)kWarps + (threadIdx.x >> 5); s < nspans;
       s += (unsigned long long)gridDim.x * kWarps) {
    const long long b0 = (long long)(s * kSpan);
    const long long g0 = b0 / 16;
    // Stage the halo and the span (bytes outside the text are zero).
    __syncwarp();
#pragma unroll
    for (int q = 0; q < kSpan / kSub; q++)
      *reinterpret_cast<uint4*>(st + kHalo + q * kSub + lane * 16) = tx.granule(g0 + q * (kSub / 16) + lane);
    if (lane < kHalo / 16) {
      const long long gh = g0 - kHalo / 16 + lane;
      *reinterpret_cast<uint4*>(st + lane * 16) = gh >= 0 ? tx.granule(gh) : make_uint4(0u, 0u, 0u, 0u);
    }
    __syncwarp();
    const LoadPos p0 = combine(block_tot[s / kScanBlock], pre[s]);
    const unsigned long long row_base = p0.rows;
    uint32_t row = 0;  // relative to row_base
    uint32_t col = p0.cols;
    int pend = pending_start(tx, st, b0, (uint8_t)cd, (uint8_t)rd, lane);  // relative to b0
    int nlist = 0;
#pragma unroll 1
    for (int q = 0; q < kSpan / kSub; q++) {
      const int gbr = q * kSub + lane * 16;  // the granule's byte 0, relative to b0
      const uint4 w = *reinterpret_cast<const uint4*>(st + kHalo + gbr);
      const uint32_t valid = tx.valid16(b0 + gbr);
      const uint32_t cd16 = eq_mask16(w, cdx) & valid;
      const uint32_t rd16 = eq_mask16(w, rdx) & valid;
      const uint32_t dm = cd16 | rd16;
      // Packed inclusive scan: row delimiters (low 16 bits), column delimiters (high 16).
      const uint32_t own = (uint32_t)__popc(rd16) | ((uint32_t)__popc(cd16) << 16);
      uint32_t inc = own;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
      }
      const uint32_t exc = inc - own;
      const uint32_t cd_before = exc >> 16;
      // The column at the granule's start: column delimiters since the last
      // row delimiter of an earlier lane, else since the sub-tile's start.
      // y = this lane's column delimiters up to its last row delimiter, counted
      // from the sub-tile's start.
      const uint32_t y = (inc >> 16) - __popc(cd16 >> (32 - __clz(rd16)));
      const uint32_t rbal = __ballot_sync(0xffffffffu, rd16 != 0);
      const uint32_t rbelow = rbal & lt;
      const uint32_t y_last = __shfl_sync(0xffffffffu, y, rbelow ? 31 - __clz(rbelow) : 0);
      const uint32_t c0 = rbelow ? cd_before - y_last : col + cd_before;
      const uint32_t r0 = row + (exc & 0xFFFFu);
      // Where the lane's first field began.
      const uint32_t dbal = __ballot_sync(0xffffffffu, dm != 0);
      const uint32_t dbelow = dbal & lt;
      const int lastpos = gbr + 31 - __clz(dm);  // meaningful when dm != 0
      const int lp = __shfl_sync(0xffffffffu, lastpos, dbelow ? 31 - __clz(dbelow) : 0);
      const int start0 = dbelow ? lp + 1 : pend;
      // List the lane's fields in text order; each field's row, column and
      // start follow from the masks below its column delimiter.
      int slot = nlist + (int)cd_before;
      for (uint32_t cm = cd16; cm; cm &= cm - 1, slot++) {
        const int j = __ffs(cm) - 1;
        const uint32_t below = (1u << j) - 1u;
        const uint32_t rb = rd16 & below, db = dm & below;
        const uint32_t r = r0 + __popc(rb);
        const uint32_t c = rb ? __popc(cd16 & below & ~((2u << (31 - __clz(rb))) - 1u)) : c0 + __popc(cd16 & below);
        const int fs = db ? gbr + 32 - __clz(db) : start0;  // the field's first byte
        const int fe = gbr + j;                             // its column delimiter
        uint32_t f = kNoField;
        if (fe - fs > kMaxItem)                              // also an unknown start
          raise_error(error, DERR_LOAD_ITEM);
        else if (c < ncols && row_base + r < nrows)
          f = pack_field(fs, fe, c);
        lf[slot] = f;
        lr[slot] = r;
      }
      // Carry the row, column and pending item into the next sub-tile.
      const uint32_t tot = __shfl_sync(0xffffffffu, inc, 31);
      const uint32_t y_end = __shfl_sync(0xffffffffu, y, rbal ? 31 - __clz(rbal) : 0);
      col = rbal ? (tot >> 16) - y_end : col + (tot >> 16);
      row += tot & 0xFFFFu;
      const int lp_end = __shfl_sync(0xffffffffu, lastpos, dbal ? 31 - __clz(dbal) : 0);
      if (dbal) pend = lp_end + 1;
      nlist += (int)(tot >> 16);
      if (nlist < kListFlush && q + 1 < kSpan / kSub) continue;
      // Convert the listed fields, 32 at a time.
      __syncwarp();
      for (int k = lane; k < nlist; k += 32) {
        const uint32_t f = lf[k];
        if (f == kNoField) continue;
        const int fs = (int)(f & 0x1FFFu) - kSpan, fe = (int)((f >> 13) & 0xFFFu);
        const uint32_t c = f >> 25;
        const bool wd = wide[c];
        long long val = 0;
        if (fs < -kHalo || !convert_staged<kFree>(st + kHalo + fs, st + kHalo + fe, wd, val))
          val = convert_global(tx, b0 + fs, b0 + fe);
        const unsigned long long r = row_base + lr[k];
        if (wd)
          reinterpret_cast<long long*>(colp[c])[r] = val;
        else
          reinterpret_cast<int32_t*>(colp[c])[r] = (int32_t)(uint32_t)(unsigned long long)val;
      }
      __syncwarp();
      nlist = 0;
    }
  }
}

template <typename K>
int grid_for(K kernel, std::atomic<int>* per_sm_cache, unsigned long long spans) {
  // Blocks per SM depend on the kernel and the architecture only; a race
  // between threads computes the same value twice.
  int per_sm = per_sm_cache->load(std::memory_order_relaxed);
  if (!per_sm) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWarps * 32, 0) != cudaSuccess || per_sm < 1)
      per_sm = 1;
    per_sm_cache->store(per_sm, std::memory_order_relaxed);
  }
  const unsigned long long want = (spans + kWarps - 1) / kWarps;
  const unsigned long long cap = (unsigned long long)num_sms() * per_sm;
  return (int)(want < 1 ? 1 : want < cap ? want : cap);
}

std::atomic<int> summary_per_sm{0}, parse_per_sm[2] = {{0}, {0}};

}  // namespace

// Spans of the text on its 16-byte grid (the grid may start up to 15 bytes
// before the text, so one more span than the bytes alone need may be used).
size_t load_chunks(unsigned long long bytes) { return bytes ? (bytes + 15 + kSpan - 1) / kSpan : 0; }

size_t load_scratch_entries(unsigned long long bytes) {
  const unsigned long long n = load_chunks(bytes);
  return 2 * n + (n + kScanBlock - 1) / kScanBlock + 1;
}

cudaError_t launch_load_index(const uint8_t* text, unsigned long long bytes, char cd, char rd, LoadPos* scratch,
                              cudaStream_t s) {
  const unsigned long long n = load_chunks(bytes);
  if (n == 0) return cudaSuccess;
  LoadPos* sum = scratch;
  LoadPos* pre = scratch + n;
  LoadPos* tot = scratch + 2 * n;
  const unsigned long long nb = (n + kScanBlock - 1) / kScanBlock;
  note_launch(3);
  load_summary_kernel<<<grid_for(load_summary_kernel, &summary_per_sm, n), kWarps * 32, 0, s>>>(text, bytes, cd, rd,
                                                                                               n, sum);
  load_scan_block_kernel<<<(unsigned)nb, kScanBlock, 0, s>>>(sum, n, pre, tot);
  load_scan_totals_kernel<<<1, kScanBlock, 0, s>>>(tot, nb);
  return cudaGetLastError();
}

const LoadPos* load_total(const LoadPos* scratch, unsigned long long bytes) {
  const unsigned long long n = load_chunks(bytes);
  return scratch + 2 * n + (n + kScanBlock - 1) / kScanBlock;
}

cudaError_t launch_load_parse(const uint8_t* text, unsigned long long bytes, char cd, char rd,
                              const LoadPos* scratch, const LoadOut& out, int* error, cudaStream_t s) {
  const unsigned long long n = load_chunks(bytes);
  if (n == 0) return cudaSuccess;
  // A field never holds a row delimiter and always ends at a column
  // delimiter: when that is no digit, sign or space, it ends every walk.
  const uint8_t u = (uint8_t)cd;
  const bool numeric = (u >= '0' && u <= '9') || u == '+' || u == '-' || u == ' ' || (u >= '\t' && u <= '\r');
  note_launch();
  if (!numeric)
    load_parse_kernel<true><<<grid_for(load_parse_kernel<true>, &parse_per_sm[1], n), kWarps * 32, 0, s>>>(
        text, bytes, cd, rd, n, scratch + n, scratch + 2 * n, out, error);
  else
    load_parse_kernel<false><<<grid_for(load_parse_kernel<false>, &parse_per_sm[0], n), kWarps * 32, 0, s>>>(
        text, bytes, cd, rd, n, scratch + n, scratch + 2 * n, out, error);
  return cudaGetLastError();
}

}  // namespace svm
