// Dimension-side kernels: Filter+Map pipelines with order-preserving
// compaction, the reference-table emulation used by REF_COMPAT joins, and the
// dense / hash dimension-table builds.
#include <climits>

#include "kern_common.cuh"
#include "kernels.h"

namespace svm {

// ================================================================ select
// One tile = 256 threads x 4 consecutive rows.  Pass 1 counts rows passing the
// conjuncts per tile; after an exclusive scan of the counts, pass 2 writes the
// projected rows at the tile's offset in row order (the reference's CPU path
// emits rows at j in order, codegen/codegen.cpp:151-180).
constexpr int kSelThreads = 256;
constexpr int kSelRows = 4;
constexpr long long kSelTile = kSelThreads * kSelRows;

unsigned long long select_tiles(long long nrows) {
  return (unsigned long long)((nrows + kSelTile - 1) / kSelTile);
}

// The row's source operands, its conjuncts, then (a join-map pipeline) each
// join's probe in order -- a row whose key is missing from a table is
// dropped, as the reference's generated join block clears `cond`
// (codegen/codegen.cpp:121-149) -- and the joined payload operands.
__device__ __forceinline__ bool select_row(const SelectParams& p, long long r, int32_t* opnd) {
  for (int c = 0; c < p.ncols_in; c++) opnd[c] = __ldg(p.cols[c] + r);
  for (int k = 0; k < p.npred; k++)
    if (!eval_prog(p.pred[k], opnd, p.error)) return false;
  if (p.ndims == 0) return true;
  uint32_t ent[kMaxDims];
  for (int d = 0; d < p.ndims; d++)
    if (!probe_dim(p.dims[d], nullptr, opnd[p.join_opnd[d]], ent[d])) return false;
  for (int k = p.ncols_in; k < p.nopnd; k++) {
    const Operand o = p.dop[k - p.ncols_in];
    uint32_t e = ent[0];
    for (int d = 1; d < kMaxDims; d++)
      if (o.slot == d) e = ent[d];
    opnd[k] = payload_value(p.dims[o.slot], o.field, e);
  }
  return true;
}

__global__ void select_count_kernel(SelectParams p) {
  __shared__ unsigned int warp_cnt[kSelThreads / 32];
  __shared__ unsigned int warp_b0[kSelThreads / 32];
  long long base = blockIdx.x * kSelTile + threadIdx.x * (long long)kSelRows;
  int32_t opnd[16];
  unsigned int cnt = 0, b0 = 0;
  for (int k = 0; k < kSelRows; k++) {
    long long r = base + k;
    if (r < p.nrows && select_row(p, r, opnd)) {
      cnt++;
      if (r < p.bulk0_rows) b0++;
    }
  }
  for (int o = 16; o; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    b0 += __shfl_xor_sync(0xffffffffu, b0, o);
  }
  if ((threadIdx.x & 31) == 0) {
    warp_cnt[threadIdx.x >> 5] = cnt;
    warp_b0[threadIdx.x >> 5] = b0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int t = 0, tb = 0;
    for (int w = 0; w < kSelThreads / 32; w++) {
      t += warp_cnt[w];
      tb += warp_b0[w];
    }
    p.tile_count[blockIdx.x] = t;
    if (tb) atomicAdd(p.bulk0_count, (unsigned long long)tb);
  }
}

__global__ void select_write_kernel(SelectParams p) {
  __shared__ unsigned int warp_tot[kSelThreads / 32];
  long long base = blockIdx.x * kSelTile + threadIdx.x * (long long)kSelRows;
  int32_t opnd[16];
  unsigned pass = 0;
  for (int k = 0; k < kSelRows; k++) {
    long long r = base + k;
    if (r < p.nrows && select_row(p, r, opnd)) pass |= 1u << k;
  }
  unsigned int c = __popc(pass);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned int x = c;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  unsigned int before = 0;
  for (int w = 0; w < wid; w++) before += warp_tot[w];
  unsigned long long pos = p.tile_offset[blockIdx.x] + before + x - c;
  for (int k = 0; k < kSelRows; k++) {
    if (!(pass >> k & 1u)) continue;
    long long r = base + k;
    if (p.ndims)
      select_row(p, r, opnd);  // the joined operands again (the row passed in the first walk)
    else
      for (int cc = 0; cc < p.ncols_in; cc++) opnd[cc] = __ldg(p.cols[cc] + r);
    for (int o = 0; o < p.nout; o++) {
      const Prog& pr = p.proj[o];
      p.out[o][pos] = (pr.n == 1 && pr.op[0] == X_OPND) ? opnd[pr.arg[0]] : eval_prog(pr, opnd, p.error);
    }
    pos++;
  }
}

cudaError_t launch_select_count(const SelectParams& p, cudaStream_t s) {
  unsigned long long t = select_tiles(p.nrows);
  if (t == 0) return cudaSuccess;
  note_launch();
  select_count_kernel<<<(unsigned)t, kSelThreads, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_select_write(const SelectParams& p, cudaStream_t s) {
  unsigned long long t = select_tiles(p.nrows);
  if (t == 0) return cudaSuccess;
  note_launch();
  select_write_kernel<<<(unsigned)t, kSelThreads, 0, s>>>(p);
  return cudaGetLastError();
}

// ================================================================ REF_COMPAT emulation
// The reference builds each join table on the host by inserting the joined
// object's bulk-0 rows in row order into ht_size slots, each row taking the
// first free slot among the 10 starting at Hash(key) % ht_size and being left
// out when all 10 are taken (com/cpp/com.hpp:168-174, cpu-runtime.hpp:80-91).
//
// Rows interact only through the slots their 10-slot windows cover, so the
// slot ring splits into independent runs of covered slots.  Each run is
// replayed sequentially (its rows in row order) by one thread; runs replay in
// parallel.  The result is exactly the sequential outcome.
namespace {
struct RcLayout {
  size_t hrow, cnt, start, maxtmp, runoff, scantmp, cursor, members, occ, total;
};
RcLayout rc_layout(long long n, unsigned ht) {
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  RcLayout L{};
  size_t o = 0;
  L.hrow = o; o += al(4 * (size_t)n);
  L.cnt = o; o += al(4 * (size_t)ht);
  L.start = o; o += al(4 * (size_t)ht);
  L.maxtmp = o; o += al(4 * max_tmp_words(ht));
  L.runoff = o; o += al(8 * ((size_t)ht + 1));
  L.scantmp = o; o += al(8 * scan_tmp_words(ht));
  L.cursor = o; o += al(4 * (size_t)ht);
  L.members = o; o += al(4 * (size_t)n);
  L.occ = o; o += al((size_t)ht);
  L.total = o;
  return L;
}
}  // namespace

size_t refcompat_scratch_bytes(long long n, unsigned ht_size) { return rc_layout(n, ht_size).total; }

__global__ void rc_hash_kernel(const int32_t* key, long long n, unsigned ht, int sgn, uint32_t* hrow,
                               uint32_t* cnt) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    uint32_t h = ref_hash_i32(key[r], sgn) % ht;
    hrow[r] = h;
    atomicAdd(cnt + h, 1u);
  }
}

__global__ void rc_start_kernel(const uint32_t* cnt, unsigned ht, int32_t* start) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < ht;
       s += (long long)gridDim.x * blockDim.x) {
    // covered(x): some row has its home in [x-9, x] (cyclically).
    bool cov = false, cov_prev = false;
    for (int j = 0; j < 10; j++) {
      long long a = ((s - j) % (long long)ht + ht) % ht;
      long long b = ((s - 1 - j) % (long long)ht + ht) % ht;
      cov |= cnt[a] != 0;
      cov_prev |= cnt[b] != 0;
    }
    start[s] = (cov && !cov_prev) ? (int32_t)s : -1;
  }
}

__global__ void rc_fix_runs_kernel(int32_t* runstart, unsigned ht) {
  int32_t last = runstart[ht - 1];          // the final run's start (or -1: one cyclic run)
  int32_t wrap = last < 0 ? 0 : last;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < ht;
       s += (long long)gridDim.x * blockDim.x)
    if (runstart[s] < 0) runstart[s] = wrap;
}

__global__ void rc_count_kernel(const uint32_t* hrow, long long n, const int32_t* runstart,
                                uint32_t* cnt) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x)
    atomicAdd(cnt + runstart[hrow[r]], 1u);
}

__global__ void rc_scatter_kernel(const uint32_t* hrow, long long n, const int32_t* runstart,
                                  const unsigned long long* runoff, uint32_t* cursor,
                                  uint32_t* members) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    int32_t run = runstart[hrow[r]];
    unsigned long long pos = runoff[run] + atomicAdd(cursor + run, 1u);
    members[pos] = (uint32_t)r;
  }
}

__device__ void sift_down(uint32_t* a, long long root, long long end) {
  while (2 * root + 1 < end) {
    long long child = 2 * root + 1;
    if (child + 1 < end && a[child] < a[child + 1]) child++;
    if (a[root] >= a[child]) return;
    uint32_t t = a[root];
    a[root] = a[child];
    a[child] = t;
    root = child;
  }
}

__global__ void rc_replay_kernel(const uint32_t* cnt, const unsigned long long* runoff,
                                 uint32_t* members, const uint32_t* hrow, unsigned ht, uint8_t* occ,
                                 uint8_t* dropped) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < ht;
       s += (long long)gridDim.x * blockDim.x) {
    uint32_t m = cnt[s];
    if (m == 0) continue;
    uint32_t* a = members + runoff[s];
    // Members in row order (heap sort; runs are short except on hostile keys).
    if (m <= 32) {
      for (uint32_t i = 1; i < m; i++) {
        uint32_t v = a[i];
        int j = (int)i - 1;
        while (j >= 0 && a[j] > v) {
          a[j + 1] = a[j];
          j--;
        }
        a[j + 1] = v;
      }
    } else {
      for (long long i = m / 2 - 1; i >= 0; i--) sift_down(a, i, m);
      for (long long e = (long long)m - 1; e > 0; e--) {
        uint32_t t = a[0];
        a[0] = a[e];
        a[e] = t;
        sift_down(a, 0, e);
      }
    }
    for (uint32_t i = 0; i < m; i++) {
      uint32_t r = a[i];
      uint32_t slot = hrow[r];
      bool placed = false;
      for (int step = 0; step < 10; step++) {
        if (!occ[slot]) {
          occ[slot] = 1;
          placed = true;
          break;
        }
        slot = slot + 1 == ht ? 0 : slot + 1;
      }
      if (!placed) dropped[r] = 1;
    }
  }
}

cudaError_t launch_refcompat(const int32_t* key, long long n, unsigned ht, int signed_char,
                             uint8_t* dropped, void* scratch, cudaStream_t s) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(dropped, 0, n > 0 ? (size_t)n : 1, s)) != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
  RcLayout L = rc_layout(n, ht);
  char* b = (char*)scratch;
  uint32_t* hrow = (uint32_t*)(b + L.hrow);
  uint32_t* cnt = (uint32_t*)(b + L.cnt);
  int32_t* start = (int32_t*)(b + L.start);
  int32_t* maxtmp = (int32_t*)(b + L.maxtmp);
  unsigned long long* runoff = (unsigned long long*)(b + L.runoff);
  unsigned long long* scantmp = (unsigned long long*)(b + L.scantmp);
  uint32_t* cursor = (uint32_t*)(b + L.cursor);
  uint32_t* members = (uint32_t*)(b + L.members);
  uint8_t* occ = (uint8_t*)(b + L.occ);
  int grid = num_sms() * 4;
  if ((e = cudaMemsetAsync(cnt, 0, 4 * (size_t)ht, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(cursor, 0, 4 * (size_t)ht, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(occ, 0, (size_t)ht, s)) != cudaSuccess) return e;
  note_launch(6);
  rc_hash_kernel<<<grid, 256, 0, s>>>(key, n, ht, signed_char, hrow, cnt);
  rc_start_kernel<<<grid, 256, 0, s>>>(cnt, ht, start);
  if ((e = launch_inclusive_max(start, ht, start, maxtmp, s)) != cudaSuccess) return e;
  rc_fix_runs_kernel<<<grid, 256, 0, s>>>(start, ht);
  if ((e = cudaMemsetAsync(cnt, 0, 4 * (size_t)ht, s)) != cudaSuccess) return e;
  rc_count_kernel<<<grid, 256, 0, s>>>(hrow, n, start, cnt);
  if ((e = launch_exclusive_scan(cnt, ht, runoff, scantmp, s)) != cudaSuccess) return e;
  rc_scatter_kernel<<<grid, 256, 0, s>>>(hrow, n, start, runoff, cursor, members);
  rc_replay_kernel<<<grid, 128, 0, s>>>(cnt, runoff, members, hrow, ht, occ, dropped);
  return cudaGetLastError();
}

// ================================================================ table builds
__device__ __forceinline__ bool build_row_live(const BuildInput& in, long long r) {
  return !(in.dropped && in.dropped[r]);
}

__global__ void build_stats_kernel(BuildInput in, int32_t* out) {
  int32_t mn[1 + kMaxKeys + 2 * kMaxMetrics], mx[1 + kMaxKeys + 2 * kMaxMetrics];
  int nf = 1 + in.npay;
  for (int f = 0; f < nf; f++) {
    mn[f] = INT_MAX;
    mx[f] = INT_MIN;
  }
  unsigned int live = 0;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < in.n;
       r += (long long)gridDim.x * blockDim.x) {
    if (!build_row_live(in, r)) continue;
    live++;
    int32_t k = in.key[r];
    mn[0] = min(mn[0], k);
    mx[0] = max(mx[0], k);
    for (int f = 0; f < in.npay; f++) {
      int32_t v = in.pay[f][r];
      mn[1 + f] = min(mn[1 + f], v);
      mx[1 + f] = max(mx[1 + f], v);
    }
  }
  for (int o = 16; o; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
  for (int f = 0; f < nf; f++) {
    for (int o = 16; o; o >>= 1) {
      mn[f] = min(mn[f], __shfl_xor_sync(0xffffffffu, mn[f], o));
      mx[f] = max(mx[f], __shfl_xor_sync(0xffffffffu, mx[f], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int f = 0; f < nf; f++) {
      atomicMin(out + 2 * f, mn[f]);
      atomicMax(out + 2 * f + 1, mx[f]);
    }
    atomicAdd((unsigned int*)(out + 2 * nf), live);
  }
}

cudaError_t launch_build_stats(const BuildInput& in, int32_t* out, cudaStream_t s) {
  if (in.n == 0) return cudaSuccess;
  note_launch();
  build_stats_kernel<<<num_sms() * 4, 256, 0, s>>>(in, out);
  return cudaGetLastError();
}

__device__ __forceinline__ uint32_t pack_entry(const BuildInput& in, const DimDesc& d, long long r) {
  uint32_t e = 1u;
  for (int f = 0; f < d.npay; f++) {
    const PayloadField& p = d.pay[f];
    if (p.bits == 0) continue;
    uint32_t v = p.col ? (uint32_t)r : (uint32_t)(in.pay[f][r] - p.min);
    e |= v << p.shift;
  }
  return e;
}

__global__ void dense_owner_kernel(BuildInput in, DimDesc d, int32_t* owner) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < in.n;
       r += (long long)gridDim.x * blockDim.x) {
    if (!build_row_live(in, r)) continue;
    uint32_t idx = (uint32_t)in.key[r] - (uint32_t)d.key_min;
    atomicMin(owner + idx, (int32_t)r);
  }
}

__global__ void dense_fill_kernel(BuildInput in, DimDesc d, const int32_t* owner, uint32_t* words) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < in.n;
       r += (long long)gridDim.x * blockDim.x) {
    if (!build_row_live(in, r)) continue;
    uint32_t idx = (uint32_t)in.key[r] - (uint32_t)d.key_min;
    if (owner[idx] != (int32_t)r) continue;
    uint64_t bit = (uint64_t)idx * (uint32_t)d.entry_bits;
    atomicOr(words + (bit >> 5), pack_entry(in, d, r) << (bit & 31));
  }
}

cudaError_t launch_build_dense(const BuildInput& in, const DimDesc& d, int32_t* owner,
                               uint32_t* words, cudaStream_t s) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(owner, 0x7F, 4 * (size_t)d.span, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(words, 0, 4 * (size_t)d.table_words, s)) != cudaSuccess) return e;
  if (in.n == 0) return cudaSuccess;
  int grid = num_sms() * 4;
  note_launch(2);
  dense_owner_kernel<<<grid, 256, 0, s>>>(in, d, owner);
  dense_fill_kernel<<<grid, 256, 0, s>>>(in, d, owner, words);
  return cudaGetLastError();
}

__global__ void hash_insert_kernel(BuildInput in, DimDesc d, unsigned long long* slots, int* error) {
  uint32_t mask = d.span - 1u;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < in.n;
       r += (long long)gridDim.x * blockDim.x) {
    if (!build_row_live(in, r)) continue;
    int32_t key = in.key[r];
    unsigned long long mine = ((unsigned long long)(uint32_t)key << 32) | (unsigned long long)(r + 1);
    uint32_t slot = mix32((uint32_t)key) & mask;
    bool done = false;
    for (uint32_t n = 0; n <= mask && !done; n++) {
      unsigned long long cur = atomicCAS(slots + slot, 0ull, mine);
      if (cur == 0ull) {
        done = true;
      } else if ((uint32_t)(cur >> 32) == (uint32_t)key) {
        // Same key: the lowest row keeps the slot.
        while ((cur & 0xffffffffull) > (unsigned long long)(r + 1)) {
          unsigned long long old = atomicCAS(slots + slot, cur, mine);
          if (old == cur) break;
          cur = old;
        }
        done = true;
      } else {
        slot = (slot + 1u) & mask;
      }
    }
    if (!done) raise_error(error, DERR_HASH_FULL);
  }
}

__global__ void hash_fill_kernel(BuildInput in, DimDesc d, const unsigned long long* slots,
                                 uint32_t* words) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < d.span;
       s += (long long)gridDim.x * blockDim.x) {
    unsigned long long v = slots[s];
    uint32_t k = 0, e = 0;
    if (v) {
      long long r = (long long)(v & 0xffffffffull) - 1;
      k = (uint32_t)(v >> 32);
      e = pack_entry(in, d, r);
    }
    words[2 * s] = k;
    words[2 * s + 1] = e;
  }
}

cudaError_t launch_build_hash(const BuildInput& in, const DimDesc& d, unsigned long long* slots,
                              uint32_t* words, int* error, cudaStream_t s) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(slots, 0, 8 * (size_t)d.span, s)) != cudaSuccess) return e;
  int grid = num_sms() * 4;
  if (in.n > 0) {
    note_launch();
    hash_insert_kernel<<<grid, 256, 0, s>>>(in, d, slots, error);
  }
  note_launch();
  hash_fill_kernel<<<grid, 256, 0, s>>>(in, d, slots, words);
  return cudaGetLastError();
}

}  // namespace svm
