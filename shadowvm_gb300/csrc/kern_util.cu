// Utility kernels: seeded data generation, column min/max, prefix scans.
#include <atomic>
#include <climits>
#include <mutex>
#include <set>
#include <tuple>

#include "kern_common.cuh"
#include "kernels.h"

namespace svm {

static std::atomic<unsigned long long> g_launches{0};
void note_launch(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
unsigned long long launches_total() { return g_launches.load(); }

// Per-device caches: the current device's SM count, and the dynamic
// shared-memory limit raised once per (device, kernel), since a function
// attribute applies only to the device that was current when it was set.
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_dev_mu;
int g_sms[kMaxDevices] = {};
std::set<std::tuple<int, const void*, int>> g_smem_attr;

int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
  return dev;
}
}  // namespace

int num_sms() {
  const int dev = current_device();
  std::lock_guard<std::mutex> g(g_dev_mu);
  if (!g_sms[dev]) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_sms[dev] = sms > 0 ? sms : 1;
  }
  return g_sms[dev];
}

cudaError_t allow_dynamic_smem(const void* fn, int bytes) {
  const int dev = current_device();
  std::lock_guard<std::mutex> g(g_dev_mu);
  if (g_smem_attr.count(std::make_tuple(dev, fn, bytes))) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) g_smem_attr.insert(std::make_tuple(dev, fn, bytes));
  return e;
}

// ---------------------------------------------------------------- generation
__global__ void gen_uniform_kernel(int32_t* out, unsigned long long n, uint64_t key, int lo,
                                   unsigned long long span, const int32_t* lookup) {
  unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (; i < n; i += stride) {
    uint64_t u = mix64(key + i);
    uint64_t off = ((u >> 32) * span) >> 32;
    out[i] = lookup ? lookup[off] : (int32_t)((long long)lo + (long long)off);
  }
}

cudaError_t launch_gen_uniform(int32_t* out, unsigned long long n, unsigned long long seed,
                               unsigned long long stream_id, unsigned long long row0, int lo, int hi,
                               const int32_t* lookup, cudaStream_t s) {
  uint64_t key = mix64((uint64_t)seed ^ ((uint64_t)stream_id * 0xD1B54A32D192ED03ull));
  unsigned long long span = (unsigned long long)((long long)hi - (long long)lo + 1);
  int grid = num_sms() * 8;
  note_launch();
  gen_uniform_kernel<<<grid, 256, 0, s>>>(out, n, key + row0, lo, span, lookup);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- min / max
__global__ void minmax_kernel(const int32_t* in, unsigned long long n, int32_t* out) {
  int32_t mn = INT_MAX, mx = INT_MIN;
  unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (; i < n; i += stride) {
    int32_t v = in[i];
    mn = min(mn, v);
    mx = max(mx, v);
  }
  for (int o = 16; o; o >>= 1) {
    mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(out, mn);
    atomicMax(out + 1, mx);
  }
}

cudaError_t launch_minmax(const int32_t* in, unsigned long long n, int32_t* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  unsigned long long want = (n + 255) / 256;
  int grid = (int)(want < (unsigned long long)num_sms() * 8 ? want : num_sms() * 8);
  note_launch();
  minmax_kernel<<<grid, 256, 0, s>>>(in, n, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- scans
// Three-phase block scan: per-tile totals, a scan of the totals, then each tile
// rescanned with its prefix.  Tiles of kScanTile elements, 256 threads.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr unsigned long long kScanTile = kScanThreads * kScanItems;

struct SumOp {
  __device__ static unsigned long long id() { return 0ull; }
  __device__ static unsigned long long op(unsigned long long a, unsigned long long b) { return a + b; }
};
struct MaxOp {
  __device__ static long long id() { return LLONG_MIN; }
  __device__ static long long op(long long a, long long b) { return a > b ? a : b; }
};

template <typename T, typename Op>
__device__ T block_scan_exclusive(T v, T* warp_tot, T* total) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T x = v;
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x = Op::op(y, x);
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    T w = lane < kScanThreads / 32 ? warp_tot[lane] : Op::id();
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w = Op::op(y, w);
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  T before_warp = wid ? warp_tot[wid - 1] : Op::id();
  T excl = __shfl_up_sync(0xffffffffu, x, 1);
  if (lane == 0) excl = Op::id();
  *total = warp_tot[kScanThreads / 32 - 1];
  return Op::op(before_warp, excl);
}

template <typename In, typename T, typename Op>
__global__ void scan_tiles_kernel(const In* in, unsigned long long n, T* tile_tot) {
  __shared__ T wt[kScanThreads / 32];
  unsigned long long base = blockIdx.x * kScanTile + threadIdx.x * (unsigned long long)kScanItems;
  T acc = Op::id();
  for (int k = 0; k < kScanItems; k++)
    if (base + k < n) acc = Op::op(acc, (T)in[base + k]);
  T total;
  block_scan_exclusive<T, Op>(acc, wt, &total);
  if (threadIdx.x == 0) tile_tot[blockIdx.x] = total;
}

// Single block: exclusive scan of the tile totals in place.
template <typename T, typename Op>
__global__ void scan_totals_kernel(T* tot, unsigned long long ntiles) {
  __shared__ T wt[kScanThreads / 32];
  T carry = Op::id();
  for (unsigned long long b0 = 0; b0 < ntiles; b0 += kScanThreads) {
    unsigned long long i = b0 + threadIdx.x;
    T v = i < ntiles ? tot[i] : Op::id();
    T total;
    T ex = block_scan_exclusive<T, Op>(v, wt, &total);
    if (i < ntiles) tot[i] = Op::op(carry, ex);
    carry = Op::op(carry, total);
    __syncthreads();
  }
}

template <typename In, typename Out, typename T, typename Op, bool kInclusive>
__global__ void scan_apply_kernel(const In* in, unsigned long long n, const T* tile_pre, Out* out,
                                  Out* total_out) {
  __shared__ T wt[kScanThreads / 32];
  unsigned long long base = blockIdx.x * kScanTile + threadIdx.x * (unsigned long long)kScanItems;
  T vals[kScanItems];
  T acc = Op::id();
  for (int k = 0; k < kScanItems; k++) {
    vals[k] = base + k < n ? (T)in[base + k] : Op::id();
    acc = Op::op(acc, vals[k]);
  }
  T total;
  T run = Op::op(tile_pre[blockIdx.x], block_scan_exclusive<T, Op>(acc, wt, &total));
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) {
      if (kInclusive) {
        run = Op::op(run, vals[k]);
        out[base + k] = (Out)run;
      } else {
        out[base + k] = (Out)run;
        run = Op::op(run, vals[k]);
      }
    }
  }
  if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
    *total_out = (Out)Op::op(tile_pre[blockIdx.x], total);
}

size_t scan_tmp_words(unsigned long long n) { return (n + kScanTile - 1) / kScanTile + 1; }
size_t max_tmp_words(unsigned long long n) { return 2 * ((n + kScanTile - 1) / kScanTile + 1); }

cudaError_t launch_exclusive_scan(const uint32_t* in, unsigned long long n, unsigned long long* out,
                                  unsigned long long* tmp, cudaStream_t s) {
  if (n == 0) return cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
  unsigned long long ntiles = (n + kScanTile - 1) / kScanTile;
  note_launch(3);
  scan_tiles_kernel<uint32_t, unsigned long long, SumOp><<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, tmp);
  scan_totals_kernel<unsigned long long, SumOp><<<1, kScanThreads, 0, s>>>(tmp, ntiles);
  scan_apply_kernel<uint32_t, unsigned long long, unsigned long long, SumOp, false>
      <<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, tmp, out, out + n);
  return cudaGetLastError();
}

cudaError_t launch_inclusive_max(const int32_t* in, unsigned long long n, int32_t* out, int32_t* tmp,
                                 cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  unsigned long long ntiles = (n + kScanTile - 1) / kScanTile;
  long long* t = reinterpret_cast<long long*>(tmp);
  note_launch(3);
  scan_tiles_kernel<int32_t, long long, MaxOp><<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, t);
  scan_totals_kernel<long long, MaxOp><<<1, kScanThreads, 0, s>>>(t, ntiles);
  scan_apply_kernel<int32_t, int32_t, long long, MaxOp, true>
      <<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, t, out, nullptr);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- segment gather
// One warp per segment (grid-stride over segments), consecutive lanes on
// consecutive words.
__global__ void gather_segments_kernel(const Segment* segs, int nseg, uint32_t* dst) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nseg; k += warps) {
    const Segment sg = segs[k];
    for (unsigned long long w = lane; w < sg.words; w += 32) dst[sg.dst_word + w] = sg.src[w];
  }
}

cudaError_t launch_gather_segments(const Segment* segs, int nseg, uint32_t* dst, cudaStream_t s) {
  if (nseg <= 0) return cudaSuccess;
  const int blocks = (nseg + 7) / 8 < num_sms() * 8 ? (nseg + 7) / 8 : num_sms() * 8;
  note_launch();
  gather_segments_kernel<<<blocks, 256, 0, s>>>(segs, nseg, dst);
  return cudaGetLastError();
}

// out[i] = lut[in[i]] (dictionary code -> hash rank, hash rank -> hash value;
// in and out may be the same array).
__global__ void lut_gather_kernel(const int32_t* in, unsigned long long n, const int32_t* lut, int32_t* out) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    out[i] = lut[in[i]];
}

cudaError_t launch_lut_gather(const int32_t* in, unsigned long long n, const int32_t* lut, int32_t* out,
                              cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned long long want = (n + 255) / 256;
  const unsigned long long cap = (unsigned long long)num_sms() * 8;
  note_launch();
  lut_gather_kernel<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(in, n, lut, out);
  return cudaGetLastError();
}

// flags[codes[i]] = 1: which dictionary codes a column holds.
__global__ void mark_codes_kernel(const int32_t* codes, unsigned long long n, uint32_t* flags) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    flags[codes[i]] = 1u;
}

cudaError_t launch_mark_codes(const int32_t* codes, unsigned long long n, uint32_t* flags, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned long long want = (n + 255) / 256;
  const unsigned long long cap = (unsigned long long)num_sms() * 8;
  note_launch();
  mark_codes_kernel<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(codes, n, flags);
  return cudaGetLastError();
}

}  // namespace svm
