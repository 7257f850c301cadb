// Device pieces shared by the fused scan kernels: the interpreted kernel
// (kern_star.cu) and the kernels compiled per plan shape (kern_star_plan.cu).
#pragma once

#include "kern_common.cuh"

namespace svm {

constexpr int kStarThreads = (kConsumerWarps + 1) * 32;
constexpr uint32_t kWaitPolls = 1u << 22;

struct StarSmem {
  uint64_t full[kStages];
  uint64_t empty[kStages];
  long long red[kConsumerWarps][kMaxMetrics + 1];
};

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// 64-bit add into shared memory with two 32-bit atomics: the low word's
// atomic returns its exact old value, so its carry is exact, and the high
// words' adds commute -- the final value equals the 64-bit sum.
__device__ __forceinline__ void smem_add64(unsigned long long* p, unsigned long long v) {
  unsigned int* w = reinterpret_cast<unsigned int*>(p);
  const unsigned int lo = (unsigned int)v, hi = (unsigned int)(v >> 32);
  const unsigned int old = atomicAdd(w, lo);
  const unsigned int up = hi + (unsigned int)(old + lo < old);
  if (up) atomicAdd(w + 1, up);
}

// ---------------------------------------------------------------- deferred aggregation
constexpr int kAggCap = 32;  // buffered rows per warp

// A gathered value: through the read-only path from device memory, or a
// plain global load from a host-resident table's page-locked memory.
__device__ __forceinline__ int32_t load_gather(const int32_t* p, bool host) {
  if (!host) return __ldg(p);
  int32_t v;
  asm("ld.global.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

// An extractor over a buffered row's words (agg_src order).
__device__ __forceinline__ uint32_t extract_entry(const Extract& x, const uint32_t* ent, bool host) {
  if (x.dim < 0) return ent[x.slot] + (uint32_t)x.base;
  uint32_t v = (ent[x.dim] >> x.shift) & x.mask;
  if (x.col) v = (uint32_t)load_gather(x.col + v, host);
  return v + (uint32_t)x.base;
}

template <int kAgg>
__device__ __forceinline__ void aggregate_entry(const StarParams& P, const uint32_t* ent,
                                                long long (&acc)[kMaxMetrics + 1], unsigned long long* s_sum,
                                                unsigned int* s_cnt) {
  const int nm = P.nmetrics;
  int32_t val[kMaxMetrics];
#pragma unroll
  for (int m = 0; m < kMaxMetrics; m++) {
    if (m < nm) {
      const uint32_t a = extract_entry(P.xa_e[m], ent, P.host_late != 0);
      const int f = P.metrics[m].form;
      uint32_t v = a;
      if (f != MF_OPND) {
        const uint32_t b = extract_entry(P.xb_e[m], ent, P.host_late != 0);
        v = f == MF_ADD ? a + b : f == MF_SUB ? a - b : a * b;
      }
      val[m] = (int32_t)v;
    }
  }
  if (kAgg == AGG_SCALAR) {
#pragma unroll
    for (int m = 0; m < kMaxMetrics; m++)
      if (m < nm) acc[m] += (long long)val[m];
    acc[kMaxMetrics] += 1;
    return;
  }
  const unsigned long long G = P.ngroups;
  uint32_t gi = 0;
  bool in_range = true;
#pragma unroll
  for (int q = 0; q < kMaxKeys; q++) {
    if (q < P.nkeys) {
      const uint32_t off = extract_entry(P.kx_e[q], ent, P.host_late != 0);
      in_range &= off < P.krange[q];
      gi += off * (uint32_t)P.kstride[q];
    }
  }
  if (!in_range) {
    raise_error(P.error, DERR_KEY_RANGE);
    return;
  }
#pragma unroll
  for (int m = 0; m < kMaxMetrics; m++) {
    if (m < nm) {
      const unsigned long long v = (unsigned long long)(long long)val[m];
      if (kAgg == AGG_DENSE_SMEM)
        smem_add64(s_sum + m * G + gi, v);
      else
        atomicAdd(P.sums + m * G + gi, v);
    }
  }
  if (kAgg == AGG_DENSE_SMEM)
    s_cnt[gi] = 1u;
  else
    atomicAdd(P.counts + gi, 1ull);
}

// Aggregates the warp's `cnt` buffered rows, one per lane.
template <int kAgg>
__device__ __forceinline__ void flush_entries(const StarParams& P, const uint32_t* buf, int cnt, int lane,
                                              long long (&acc)[kMaxMetrics + 1], unsigned long long* s_sum,
                                              unsigned int* s_cnt) {
  __syncwarp();
  const int W = P.agg_words;
  for (int base = 0; base < cnt; base += 32)
    if (base + lane < cnt) aggregate_entry<kAgg>(P, buf + (size_t)(base + lane) * W, acc, s_sum, s_cnt);
  __syncwarp();
}

// The block's partial aggregates into the global int64 slots: the scalar
// sums reduced over the block and added once; the shared-memory groups
// added slot by slot (only the non-empty ones).
template <int kAgg>
__device__ __forceinline__ void finish_block(const StarParams& P, StarSmem& S, long long (&acc)[kMaxMetrics + 1],
                                             unsigned long long* s_sum, unsigned int* s_cnt, int tid, int warp,
                                             int lane) {
  const int nm = P.nmetrics;
  const unsigned long long G = P.ngroups;
  if (kAgg == AGG_SCALAR) {
    for (int o = 16; o; o >>= 1)
      for (int m = 0; m <= kMaxMetrics; m++) acc[m] += __shfl_xor_sync(0xffffffffu, acc[m], o);
    if (lane == 0 && warp < kConsumerWarps)
      for (int m = 0; m <= kMaxMetrics; m++) S.red[warp][m] = acc[m];
    __syncthreads();
    if (tid == 0) {
      long long tot[kMaxMetrics + 1] = {0, 0, 0, 0};
      for (int w = 0; w < kConsumerWarps; w++)
        for (int m = 0; m <= kMaxMetrics; m++) tot[m] += S.red[w][m];
      for (int m = 0; m < nm; m++)
        if (tot[m]) atomicAdd(P.sums + m, (unsigned long long)tot[m]);
      if (tot[kMaxMetrics]) atomicAdd(P.counts, (unsigned long long)tot[kMaxMetrics]);
    }
  } else if (kAgg == AGG_DENSE_SMEM) {
    __syncthreads();
    for (unsigned long long i = tid; i < G; i += blockDim.x) {
      unsigned int c = s_cnt[i];
      if (!c) continue;
      atomicAdd(P.counts + i, (unsigned long long)c);
      for (int m = 0; m < nm; m++) atomicAdd(P.sums + m * G + i, s_sum[m * G + i]);
    }
  }
}

}  // namespace svm
