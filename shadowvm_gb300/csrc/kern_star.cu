// The fused fact-table scan: range filters and dimension probes in the order
// the planner chose (most selective first), then group keys and metrics of
// the surviving rows aggregated per block (registers or shared memory) and
// merged into int64 group slots with global atomics.
//
// This replaces, for one query, the reference's generated per-row loop
// (codegen/template.cpp:61-89 filled by codegen/codegen.cpp:100-229), its
// per-bulk host compaction (core/pipeline.cu:346-357) and its per-bulk
// sort + reduce (core/pipeline.cu:360-472).
//
// Layout: a thread owns a group of 4 consecutive rows and reads each fact
// column it needs with one 16-byte streaming load (ld.global.cs).  A column is
// only fetched while some row of the group is still alive, so the columns
// read after selective steps are mostly skipped.  Dimension tables small
// enough are staged in shared memory at block start; the others are probed in
// global memory through the read-only path and stay L2-resident.
#include <climits>

#include "kern_common.cuh"
#include "kernels.h"

namespace svm {

constexpr int kStarThreads = 256;

template <int kSlots>
__device__ __forceinline__ int32_t pick(const int32_t (&val)[kMaxSteps][4], int slot, int j) {
  int32_t raw = 0;
#pragma unroll
  for (int k = 0; k < kSlots; k++)
    if (k == slot) raw = val[k][j];
  return raw;
}

__device__ __forceinline__ int32_t opnd_value(const StarParams& P, const int32_t (&val)[kMaxSteps][4],
                                              int j, Operand o) {
  int32_t raw = pick<kMaxSteps>(val, o.slot, j);
  if (o.field < 0) return raw;
  return payload_value(P.dims[P.steps[o.slot].dim], o.field, (uint32_t)raw);
}

__device__ __forceinline__ int32_t metric_value(const StarParams& P, const Metric& M,
                                                const int32_t (&val)[kMaxSteps][4], int j) {
  if (M.form == MF_PROG) {
    int32_t ov[16];
    for (int q = 0; q < P.nopnd; q++) ov[q] = opnd_value(P, val, j, P.opnds[q]);
    return eval_prog(M.prog, ov, P.error);
  }
  uint32_t a = (uint32_t)opnd_value(P, val, j, M.a);
  if (M.form == MF_OPND) return (int32_t)a;
  uint32_t b = (uint32_t)opnd_value(P, val, j, M.b);
  if (M.form == MF_ADD) return (int32_t)(a + b);
  if (M.form == MF_SUB) return (int32_t)(a - b);
  return (int32_t)(a * b);
}

template <int kAgg>
__global__ void __launch_bounds__(kStarThreads) star_kernel(const __grid_constant__ StarParams P) {
  extern __shared__ __align__(16) uint32_t smem[];

  // Stage the small dimension tables.
  for (int d = 0; d < P.ndims; d++) {
    const DimDesc& D = P.dims[d];
    if (D.smem_word_off < 0) continue;
    for (uint32_t w = threadIdx.x; w < D.table_words; w += blockDim.x)
      smem[D.smem_word_off + w] = __ldg(D.words + w);
  }
  const int nm = P.nmetrics;
  const unsigned long long G = P.ngroups;
  unsigned long long* s_sum = reinterpret_cast<unsigned long long*>(smem + ((P.smem_table_words + 3) & ~3));
  unsigned int* s_cnt = reinterpret_cast<unsigned int*>(s_sum + (kAgg == AGG_DENSE_SMEM ? nm * G : 0));
  if (kAgg == AGG_DENSE_SMEM) {
    for (unsigned long long i = threadIdx.x; i < nm * G; i += blockDim.x) s_sum[i] = 0ull;
    for (unsigned long long i = threadIdx.x; i < G; i += blockDim.x) s_cnt[i] = 0u;
  }
  __syncthreads();

  long long acc[kMaxMetrics] = {0, 0, 0};
  unsigned long long nacc = 0;

  const long long a0 = P.row_begin & ~3ll;
  const long long ngr = (P.row_end - a0 + 3) >> 2;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ngr; g += stride) {
    const long long r0 = a0 + 4 * g;
    uint32_t mask = 0xFu;
    if (r0 < P.row_begin) mask &= (0xFu << (P.row_begin - r0)) & 0xFu;
    if (r0 + 4 > P.row_end) mask &= 0xFu >> (r0 + 4 - P.row_end);
    int32_t val[kMaxSteps][4];
#pragma unroll
    for (int k = 0; k < kMaxSteps; k++) {
      if (k < P.nsteps && mask) {
        const Step& st = P.steps[k];
        int4 v = __ldcs(reinterpret_cast<const int4*>(P.cols[st.col] + r0));
        val[k][0] = v.x;
        val[k][1] = v.y;
        val[k][2] = v.z;
        val[k][3] = v.w;
        if (st.kind == STEP_RANGE) {
          uint32_t span = (uint32_t)st.hi - (uint32_t)st.lo;
#pragma unroll
          for (int j = 0; j < 4; j++)
            if ((uint32_t)val[k][j] - (uint32_t)st.lo > span) mask &= ~(1u << j);
        } else if (st.kind == STEP_PROBE) {
          const DimDesc& D = P.dims[st.dim];
#pragma unroll
          for (int j = 0; j < 4; j++) {
            if (mask >> j & 1u) {
              uint32_t e;
              if (probe_dim(D, smem, val[k][j], e))
                val[k][j] = (int32_t)e;
              else
                mask &= ~(1u << j);
            }
          }
        }
      }
    }
    if (!mask) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (!(mask >> j & 1u)) continue;
      bool keep = true;
      for (int q = 0; q < P.npost && keep; q++) {
        int32_t ov[16];
        for (int o = 0; o < P.nopnd; o++) ov[o] = opnd_value(P, val, j, P.opnds[o]);
        keep = eval_prog(P.post[q], ov, P.error) != 0;
      }
      if (!keep) continue;
      if (kAgg == AGG_SCALAR) {
        for (int m = 0; m < nm; m++) acc[m] += (long long)metric_value(P, P.metrics[m], val, j);
        nacc++;
      } else {
        unsigned long long gi = 0;
        bool ok = true;
        for (int q = 0; q < P.nkeys; q++) {
          uint32_t off = (uint32_t)opnd_value(P, val, j, P.keys[q]) - (uint32_t)P.kmin[q];
          ok &= off < P.krange[q];
          gi += (unsigned long long)off * P.kstride[q];
        }
        if (!ok) {
          raise_error(P.error, 3);
          continue;
        }
        for (int m = 0; m < nm; m++) {
          unsigned long long v = (unsigned long long)(long long)metric_value(P, P.metrics[m], val, j);
          if (kAgg == AGG_DENSE_SMEM)
            atomicAdd(s_sum + m * G + gi, v);
          else
            atomicAdd(P.sums + m * G + gi, v);
        }
        if (kAgg == AGG_DENSE_SMEM)
          atomicAdd(s_cnt + gi, 1u);
        else
          atomicAdd(P.counts + gi, 1ull);
      }
    }
  }

  if (kAgg == AGG_SCALAR) {
    __shared__ long long red[kStarThreads / 32][kMaxMetrics + 1];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long c = (long long)nacc;
    for (int o = 16; o; o >>= 1) {
      for (int m = 0; m < kMaxMetrics; m++) acc[m] += __shfl_xor_sync(0xffffffffu, acc[m], o);
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (lane == 0) {
      for (int m = 0; m < kMaxMetrics; m++) red[wid][m] = acc[m];
      red[wid][kMaxMetrics] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      long long t[kMaxMetrics + 1] = {0, 0, 0, 0};
      for (int w = 0; w < kStarThreads / 32; w++)
        for (int m = 0; m <= kMaxMetrics; m++) t[m] += red[w][m];
      for (int m = 0; m < nm; m++)
        if (t[m]) atomicAdd(P.sums + m, (unsigned long long)t[m]);
      if (t[kMaxMetrics]) atomicAdd(P.counts, (unsigned long long)t[kMaxMetrics]);
    }
  } else if (kAgg == AGG_DENSE_SMEM) {
    __syncthreads();
    for (unsigned long long i = threadIdx.x; i < G; i += blockDim.x) {
      unsigned int c = s_cnt[i];
      if (!c) continue;
      atomicAdd(P.counts + i, (unsigned long long)c);
      for (int m = 0; m < nm; m++) atomicAdd(P.sums + m * G + i, s_sum[m * G + i]);
    }
  }
}

int star_block_size() { return kStarThreads; }

size_t star_smem_bytes(const StarParams& p) {
  size_t b = (size_t)((p.smem_table_words + 3) & ~3) * 4;
  if (p.agg == AGG_DENSE_SMEM) b += (size_t)p.ngroups * (8 * p.nmetrics + 4);
  return b;
}

template <int kAgg>
static const void* star_fn() {
  return reinterpret_cast<const void*>(&star_kernel<kAgg>);
}

static const void* star_entry(int agg) {
  switch (agg) {
    case AGG_SCALAR: return star_fn<AGG_SCALAR>();
    case AGG_DENSE_SMEM: return star_fn<AGG_DENSE_SMEM>();
    default: return star_fn<AGG_DENSE_GLOBAL>();
  }
}

int star_grid_size(const StarParams& p, size_t smem) {
  static bool attr_set[3] = {false, false, false};
  int a = p.agg == AGG_SCALAR ? 0 : p.agg == AGG_DENSE_SMEM ? 1 : 2;
  const void* fn = star_entry(p.agg);
  if (!attr_set[a]) {
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr_set[a] = true;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kStarThreads, smem);
  if (per_sm < 1) per_sm = 1;
  long long groups = (p.row_end - (p.row_begin & ~3ll) + 3) >> 2;
  long long want = (groups + kStarThreads - 1) / kStarThreads;
  long long cap = (long long)num_sms() * per_sm;
  if (want < 1) want = 1;
  return (int)(want < cap ? want : cap);
}

cudaError_t launch_star(const StarParams& p, int grid, int block, size_t smem, cudaStream_t s) {
  note_launch();
  switch (p.agg) {
    case AGG_SCALAR: star_kernel<AGG_SCALAR><<<grid, block, smem, s>>>(p); break;
    case AGG_DENSE_SMEM: star_kernel<AGG_DENSE_SMEM><<<grid, block, smem, s>>>(p); break;
    case AGG_DENSE_GLOBAL: star_kernel<AGG_DENSE_GLOBAL><<<grid, block, smem, s>>>(p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------- finalize
__global__ void group_flags_kernel(const unsigned long long* counts, unsigned long long G,
                                   uint32_t* flags) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < G;
       i += (unsigned long long)gridDim.x * blockDim.x)
    flags[i] = counts[i] != 0ull;
}

struct FinalizeOut {
  int32_t* key[kMaxKeys];
  void* met[kMaxMetrics];
  int wide[kMaxMetrics];
};

__global__ void group_write_kernel(StarParams P, const unsigned long long* pos, FinalizeOut o) {
  unsigned long long G = P.ngroups;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < G;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    if (P.counts[i] == 0ull) continue;
    unsigned long long at = pos[i];
    for (int q = 0; q < P.nkeys; q++) {
      unsigned long long off = (i / P.kstride[q]) % P.krange[q];
      o.key[q][at] = (int32_t)((uint32_t)P.kmin[q] + (uint32_t)off);
    }
    for (int m = 0; m < P.nmetrics; m++) {
      unsigned long long s = P.sums[m * G + i];
      if (o.wide[m])
        reinterpret_cast<long long*>(o.met[m])[at] = (long long)s;
      else
        reinterpret_cast<int32_t*>(o.met[m])[at] = (int32_t)(uint32_t)s;
    }
  }
}

cudaError_t launch_finalize_dense(const StarParams& p, int32_t* const* key_out, void* const* met_out,
                                  const int* wide, unsigned long long* flags_tmp,
                                  unsigned long long* scan_tmp, unsigned long long* out_count,
                                  cudaStream_t s) {
  // flags_tmp holds G uint32 flags followed by G+1 uint64 positions.
  (void)out_count;
  unsigned long long G = p.ngroups;
  uint32_t* flags = reinterpret_cast<uint32_t*>(flags_tmp);
  unsigned long long* pos = flags_tmp + (G + 1) / 2 + 1;
  int grid = num_sms() * 4;
  if (key_out == nullptr) {
    note_launch();
    group_flags_kernel<<<grid, 256, 0, s>>>(p.counts, G, flags);
    return launch_exclusive_scan(flags, G, pos, scan_tmp, s);
  }
  FinalizeOut o{};
  for (int q = 0; q < p.nkeys; q++) o.key[q] = key_out[q];
  for (int m = 0; m < p.nmetrics; m++) {
    o.met[m] = met_out[m];
    o.wide[m] = wide[m];
  }
  note_launch();
  group_write_kernel<<<grid, 256, 0, s>>>(p, pos, o);
  return cudaGetLastError();
}

}  // namespace svm
