// The fused fact-table scan: range filters and dimension probes in the order
// the planner chose (cheapest per rejected row first), then group keys and
// metrics of the surviving rows aggregated per block (registers or shared
// memory) and merged into int64 group slots with global atomics.
//
// This replaces, for one query, the reference's generated per-row loop
// (codegen/template.cpp:61-89 filled by codegen/codegen.cpp:100-229), its
// per-bulk host compaction (core/pipeline.cu:346-357) and its per-bulk
// sort + reduce (core/pipeline.cu:360-472).
//
// Data movement: a persistent grid walks the fact rows in tiles of kTileRows.
// In every block one producer warp streams each fact column the query reads
// into a ring of shared-memory stages with 1-D bulk copies (cp.async.bulk,
// completion counted on an mbarrier per stage); the consumer warps work on
// the staged tile and release the stage.  The DRAM stream is therefore never
// behind a dependent probe.  Small dimension tables are staged in shared
// memory at block start; larger ones are probed in global memory and stay
// L2-resident.
//
// Execution inside a tile is vectorised with selection vectors: each consumer
// warp owns 128 rows.  The first step runs densely (4 rows per lane, one
// 16-byte shared-memory read per column); the surviving rows are compacted
// into a warp-local list (row offset + the payload words probed so far), and
// every later step and the aggregation run over that list with all 32 lanes
// busy.  Work per step is proportional to the rows still alive.
#include <climits>

#include "kern_star_common.cuh"
#include "kernels.h"

namespace svm {

// A consumer warp's selection vector: surviving row offsets (within the
// warp's 128 rows), and per probed dimension the matched table entry of each
// row, indexed by row offset (so compaction only moves the offsets).
// A consumer warp's selection vector in shared memory: the row indices of
// its live rows and, per joined dimension, the probe word of each row.
struct WarpList {
  uint32_t* pwb;  // ndims x kWarpRows
  uint16_t* row;  // kWarpRows
  __device__ __forceinline__ uint32_t* pw(int d) const { return pwb + d * kWarpRows; }
};

// Bytes of one warp's list for `ndims` joined dimensions (16-byte multiple).
__host__ __device__ __forceinline__ size_t warp_list_bytes(int ndims) {
  return (size_t)(ndims > 0 ? ndims : 1) * kWarpRows * 4 + kWarpRows * 2;
}

__device__ __forceinline__ WarpList warp_list(uint8_t* base, int warp, int ndims) {
  uint8_t* p = base + (size_t)warp * warp_list_bytes(ndims);
  WarpList L;
  L.pwb = reinterpret_cast<uint32_t*>(p);
  L.row = reinterpret_cast<uint16_t*>(p + (size_t)(ndims > 0 ? ndims : 1) * kWarpRows * 4);
  return L;
}

// Dense-table entry for `key`, or 0 (bit 0 clear) when absent.
__device__ __forceinline__ uint32_t dense_entry(const Step& D, const uint32_t* w, int32_t key, bool live) {
  uint32_t idx = (uint32_t)key - (uint32_t)D.key_min;
  live = live && idx < D.span;
  uint32_t bit = idx * (uint32_t)D.entry_bits;  // span * entry_bits < 2^32 (planner)
  uint32_t word = live ? w[bit >> 5] : 0u;
  return D.entry_bits == 32 ? word : (word >> (bit & 31)) & ((1u << D.entry_bits) - 1u);
}

__device__ __forceinline__ uint32_t hash_entry(const Step& D, const uint32_t* w, int32_t key, bool live) {
  if (!live) return 0u;
  const uint32_t cmask = D.span - 1u;
  uint32_t slot = mix32((uint32_t)key) & cmask;
  for (uint32_t n = 0; n <= cmask; n++) {
    uint2 kv = reinterpret_cast<const uint2*>(w)[slot];
    if (kv.y == 0u) return 0u;
    if ((int32_t)kv.x == key) return kv.y;
    slot = (slot + 1u) & cmask;
  }
  return 0u;
}

// Looks up 4 keys (lanes' `live` flags) in table D; entries with bit 0 clear
// are misses.  Dense lookups are issued together (4 loads in flight).
__device__ __forceinline__ void lookup4(const Step& D, const uint32_t* tables, const int32_t (&key)[4],
                                        const bool (&live)[4], uint32_t (&e)[4]) {
  // Fully unrolled over the 4 keys: the arrays stay in registers.
  const uint32_t* w = D.smem_word_off >= 0 ? tables + D.smem_word_off : D.words;
  if (D.layout == LAYOUT_DENSE) {
#pragma unroll
    for (int j = 0; j < 4; j++) e[j] = dense_entry(D, w, key[j], live[j]);
  } else {
#pragma unroll
    for (int j = 0; j < 4; j++) e[j] = hash_entry(D, w, key[j], live[j]);
  }
}

__device__ __forceinline__ int32_t opnd_value(const StarParams& P, const int32_t* wstage, int row,
                                              const uint32_t (&pw)[kMaxDims], Operand o) {
  if (o.field < 0) return wstage[o.slot * kTileRows + row];
  uint32_t e = pw[0];
#pragma unroll
  for (int d = 1; d < kMaxDims; d++)
    if (o.slot == d) e = pw[d];
  return payload_value(P.dims[o.slot], o.field, e);
}

// A flattened operand: one staged value or one payload field, no indirection.
__device__ __forceinline__ uint32_t extract(const Extract& x, const int32_t* wstage, int row,
                                            const uint32_t (&pw)[kMaxDims]) {
  if (x.dim < 0) return (uint32_t)wstage[x.slot * kTileRows + row] + (uint32_t)x.base;
  uint32_t e = pw[0];
#pragma unroll
  for (int d = 1; d < kMaxDims; d++)
    if (x.dim == d) e = pw[d];
  uint32_t v = (e >> x.shift) & x.mask;
  if (x.col) v = (uint32_t)__ldg(x.col + v);
  return v + (uint32_t)x.base;
}

template <bool kProg>
__device__ __forceinline__ int32_t metric_value(const StarParams& P, const Metric& M, const int32_t* wstage,
                                                int row, const uint32_t (&pw)[kMaxDims]) {
  if (kProg && M.form == MF_PROG) {
    int32_t ov[16];
    for (int q = 0; q < P.nopnd; q++) ov[q] = opnd_value(P, wstage, row, pw, P.opnds[q]);
    return eval_prog(M.prog, ov, P.error);
  }
  uint32_t a = extract(M.xa, wstage, row, pw);
  if (M.form == MF_OPND) return (int32_t)a;
  uint32_t b = extract(M.xb, wstage, row, pw);
  if (M.form == MF_ADD) return (int32_t)(a + b);
  if (M.form == MF_SUB) return (int32_t)(a - b);
  return (int32_t)(a * b);
}

template <int kAgg, bool kProg>
__device__ __forceinline__ void aggregate_row(const StarParams& P, const int32_t* wstage, int row,
                                              const uint32_t (&pw)[kMaxDims], long long (&acc)[kMaxMetrics + 1],
                                              unsigned long long* s_sum, unsigned int* s_cnt) {
  if (kProg) {
    for (int q = 0; q < P.npost; q++) {
      int32_t ov[16];
      for (int o = 0; o < P.nopnd; o++) ov[o] = opnd_value(P, wstage, row, pw, P.opnds[o]);
      if (!eval_prog(P.post[q], ov, P.error)) return;
    }
  }
  const int nm = P.nmetrics;
  if (kAgg == AGG_SCALAR) {
#pragma unroll
    for (int m = 0; m < kMaxMetrics; m++)
      if (m < nm) acc[m] += (long long)metric_value<kProg>(P, P.metrics[m], wstage, row, pw);
    acc[kMaxMetrics] += 1;
    return;
  }
  const unsigned long long G = P.ngroups;
  // Dense group index (G <= 2^26): keys read through their flattened
  // extractors with compile-time indices.
  uint32_t gi = 0;
  bool in_range = true;
#pragma unroll
  for (int q = 0; q < kMaxKeys; q++) {
    if (q < P.nkeys) {
      const uint32_t off = extract(P.kx[q], wstage, row, pw);
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
      unsigned long long v = (unsigned long long)(long long)metric_value<kProg>(P, P.metrics[m], wstage, row, pw);
      if (kAgg == AGG_DENSE_SMEM)
        smem_add64(s_sum + m * G + gi, v);
      else
        atomicAdd(P.sums + m * G + gi, v);
    }
  }
  // Only "the group has a row" is read back: a plain store marks it.
  if (kAgg == AGG_DENSE_SMEM)
    s_cnt[gi] = 1u;
  else
    atomicAdd(P.counts + gi, 1ull);
}

// kFuse consecutive filter steps over the first n entries of the warp's
// selection vector (kChunks * 32 >= n): each lane takes one entry per chunk;
// every lookup of the fused steps is issued before any result is used (the
// steps are evaluated independently and their outcomes AND-ed); survivors are
// compacted in place.  Returns the new list length.
template <int kChunks, int kFuse>
__device__ __forceinline__ int list_step(const Step* sts, const int32_t* wstage, const uint32_t* tables,
                                         const WarpList& L, int n, int lane, uint32_t lt) {
  bool live[4];
  uint16_t row[4];
  uint32_t e[kFuse][4];
  bool ok[kFuse][4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const int idx = 32 * c + lane;
    live[c] = c < kChunks && idx < n;
    row[c] = live[c] ? L.row[idx] : (uint16_t)0;
  }
#pragma unroll
  for (int f = 0; f < kFuse; f++) {
    const Step& st = sts[f];
    const uint32_t span = (uint32_t)st.hi - (uint32_t)st.lo;
    int32_t key[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      key[c] = live[c] ? wstage[st.col * kTileRows + row[c]] : 0;
      ok[f][c] = live[c] && (uint32_t)key[c] - (uint32_t)st.lo <= span;
      e[f][c] = 0u;
    }
    if (st.kind == STEP_PROBE) {
      const uint32_t* w = st.smem_word_off >= 0 ? tables + st.smem_word_off : st.words;
      if (st.layout == LAYOUT_DENSE) {
#pragma unroll
        for (int c = 0; c < kChunks; c++) e[f][c] = dense_entry(st, w, key[c], ok[f][c]);
      } else {
#pragma unroll
        for (int c = 0; c < kChunks; c++) e[f][c] = hash_entry(st, w, key[c], ok[f][c]);
      }
    }
  }
#pragma unroll
  for (int f = 0; f < kFuse; f++) {
    const Step& st = sts[f];
#pragma unroll
    for (int c = 0; c < kChunks; c++)
      live[c] = live[c] && ok[f][c] && (st.kind != STEP_PROBE || (e[f][c] & 1u));
  }
#pragma unroll
  for (int f = 0; f < kFuse; f++) {
    const Step& st = sts[f];
    if (st.kind == STEP_PROBE) {
#pragma unroll
      for (int c = 0; c < kChunks; c++)
        if (live[c]) L.pw(st.dim)[row[c]] = e[f][c];
    }
  }
  int pos[4];
  int m = 0;
#pragma unroll
  for (int c = 0; c < kChunks; c++) {
    const uint32_t b = __ballot_sync(0xffffffffu, live[c]);
    pos[c] = m + __popc(b & lt);
    m += __popc(b);
  }
  __syncwarp();
#pragma unroll
  for (int c = 0; c < kChunks; c++)
    if (live[c]) L.row[pos[c]] = row[c];
  __syncwarp();
  return m;
}

template <int kAgg, bool kProg>
__global__ void __launch_bounds__(kStarThreads, 3) star_kernel(const __grid_constant__ StarParams P) {
  extern __shared__ __align__(128) uint8_t dyn[];
  __shared__ StarSmem S;
  // The filter steps, copied once per block: the step loop reads them with a
  // runtime index, which from the kernel parameters costs a constant-bank
  // load per field per warp and tile (3.87 -> 3.57 ms on the 600 M-row
  // four-dimension star query when read from shared memory instead).
  __shared__ Step s_steps[kMaxSteps];
  static_assert(sizeof(Step) % 4 == 0, "steps are copied as 32-bit words");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ncols = P.ncols, nst = P.nstages;
  const size_t ring_bytes = (size_t)nst * ncols * kTileRows * 4;
  int32_t* ring = reinterpret_cast<int32_t*>(dyn);
  uint8_t* lists = dyn + ring_bytes;
  uint32_t* tables = reinterpret_cast<uint32_t*>(lists + kConsumerWarps * warp_list_bytes(P.ndims));
  unsigned long long* s_sum =
      reinterpret_cast<unsigned long long*>(tables + ((P.smem_table_words + 3) & ~3));
  const int nm = P.nmetrics;
  const unsigned long long G = P.ngroups;
  unsigned int* s_cnt = reinterpret_cast<unsigned int*>(s_sum + (kAgg == AGG_DENSE_SMEM ? nm * G : 0));
  // Deferred-aggregation buffers: kAggCap rows of agg_words words per consumer warp.
  uint32_t* aggbuf = reinterpret_cast<uint32_t*>(s_cnt + (kAgg == AGG_DENSE_SMEM ? G : 0));
  const bool deferred = !kProg && P.agg_words > 0;

  for (int i = tid; i < P.nsteps * (int)(sizeof(Step) / 4); i += blockDim.x)
    reinterpret_cast<uint32_t*>(s_steps)[i] = reinterpret_cast<const uint32_t*>(P.steps)[i];
  if (tid == 0) {
    for (int s = 0; s < nst; s++) {
      mbar_init(&S.full[s], 1);
      mbar_init(&S.empty[s], kConsumerWarps);
    }
    mbar_fence_init();
  }
  for (int d = 0; d < P.ndims; d++) {
    const DimDesc& D = P.dims[d];
    if (D.smem_word_off < 0) continue;
    for (uint32_t w = tid; w < D.table_words; w += blockDim.x) tables[D.smem_word_off + w] = __ldg(D.words + w);
  }
  if (kAgg == AGG_DENSE_SMEM) {
    for (unsigned long long i = tid; i < nm * G; i += blockDim.x) s_sum[i] = 0ull;
    for (unsigned long long i = tid; i < G; i += blockDim.x) s_cnt[i] = 0u;
  }
  __syncthreads();

  const long long a0 = P.row_begin & ~3ll;
  const long long end4 = (P.row_end + 3) & ~3ll;  // copies stop at the 4-row boundary past row_end
  const long long ntiles = (P.row_end - a0 + kTileRows - 1) / kTileRows;
  const uint32_t polls = P.wait_polls ? P.wait_polls : kWaitPolls;
  long long acc[kMaxMetrics + 1] = {0, 0, 0, 0};

  if (warp == kConsumerWarps) {
    // ---------------- producer: one lane issues the bulk copies
    if (lane == 0 && !P.stall_copies) {
      long long issued = 0;
      RingPos rp;
      for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, issued++, rp.next(nst)) {
        const int s = rp.s;
        if (issued >= nst && !mbar_wait_bounded(&S.empty[s], rp.phase ^ 1u, polls)) {
          raise_error(P.error, DERR_TIMEOUT);
          break;
        }
        long long start = a0 + t * kTileRows;
        long long stop = start + kTileRows < end4 ? start + kTileRows : end4;
        uint32_t bytes = (uint32_t)((stop - start) * 4);
        mbar_arrive_expect_tx(&S.full[s], bytes * (uint32_t)ncols);
        for (int c = 0; c < ncols; c++)
          bulk_g2s(ring + ((size_t)s * ncols + c) * kTileRows, P.cols[c] + start, bytes, &S.full[s]);
      }
      // Every issued copy lands before the block exits.
      long long first = issued > nst ? issued - nst : 0;
      for (long long q = first; q < issued; q++)
        mbar_wait_bounded(&S.full[q % nst], (uint32_t)((q / nst) & 1), polls);
    }
  } else {
    // ---------------- consumers
    const WarpList L = warp_list(lists, warp, P.ndims);
    const uint32_t lt = lanemask_lt();
    uint32_t* buf = aggbuf + (size_t)warp * kAggCap * (deferred ? P.agg_words : 0);
    int cnt = 0;  // rows buffered (deferred aggregation)
    RingPos rp;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, rp.next(nst)) {
      const int s = rp.s;
      if (!mbar_wait_bounded(&S.full[s], rp.phase, polls)) {
        raise_error(P.error, DERR_TIMEOUT);
        break;
      }
      // This warp's rows: [start + 128*warp, +128); lane owns 4 of them in the dense step.
      const int32_t* wstage = ring + (size_t)s * ncols * kTileRows + warp * kWarpRows;
      const long long r0 = a0 + t * kTileRows + warp * kWarpRows + 4 * lane;
      uint32_t mask = 0xFu;
      if (r0 < P.row_begin) mask &= (0xFu << (unsigned)(P.row_begin - r0 > 4 ? 4 : P.row_begin - r0)) & 0xFu;
      if (r0 + 4 > P.row_end) mask &= r0 >= P.row_end ? 0u : 0xFu >> (unsigned)(r0 + 4 - P.row_end);

      // ---- every filter step over the lane's 4 rows, predicated on the rows
      // still live: a probe's loads go out only for live rows, its entries
      // are kept per row in shared memory; the warp stops once no row lives.
      for (int k = 0; k < P.nsteps; k++) {
        if (!__any_sync(0xffffffffu, mask)) break;
        const Step& st = s_steps[k];
        const int4 v = reinterpret_cast<const int4*>(wstage + st.col * kTileRows)[lane];
        const int32_t key[4] = {v.x, v.y, v.z, v.w};
        const uint32_t span = (uint32_t)st.hi - (uint32_t)st.lo;
        bool live[4];
#pragma unroll
        for (int j = 0; j < 4; j++) live[j] = (mask >> j & 1u) && (uint32_t)key[j] - (uint32_t)st.lo <= span;
        if (st.kind == STEP_PROBE) {
          uint32_t e[4];
          lookup4(st, tables, key, live, e);
#pragma unroll
          for (int j = 0; j < 4; j++) live[j] = live[j] && (e[j] & 1u);
          *reinterpret_cast<uint4*>(&L.pw(st.dim)[4 * lane]) = make_uint4(e[0], e[1], e[2], e[3]);
        }
        mask = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) mask |= (uint32_t)live[j] << j;
      }
      // ---- the survivors as a selection list
      int n = 0;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const uint32_t b = __ballot_sync(0xffffffffu, mask >> j & 1u);
        if (mask >> j & 1u) L.row[n + __popc(b & lt)] = (uint16_t)(4 * lane + j);
        n += __popc(b);
      }
      __syncwarp();

      // ---- aggregate the survivors: buffered (their operand words) and
      // aggregated 32 rows at a time, or in place
      if (deferred && n <= kAggCap) {
        if (cnt + n > kAggCap) {
          flush_entries<kAgg>(P, buf, cnt, lane, acc, s_sum, s_cnt);
          cnt = 0;
        }
        const int W = P.agg_words;
        for (int idx = lane; idx < n; idx += 32) {
          const int row = L.row[idx];
          uint32_t* ent = buf + (size_t)(cnt + idx) * W;
          for (int k = 0; k < W; k++) {
            const int code = P.agg_src[k];
            ent[k] = code < 8 ? L.pw(code)[row] : (uint32_t)wstage[(code - 8) * kTileRows + row];
          }
        }
        cnt += n;
      } else {
        for (int base = 0; base < n; base += 32) {
          const int idx = base + lane;
          if (idx < n) {
            const int row = L.row[idx];
            uint32_t pw[kMaxDims];
#pragma unroll
            for (int d = 0; d < kMaxDims; d++) pw[d] = d < P.ndims ? L.pw(d)[row] : 0u;
            aggregate_row<kAgg, kProg>(P, wstage, row, pw, acc, s_sum, s_cnt);
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.empty[s]);
    }
    if (deferred && cnt) flush_entries<kAgg>(P, buf, cnt, lane, acc, s_sum, s_cnt);
  }

  finish_block<kAgg>(P, S, acc, s_sum, s_cnt, tid, warp, lane);
}

int star_block_size() { return kStarThreads; }

size_t star_smem_bytes(const StarParams& p) {
  size_t b = (size_t)p.nstages * p.ncols * kTileRows * 4;
  b += warp_list_bytes(p.ndims) * kConsumerWarps;
  b += (size_t)((p.smem_table_words + 3) & ~3) * 4;
  if (p.agg == AGG_DENSE_SMEM) b += (size_t)p.ngroups * (8 * p.nmetrics + 4);
  b = (b + 15) & ~size_t(15);
  b += (size_t)kConsumerWarps * kAggCap * p.agg_words * 4;
  return b;
}

// Plans without bytecode (no residual predicate, no general metric) run the
// lean instantiation.
static bool plan_needs_prog(const StarParams& p) {
  if (p.npost > 0) return true;
  for (int m = 0; m < p.nmetrics; m++)
    if (p.metrics[m].form == MF_PROG) return true;
  return false;
}

template <bool kProg>
static const void* star_entry_t(int agg) {
  switch (agg) {
    case AGG_SCALAR: return reinterpret_cast<const void*>(&star_kernel<AGG_SCALAR, kProg>);
    case AGG_DENSE_SMEM: return reinterpret_cast<const void*>(&star_kernel<AGG_DENSE_SMEM, kProg>);
    default: return reinterpret_cast<const void*>(&star_kernel<AGG_DENSE_GLOBAL, kProg>);
  }
}

int star_blocks_per_sm(const StarParams& p, size_t smem) {
  const bool prog = plan_needs_prog(p);
  const void* fn = prog ? star_entry_t<true>(p.agg) : star_entry_t<false>(p.agg);
  allow_dynamic_smem(fn, 210 * 1024);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kStarThreads, smem);
  return per_sm;
}

int star_grid_size(const StarParams& p, size_t smem) {
  int per_sm = star_blocks_per_sm(p, smem);
  if (per_sm < 1) per_sm = 1;
  long long tiles = (p.row_end - (p.row_begin & ~3ll) + kTileRows - 1) / kTileRows;
  long long cap = (long long)num_sms() * per_sm;
  if (tiles < 1) tiles = 1;
  return (int)(tiles < cap ? tiles : cap);
}

cudaError_t launch_star(const StarParams& p, int grid, int block, size_t smem, cudaStream_t s) {
  note_launch();
  const bool prog = plan_needs_prog(p);
  switch (p.agg * 2 + (prog ? 1 : 0)) {
    case AGG_SCALAR * 2: star_kernel<AGG_SCALAR, false><<<grid, block, smem, s>>>(p); break;
    case AGG_SCALAR * 2 + 1: star_kernel<AGG_SCALAR, true><<<grid, block, smem, s>>>(p); break;
    case AGG_DENSE_SMEM * 2: star_kernel<AGG_DENSE_SMEM, false><<<grid, block, smem, s>>>(p); break;
    case AGG_DENSE_SMEM * 2 + 1: star_kernel<AGG_DENSE_SMEM, true><<<grid, block, smem, s>>>(p); break;
    case AGG_DENSE_GLOBAL * 2: star_kernel<AGG_DENSE_GLOBAL, false><<<grid, block, smem, s>>>(p); break;
    case AGG_DENSE_GLOBAL * 2 + 1: star_kernel<AGG_DENSE_GLOBAL, true><<<grid, block, smem, s>>>(p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ================================================================ batched queries
// One persistent launch for a batch of fact pipelines over one fact table.
// The producer hands tiles out dynamically (an atomic tile counter, so blocks
// that drew tiles covered by many queries take fewer tiles) and streams the
// union of the batch's columns; a tile index of -1 in a stage ends the scan.
// Each consumer warp then runs, for every query whose range covers its 128
// rows, the same dense-step / selection-vector / aggregation pipeline as the
// single-query kernel, into that query's own int64 slots.

__device__ __forceinline__ void batch_query_slice(const BatchQuery& Q, const BatchParams& B, const int32_t* wstage,
                                                  long long slice_start, const WarpList& L, int lane, uint32_t lt) {
  const long long r0 = slice_start + 4 * lane;
  uint32_t mask = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) mask |= (uint32_t)(r0 + j >= Q.row_begin && r0 + j < Q.row_end) << j;
  if (!__any_sync(0xffffffffu, mask)) return;
  uint32_t e0[4] = {0u, 0u, 0u, 0u};
  int d0 = -1;
  if (Q.nsteps > 0) {
    const Step& st = Q.steps[0];
    const int4 v = reinterpret_cast<const int4*>(wstage + st.col * kTileRows)[lane];
    const int32_t key[4] = {v.x, v.y, v.z, v.w};
    const uint32_t span = (uint32_t)st.hi - (uint32_t)st.lo;
    bool live[4];
#pragma unroll
    for (int j = 0; j < 4; j++) live[j] = (mask >> j & 1u) && (uint32_t)key[j] - (uint32_t)st.lo <= span;
    if (st.kind == STEP_PROBE) {
      d0 = st.dim;
      lookup4(st, nullptr, key, live, e0);
#pragma unroll
      for (int j = 0; j < 4; j++) live[j] = live[j] && (e0[j] & 1u);
    }
    mask = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) mask |= (uint32_t)live[j] << j;
  }
  __syncwarp();
  if (d0 >= 0) *reinterpret_cast<uint4*>(&L.pw(d0)[4 * lane]) = make_uint4(e0[0], e0[1], e0[2], e0[3]);
  int n = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const uint32_t b = __ballot_sync(0xffffffffu, mask >> j & 1u);
    if (mask >> j & 1u) L.row[n + __popc(b & lt)] = (uint16_t)(4 * lane + j);
    n += __popc(b);
  }
  __syncwarp();
  for (int k = 1; k < Q.nsteps && n > 0; k++) {
    const Step* st = &Q.steps[k];
    if (n <= 32)
      n = list_step<1, 1>(st, wstage, nullptr, L, n, lane, lt);
    else if (n <= 64)
      n = list_step<2, 1>(st, wstage, nullptr, L, n, lane, lt);
    else
      n = list_step<4, 1>(st, wstage, nullptr, L, n, lane, lt);
  }
  if (n == 0) return;
  unsigned long long* sums = B.slots + Q.slot_off;
  const unsigned long long G = Q.ngroups;
  const int nm = Q.nmetrics;
  long long acc[kMaxMetrics] = {0, 0, 0};
  for (int base = 0; base < n; base += 32) {
    const int idx = base + lane;
    if (idx >= n) continue;
    const int row = L.row[idx];
    uint32_t pw[kMaxDims];
#pragma unroll
    for (int d = 0; d < kMaxDims; d++) pw[d] = L.pw(d)[row];
    uint32_t gi = 0;
    bool in_range = true;
#pragma unroll
    for (int q = 0; q < kMaxKeys; q++) {
      if (q < Q.nkeys) {
        const uint32_t off = extract(Q.kx[q], wstage, row, pw);
        in_range &= off < Q.krange[q];
        gi += off * Q.kstride[q];
      }
    }
    if (!in_range) {
      raise_error(B.error, DERR_KEY_RANGE);
      continue;
    }
#pragma unroll
    for (int m = 0; m < kMaxMetrics; m++) {
      if (m < nm) {
        uint32_t a = extract(Q.xa[m], wstage, row, pw), v = a;
        if (Q.mform[m] != MF_OPND) {
          uint32_t b2 = extract(Q.xb[m], wstage, row, pw);
          v = Q.mform[m] == MF_ADD ? a + b2 : Q.mform[m] == MF_SUB ? a - b2 : a * b2;
        }
        if (Q.nkeys == 0)
          acc[m] += (long long)(int32_t)v;
        else
          atomicAdd(sums + m * G + gi, (unsigned long long)(long long)(int32_t)v);
      }
    }
    if (Q.nkeys) sums[(size_t)nm * G + gi] = 1ull;  // the group has a row
  }
  if (Q.nkeys == 0) {
#pragma unroll
    for (int m = 0; m < kMaxMetrics; m++) {
      if (m < nm) {
        long long s = acc[m];
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && s) atomicAdd(sums + m, (unsigned long long)s);
      }
    }
  }
}

__global__ void __launch_bounds__(kStarThreads, 2) batch_kernel(const __grid_constant__ BatchParams B) {
  extern __shared__ __align__(128) uint8_t dyn[];
  __shared__ uint64_t full[kStages], empty[kStages];
  __shared__ long long stage_tile[kStages];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ncols = B.ncols, nst = B.nstages;
  int32_t* ring = reinterpret_cast<int32_t*>(dyn);
  uint8_t* lists = dyn + (size_t)nst * ncols * kTileRows * 4;
  if (tid == 0) {
    for (int s = 0; s < nst; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumerWarps);
    }
    mbar_fence_init();
  }
  __syncthreads();
  const long long a0 = B.row_begin & ~3ll;
  const long long end4 = (B.row_end + 3) & ~3ll;
  const long long ntiles = (B.row_end - a0 + kTileRows - 1) / kTileRows;

  if (warp == kConsumerWarps) {
    if (lane == 0) {
      long long issued = 0;
      RingPos rp;
      for (;; issued++, rp.next(nst)) {
        const int s = rp.s;
        if (issued >= nst && !mbar_wait_bounded(&empty[s], rp.phase ^ 1u, kWaitPolls)) {
          raise_error(B.error, DERR_TIMEOUT);
          break;
        }
        const long long t = (long long)atomicAdd(B.tile_counter, 1ull);
        if (t >= ntiles) {
          stage_tile[s] = -1;  // end of the scan
          mbar_arrive(&full[s]);
          issued++;
          break;
        }
        stage_tile[s] = t;
        const long long start = a0 + t * kTileRows;
        const long long stop = start + kTileRows < end4 ? start + kTileRows : end4;
        const uint32_t bytes = (uint32_t)((stop - start) * 4);
        mbar_arrive_expect_tx(&full[s], bytes * (uint32_t)ncols);
        for (int c = 0; c < ncols; c++)
          bulk_g2s(ring + ((size_t)s * ncols + c) * kTileRows, B.cols[c] + start, bytes, &full[s]);
      }
      const long long first = issued > nst ? issued - nst : 0;
      for (long long q = first; q < issued; q++)
        mbar_wait_bounded(&full[q % nst], (uint32_t)((q / nst) & 1), kWaitPolls);
    }
    return;
  }
  const WarpList L = warp_list(lists, warp, kMaxDims);
  const uint32_t lt = lanemask_lt();
  for (RingPos rp;; rp.next(nst)) {
    const int s = rp.s;
    if (!mbar_wait_bounded(&full[s], rp.phase, kWaitPolls)) {
      raise_error(B.error, DERR_TIMEOUT);
      break;
    }
    const long long t = stage_tile[s];
    if (t < 0) break;
    const int32_t* wstage = ring + (size_t)s * ncols * kTileRows + warp * kWarpRows;
    const long long slice_start = a0 + t * kTileRows + warp * kWarpRows;
    for (int base = 0; base < B.nqueries; base += 32) {
      const int q = base + lane;
      bool act = false;
      if (q < B.nqueries) {
        const BatchQuery& Q = B.queries[q];
        act = Q.row_begin < slice_start + kWarpRows && Q.row_end > slice_start;
      }
      uint32_t bq = __ballot_sync(0xffffffffu, act);
      while (bq) {
        const int qi = base + __ffs(bq) - 1;
        bq &= bq - 1;
        batch_query_slice(B.queries[qi], B, wstage, slice_start, L, lane, lt);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

size_t batch_smem_bytes(const BatchParams& b) {
  return (size_t)b.nstages * b.ncols * kTileRows * 4 + warp_list_bytes(kMaxDims) * kConsumerWarps;
}

int batch_grid_size(const BatchParams& b, size_t smem) {
  allow_dynamic_smem(reinterpret_cast<const void*>(&batch_kernel), 210 * 1024);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, kStarThreads, smem);
  return num_sms() * (per_sm < 1 ? 1 : per_sm);
}

cudaError_t launch_batch(const BatchParams& b, int grid, size_t smem, cudaStream_t s) {
  note_launch();
  batch_kernel<<<grid, kStarThreads, smem, s>>>(b);
  return cudaGetLastError();
}

// Groups of all queries numbered one after the other (BatchQuery::group_off).
__device__ __forceinline__ int batch_query_of(const BatchQuery* Q, int nq, unsigned long long g) {
  int lo = 0, hi = nq - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (Q[mid].group_off <= g)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__global__ void batch_flags_kernel(const BatchQuery* Q, int nq, const unsigned long long* slots,
                                   unsigned long long total, uint32_t* flags) {
  for (unsigned long long g = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; g < total;
       g += (unsigned long long)gridDim.x * blockDim.x) {
    const BatchQuery& q = Q[batch_query_of(Q, nq, g)];
    const unsigned long long gi = g - q.group_off;
    // A query without keys has exactly one result row.
    flags[g] = q.nkeys == 0 ? 1u : (uint32_t)(slots[q.slot_off + (size_t)q.nmetrics * q.ngroups + gi] != 0ull);
  }
}

__global__ void batch_write_kernel(const BatchQuery* Q, int nq, const unsigned long long* slots,
                                   unsigned long long total, const uint32_t* flags, const unsigned long long* pos,
                                   BatchOut o) {
  for (unsigned long long g = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; g < total;
       g += (unsigned long long)gridDim.x * blockDim.x) {
    if (!flags[g]) continue;
    const BatchQuery& q = Q[batch_query_of(Q, nq, g)];
    const unsigned long long gi = g - q.group_off, at = pos[g];
    for (int k = 0; k < q.nkeys; k++)
      o.key[k][at] = (int32_t)((uint32_t)q.kmin[k] + (uint32_t)((gi / q.kstride[k]) % q.krange[k]));
    for (int m = 0; m < q.nmetrics; m++) o.sum[m][at] = (long long)slots[q.slot_off + (size_t)m * q.ngroups + gi];
  }
}

__global__ void batch_bounds_kernel(const BatchQuery* Q, int nq, const unsigned long long* pos,
                                    unsigned long long total, unsigned long long* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= nq; i += gridDim.x * blockDim.x)
    out[i] = pos[i < nq ? Q[i].group_off : total];
}

cudaError_t launch_batch_bounds(const BatchQuery* Q, int nq, const unsigned long long* pos, unsigned long long total,
                                unsigned long long* out, cudaStream_t s) {
  note_launch();
  batch_bounds_kernel<<<(nq + 256) / 256, 256, 0, s>>>(Q, nq, pos, total, out);
  return cudaGetLastError();
}

cudaError_t launch_batch_finalize(const BatchQuery* Q, int nq, const unsigned long long* slots,
                                  unsigned long long total, uint32_t* flags, unsigned long long* pos,
                                  unsigned long long* scan_tmp, const BatchOut* out, cudaStream_t s) {
  const int grid = num_sms() * 4;
  if (!out) {
    note_launch();
    batch_flags_kernel<<<grid, 256, 0, s>>>(Q, nq, slots, total, flags);
    return launch_exclusive_scan(flags, total, pos, scan_tmp, s);
  }
  note_launch();
  batch_write_kernel<<<grid, 256, 0, s>>>(Q, nq, slots, total, flags, pos, *out);
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
