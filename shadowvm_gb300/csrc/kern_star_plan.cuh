// The fused scan compiled per plan shape: the kernel template and its
// registry entry type, shared by the translation units that instantiate
// shapes (kern_star_plan.cu, kern_star_plan_mix.cu).
#pragma once

#include <climits>
#include <type_traits>

#include "kern_star_common.cuh"
#include "kernels.h"

namespace svm {
namespace plan {

// Step codes (the host side is star_plan_code): bits 0-1 the kind, bits 2-4
// log2 of a dense table's entry width, bit 5 a fact-side range folded into a
// probe on the same column.
enum : int { SC_NONE = 0, SC_RANGE = 1, SC_SMEM = 2, SC_L2 = 3 };

template <int kCode>
struct StepCode {
  static constexpr int kind = kCode & 3;
  static constexpr int bits_log2 = (kCode >> 2) & 7;
  static constexpr int bits = 1 << bits_log2;
  static constexpr bool ranged = ((kCode >> 5) & 1) != 0;
  static constexpr bool probe = kind == SC_SMEM || kind == SC_L2;
};

__host__ __device__ constexpr int plan_warp_rows(int rows_per_lane) { return 32 * rows_per_lane; }

// One consumer warp's survivor list: row offsets within the warp's rows and,
// per joined dimension, each row's table entry (indexed by row offset), in
// 8- or 16-bit words when every entry fits them (entry_bytes 1, 2 or 4).
__host__ __device__ inline size_t plan_list_bytes(int ndims, int rows_per_lane, int entry_bytes) {
  const size_t wr = (size_t)plan_warp_rows(rows_per_lane);
  return ((size_t)(ndims > 0 ? ndims : 1) * wr * entry_bytes + wr * 2 + 15) & ~size_t(15);
}

// The bytes a kept entry takes: the narrowest of 1, 2 and 4 that holds every
// probe step's entries (the host side is star_plan_smem_bytes).
__host__ __device__ constexpr int plan_entry_bytes(int max_entry_bits) {
  return max_entry_bits <= 8 ? 1 : max_entry_bits <= 16 ? 2 : 4;
}

template <int kR, typename PwT>
struct PlanList {
  PwT* pwb;
  uint16_t* row;
  __device__ __forceinline__ PwT* pw(int d) const { return pwb + d * plan_warp_rows(kR); }
};

// The kept-entry word of a shape: the narrowest that holds every probe
// step's entries.
template <int A, int B, int C, int D>
struct PlanEntryWord {
  static constexpr int bits(int code) { return ((code & 3) >= SC_SMEM) ? (1 << ((code >> 2) & 7)) : 0; }
  static constexpr int max2(int a, int b) { return a > b ? a : b; }
  static constexpr int bytes = plan_entry_bytes(max2(max2(bits(A), bits(B)), max2(bits(C), bits(D))));
  using type = typename std::conditional<bytes == 1, uint8_t,
                                         typename std::conditional<bytes == 2, uint16_t, uint32_t>::type>::type;
};

template <typename PwT, int kR>
__device__ __forceinline__ void store_entries(PwT* out, int lane, const uint32_t (&e)[kR]);

template <>
__device__ __forceinline__ void store_entries<uint32_t, 4>(uint32_t* out, int lane, const uint32_t (&e)[4]) {
  *reinterpret_cast<uint4*>(out + 4 * lane) = make_uint4(e[0], e[1], e[2], e[3]);
}
template <>
__device__ __forceinline__ void store_entries<uint32_t, 8>(uint32_t* out, int lane, const uint32_t (&e)[8]) {
  *reinterpret_cast<uint4*>(out + 4 * lane) = make_uint4(e[0], e[1], e[2], e[3]);
  *reinterpret_cast<uint4*>(out + 128 + 4 * lane) = make_uint4(e[4], e[5], e[6], e[7]);
}
template <>
__device__ __forceinline__ void store_entries<uint8_t, 4>(uint8_t* out, int lane, const uint32_t (&e)[4]) {
  *reinterpret_cast<uint32_t*>(out + 4 * lane) = e[0] | e[1] << 8 | e[2] << 16 | e[3] << 24;
}
template <>
__device__ __forceinline__ void store_entries<uint8_t, 8>(uint8_t* out, int lane, const uint32_t (&e)[8]) {
  *reinterpret_cast<uint32_t*>(out + 4 * lane) = e[0] | e[1] << 8 | e[2] << 16 | e[3] << 24;
  *reinterpret_cast<uint32_t*>(out + 128 + 4 * lane) = e[4] | e[5] << 8 | e[6] << 16 | e[7] << 24;
}
template <>
__device__ __forceinline__ void store_entries<uint16_t, 4>(uint16_t* out, int lane, const uint32_t (&e)[4]) {
  *reinterpret_cast<uint2*>(out + 4 * lane) = make_uint2(e[0] | e[1] << 16, e[2] | e[3] << 16);
}
template <>
__device__ __forceinline__ void store_entries<uint16_t, 8>(uint16_t* out, int lane, const uint32_t (&e)[8]) {
  *reinterpret_cast<uint2*>(out + 4 * lane) = make_uint2(e[0] | e[1] << 16, e[2] | e[3] << 16);
  *reinterpret_cast<uint2*>(out + 128 + 4 * lane) = make_uint2(e[4] | e[5] << 16, e[6] | e[7] << 16);
}

// Row offset (within the warp's rows) of row j of lane `lane`.
template <int kR>
__device__ __forceinline__ int plan_row(int lane, int j) {
  return (j >> 2) * 128 + lane * 4 + (j & 3);
}

// One compiled filter step over the lane's kR rows: keeps the rows of `mask`
// that pass, and stores each probed row's table entry when the table has a
// payload.  A probe's loads go out only for rows still live; all kR of them
// are issued before any is used.
template <int kCode, int kR, typename PwT>
__device__ __forceinline__ void plan_step(const Step& st, const int32_t* wstage, const uint32_t* tables,
                                          const PlanList<kR, PwT>& L, int lane, uint32_t& mask) {
  using C = StepCode<kCode>;
  constexpr int kTR = kConsumerWarps * plan_warp_rows(kR);
  const int32_t* col = wstage + st.col * kTR;
  int32_t key[kR];
#pragma unroll
  for (int q = 0; q < kR / 4; q++) {
    const int4 v = reinterpret_cast<const int4*>(col + q * 128)[lane];
    key[4 * q + 0] = v.x;
    key[4 * q + 1] = v.y;
    key[4 * q + 2] = v.z;
    key[4 * q + 3] = v.w;
  }
  bool live[kR];
#pragma unroll
  for (int j = 0; j < kR; j++) live[j] = (mask >> j) & 1u;
  if (C::kind == SC_RANGE || C::ranged) {
    const uint32_t lo = (uint32_t)st.lo, span = (uint32_t)st.hi - (uint32_t)st.lo;
#pragma unroll
    for (int j = 0; j < kR; j++) live[j] = live[j] && (uint32_t)key[j] - lo <= span;
  }
  if (C::probe) {
    const uint32_t kmin = (uint32_t)st.key_min, span = st.span;
    uint32_t wi[kR], sh[kR], word[kR];
#pragma unroll
    for (int j = 0; j < kR; j++) {
      const uint32_t idx = (uint32_t)key[j] - kmin;
      live[j] = live[j] && idx < span;
      const uint32_t bit = idx << C::bits_log2;  // span << bits_log2 < 2^32 (planner)
      wi[j] = bit >> 5;
      sh[j] = bit & 31u;
    }
    if (C::kind == SC_SMEM) {
      const uint32_t* w = tables + st.smem_word_off;
#pragma unroll
      for (int j = 0; j < kR; j++) word[j] = live[j] ? w[wi[j]] : 0u;
    } else {
      const uint32_t* w = st.words;
#pragma unroll
      for (int j = 0; j < kR; j++) word[j] = live[j] ? __ldg(w + wi[j]) : 0u;
    }
    uint32_t e[kR];
#pragma unroll
    for (int j = 0; j < kR; j++) {
      e[j] = C::bits == 32 ? word[j] : (word[j] >> sh[j]) & ((1u << (C::bits & 31)) - 1u);
      live[j] = live[j] && (e[j] & 1u);
    }
    if (C::bits > 1) store_entries<PwT, kR>(L.pw(st.dim), lane, e);
  }
  mask = 0;
#pragma unroll
  for (int j = 0; j < kR; j++) mask |= (uint32_t)live[j] << j;
}

template <int kCode, int kR, typename PwT>
__device__ __forceinline__ void plan_step_if(const Step& st, const int32_t* wstage, const uint32_t* tables,
                                             const PlanList<kR, PwT>& L, int lane, uint32_t& mask) {
  if (kCode == SC_NONE) return;
  if (!__any_sync(0xffffffffu, mask)) return;
  plan_step<kCode, kR, PwT>(st, wstage, tables, L, lane, mask);
}

// The warp's live rows after the dense steps, as a list of row offsets in
// row order (L.row); returns their count.  Lane L's rows of a 128-row slice
// are 4L..4L+3, so a lane's place in the list is the live rows of the lanes
// before it: their counts (0..4) summed from three ballots of the count bits.
template <int kR, typename PwT>
__device__ __forceinline__ int plan_sorted_list(const PlanList<kR, PwT>& L, int lane, uint32_t lt, uint32_t mask) {
  int n = 0;
#pragma unroll
  for (int q = 0; q < kR / 4; q++) {
    const uint32_t m4 = (mask >> (4 * q)) & 15u;
    const uint32_t c = (uint32_t)__popc(m4);
    const uint32_t b0 = __ballot_sync(0xffffffffu, c & 1u), b1 = __ballot_sync(0xffffffffu, c & 2u),
                   b2 = __ballot_sync(0xffffffffu, c & 4u);
    int pos = n + __popc(b0 & lt) + 2 * __popc(b1 & lt) + 4 * __popc(b2 & lt);
#pragma unroll
    for (int jj = 0; jj < 4; jj++)
      if ((m4 >> jj) & 1u) L.row[pos++] = (uint16_t)(q * 128 + lane * 4 + jj);
    n += __popc(b0) + 2 * __popc(b1) + 4 * __popc(b2);
  }
  __syncwarp();
  return n;
}

// One compiled filter step over the warp's list of live rows (n of them):
// lane L takes entries L, L + 32, L + 64 and L + 96 of each 128, so four
// probe loads are in flight per lane; the survivors are compacted in place,
// in row order, and each keeps its table entry (by row offset) when the
// table has a payload.  Returns the survivors' count.
template <int kCode, int kR, typename PwT>
__device__ __forceinline__ int plan_list_step(const Step& st, const int32_t* wstage, const uint32_t* tables,
                                              const PlanList<kR, PwT>& L, int lane, uint32_t lt, int n) {
  using C = StepCode<kCode>;
  if (C::kind == SC_NONE || n == 0) return n;
  constexpr int kTR = kConsumerWarps * plan_warp_rows(kR);
  constexpr int kU = 4;
  const int32_t* col = wstage + st.col * kTR;
  int out = 0;
  for (int r0 = 0; r0 < n; r0 += 32 * kU) {
    int row[kU];
    bool live[kU];
    uint32_t key[kU], e[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int i = r0 + u * 32 + lane;
      live[u] = i < n;
      row[u] = live[u] ? (int)L.row[i] : 0;
      key[u] = (uint32_t)col[row[u]];
      e[u] = 0u;
    }
    if (C::kind == SC_RANGE || C::ranged) {
      const uint32_t lo = (uint32_t)st.lo, span = (uint32_t)st.hi - (uint32_t)st.lo;
#pragma unroll
      for (int u = 0; u < kU; u++) live[u] = live[u] && key[u] - lo <= span;
    }
    if (C::probe) {
      const uint32_t kmin = (uint32_t)st.key_min, span = st.span;
      uint32_t word[kU], sh[kU];
#pragma unroll
      for (int u = 0; u < kU; u++) {
        const uint32_t idx = key[u] - kmin;
        live[u] = live[u] && idx < span;
        const uint32_t bit = idx << C::bits_log2;
        sh[u] = bit & 31u;
        const uint32_t wi = bit >> 5;
        if (C::kind == SC_SMEM)
          word[u] = live[u] ? tables[st.smem_word_off + wi] : 0u;
        else
          word[u] = live[u] ? __ldg(st.words + wi) : 0u;
      }
#pragma unroll
      for (int u = 0; u < kU; u++) {
        e[u] = C::bits == 32 ? word[u] : (word[u] >> sh[u]) & ((1u << (C::bits & 31)) - 1u);
        live[u] = live[u] && (e[u] & 1u);
      }
    }
    __syncwarp();  // every entry of this round is read before any is overwritten
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const uint32_t b = __ballot_sync(0xffffffffu, live[u]);
      if (live[u]) {
        L.row[out + __popc(b & lt)] = (uint16_t)row[u];
        if (C::probe && C::bits > 1) L.pw(st.dim)[row[u]] = (PwT)e[u];
      }
      out += __popc(b);
    }
    __syncwarp();
  }
  return out;
}

// kC: the step after which the warp's live rows become a list (0..2: the
// later steps run over the list; 3: every step runs over all the warp's
// rows; 4: a list after step 0, then steps 1 and 2 over it in one pass).
// Two compiled filter steps over the warp's list in one pass: each entry's
// lookups for both steps are issued before either result is used (the
// second step's table is read for rows the first will drop), so the two
// probes cost one round trip to L2 instead of two.  Otherwise as
// plan_list_step.
template <int kA, int kB, int kR, typename PwT>
__device__ __forceinline__ int plan_list_step2(const Step& sa, const Step& sb, const int32_t* wstage,
                                               const uint32_t* tables, const PlanList<kR, PwT>& L, int lane,
                                               uint32_t lt, int n) {
  using A = StepCode<kA>;
  using Bc = StepCode<kB>;
  if (n == 0) return 0;
  constexpr int kTR = kConsumerWarps * plan_warp_rows(kR);
  constexpr int kU = 4;
  const int32_t* ca = wstage + sa.col * kTR;
  const int32_t* cb = wstage + sb.col * kTR;
  int out = 0;
  for (int r0 = 0; r0 < n; r0 += 32 * kU) {
    int row[kU];
    bool live[kU];
    uint32_t wa[kU], sha[kU], wb[kU], shb[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int i = r0 + u * 32 + lane;
      live[u] = i < n;
      row[u] = live[u] ? (int)L.row[i] : 0;
      const uint32_t ka = (uint32_t)ca[row[u]], kb = (uint32_t)cb[row[u]];
      bool la = live[u], lb = live[u];
      if (A::kind == SC_RANGE || A::ranged) la = la && ka - (uint32_t)sa.lo <= (uint32_t)sa.hi - (uint32_t)sa.lo;
      if (Bc::kind == SC_RANGE || Bc::ranged) lb = lb && kb - (uint32_t)sb.lo <= (uint32_t)sb.hi - (uint32_t)sb.lo;
      wa[u] = 0u;
      sha[u] = 0u;
      wb[u] = 0u;
      shb[u] = 0u;
      if (A::probe) {
        const uint32_t idx = ka - (uint32_t)sa.key_min;
        la = la && idx < sa.span;
        const uint32_t bit = idx << A::bits_log2;
        sha[u] = bit & 31u;
        if (A::kind == SC_SMEM)
          wa[u] = la ? tables[sa.smem_word_off + (bit >> 5)] : 0u;
        else
          wa[u] = la ? __ldg(sa.words + (bit >> 5)) : 0u;
      }
      if (Bc::probe) {
        const uint32_t idx = kb - (uint32_t)sb.key_min;
        lb = lb && idx < sb.span;
        const uint32_t bit = idx << Bc::bits_log2;
        shb[u] = bit & 31u;
        if (Bc::kind == SC_SMEM)
          wb[u] = lb ? tables[sb.smem_word_off + (bit >> 5)] : 0u;
        else
          wb[u] = lb ? __ldg(sb.words + (bit >> 5)) : 0u;
      }
      live[u] = la && lb;
    }
    uint32_t ea[kU], eb[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      ea[u] = A::bits == 32 ? wa[u] : (wa[u] >> sha[u]) & ((1u << (A::bits & 31)) - 1u);
      eb[u] = Bc::bits == 32 ? wb[u] : (wb[u] >> shb[u]) & ((1u << (Bc::bits & 31)) - 1u);
      if (A::probe) live[u] = live[u] && (ea[u] & 1u);
      if (Bc::probe) live[u] = live[u] && (eb[u] & 1u);
    }
    __syncwarp();  // every entry of this round is read before any is overwritten
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const uint32_t b = __ballot_sync(0xffffffffu, live[u]);
      if (live[u]) {
        L.row[out + __popc(b & lt)] = (uint16_t)row[u];
        if (A::probe && A::bits > 1) L.pw(sa.dim)[row[u]] = (PwT)ea[u];
        if (Bc::probe && Bc::bits > 1) L.pw(sb.dim)[row[u]] = (PwT)eb[u];
      }
      out += __popc(b);
    }
    __syncwarp();
  }
  return out;
}

// Copies a probe step's kept entry of `row` into the next buffered word when
// the step's entries carry a payload (the host puts those words first, in
// step order, so `k` is a compile-time index here).
template <int kCode, int kR, typename PwT>
__device__ __forceinline__ void append_entry(const Step& st, const PlanList<kR, PwT>& L, int row, uint32_t* ent,
                                             int& k) {
  using C = StepCode<kCode>;
  if (C::probe && C::bits > 1) ent[k++] = (uint32_t)L.pw(st.dim)[row];
}

template <int kAgg, int kR, int kMinB, int kC, int S0, int S1, int S2, int S3>
__global__ void __launch_bounds__(kStarThreads, kMinB) star_plan_kernel(const __grid_constant__ StarParams P) {
  using PwT = typename PlanEntryWord<S0, S1, S2, S3>::type;
  constexpr int kWR = plan_warp_rows(kR);
  constexpr int kTR = kConsumerWarps * kWR;
  extern __shared__ __align__(128) uint8_t dyn[];
  __shared__ StarSmem S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ncols = P.ncols, nst = P.nstages;
  int32_t* ring = reinterpret_cast<int32_t*>(dyn);
  const size_t lb = plan_list_bytes(P.ndims, kR, (int)sizeof(PwT));
  uint8_t* lists = dyn + (size_t)nst * ncols * kTR * 4;
  uint32_t* tables = reinterpret_cast<uint32_t*>(lists + kConsumerWarps * lb);
  unsigned long long* s_sum =
      reinterpret_cast<unsigned long long*>(tables + ((P.smem_table_words + 3) & ~3));
  const int nm = P.nmetrics;
  const unsigned long long G = P.ngroups;
  unsigned int* s_cnt = reinterpret_cast<unsigned int*>(s_sum + (kAgg == AGG_DENSE_SMEM ? nm * G : 0));
  uint32_t* aggbuf = reinterpret_cast<uint32_t*>(s_cnt + (kAgg == AGG_DENSE_SMEM ? G : 0));

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
  const long long ntiles = (P.row_end - a0 + kTR - 1) / kTR;
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
        const long long start = a0 + t * kTR;
        const long long stop = start + kTR < end4 ? start + kTR : end4;
        const uint32_t bytes = (uint32_t)((stop - start) * 4);
        mbar_arrive_expect_tx(&S.full[s], bytes * (uint32_t)ncols);
        for (int c = 0; c < ncols; c++)
          bulk_g2s(ring + ((size_t)s * ncols + c) * kTR, P.cols[c] + start, bytes, &S.full[s]);
      }
      // Every issued copy lands before the block exits.
      const long long first = issued > nst ? issued - nst : 0;
      for (long long q = first; q < issued; q++)
        mbar_wait_bounded(&S.full[q % nst], (uint32_t)((q / nst) & 1), polls);
    }
  } else {
    // ---------------- consumers
    PlanList<kR, PwT> L;
    L.pwb = reinterpret_cast<PwT*>(lists + (size_t)warp * lb);
    L.row = reinterpret_cast<uint16_t*>(lists + (size_t)warp * lb +
                                        (size_t)(P.ndims > 0 ? P.ndims : 1) * kWR * sizeof(PwT));
    const uint32_t lt = lanemask_lt();
    const int W = P.agg_words;
    uint32_t* buf = aggbuf + (size_t)warp * kAggCap * W;
    int cnt = 0;  // rows buffered
    RingPos rp;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, rp.next(nst)) {
      const int s = rp.s;
      if (!mbar_wait_bounded(&S.full[s], rp.phase, polls)) {
        raise_error(P.error, DERR_TIMEOUT);
        break;
      }
      const int32_t* wstage = ring + (size_t)s * ncols * kTR + warp * kWR;
      const long long base = a0 + t * kTR + warp * kWR;
      uint32_t mask;
      if (base >= P.row_begin && base + kWR <= P.row_end) {
        mask = (1u << kR) - 1u;
      } else {
        mask = 0;
#pragma unroll
        for (int j = 0; j < kR; j++) {
          const long long r = base + plan_row<kR>(lane, j);
          mask |= (uint32_t)(r >= P.row_begin && r < P.row_end) << j;
        }
      }
      int n = 0;
      plan_step_if<S0, kR, PwT>(P.steps[0], wstage, tables, L, lane, mask);
      if (kC == 0 || kC == 4) n = plan_sorted_list<kR, PwT>(L, lane, lt, mask);
      if (kC == 4) {
        n = plan_list_step2<S1, S2, kR, PwT>(P.steps[1], P.steps[2], wstage, tables, L, lane, lt, n);
        n = plan_list_step<S3, kR, PwT>(P.steps[3], wstage, tables, L, lane, lt, n);
      } else {
        if (kC < 1)
          n = plan_list_step<S1, kR, PwT>(P.steps[1], wstage, tables, L, lane, lt, n);
        else
          plan_step_if<S1, kR, PwT>(P.steps[1], wstage, tables, L, lane, mask);
        if (kC == 1) n = plan_sorted_list<kR, PwT>(L, lane, lt, mask);
        if (kC < 2)
          n = plan_list_step<S2, kR, PwT>(P.steps[2], wstage, tables, L, lane, lt, n);
        else
          plan_step_if<S2, kR, PwT>(P.steps[2], wstage, tables, L, lane, mask);
        if (kC == 2) n = plan_sorted_list<kR, PwT>(L, lane, lt, mask);
        if (kC < 3) {
          n = plan_list_step<S3, kR, PwT>(P.steps[3], wstage, tables, L, lane, lt, n);
        } else {
          plan_step_if<S3, kR, PwT>(P.steps[3], wstage, tables, L, lane, mask);
          // ---- the survivors as a list of row offsets
#pragma unroll
          for (int j = 0; j < kR; j++) {
            const uint32_t b = __ballot_sync(0xffffffffu, (mask >> j) & 1u);
            if ((mask >> j) & 1u) L.row[n + __popc(b & lt)] = (uint16_t)plan_row<kR>(lane, j);
            n += __popc(b);
          }
          __syncwarp();
        }
      }
      // ---- their operand words into the warp's buffer, aggregated 32 rows at a time
      for (int done = 0; done < n;) {
        const int take = n - done < kAggCap - cnt ? n - done : kAggCap - cnt;
        if (lane < take) {
          const int row = L.row[done + lane];
          uint32_t* ent = buf + (size_t)(cnt + lane) * W;
          int k = 0;
          append_entry<S0, kR, PwT>(P.steps[0], L, row, ent, k);
          append_entry<S1, kR, PwT>(P.steps[1], L, row, ent, k);
          append_entry<S2, kR, PwT>(P.steps[2], L, row, ent, k);
          append_entry<S3, kR, PwT>(P.steps[3], L, row, ent, k);
          for (; k < W; k++) {
            const int code = P.agg_src[k];
            ent[k] = code < 8               ? (uint32_t)L.pw(code)[row]
                     : code == kAggRowWord ? (uint32_t)(base + row)
                                           : (uint32_t)wstage[(code - 8) * kTR + row];
          }
        }
        cnt += take;
        done += take;
        if (cnt == kAggCap) {
          flush_entries<kAgg>(P, buf, cnt, lane, acc, s_sum, s_cnt);
          cnt = 0;
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&S.empty[s]);
    }
    if (cnt) flush_entries<kAgg>(P, buf, cnt, lane, acc, s_sum, s_cnt);
  }
  finish_block<kAgg>(P, S, acc, s_sum, s_cnt, tid, warp, lane);
}

// ---------------------------------------------------------------- registry
constexpr int R_ = SC_RANGE;
constexpr int smem(int bits_log2) { return SC_SMEM | bits_log2 << 2; }
constexpr int l2(int bits_log2) { return SC_L2 | bits_log2 << 2; }

struct PlanEntry {
  int agg, rows, minb, list_after, s[4];
  const void* fn;
};

}  // namespace plan
}  // namespace svm

#define SVM_PLAN(AGG, R, MB, A, B, C, D)                                             \
  {AGG, R, MB, 3, {A, B, C, D},                                                      \
   reinterpret_cast<const void*>(&::svm::plan::star_plan_kernel<AGG, R, MB, 3, A, B, C, D>)}
// A shape with 8 rows per lane for 2 blocks per SM whose live rows become a
// list after step KC.
#define SVM_PLAN_LIST(AGG, KC, A, B, C, D)                                          \
  {AGG, 8, 2, KC, {A, B, C, D},                                                      \
   reinterpret_cast<const void*>(&::svm::plan::star_plan_kernel<AGG, 8, 2, KC, A, B, C, D>)}
// Each shape with 4 rows per lane for 3 or 4 blocks per SM, and 8 rows per lane for 2.
#define SVM_PLAN_R(AGG, A, B, C, D) \
  SVM_PLAN(AGG, 4, 3, A, B, C, D), SVM_PLAN(AGG, 4, 4, A, B, C, D), SVM_PLAN(AGG, 8, 2, A, B, C, D)
// The same, and the form with 8 rows per lane whose steps after the first
// run over a list of the live rows.
#define SVM_PLAN_RL(AGG, A, B, C, D) SVM_PLAN_R(AGG, A, B, C, D), SVM_PLAN_LIST(AGG, 0, A, B, C, D)
