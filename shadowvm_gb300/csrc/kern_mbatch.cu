// Batched star queries with merged probe tables.
//
// One persistent block per SM scans the union of a batch's fact columns once
// (bulk-copy ring, dynamic tile hand-out).  Four fill warps run one tile
// ahead of the consumers: once a tile has landed they look every row up in
// each merged probe table the tile's queries need (ProbeGroup: the dense
// dimension tables probed through one fact column, concatenated per key) with
// asynchronous gathers into one of two merged-word buffers, whose completion
// an mbarrier tracks.  The consumer warps turn each needed table's present
// bits into a 1024-bit row bitmap (a 32 x 32 bit transpose per 32 rows), then
// take the tile's queries one at a time; every query's descriptor stays in
// shared memory for the whole launch.  A query's probe steps are one AND of a
// bitmap word per lane; its range steps test staged fact values, with ballots
// over every row while many rows live, else only the live rows; only its
// surviving rows reach the int64 group slots.  The lookups are thus shared by
// every query of the batch and overlap the previous tile's query work.
#include <climits>

#include "kern_common.cuh"
#include "kernels.h"

namespace svm {
namespace {

// The block is 32 warps: kCW consumer warps and 32 - kCW fill warps (the
// first fill warp also issues the bulk copies); the split is a template
// parameter the launch tuner chooses (28 + 4 or 24 + 8).
constexpr int kMBThreads = 1024;
constexpr uint32_t kPolls = 1u << 22;

template <int kCW>
__device__ __forceinline__ void consumer_bar() {
  asm volatile("bar.sync 1, %0;" ::"n"(kCW * 32) : "memory");
}

__device__ __forceinline__ uint32_t lane_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

constexpr int kChunks = kTileRows / 32;     // bitmap words per tile
// Merged words are stored by swizzled row position: row r at slot
// (r % 32) * 32 + ((r / 32) ^ (r % 32)) of a group's region.  The 32 rows a
// lane owns (lane L: rows L, L + 32, ..., L + 992) then sit in one 32-slot
// block, so one transpose of a block yields a lane's bitmap words directly,
// and both the fill (consecutive rows) and the transpose (one block) touch
// 32 distinct banks.
constexpr int kSlots = kTileRows;           // slots per group region (row-major words)
__device__ __forceinline__ int row_slot(int r) { return ((r & 31) << 5) | ((r >> 5) ^ (r & 31)); }
constexpr int kBmStride = kChunks + 1;      // a table's bitmap row, padded (conflict-free stores)
static_assert(sizeof(MQuery) == 240 && sizeof(MExtract) == 12, "descriptor layout");
constexpr int kDenseRows = 256;             // live rows above which a range test runs on every row
constexpr int kAggRing = 64;                // surviving-row ring per consumer warp (uint16 rows)

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// A value for the aggregation: a staged fact value, or a payload field of a
// merged probe word (optionally a row index into a gather column), plus
// `base`.  Word w of row r of a group sits at
// group_first_word * kSlots + row_slot(r) * words + w.
__device__ __forceinline__ uint32_t mx(const MExtract& x, const BatchParams& B, const int32_t* stage,
                                       const uint32_t* mw, int row) {
  if (x.src < 0) return (uint32_t)stage[x.slot * kTileRows + row] + (uint32_t)x.base;
  uint32_t v = (mw[x.src * kSlots + row_slot(row) * (x.sg & 15) + x.slot] >> x.shift) & x.mask;
  if (x.sg >> 4) v = (uint32_t)__ldg(B.gcol[(x.sg >> 4) - 1] + v);
  return v + (uint32_t)x.base;
}

// Asynchronous gather of 4, 8 or 16 bytes; with `valid` false it writes zeros
// and reads nothing.
// The merged tables are gathered with an L2 evict-last policy, the fact
// stream with evict-first, so the scan does not push the tables out of L2.
template <int kBytes>
__device__ __forceinline__ void cp_async_zfill(void* dst, const void* src, bool valid, uint64_t policy) {
  if (kBytes == 16)
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2, %3;" ::"r"(smem_u32(dst)), "l"(src),
                 "r"(valid ? 16 : 0), "l"(policy)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], %2, %3, %4;" ::"r"(smem_u32(dst)), "l"(src),
                 "n"(kBytes), "r"(valid ? kBytes : 0), "l"(policy)
                 : "memory");
}

__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ void bulk_g2s_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                              uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

// Starts the lookup of one row in a merged table: the entry's words are
// copied to the row's slot of the group's region (zeros when the key is
// outside the table).  Entries of 4 or 8 words go in 16-byte pieces, other
// even widths in 8-byte pieces, odd widths word by word.
__device__ __forceinline__ void fill_issue(const ProbeGroup& G, const int32_t* stage, uint32_t* mwb, int row,
                                           uint64_t pol) {
  const uint32_t off = (uint32_t)stage[G.col * kTileRows + row] - (uint32_t)G.key_min;
  const bool in = off < G.span;
  const int W = G.words;
  const uint32_t* src = G.table + (size_t)(in ? off : 0u) * W;
  uint32_t* dst = mwb + G.word_off * kSlots + row_slot(row) * W;
  if ((W & 3) == 0) {
    for (int h = 0; h < W; h += 4) cp_async_zfill<16>(dst + h, src + h, in, pol);
  } else if ((W & 1) == 0) {
    for (int h = 0; h < W; h += 2) cp_async_zfill<8>(dst + h, src + h, in, pol);
  } else {
    for (int h = 0; h < W; h++) cp_async_zfill<4>(dst + h, src + h, in, pol);
  }
}

// Each lane's completed gathers count one arrival on `bar`.
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// 32 x 32 bit transpose across a warp: lane i holds row i on entry (bit j =
// element (i, j)) and column i on return (bit j = element (j, i)).  Five
// exchange steps, each swapping the off-diagonal blocks of half the size.
__device__ __forceinline__ uint32_t transpose32(uint32_t x, int lane) {
  const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int k = 0; k < 5; k++) {
    const int s = 16 >> k;
    const uint32_t m = masks[k];
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, s);
    x = (lane & s) ? ((x & ~m) | ((y & ~m) >> s)) : ((x & m) | ((y & m) << s));
  }
  return x;
}

// One query over one staged tile (local rows [lo, hi)).  Lane L owns rows
// L + 32 i (i = 0..31) as bit i of one mask word, so every per-row shared
// memory read of a lane hits its own bank.
__device__ __forceinline__ void mquery_tile(const MQuery& Q, const BatchParams& B, const int32_t* stage,
                                            const uint32_t* mw, const uint32_t* bm, int lo, int hi, int lane,
                                            uint32_t lt, uint16_t* ring) {
  // bits i with lo <= L + 32 i < hi
  const int ia = lo > lane ? (lo - lane + 31) >> 5 : 0;
  const int ib = hi > lane ? ((hi - 1 - lane) >> 5) + 1 : 0;  // exclusive
  uint32_t m = ia >= ib ? 0u : (ib - ia == 32 ? 0xFFFFFFFFu : ((1u << (ib - ia)) - 1u) << ia);
  const int np = Q.nprobe, nr = Q.nrange;
  for (int p = 0; p < np; p++) m &= bm[Q.probe_tab[p] * kBmStride + lane];
  for (int r = 0; r < nr; r++) {
    const int live = __reduce_add_sync(0xffffffffu, __popc(m));
    if (!live) return;
    const int32_t* cv = stage + Q.range_col[r] * kTileRows;
    const uint32_t rlo = (uint32_t)Q.range_lo[r];
    const uint32_t span = (uint32_t)Q.range_hi[r] - rlo;
    if (live > kDenseRows) {
      uint32_t keep = 0;
#pragma unroll 8
      for (int i = 0; i < kChunks; i++) keep |= (uint32_t)((uint32_t)cv[32 * i + lane] - rlo <= span) << i;
      m &= keep;
    } else {
      for (uint32_t bb = m; bb; bb &= bb - 1) {
        const int j = __ffs(bb) - 1;
        if ((uint32_t)cv[32 * j + lane] - rlo > span) m &= ~(1u << j);
      }
    }
  }
  if (!__any_sync(0xffffffffu, m)) return;
  const int nkeys = Q.nkeys, nm = Q.nmetrics;
  unsigned long long* sums = B.slots + Q.slot_off;
  const unsigned long long G = Q.ngroups;
  // The keys' operands, read once per query and tile (the metrics' stay in
  // the shared-memory descriptor).
  MExtract kx[kMaxKeys];
  uint32_t kr[kMaxKeys], ks[kMaxKeys];
#pragma unroll
  for (int q = 0; q < kMaxKeys; q++) {
    kx[q] = Q.kx[q];
    kr[q] = Q.krange[q];
    ks[q] = Q.kstride[q];
  }
  const MExtract* xa = Q.xa;
  const MExtract* xb = Q.xb;
  const uint8_t* mf = Q.mform;
  long long acc[kMaxMetrics] = {0, 0, 0};
  auto aggregate = [&](int row) {
    uint32_t gi = 0;
    bool in_range = true;
#pragma unroll
    for (int q = 0; q < kMaxKeys; q++) {
      if (q < nkeys) {
        const uint32_t off = mx(kx[q], B, stage, mw, row);
        in_range &= off < kr[q];
        gi += off * ks[q];
      }
    }
    if (!in_range) {
      raise_error(B.error, DERR_KEY_RANGE);
      return;
    }
#pragma unroll
    for (int mi = 0; mi < kMaxMetrics; mi++) {
      if (mi < nm) {
        const uint32_t va = mx(xa[mi], B, stage, mw, row);
        uint32_t v = va;
        const int f = mf[mi];
        if (f != MF_OPND) {
          const uint32_t vb = mx(xb[mi], B, stage, mw, row);
          v = f == MF_ADD ? va + vb : f == MF_SUB ? va - vb : va * vb;
        }
        if (nkeys == 0)
          acc[mi] += (long long)(int32_t)v;
        else
          atomicAdd(sums + (size_t)mi * G + gi, (unsigned long long)(long long)(int32_t)v);
      }
    }
    if (nkeys) sums[(size_t)nm * G + gi] = 1ull;  // the group has a row
  };
  // The warp's surviving rows, balanced over its lanes: a lane walking only
  // its own rows would hold the warp for as many steps as its busiest lane.
  // Each step appends every lane's next row (one per lane, consecutive
  // entries from distinct lanes) to the warp's 64-entry ring; every 32
  // entries, and once at the end, the lanes take one entry each.
  uint32_t bb = m, wp = 0, rp = 0;  // ring write / read positions (warp-uniform)
  for (;;) {
    const uint32_t has = __ballot_sync(0xffffffffu, bb != 0u);
    if (bb) {
      const int j = __ffs(bb) - 1;
      bb &= bb - 1;
      ring[(wp + __popc(has & lt)) & (kAggRing - 1)] = (uint16_t)(32 * j + lane);
    }
    wp += __popc(has);
    if (wp - rp >= 32u || (has == 0u && wp != rp)) {
      __syncwarp();
      const uint32_t n = wp - rp < 32u ? wp - rp : 32u;
      if ((uint32_t)lane < n) aggregate(ring[(rp + lane) & (kAggRing - 1)]);
      rp += n;
      __syncwarp();  // read before the next steps overwrite the slots
    }
    if (has == 0u) break;
  }
  if (nkeys == 0) {
#pragma unroll
    for (int mi = 0; mi < kMaxMetrics; mi++) {
      if (mi < nm) {
        long long sacc = acc[mi];
        for (int o = 16; o; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
        if (lane == 0 && sacc) atomicAdd(sums + mi, (unsigned long long)sacc);
      }
    }
  }
}

// The queries active on the tile starting at `tile_start` and the probe
// groups they need (every lane of the calling warp gets `need`; with `list`
// the active query indices are written to act[0, na)).
__device__ __forceinline__ uint32_t tile_queries(const long long* qlo, const long long* qhi, const uint32_t* qg,
                                                 int nq, long long tile_start, uint16_t* act, bool list, int lane,
                                                 uint32_t lt, int* na_out) {
  const long long tile_end = tile_start + kTileRows;
  uint32_t need = 0;
  int na = 0;
  for (int base = 0; base < nq; base += 32) {
    const int q = base + lane;
    const bool a = q < nq && qlo[q] < tile_end && qhi[q] > tile_start;
    if (a) need |= qg[q];
    const uint32_t bq = __ballot_sync(0xffffffffu, a);
    if (list && a) act[na + __popc(bq & lt)] = (uint16_t)q;
    na += __popc(bq);
  }
  *na_out = na;
  return __reduce_or_sync(0xffffffffu, need);
}

template <int kCW>
__global__ void __launch_bounds__(kMBThreads, 1) mbatch_kernel(const __grid_constant__ BatchParams B) {
  constexpr int kMBatchWarps = kCW;              // consumer warps
  constexpr int kFillWarps = 32 - kCW;           // fill warps (the first also issues the bulk copies)
  constexpr int kFillRows = kTileRows / kFillWarps;
  static_assert(kTileRows % kFillWarps == 0, "fill warps split a tile evenly");
  extern __shared__ __align__(128) uint8_t dyn[];
  __shared__ uint64_t full[kStages], empty[kStages];
  __shared__ uint64_t fill_full[2], fill_empty[2];
  __shared__ long long stage_tile[kStages];
  __shared__ long long s_tile;
  __shared__ int s_next, s_na;
  __shared__ uint32_t s_need;
  __shared__ int s_list_na[2];          // per lookup buffer: the fill's list of the tile's queries
  __shared__ uint32_t s_list_need[2];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ncols = B.ncols, nst = B.nstages, nq = B.nqueries;
  const size_t mw_words = (size_t)B.nmwords * kSlots;
  int32_t* ring = reinterpret_cast<int32_t*>(dyn);
  uint32_t* mwbuf = reinterpret_cast<uint32_t*>(dyn + (size_t)nst * ncols * kTileRows * 4);  // two buffers
  uint32_t* bm = mwbuf + 2 * mw_words;
  MQuery* sq = reinterpret_cast<MQuery*>(bm + kMaxMergedTables * kBmStride);  // every query's descriptor
  long long* qlo = reinterpret_cast<long long*>(sq + nq);
  long long* qhi = qlo + nq;
  uint32_t* qg = reinterpret_cast<uint32_t*>(qhi + nq);
  uint16_t* act = reinterpret_cast<uint16_t*>(qg + nq);  // two lists of nq, one per lookup buffer
  uint16_t* aggring = act + 2 * nq;                       // kAggRing per consumer warp
  if (tid == 0) {
    for (int s = 0; s < nst; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&fill_full[b], 32 * kFillWarps + 1);  // each fill lane's gathers + the list
      mbar_init(&fill_empty[b], 1);
    }
    mbar_fence_init();
  }
  for (int i = tid; i < nq * (int)(sizeof(MQuery) / 16); i += kMBThreads)
    reinterpret_cast<uint4*>(sq)[i] = reinterpret_cast<const uint4*>(B.mq)[i];
  for (int q = tid; q < nq; q += kMBThreads) {
    qlo[q] = B.mq[q].row_begin;
    qhi[q] = B.mq[q].row_end;
    qg[q] = B.mq[q].gmask;
  }
  __syncthreads();
  const long long a0 = B.row_begin & ~3ll;
  const long long end4 = (B.row_end + 3) & ~3ll;
  const long long ntiles = (B.row_end - a0 + kTileRows - 1) / kTileRows;
  const uint32_t lt = lane_lt();

  if (warp >= kMBatchWarps) {
    // Fill warps.  Lane 0 of the first claims tiles and issues their bulk
    // copies; each fill warp issues the lookups of its quarter of a tile's
    // rows once the tile has landed.
    const int fw = warp - kMBatchWarps;
    const bool tma = fw == 0;
    const uint64_t pol_tab = policy_evict_last(), pol_fact = policy_evict_first();
    long long last_real = -1, last_seen = -1;  // lane 0: last tile copied / last tile waited for
    RingPos ip;                                 // lane 0: the ring position of the next issue
    auto issue_tile = [&](long long i) -> bool {  // lane 0 only, i = 0, 1, 2, ...; false on a timeout
      const int s = ip.s;
      const uint32_t ph = ip.phase;
      ip.next(nst);
      if (i >= nst && !mbar_wait_bounded(&empty[s], ph ^ 1u, kPolls)) return false;
      const long long t = (long long)atomicAdd(B.tile_counter, 1ull);
      if (t >= ntiles) {
        stage_tile[s] = -1;  // end of the scan
        mbar_arrive(&full[s]);
        return true;
      }
      stage_tile[s] = t;
      const long long start = a0 + t * kTileRows;
      const long long stop = start + kTileRows < end4 ? start + kTileRows : end4;
      const uint32_t bytes = (uint32_t)((stop - start) * 4);
      mbar_arrive_expect_tx(&full[s], bytes * (uint32_t)ncols);
      for (int c = 0; c < ncols; c++)
        bulk_g2s_hint(ring + ((size_t)s * ncols + c) * kTileRows, B.cols[c] + start, bytes, &full[s], pol_fact);
      last_real = i;
      return true;
    };
    int ok = 1;
    if (tma && lane == 0) ok = issue_tile(0);
    ok = __shfl_sync(0xffffffffu, ok, 0);
    RingPos rp;
    for (long long i = 0; ok; i++, rp.next(nst)) {
      const int s = rp.s, b = (int)(i & 1);
      bool good = mbar_wait_bounded(&full[s], rp.phase, kPolls);
      if (good && i >= 2) good = mbar_wait_bounded(&fill_empty[b], (uint32_t)((i / 2 - 1) & 1), kPolls);
      if (!__all_sync(0xffffffffu, good)) {
        if (lane == 0) raise_error(B.error, DERR_TIMEOUT);
        break;
      }
      last_seen = i;
      const long long t = stage_tile[s];
      if (t < 0) {
        if (tma && lane == 0) mbar_arrive(&fill_full[b]);  // the list's arrival
        mbar_arrive(&fill_full[b]);  // every fill lane: lets the consumers reach the end marker
        break;
      }
      // Fill warp 0 lists the tile's queries for the consumers (one tile
      // ahead of them), so no consumer warp holds the others while it lists.
      int na;
      const uint32_t need =
          tile_queries(qlo, qhi, qg, nq, a0 + t * kTileRows, act + (size_t)b * nq, tma, lane, lt, &na);
      if (tma) {
        if (lane == 0) {
          s_list_na[b] = na;
          s_list_need[b] = need;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&fill_full[b]);  // the list
      }
      const int32_t* stage = ring + (size_t)s * ncols * kTileRows;
      uint32_t* mwb = mwbuf + (size_t)b * mw_words;
      // The next tile's copies.  With three or more stages its slot held
      // tile i - 2 (or nothing yet), which the consumers released together
      // with the lookup buffer waited for above, so the copies go out before
      // this tile's lookups and overlap them; with two stages the slot is
      // the consumers' current tile, and the copies follow the lookups.
      const bool early = nst >= 3;
      auto next_tile = [&]() {
        if (lane == 0) ok = issue_tile(i + 1);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok && lane == 0) raise_error(B.error, DERR_TIMEOUT);
      };
      if (tma && early) next_tile();
      for (uint32_t mm = need; mm; mm &= mm - 1) {
        // A register copy: the gathers' asm clobbers memory, which would
        // otherwise reload the group's fields for every row.
        const ProbeGroup G = B.probe[__ffs(mm) - 1];
        for (int row = fw * kFillRows + lane; row < (fw + 1) * kFillRows; row += 32)
          fill_issue(G, stage, mwb, row, pol_tab);
      }
      cp_async_arrive(&fill_full[b]);
      if (tma && !early) next_tile();
    }
    // Every copy issued lands before the block may exit (a tile issued but
    // never waited for exists only after a timeout).
    if (tma && lane == 0 && last_real > last_seen)
      mbar_wait_bounded(&full[last_real % nst], (uint32_t)((last_real / nst) & 1), kPolls);
    cp_async_wait_all();
    return;
  }

  RingPos rp;
  for (long long i = 0;; i++, rp.next(nst)) {
    const int s = rp.s, b = (int)(i & 1);
    const uint32_t sp = rp.phase, bp = (uint32_t)((i / 2) & 1);
    // Warp 0 waits for the tile and hands its query list (written by the
    // fill warps) to the other warps.
    if (warp == 0 && lane == 0) {
      const bool good = mbar_wait_bounded(&fill_full[b], bp, kPolls) && mbar_wait_bounded(&full[s], sp, kPolls);
      const long long t0 = good ? stage_tile[s] : -2;
      s_next = 0;
      s_tile = t0;
      s_na = t0 >= 0 ? s_list_na[b] : 0;
      s_need = t0 >= 0 ? s_list_need[b] : 0u;
    }
    consumer_bar<kCW>();
    const long long t = s_tile;
    if (t < 0) {
      if (t == -2 && tid == 0) raise_error(B.error, DERR_TIMEOUT);
      break;
    }
    if (tid != 0) {  // both phases are complete: these acquire the copies at once
      mbar_wait_bounded(&full[s], sp, kPolls);
      mbar_wait_bounded(&fill_full[b], bp, kPolls);
    }
    const int32_t* stage = ring + (size_t)s * ncols * kTileRows;
    const uint32_t* mw = mwbuf + (size_t)b * mw_words;
    const long long tile_start = a0 + t * kTileRows, tile_end = tile_start + kTileRows;
    const int na = s_na;
    const uint32_t need = s_need;
    // Each needed table's present bits as a row bitmap: word 0 of each row's
    // entry, transposed per 32 rows.
    const int ng = __popc(need);
    for (int it = warp; it < ng * kChunks; it += kMBatchWarps) {
      const int gsel = it / kChunks, chunk = it % kChunks;
      uint32_t mm = need;
      for (int z = 0; z < gsel; z++) mm &= mm - 1;
      const int g = __ffs(mm) - 1;
      const ProbeGroup& G = B.probe[g];
      // column `chunk` = the rows chunk + 32 i a lane owns: lane i reads row
      // chunk + 32 i; after the transpose lane t holds table t's word.
      const uint32_t present = transpose32(mw[G.word_off * kSlots + row_slot(chunk + 32 * lane) * G.words], lane);
      const int t0 = B.gtab0[g];
      if (lane < B.gtab0[g + 1] - t0) bm[(t0 + lane) * kBmStride + chunk] = present;
    }
    consumer_bar<kCW>();
    // Queries, claimed one at a time.
    for (;;) {
      int k = 0;
      if (lane == 0) k = atomicAdd(&s_next, 1);
      k = __shfl_sync(0xffffffffu, k, 0);
      if (k >= na) break;
      const int q = act[(size_t)b * nq + k];
      const long long lo = qlo[q] > tile_start ? qlo[q] - tile_start : 0;
      const long long hi = qhi[q] < tile_end ? qhi[q] - tile_start : kTileRows;
      mquery_tile(sq[q], B, stage, mw, bm, (int)lo, (int)hi, lane, lt, aggring + warp * kAggRing);
    }
    consumer_bar<kCW>();
    if (tid == 0) {
      mbar_arrive(&empty[s]);
      mbar_arrive(&fill_empty[b]);
    }
  }
}

__global__ void merge_build_kernel(const __grid_constant__ MergeBuild M, uint32_t* out) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < M.span;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t w[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
    bool have = false;  // the shared field holds a present source's value
    uint32_t sv = 0u, bad = 0u;
    for (int i = 0; i < M.nsrc; i++) {
      const MergeSrc& S = M.src[i];
      const long long idx = (long long)M.key_min + (long long)k - (long long)S.key_min;
      if (idx < 0 || idx >= (long long)S.span) continue;
      const unsigned long long bit = (unsigned long long)idx * (unsigned)S.entry_bits;
      uint32_t e = S.words[bit >> 5] >> (bit & 31);
      if (S.entry_bits < 32) e &= (1u << S.entry_bits) - 1u;
      w[0] |= (e & 1u) << S.present_bit;
      uint32_t pay = S.pay_bits >= 32 ? e >> 1 : (e >> 1) & ((1u << S.pay_bits) - 1u);
      if (S.shared) {
        // Only a present key's value counts; every present source must agree.
        if (!(e & 1u)) continue;
        pay += (uint32_t)S.val_off;
        if (have) {
          if (pay != sv) bad |= 1u << i;
          continue;
        }
        have = true;
        sv = pay;
      }
#pragma unroll
      for (int z = 0; z < 8; z++)
        if (z == S.pay_word && S.pay_bits > 0) w[z] |= pay << S.pay_bit;
    }
    for (int z = 0; z < M.words; z++) out[k * M.words + z] = w[z];
    if (bad) atomicOr(M.conflict, bad);
  }
}

}  // namespace

cudaError_t launch_merge_build(const MergeBuild& m, uint32_t* out, cudaStream_t s) {
  if (m.span == 0) return cudaSuccess;
  unsigned long long blocks = (m.span + 255) / 256;
  const unsigned long long cap = (unsigned long long)num_sms() * 8;
  note_launch();
  merge_build_kernel<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(m, out);
  return cudaGetLastError();
}

namespace {
int cwarps_of(const BatchParams& b) { return b.cwarps == 24 ? 24 : 28; }
const void* mbatch_fn(const BatchParams& b) {
  return cwarps_of(b) == 24 ? reinterpret_cast<const void*>(&mbatch_kernel<24>)
                            : reinterpret_cast<const void*>(&mbatch_kernel<28>);
}
}  // namespace

size_t mbatch_smem_bytes(const BatchParams& b) {
  return (size_t)b.nstages * b.ncols * kTileRows * 4 + 2 * (size_t)b.nmwords * kSlots * 4 +
         (size_t)kMaxMergedTables * kBmStride * 4 + (size_t)b.nqueries * (sizeof(MQuery) + 8 + 8 + 4 + 4) +
         (size_t)cwarps_of(b) * kAggRing * 2 + 16;
}

int mbatch_grid_size(const BatchParams& b, size_t smem) {
  const void* fn = mbatch_fn(b);
  allow_dynamic_smem(fn, 226 * 1024);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kMBThreads, smem);
  return num_sms() * per_sm;
}

void mbatch_attributes(int* regs, int* max_threads, size_t* static_smem) {
  cudaFuncAttributes a{};
  cudaFuncGetAttributes(&a, reinterpret_cast<const void*>(&mbatch_kernel<28>));
  *regs = a.numRegs;
  *max_threads = a.maxThreadsPerBlock;
  *static_smem = a.sharedSizeBytes;
}

cudaError_t launch_mbatch(const BatchParams& b, int grid, size_t smem, cudaStream_t s) {
  note_launch();
  void* args[] = {const_cast<BatchParams*>(&b)};
  return cudaLaunchKernel(mbatch_fn(b), dim3(grid), dim3(kMBThreads), args, smem, s);
}

}  // namespace svm
