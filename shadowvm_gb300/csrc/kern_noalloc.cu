// svm_scan_aggregate_noalloc: the fused scan (kern_star.cu) over caller-owned
// device columns with all of its scratch in one file-scope device array, for
// callers that cannot allocate device memory on their query path.  Nothing
// here calls cudaMalloc, cudaFree or an allocating library routine.
#include <climits>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "ctx.h"
#include "kernels.h"

namespace svm {
namespace {

// The scratch: every GPU that loads the library holds it until exit.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[SVM_NOALLOC_SCRATCH_WORDS];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned long long* g_scratch_addr[kMaxDevices] = {};

// The array's device address on device `dev`.  In host code
// `g_noalloc_scratch` names a host-side stand-in, not device memory, so the
// address is looked up once per device, with that device current.
// svm_init does it for its context's device; a later call only reads it.
svm_status scratch_address(Ctx* x, int dev, unsigned long long** out) {
  if (dev < 0 || dev >= kMaxDevices) return x->fail(SVM_E_INVALID_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_addr[dev]) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (!e && cur != dev) e = cudaSetDevice(dev);
    void* p = nullptr;
    if (!e) e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return x->cuda_fail(e ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
    g_scratch_addr[dev] = static_cast<unsigned long long*>(p);
  }
  *out = g_scratch_addr[dev];
  return SVM_OK;
}

}  // namespace

// Called by svm_init with the context's device current: looks the static
// scratch up once per device, so that no query-path call loads the module
// (which, under lazy module loading, is when the driver places the array).
svm_status noalloc_prepare(Ctx* x) {
  unsigned long long* p;
  return scratch_address(x, x->device, &p);
}

}  // namespace svm

using namespace svm;

extern "C" svm_status svm_scan_aggregate_noalloc(svm_ctx* c, const svm_noalloc_scan* q, int32_t* const* key_out,
                                                 long long* const* sum_out, unsigned long long max_rows,
                                                 unsigned long long* nrows_out) {
  if (!c || !q || !nrows_out) return SVM_E_INVALID_ARG;
  Ctx* x = &c->impl;
  std::lock_guard<std::recursive_mutex> guard(x->mu);
  cudaSetDevice(x->device);
  x->err.clear();
  *nrows_out = 0;
  const int nkeys = q->nkeys, nm = q->nmetrics;
  if (q->ncols < 1 || !q->cols) return x->fail(SVM_E_INVALID_ARG, "noalloc scan: no columns");
  if (nkeys < 0 || nkeys > kMaxKeys) return x->fail(SVM_E_INVALID_ARG, "noalloc scan: 0..3 keys");
  if (nm < 1 || nm > kMaxMetrics) return x->fail(SVM_E_INVALID_ARG, "noalloc scan: 1..3 metrics");
  if (q->nranges < 0 || q->nranges > kMaxSteps) return x->fail(SVM_E_INVALID_ARG, "noalloc scan: 0..8 ranges");
  if (!sum_out || (nkeys && !key_out)) return x->fail(SVM_E_INVALID_ARG, "noalloc scan: missing outputs");

  StarParams P{};
  std::vector<int> slot_col;  // StarParams::cols slot -> caller column
  auto slot_of = [&](int col, int* slot) -> bool {
    if (col < 0 || col >= q->ncols || !q->cols[col]) return false;
    if (reinterpret_cast<uintptr_t>(q->cols[col]) & 15) return false;
    for (size_t i = 0; i < slot_col.size(); i++)
      if (slot_col[i] == col) {
        *slot = (int)i;
        return true;
      }
    if (slot_col.size() == (size_t)kMaxSteps) return false;
    slot_col.push_back(col);
    *slot = (int)slot_col.size() - 1;
    return true;
  };
  const char* bad_col = "noalloc scan: a column index is out of range, its pointer is null or not "
                        "16-byte aligned, or more than 8 distinct columns are used";
  P.nsteps = q->nranges;
  for (int i = 0; i < q->nranges; i++) {
    Step& st = P.steps[i];
    st.kind = STEP_RANGE;
    if (!slot_of(q->range_col[i], &st.col)) return x->fail(SVM_E_INVALID_ARG, bad_col);
    st.lo = q->range_lo[i];
    st.hi = q->range_hi[i];
  }
  unsigned long long G = 1;
  for (int k = 0; k < nkeys; k++) {
    int s;
    if (!slot_of(q->key_col[k], &s)) return x->fail(SVM_E_INVALID_ARG, bad_col);
    if (q->key_max[k] < q->key_min[k]) return x->fail(SVM_E_INVALID_ARG, "noalloc scan: key_max < key_min");
    P.keys[k] = Operand{(int8_t)s, -1};
    P.kmin[k] = q->key_min[k];
    unsigned long long r = (unsigned long long)((long long)q->key_max[k] - q->key_min[k] + 1);
    if (r > (1ull << 26) || G * r > (1ull << 26)) return x->fail(SVM_E_INVALID_ARG, "noalloc scan: too many groups");
    P.krange[k] = (uint32_t)r;
    G *= r;
  }
  unsigned long long stride = 1;
  for (int k = nkeys - 1; k >= 0; k--) {
    P.kstride[k] = stride;
    stride *= P.krange[k];
  }
  P.nkeys = nkeys;
  P.ngroups = G;
  P.nmetrics = nm;
  for (int m = 0; m < nm; m++) {
    Metric& M = P.metrics[m];
    int op = q->metric_op[m], s;
    if (op < SVM_METRIC_COL || op > SVM_METRIC_MUL) return x->fail(SVM_E_INVALID_ARG, "noalloc scan: bad metric op");
    M.form = op == SVM_METRIC_COL ? MF_OPND : op == SVM_METRIC_ADD ? MF_ADD : op == SVM_METRIC_SUB ? MF_SUB : MF_MUL;
    if (!slot_of(q->metric_a[m], &s)) return x->fail(SVM_E_INVALID_ARG, bad_col);
    M.a = Operand{(int8_t)s, -1};
    if (op != SVM_METRIC_COL) {
      if (!slot_of(q->metric_b[m], &s)) return x->fail(SVM_E_INVALID_ARG, bad_col);
      M.b = Operand{(int8_t)s, -1};
    }
  }
  // Scratch words: error word, sums, counts, then (with keys) compaction flags,
  // positions and the scan's tile totals.
  const size_t fin_words = nkeys ? (G + 1) / 2 + 1 + G + 1 : 0;
  const size_t scan_words = nkeys ? scan_tmp_words(G) : 0;
  const size_t need = 1 + (size_t)nm * G + G + fin_words + scan_words;
  if (need > SVM_NOALLOC_SCRATCH_WORDS)
    return x->fail(SVM_E_INVALID_ARG, "noalloc scan: " + std::to_string(G) + " groups x " + std::to_string(nm) +
                                          " metrics need " + std::to_string(need) + " scratch words; the static "
                                          "scratch holds " + std::to_string(SVM_NOALLOC_SCRATCH_WORDS));
  if (nkeys == 0 && q->nrows > 0 && max_rows < 1)
    return x->fail(SVM_E_INVALID_ARG, "noalloc scan: max_rows is 0 but a query without keys writes one row");
  unsigned long long* scratch;
  svm_status st = scratch_address(x, x->device, &scratch);
  if (st) return st;
  if (q->nrows == 0) return SVM_OK;  // no rows: no bulk, no result row

  P.ncols = (int)slot_col.size();
  for (size_t i = 0; i < slot_col.size(); i++) P.cols[i] = q->cols[slot_col[i]];
  // A contradictory range (lo > hi) passes no row: scan nothing.
  bool empty = false;
  for (int i = 0; i < q->nranges; i++) empty |= q->range_lo[i] > q->range_hi[i];
  P.row_begin = 0;
  P.row_end = empty ? 0 : (long long)q->nrows;
  P.error = reinterpret_cast<int*>(scratch);
  P.sums = scratch + 1;
  P.counts = P.sums + (size_t)nm * G;
  unsigned long long* fin = P.counts + G;
  unsigned long long* scant = fin + fin_words;
  P.agg = nkeys == 0 ? AGG_SCALAR
                     : G * (8ull * nm + 4) <= (unsigned long long)kSmemAggBytes ? AGG_DENSE_SMEM : AGG_DENSE_GLOBAL;
  flatten_plan(P);
  int best_blocks = 0, best_st = 0;
  for (int nst = kStages; nst >= 2; nst--) {
    P.nstages = nst;
    size_t sm = star_smem_bytes(P);
    int blocks = sm <= 200 * 1024 ? star_blocks_per_sm(P, sm) : 0;
    if (blocks > best_blocks) {
      best_blocks = blocks;
      best_st = nst;
    }
  }
  if (best_blocks == 0) return x->fail(SVM_E_UNSUPPORTED, "noalloc scan: shared-memory plan too large");
  P.nstages = best_st;
  const size_t smem = star_smem_bytes(P);

  // The array keeps the previous call's contents: clear the error word and the slots.
  cudaError_t e = cudaMemsetAsync(scratch, 0, (1 + (size_t)(nm + 1) * G) * 8, x->stream);
  if (!e) e = launch_star(P, star_grid_size(P, smem), star_block_size(), smem, x->stream);
  if (e) return x->cuda_fail(e, "noalloc scan");
  unsigned long long rows = 0;
  // The kernel's error word is read before the result is used: a key outside
  // its range or a wait that gave up is reported as such, not as a row count.
  auto device_error = [&](int h) {
    const char* m;
    const svm_status s = device_error_status(h, &m);
    return x->fail(s, std::string("noalloc scan: ") +
                          (h == DERR_KEY_RANGE ? "a key value lies outside [key_min, key_max]" : m));
  };
  int h = 0;
  if (nkeys == 0) {
    for (int m = 0; m < nm && !e; m++)
      e = cudaMemcpyAsync(sum_out[m], P.sums + m, 8, cudaMemcpyDeviceToDevice, x->stream);
    rows = 1;
  } else {
    e = launch_finalize_dense(P, nullptr, nullptr, nullptr, fin, scant, nullptr, x->stream);
    unsigned long long* pos = fin + (G + 1) / 2 + 1;
    if (!e) e = cudaMemcpyAsync(&rows, pos + G, 8, cudaMemcpyDeviceToHost, x->stream);
    if (!e) e = cudaMemcpyAsync(&h, P.error, sizeof(int), cudaMemcpyDeviceToHost, x->stream);
    if (!e) e = cudaStreamSynchronize(x->stream);
    if (e) return x->cuda_fail(e, "noalloc scan");
    if (h) return device_error(h);
    if (rows > max_rows)
      return x->fail(SVM_E_INVALID_ARG, "noalloc scan: " + std::to_string(rows) + " result rows exceed max_rows " +
                                            std::to_string(max_rows));
    int wide[kMaxMetrics] = {1, 1, 1};
    void* mo[kMaxMetrics] = {};
    for (int m = 0; m < nm; m++) mo[m] = sum_out[m];
    e = launch_finalize_dense(P, key_out, mo, wide, fin, scant, nullptr, x->stream);
  }
  if (!e) e = cudaMemcpyAsync(&h, P.error, sizeof(int), cudaMemcpyDeviceToHost, x->stream);
  if (!e) e = cudaStreamSynchronize(x->stream);
  if (e) return x->cuda_fail(e, "noalloc scan");
  if (h) return device_error(h);
  *nrows_out = rows;
  return SVM_OK;
}
