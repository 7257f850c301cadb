// The C ABI (include/svm_capi.h): context, object store, profiling.
#include <algorithm>
#include <climits>
#include <cstring>

#include "ctx.h"
#include "kernels.h"
#include "strdict.h"

namespace svm {

DevBuf::~DevBuf() {
  if (!p || !owned) return;
  if (ctx)
    ctx->release(p, bytes);
  else
    cudaFree(p);
}

namespace {
constexpr size_t kPoolMaxBlock = size_t(512) << 20;  // larger blocks are freed at once
constexpr size_t kPoolCap = size_t(4) << 30;         // pooled bytes kept at most

// Size classes: four per doubling above 4 KB (at most 25% rounding).
size_t size_class(size_t bytes) {
  if (bytes <= 4096) return (bytes + 255) & ~size_t(255);
  size_t p2 = 4096;
  while (p2 * 2 < bytes) p2 *= 2;
  const size_t q = p2 / 4;
  return (bytes + q - 1) / q * q;
}
}  // namespace

void Ctx::release(void* p, size_t bytes) {
  in_use -= bytes;
  if (bytes <= kPoolMaxBlock && pooled + bytes <= kPoolCap) {
    pool.emplace(bytes, p);
    pooled += bytes;
    return;
  }
  cudaFree(p);
}

void Ctx::trim_pool(size_t keep) {
  while (pooled > keep && !pool.empty()) {
    auto it = std::prev(pool.end());  // largest first
    cudaFree(it->second);
    pooled -= it->first;
    pool.erase(it);
  }
}

svm_status Ctx::cuda_fail(cudaError_t e, const char* what) {
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return SVM_E_CUDA;
}

svm_status Ctx::alloc(size_t bytes, DevBufPtr* out, bool zero) {
  if (bytes == 0) bytes = 256;
  if (bytes <= kPoolMaxBlock) bytes = size_class(bytes);
  if (cfg.hbm_budget_bytes && in_use + bytes > cfg.hbm_budget_bytes)
    return fail(SVM_E_OOM_BUDGET, "HBM budget exceeded: " + std::to_string(in_use) + " + " +
                                      std::to_string(bytes) + " > " + std::to_string(cfg.hbm_budget_bytes));
  auto b = std::make_shared<DevBuf>();
  cudaError_t e = cudaSuccess;
  auto hit = pool.find(bytes);
  if (hit != pool.end()) {
    b->p = hit->second;
    pooled -= bytes;
    pool.erase(hit);
  } else {
    if (cfg.hbm_budget_bytes && in_use + pooled + bytes > cfg.hbm_budget_bytes)
      trim_pool(cfg.hbm_budget_bytes > in_use + bytes ? cfg.hbm_budget_bytes - in_use - bytes : 0);
    e = cudaMalloc(&b->p, bytes);
    if (e == cudaErrorMemoryAllocation && pooled) {
      cudaGetLastError();
      trim_pool(0);
      e = cudaMalloc(&b->p, bytes);
    }
  }
  if (e != cudaSuccess) {
    b->p = nullptr;
    cudaGetLastError();
    return cuda_fail(e, "cudaMalloc");
  }
  b->ctx = this;
  b->bytes = bytes;
  in_use += bytes;
  if (zero && (e = cudaMemsetAsync(b->p, 0, bytes, stream)) != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  *out = b;
  return SVM_OK;
}

svm_status Ctx::upload(void* dst, const void* src, size_t bytes) {
  constexpr size_t kPiece = size_t(64) << 20;
  cudaError_t e;
  if (bytes < kPiece) {
    e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream);
    return e ? cuda_fail(e, "cudaMemcpyAsync") : SVM_OK;
  }
  if (!copy_stream[0]) {
    for (int i = 0; i < kCopyStreams; i++) {
      if ((e = cudaStreamCreateWithFlags(&copy_stream[i], cudaStreamNonBlocking))) return cuda_fail(e, "copy stream");
    }
    for (int i = 0; i <= kCopyStreams; i++)
      if ((e = cudaEventCreateWithFlags(&copy_event[i], cudaEventDisableTiming))) return cuda_fail(e, "copy event");
  }
  // copy streams wait for the work already on `stream` ...
  if ((e = cudaEventRecord(copy_event[kCopyStreams], stream))) return cuda_fail(e, "cudaEventRecord");
  for (int i = 0; i < kCopyStreams; i++)
    if ((e = cudaStreamWaitEvent(copy_stream[i], copy_event[kCopyStreams], 0))) return cuda_fail(e, "wait");
  size_t off = 0;
  for (int piece = 0; off < bytes; piece++, off += kPiece) {
    const size_t n = bytes - off < kPiece ? bytes - off : kPiece;
    e = cudaMemcpyAsync((char*)dst + off, (const char*)src + off, n, cudaMemcpyHostToDevice,
                        copy_stream[piece % kCopyStreams]);
    if (e) return cuda_fail(e, "cudaMemcpyAsync");
  }
  // ... and `stream` waits for every piece.
  for (int i = 0; i < kCopyStreams; i++) {
    if ((e = cudaEventRecord(copy_event[i], copy_stream[i]))) return cuda_fail(e, "cudaEventRecord");
    if ((e = cudaStreamWaitEvent(stream, copy_event[i], 0))) return cuda_fail(e, "wait");
  }
  return SVM_OK;
}

svm_status Ctx::pinned_take(size_t bytes, PinnedBlock* out) {
  size_t best = pinned_pool.size();
  for (size_t i = 0; i < pinned_pool.size(); i++)
    if (pinned_pool[i].bytes >= bytes && (best == pinned_pool.size() || pinned_pool[i].bytes < pinned_pool[best].bytes))
      best = i;
  if (best < pinned_pool.size()) {
    *out = pinned_pool[best];
    pinned_pool.erase(pinned_pool.begin() + (long)best);
    return SVM_OK;
  }
  size_t want = 4096;
  while (want < bytes) want *= 2;
  void* p = nullptr;
  cudaError_t e = cudaMallocHost(&p, want);
  if (e) return cuda_fail(e, "cudaMallocHost");
  out->p = p;
  out->bytes = want;
  return SVM_OK;
}

void Ctx::pinned_give(PinnedBlock* b) {
  if (b->p) pinned_pool.push_back(*b);
  *b = PinnedBlock{};
}

svm_status Ctx::pinned_reserve(size_t bytes) {
  if (pinned_bytes >= bytes) return SVM_OK;
  if (pinned) cudaFreeHost(pinned);
  pinned = nullptr;
  pinned_bytes = 0;
  size_t want = std::max(bytes, pinned_bytes * 2);
  cudaError_t e = cudaMallocHost(&pinned, want);
  if (e) {
    pinned = nullptr;
    return cuda_fail(e, "cudaMallocHost");
  }
  pinned_bytes = want;
  return SVM_OK;
}

svm_status Ctx::scratch_reserve(size_t bytes) {
  if (scratch && scratch->bytes >= bytes) return SVM_OK;
  if (scratch) {
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  }
  scratch.reset();
  size_t want = bytes < (64u << 20) ? (64u << 20) : bytes + (bytes >> 2);
  return alloc(want, &scratch);
}

svm_status Ctx::scratch_take(size_t bytes, void** out) {
  size_t off = (scratch_used + 255) & ~size_t(255);
  if (!scratch || off + bytes > scratch->bytes)
    return fail(SVM_E_INVALID_ARG, "internal: scratch arena too small");
  *out = (char*)scratch->p + off;
  scratch_used = off + bytes;
  return SVM_OK;
}

void Ctx::purge_rank_cache() {
  for (auto it = rank_cache.begin(); it != rank_cache.end();)
    it = it->second.codes.use_count() == 1 ? rank_cache.erase(it) : std::next(it);
}

svm_status Ctx::column_stats(const ObjectPtr& o, int c, ColStats* out) {
  if (o->stats.size() < o->types.size()) o->stats.resize(o->types.size());
  if (!o->stats[c].valid) {
    if (o->types[c] != SVM_INT32 && o->types[c] != SVM_STRING)
      return fail(SVM_E_UNSUPPORTED, "column statistics need an int32 column");
    int32_t h[2] = {INT_MAX, INT_MIN};
    DevBufPtr d;
    svm_status st = alloc(8, &d);
    if (st) return st;
    const int32_t* colp = (const int32_t*)o->col(c);
    cudaError_t e = cudaSuccess;
    if (o->host) {  // a device copy of the whole column, kept for the object's scans
      DevBufPtr& dc = o->dev_copy[c];
      const DevBufPtr& hb = o->storage[c];
      if (!hb->p && o->nrows) return fail(SVM_E_INVALID_ARG, "a host-resident column the query reads has no data");
      if (!dc) {
        if ((st = alloc(hb->bytes + 256, &dc))) return st;
        if (hb->bytes) e = cudaMemcpyAsync(dc->p, hb->p, hb->bytes, cudaMemcpyHostToDevice, stream);
      }
      colp = (const int32_t*)dc->p + o->row0;
    }
    if (!e) e = cudaMemcpyAsync(d->p, h, 8, cudaMemcpyHostToDevice, stream);
    if (!e) e = launch_minmax(colp, o->nrows, (int32_t*)d->p, stream);
    if (!e) e = cudaMemcpyAsync(h, d->p, 8, cudaMemcpyDeviceToHost, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) return cuda_fail(e, "column statistics");
    o->stats[c].valid = true;
    o->stats[c].min = h[0];
    o->stats[c].max = h[1];
  }
  *out = o->stats[c];
  return SVM_OK;
}

void Ctx::prof_begin(int cls, cudaEvent_t* a) {
  *a = nullptr;
  if (!profiling) return;
  if (event_pool.empty()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    event_pool.push_back(e);
  }
  *a = event_pool.back();
  event_pool.pop_back();
  cudaEventRecord(*a, stream);
  (void)cls;
}

void Ctx::prof_end(int cls, cudaEvent_t a) {
  if (!profiling || !a) return;
  cudaEvent_t b;
  if (event_pool.empty()) {
    cudaEventCreate(&b);
  } else {
    b = event_pool.back();
    event_pool.pop_back();
  }
  cudaEventRecord(b, stream);
  pending.push_back({cls, a, b});
}

void Ctx::prof_collect() {
  if (pending.empty()) return;
  cudaStreamSynchronize(stream);
  for (auto& pe : pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, pe.a, pe.b);
    prof_launches[pe.cls]++;
    prof_ms[pe.cls] += ms;
    event_pool.push_back(pe.a);
    event_pool.push_back(pe.b);
  }
  pending.clear();
}

}  // namespace svm

using svm::Ctx;
using svm::ObjectPtr;

static Ctx* C(svm_ctx* c) { return &c->impl; }

extern "C" {

int svm_abi_version(void) { return SVM_ABI_VERSION; }

void svm_config_default(svm_config* cfg) {
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->device = 0;
  cfg->hbm_budget_bytes = 0;
  cfg->tuple_per_bulk = 2000000ull;  // com/cpp/com.cu:13
  cfg->join_mode = SVM_JOIN_REF_COMPAT;
  cfg->hash_char_signed = 1;
  cfg->batch_policy = SVM_BATCH_AUTO;
  cfg->autotune = 1;
}

svm_status svm_init(const svm_config* cfg, svm_ctx** out) {
  if (!out) return SVM_E_INVALID_ARG;
  *out = nullptr;
  svm_config c;
  if (cfg)
    c = *cfg;
  else
    svm_config_default(&c);
  if (c.tuple_per_bulk == 0 || c.tuple_per_bulk > (1ull << 31) / svm::kHashRate) return SVM_E_INVALID_ARG;
  if (c.join_mode != SVM_JOIN_REF_COMPAT && c.join_mode != SVM_JOIN_EXACT) return SVM_E_INVALID_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || c.device < 0 || c.device >= n) {
    cudaGetLastError();
    return SVM_E_CUDA;
  }
  if (cudaSetDevice(c.device) != cudaSuccess) return SVM_E_CUDA;
  svm_ctx* h = new svm_ctx();
  Ctx* x = &h->impl;
  x->cfg = c;
  x->device = c.device;
  if (cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&x->d_error, sizeof(int)) != cudaSuccess ||
      cudaMemset(x->d_error, 0, sizeof(int)) != cudaSuccess || svm::noalloc_prepare(x) != SVM_OK) {
    delete h;
    return SVM_E_CUDA;
  }
  *out = h;
  return SVM_OK;
}

void svm_destroy(svm_ctx* c) {
  if (!c) return;
  Ctx* x = C(c);
  cudaSetDevice(x->device);
  if (x->stream) cudaStreamSynchronize(x->stream);
  x->prof_collect();
  x->objects.clear();
  x->merged_cache.clear();
  x->dim_cache.clear();
  x->scratch.reset();
  x->trim_pool(0);
  if (x->pinned) cudaFreeHost(x->pinned);
  for (auto& b : x->pinned_pool) cudaFreeHost(b.p);
  x->pinned_pool.clear();
  for (int i = 0; i < svm::Ctx::kCopyStreams; i++)
    if (x->copy_stream[i]) cudaStreamDestroy(x->copy_stream[i]);
  for (int i = 0; i <= svm::Ctx::kCopyStreams; i++)
    if (x->copy_event[i]) cudaEventDestroy(x->copy_event[i]);
  for (auto e : x->event_pool) cudaEventDestroy(e);
  if (x->d_error) cudaFree(x->d_error);
  if (x->stream) cudaStreamDestroy(x->stream);
  delete c;
}

const char* svm_last_error(const svm_ctx* c) { return c ? c->impl.err.c_str() : "null context"; }

void* svm_stream(svm_ctx* c) { return c ? (void*)c->impl.stream : nullptr; }

unsigned long long svm_bytes_in_use(const svm_ctx* c) { return c ? c->impl.in_use : 0; }

svm_status svm_object_put_columns(svm_ctx* c, const char* id, int ncols, const svm_column_desc* cols,
                                  unsigned long long nrows, const void* const* columns, int on_device) {
  if (!c || !id || ncols <= 0 || ncols > 64 || !cols) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  auto o = std::make_shared<svm::Object>();
  o->id = id;
  o->version = x->next_version++;
  o->ncols = ncols;
  o->nrows = nrows;
  o->has_bulks = nrows > 0;
  o->bulk0_rows = nrows < x->cfg.tuple_per_bulk ? nrows : x->cfg.tuple_per_bulk;
  o->source_rows = nrows;
  unsigned long long padded = (nrows + 63) / 64 * 64 + 64;
  for (int k = 0; k < ncols; k++) {
    const int t = cols[k].type;
    if (t != SVM_INT32 && t != SVM_INT64 && t != SVM_STRING)
      return x->fail(SVM_E_UNSUPPORTED, "object columns must be Int32, Int64 or String");
    if (t == SVM_STRING && (cols[k].val_size <= 0 || cols[k].val_size > 4096))
      return x->fail(SVM_E_INVALID_ARG, "a String column needs a width (val_size) of 1..4096 bytes");
  }
  // Replacing an object of the same shape that no view shares: reuse its storage.
  ObjectPtr old = x->find(id);
  bool reuse = old && !old->host && old->ncols == ncols && old->nrows == nrows && old->row0 == 0 &&
               (int)old->storage.size() == ncols;
  for (int k = 0; reuse && k < ncols; k++)
    reuse = old->types[k] == cols[k].type && old->storage[k].use_count() == 1;
  for (int k = 0; k < ncols; k++) {
    const int t = cols[k].type;
    o->types.push_back(t);
    svm::DevBufPtr b;
    size_t el = t == SVM_INT64 ? 8 : 4;  // String columns hold int32 dictionary codes
    if (reuse) {
      b = old->storage[k];
      if (!(columns && columns[k] && nrows)) {
        cudaError_t e = cudaMemsetAsync(b->p, 0, b->bytes, x->stream);
        if (e) return x->cuda_fail(e, "cudaMemsetAsync");
      }
    } else {
      svm_status st = x->alloc(padded * el, &b, true);
      if (st) return st;
    }
    if (t == SVM_STRING) {
      // Dictionary-encode the fixed-width values (a device column arrives
      // on the host first); a column left unset holds the all-NUL value.
      const int w = (int)cols[k].val_size;
      svm::StrCol sc;
      sc.width = w;
      std::vector<int32_t> codes;
      if (columns && columns[k] && nrows) {
        std::vector<char> hostv;
        const char* vals = (const char*)columns[k];
        if (on_device) {
          hostv.resize(nrows * (size_t)w);
          cudaError_t e = cudaMemcpy(hostv.data(), vals, hostv.size(), cudaMemcpyDeviceToHost);
          if (e) return x->cuda_fail(e, "string column read");
          vals = hostv.data();
        }
        sc.dict = svm::build_dict(vals, nrows, w, &codes);
        svm_status st = x->upload(b->p, codes.data(), nrows * 4);
        if (st) return st;
      } else {  // every row the all-NUL value, code 0 (the storage is zeroed)
        std::vector<char> zero((size_t)w, 0);
        sc.dict = svm::build_dict(zero.data(), 1, w, &codes);
      }
      o->strs[k] = sc;
    } else if (columns && columns[k] && nrows) {
      if (on_device) {
        cudaError_t e = cudaMemcpyAsync(b->p, columns[k], nrows * el, cudaMemcpyDeviceToDevice, x->stream);
        if (e) return x->cuda_fail(e, "cudaMemcpyAsync");
      } else {
        svm_status st = x->upload(b->p, columns[k], nrows * el);
        if (st) return st;
      }
    }
    o->storage.push_back(b);
  }
  cudaError_t e = cudaStreamSynchronize(x->stream);
  if (e) return x->cuda_fail(e, "object upload");
  x->put_object(id, o);
  x->purge_rank_cache();
  return SVM_OK;
}

svm_status svm_object_put_host(svm_ctx* c, const char* id, int ncols, const int* types,
                               unsigned long long nrows, const void* const* columns) {
  if (!c || !id || ncols <= 0 || ncols > 64 || !types || !columns) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  x->err.clear();
  auto o = std::make_shared<svm::Object>();
  o->id = id;
  o->version = x->next_version++;
  o->ncols = ncols;
  o->nrows = nrows;
  o->host = true;
  o->has_bulks = nrows > 0;
  o->bulk0_rows = nrows < x->cfg.tuple_per_bulk ? nrows : x->cfg.tuple_per_bulk;
  o->source_rows = nrows;
  for (int k = 0; k < ncols; k++) {
    const int t = types[k];
    if (t != SVM_INT32 && t != SVM_INT64)
      return x->fail(SVM_E_UNSUPPORTED, "host-resident object columns must be Int32 or Int64");
    const size_t el = t == SVM_INT64 ? 8 : 4;
    if (columns[k] && nrows) {
      if ((uintptr_t)columns[k] % el)
        return x->fail(SVM_E_INVALID_ARG, "column " + std::to_string(k) + " is not aligned to its element size");
      cudaPointerAttributes a{};
      if (cudaPointerGetAttributes(&a, columns[k]) != cudaSuccess || a.type != cudaMemoryTypeHost) {
        cudaGetLastError();
        return x->fail(SVM_E_INVALID_ARG,
                       "column " + std::to_string(k) + " is not page-locked host memory (cudaHostAlloc / cudaHostRegister)");
      }
    }
    auto b = std::make_shared<svm::DevBuf>();
    b->p = const_cast<void*>(columns[k]);
    b->bytes = columns[k] ? nrows * el : 0;
    b->owned = false;
    o->types.push_back(t);
    o->storage.push_back(b);
  }
  x->put_object(id, o);
  return SVM_OK;
}

svm_status svm_object_put(svm_ctx* c, const char* id, int ncols, const int* types,
                          unsigned long long nrows, const void* const* columns, int on_device) {
  if (!c || !id || ncols <= 0 || ncols > 64 || !types) return SVM_E_INVALID_ARG;
  std::vector<svm_column_desc> cols(ncols);
  for (int k = 0; k < ncols; k++) {
    if (types[k] != SVM_INT32 && types[k] != SVM_INT64)
      return C(c)->fail(SVM_E_UNSUPPORTED, "object columns must be Int32 or Int64 (String columns: svm_object_put_columns)");
    cols[k] = svm_column_desc{types[k], types[k] == SVM_INT64 ? 8 : 4};
  }
  return svm_object_put_columns(c, id, ncols, cols.data(), nrows, columns, on_device);
}

svm_status svm_object_load_text(svm_ctx* c, const char* id, int ncols, const int* types, const char* text,
                                unsigned long long bytes, int on_device, char col_delim, char row_delim,
                                unsigned long long* nrows_out) {
  if (!c || !id || ncols <= 0 || ncols > svm::kLoadMaxCols || !types || (bytes && !text)) return SVM_E_INVALID_ARG;
  if (col_delim == row_delim) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  x->err.clear();
  for (int k = 0; k < ncols; k++)
    if (types[k] != SVM_INT32 && types[k] != SVM_INT64)
      return x->fail(SVM_E_UNSUPPORTED, "text loader: columns must be Int32 or Int64 (strings are not loaded)");
  // Host text is uploaded first; device text is read where it is.
  svm::DevBufPtr tbuf;
  svm_status st = SVM_OK;
  cudaError_t e = cudaSuccess;
  const uint8_t* dtext = (const uint8_t*)text;
  if (!on_device && bytes) {
    if ((st = x->alloc(bytes, &tbuf, false)) || (st = x->upload(tbuf->p, text, bytes))) return st;
    dtext = (const uint8_t*)tbuf->p;
  }
  // Span index and the row count.
  x->scratch_reset();
  const size_t entries = svm::load_scratch_entries(bytes);
  if ((st = x->scratch_reserve(entries * sizeof(svm::LoadPos) + 1024))) return st;
  void* scr;
  if ((st = x->scratch_take(entries * sizeof(svm::LoadPos), &scr))) return st;
  svm::LoadPos total{0ull, 0u, 0u};
  cudaEvent_t ev;
  x->prof_begin(SVM_K_OTHER, &ev);
  e = svm::launch_load_index(dtext, bytes, col_delim, row_delim, (svm::LoadPos*)scr, x->stream);
  x->prof_end(SVM_K_OTHER, ev);
  if (!e && bytes)
    e = cudaMemcpyAsync(&total, svm::load_total((const svm::LoadPos*)scr, bytes), sizeof(total),
                        cudaMemcpyDeviceToHost, x->stream);
  if (!e) e = cudaStreamSynchronize(x->stream);
  if (e) return x->cuda_fail(e, "text loader index");
  // The object, every column zero until a field fills it.
  auto o = std::make_shared<svm::Object>();
  o->id = id;
  o->version = x->next_version++;
  o->ncols = ncols;
  o->nrows = total.rows;
  o->has_bulks = total.rows > 0;
  o->bulk0_rows = total.rows < x->cfg.tuple_per_bulk ? total.rows : x->cfg.tuple_per_bulk;
  o->source_rows = total.rows;
  const unsigned long long prow = (total.rows + 63) / 64 * 64 + 64;
  svm::LoadOut out{};
  out.ncols = ncols;
  out.nrows = total.rows;
  for (int k = 0; k < ncols; k++) {
    svm::DevBufPtr b;
    if ((st = x->alloc(prow * (types[k] == SVM_INT64 ? 8 : 4), &b, true))) return st;
    o->types.push_back(types[k]);
    o->storage.push_back(b);
    out.col[k] = b->p;
    out.wide[k] = types[k] == SVM_INT64;
  }
  int zero = 0;
  e = cudaMemcpyAsync(x->d_error, &zero, sizeof(int), cudaMemcpyHostToDevice, x->stream);
  if (!e) {
    x->prof_begin(SVM_K_LOAD, &ev);
    e = svm::launch_load_parse(dtext, bytes, col_delim, row_delim, (const svm::LoadPos*)scr, out, x->d_error,
                               x->stream);
    x->prof_end(SVM_K_LOAD, ev);
  }
  int h = 0;
  if (!e) e = cudaMemcpyAsync(&h, x->d_error, sizeof(int), cudaMemcpyDeviceToHost, x->stream);
  if (!e) e = cudaStreamSynchronize(x->stream);
  if (e) return x->cuda_fail(e, "text loader parse");
  if (h) return x->fail(SVM_E_INVALID_ARG, "text loader: an item longer than 4095 bytes");
  x->put_object(id, o);
  if (nrows_out) *nrows_out = total.rows;
  return SVM_OK;
}

svm_status svm_object_gen_uniform(svm_ctx* c, const char* id, int col, unsigned long long seed,
                                  unsigned long long stream, unsigned long long row0, int lo, int hi,
                                  const int* lookup) {
  if (!c || !id || hi < lo) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  ObjectPtr o = x->find(id);
  if (!o) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + id);
  if (o->host) return x->fail(SVM_E_UNSUPPORTED, "gen_uniform: object " + std::string(id) + " lives in host memory");
  if (col < 0 || col >= o->ncols || o->types[col] != SVM_INT32)
    return x->fail(SVM_E_INVALID_ARG, "gen_uniform needs an int32 column");
  svm::DevBufPtr lut;
  if (lookup) {
    size_t n = (size_t)((long long)hi - lo + 1) * 4;
    svm_status st = x->alloc(n, &lut);
    if (st) return st;
    cudaError_t e = cudaMemcpyAsync(lut->p, lookup, n, cudaMemcpyHostToDevice, x->stream);
    if (e) return x->cuda_fail(e, "cudaMemcpyAsync");
  }
  cudaEvent_t ev;
  x->prof_begin(SVM_K_OTHER, &ev);
  cudaError_t e = svm::launch_gen_uniform((int32_t*)o->col(col), o->nrows, seed, stream, row0, lo, hi,
                                          lut ? (const int32_t*)lut->p : nullptr, x->stream);
  x->prof_end(SVM_K_OTHER, ev);
  if (!e) e = cudaStreamSynchronize(x->stream);
  if (e) return x->cuda_fail(e, "gen_uniform");
  if ((int)o->stats.size() > col) o->stats[col].valid = false;
  o->version = x->next_version++;
  return SVM_OK;
}

svm_status svm_object_view(svm_ctx* c, const char* id, const char* base, unsigned long long row0,
                           unsigned long long nrows) {
  if (!c || !id || !base) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  ObjectPtr b = x->find(base);
  if (!b) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + base);
  if (row0 > b->nrows || nrows > b->nrows - row0) return x->fail(SVM_E_INVALID_ARG, "view out of range");
  auto o = std::make_shared<svm::Object>(*b);
  o->id = id;
  o->version = x->next_version++;
  o->row0 = b->row0 + row0;
  o->nrows = nrows;
  o->has_bulks = nrows > 0;
  o->bulk0_rows = nrows < x->cfg.tuple_per_bulk ? nrows : x->cfg.tuple_per_bulk;
  o->source_rows = nrows;
  // Column statistics of the base bound the view's values.
  x->put_object(id, o);
  return SVM_OK;
}

svm_status svm_object_info(svm_ctx* c, const char* id, int* ncols, unsigned long long* nrows) {
  if (!c || !id) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  ObjectPtr o = x->find(id);
  if (!o) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + id);
  if (ncols) *ncols = o->ncols;
  if (nrows) *nrows = o->nrows;
  return SVM_OK;
}

svm_status svm_object_types(svm_ctx* c, const char* id, int* types, int max_cols) {
  if (!c || !id || !types) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  ObjectPtr o = x->find(id);
  if (!o) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + id);
  for (int k = 0; k < o->ncols && k < max_cols; k++) types[k] = o->types[k];
  return SVM_OK;
}

svm_status svm_object_read(svm_ctx* c, const char* id, int col, unsigned long long row0,
                           unsigned long long n, void* host_out) {
  if (!c || !id || (!host_out && n)) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  ObjectPtr o = x->find(id);
  if (!o) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + id);
  if (o->host) return x->fail(SVM_E_UNSUPPORTED, "object " + std::string(id) + " lives in host memory (svm_object_put_host): read it in place");
  if (col < 0 || col >= o->ncols || row0 > o->nrows || n > o->nrows - row0)
    return x->fail(SVM_E_INVALID_ARG, "read out of range");
  if (!n) return SVM_OK;
  size_t el = o->elem(col);
  if (o->is_string(col)) {  // codes back to fixed-width values (NUL-padded to the column's width)
    std::vector<int32_t> codes(n);
    cudaError_t e = cudaMemcpyAsync(codes.data(), o->col(col) + row0 * el, n * el, cudaMemcpyDeviceToHost, x->stream);
    if (!e) e = cudaStreamSynchronize(x->stream);
    if (e) return x->cuda_fail(e, "object read");
    const svm::StrCol& sc = o->strs.at(col);
    const int w = sc.width, dw = sc.dict->width < w ? sc.dict->width : w;
    char* out = (char*)host_out;
    for (unsigned long long i = 0; i < n; i++) {
      char* dst = out + i * (unsigned long long)w;
      const uint32_t k = (uint32_t)codes[i];
      if (k >= sc.dict->count) return x->fail(SVM_E_DEVICE, "string code out of its dictionary");
      std::memcpy(dst, sc.dict->value(k), (size_t)dw);
      std::memset(dst + dw, 0, (size_t)(w - dw));
    }
    return SVM_OK;
  }
  cudaError_t e = cudaMemcpyAsync(host_out, o->col(col) + row0 * el, n * el, cudaMemcpyDeviceToHost, x->stream);
  if (!e) e = cudaStreamSynchronize(x->stream);
  if (e) return x->cuda_fail(e, "object read");
  return SVM_OK;
}

svm_status svm_object_columns(svm_ctx* c, const char* id, svm_column_desc* cols, int max_cols) {
  if (!c || !id || !cols) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  ObjectPtr o = x->find(id);
  if (!o) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + id);
  for (int k = 0; k < o->ncols && k < max_cols; k++) {
    cols[k].type = o->types[k];
    cols[k].val_size = o->is_string(k) ? o->strs.at(k).width : (long long)o->elem(k);
  }
  return SVM_OK;
}

svm_status svm_object_device_ptr(svm_ctx* c, const char* id, int col, void** dptr) {
  if (!c || !id || !dptr) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  ObjectPtr o = x->find(id);
  if (!o) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + id);
  if (o->host) return x->fail(SVM_E_UNSUPPORTED, "object " + std::string(id) + " lives in host memory (svm_object_put_host): read it in place");
  if (col < 0 || col >= o->ncols) return x->fail(SVM_E_INVALID_ARG, "bad column");
  *dptr = o->col(col);
  return SVM_OK;
}

svm_status svm_object_drop(svm_ctx* c, const char* id) {
  if (!c || !id) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  auto it = x->objects.find(id);
  if (it == x->objects.end()) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + id);
  // No wait for the stream: work already enqueued that reads the object
  // runs first, and its blocks go back to a pool whose next user is ordered
  // behind that work on the same stream (a block too big for the pool is
  // freed with cudaFree, which waits for the device itself).
  x->forget_plans(it->second.get());
  x->objects.erase(it);
  x->purge_rank_cache();
  // Tables built over the dropped object are keyed by its version; drop them
  // too, with the merged probe tables made from them.
  std::vector<const svm::DimTable*> gone;
  for (auto d = x->dim_cache.begin(); d != x->dim_cache.end();) {
    if (d->first.compare(0, std::strlen(id) + 1, std::string(id) + "#") == 0) {
      gone.push_back(d->second.get());
      d = x->dim_cache.erase(d);
    } else {
      ++d;
    }
  }
  if (!gone.empty())
    for (auto m = x->merged_cache.begin(); m != x->merged_cache.end();) {
      bool hit = false;
      for (const svm::DimTablePtr& t : m->second.srcs) hit |= std::find(gone.begin(), gone.end(), t.get()) != gone.end();
      m = hit ? x->merged_cache.erase(m) : std::next(m);
    }
  return SVM_OK;
}

svm_status svm_objects_read(svm_ctx* c, int n, const char* const* ids, void* host, unsigned long long cap,
                            unsigned long long* nrows_out, unsigned long long* needed) {
  if (!c || n < 0 || (n && (!ids || !nrows_out)) || !needed) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  x->err.clear();
  std::vector<svm::Segment> segs;
  unsigned long long total = 0;  // bytes; every column starts 8-byte aligned
  for (int k = 0; k < n; k++) {
    ObjectPtr o = ids[k] ? x->find(ids[k]) : nullptr;
    if (!o) return x->fail(SVM_E_NOT_FOUND, std::string("no object ") + (ids[k] ? ids[k] : "(null)"));
    if (o->host)
      return x->fail(SVM_E_UNSUPPORTED, "object " + std::string(ids[k]) + " lives in host memory (svm_object_put_host)");
    nrows_out[k] = o->nrows;
    for (int col = 0; col < o->ncols; col++) {
      if (o->is_string(col))
        return x->fail(SVM_E_UNSUPPORTED, std::string("objects read: ") + ids[k] +
                                              " has a String column (read it with svm_object_read)");
      const unsigned long long bytes = o->nrows * o->elem(col);
      if (bytes) segs.push_back(svm::Segment{(const uint32_t*)o->col(col), total / 4, bytes / 4});
      total += (bytes + 7) & ~7ull;
    }
  }
  *needed = total;
  if (!host || !total) return SVM_OK;
  if (cap < total) return x->fail(SVM_E_INVALID_ARG, "objects read: host buffer smaller than needed bytes");
  x->scratch_reset();
  const size_t sbytes = segs.size() * sizeof(svm::Segment);
  svm_status st = x->scratch_reserve(sbytes + total + 1024);
  void *dseg, *dbuf;
  if (st || (st = x->scratch_take(sbytes, &dseg)) || (st = x->scratch_take(total, &dbuf))) return st;
  if ((st = x->pinned_reserve(total))) return st;
  cudaError_t e = cudaMemcpyAsync(dseg, segs.data(), sbytes, cudaMemcpyHostToDevice, x->stream);
  if (!e) e = svm::launch_gather_segments((const svm::Segment*)dseg, (int)segs.size(), (uint32_t*)dbuf, x->stream);
  if (!e) e = cudaMemcpyAsync(x->pinned, dbuf, total, cudaMemcpyDeviceToHost, x->stream);
  if (!e) e = cudaStreamSynchronize(x->stream);
  if (e) return x->cuda_fail(e, "objects read");
  std::memcpy(host, x->pinned, total);
  return SVM_OK;
}

svm_status svm_run_pipeline(svm_ctx* c, const svm_pipeline* p) {
  if (!c || !p) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  x->err.clear();
  return svm::run_pipeline(x, p);
}

svm_status svm_run_batch(svm_ctx* c, int n, const svm_pipeline* p) {
  if (!c || (n > 0 && !p) || n < 0) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  x->err.clear();
  return svm::run_batch(x, n, p);
}

struct svm_fold {
  void* impl = nullptr;
};

svm_status svm_batch_begin(svm_ctx* c, int n, const svm_pipeline* p, int host_results, svm_fold** out) {
  if (!c || (n > 0 && !p) || n < 0 || !out) return SVM_E_INVALID_ARG;
  *out = nullptr;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  x->err.clear();
  void* f = nullptr;
  svm_status st = svm::batch_begin(x, n, p, host_results, &f);
  if (st) return st;
  *out = new svm_fold{f};
  return SVM_OK;
}

svm_status svm_batch_wait(svm_ctx* c, svm_fold* fold, unsigned long long* nrows_out, unsigned long long* needed) {
  if (!c || !fold || !fold->impl) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  // The wait for the fold's device work holds no lock, so that the next fold
  // can be planned and enqueued meanwhile.
  cudaSetDevice(x->device);
  svm::fold_sync(fold->impl);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  x->err.clear();
  return svm::batch_wait(x, fold->impl, nullptr, 0, nrows_out, needed);
}

svm_status svm_batch_release(svm_ctx* c, svm_fold* fold, void* host, unsigned long long cap) {
  if (!c || !fold) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  x->err.clear();
  svm_status st = SVM_OK;
  if (host && fold->impl) st = svm::batch_wait(x, fold->impl, host, cap, nullptr, nullptr);
  svm::batch_discard(x, fold->impl);
  delete fold;
  return st;
}

svm_status svm_pipeline_footprint(svm_ctx* c, const svm_pipeline* p, unsigned long long* bytes) {
  if (!c || !p || !bytes) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  cudaSetDevice(x->device);
  x->err.clear();
  *bytes = 0;
  return svm::pipeline_footprint(x, p, bytes);
}

unsigned long long svm_kernel_launches(void) { return svm::launches_total(); }

svm_status svm_pin_launch(svm_ctx* c, int rows_per_lane, int blocks_per_sm, int ring_stages, int tables_staged) {
  if (!c) return SVM_E_INVALID_ARG;
  if (!(rows_per_lane == -1 || rows_per_lane == 0 || rows_per_lane == 4 || rows_per_lane == 8) ||
      !(blocks_per_sm == 0 || (blocks_per_sm >= 2 && blocks_per_sm <= 4)) ||
      !(ring_stages == 0 || (ring_stages >= 2 && ring_stages <= svm::kStages)) || tables_staged < -1 ||
      tables_staged > 1)
    return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  x->pin_rows = rows_per_lane;
  x->pin_minb = blocks_per_sm;
  x->pin_stages = ring_stages;
  x->pin_staged = tables_staged;
  return SVM_OK;
}

svm_status svm_pin_list_after(svm_ctx* c, int list_after) {
  if (!c) return SVM_E_INVALID_ARG;
  if (list_after < -1 || list_after > 4) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  x->pin_list = list_after;
  return SVM_OK;
}

svm_status svm_pin_batch_launch(svm_ctx* c, int consumer_warps, int ring_stages) {
  if (!c) return SVM_E_INVALID_ARG;
  if (!(consumer_warps == 0 || consumer_warps == 24 || consumer_warps == 28) ||
      !(ring_stages == 0 || (ring_stages >= 2 && ring_stages <= svm::kStages)))
    return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  x->pin_batch_cw = consumer_warps;
  x->pin_batch_stages = ring_stages;
  return SVM_OK;
}

svm_status svm_last_launch(svm_ctx* c, char* buf, unsigned long long cap) {
  if (!c || !buf || cap == 0) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  const std::string& t = x->last_launch;
  const size_t n = t.size() < cap - 1 ? t.size() : (size_t)cap - 1;
  std::memcpy(buf, t.data(), n);
  buf[n] = 0;
  return SVM_OK;
}

svm_status svm_test_device_wait(svm_ctx* c, unsigned int wait_polls, int stall_copies) {
  if (!c) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  x->wait_polls = wait_polls;
  x->stall_copies = stall_copies != 0;
  return SVM_OK;
}

svm_status svm_profile_enable(svm_ctx* c, int on) {
  if (!c) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  x->prof_collect();
  x->profiling = on != 0;
  return SVM_OK;
}

svm_status svm_profile_reset(svm_ctx* c) {
  if (!c) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  x->prof_collect();
  for (int k = 0; k < SVM_K_COUNT; k++) {
    x->prof_launches[k] = 0;
    x->prof_ms[k] = 0;
  }
  return SVM_OK;
}

svm_status svm_profile_read(svm_ctx* c, int cls, unsigned long long* launches, double* total_ms) {
  if (!c || cls < 0 || cls >= SVM_K_COUNT) return SVM_E_INVALID_ARG;
  Ctx* x = C(c);
  std::lock_guard<std::recursive_mutex> g(x->mu);
  x->prof_collect();
  if (launches) *launches = x->prof_launches[cls];
  if (total_ms) *total_ms = x->prof_ms[cls];
  return SVM_OK;
}

}  // extern "C"
