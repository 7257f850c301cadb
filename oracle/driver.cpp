/*
 * ORACLE (test infrastructure only): runs one generated query function the way
 * the reference's CPU path does.
 *
 *   - objects are lists of Bulks laid out as RamObject::NewBulk does
 *     (object/object.cpp:55-95: page-aligned column regions in one buffer);
 *   - Pipeline::Open (core/pipeline.cu:82-137) builds one capped
 *     linear-probing table per join over bulk 0 of the joined object, written
 *     into that object's last column, HashRate x bulk capacity slots;
 *   - Pipeline::Run / TransformTask (core/pipeline.cu:139-344, CPU branch)
 *     runs one task per source bulk on a pool of `threads` workers, each task
 *     seeing source bulk i plus bulk 0 of every joined object;
 *   - Pipeline::ReduceTask (core/pipeline.cu:360-472) sorts and sums each
 *     task's emitted rows by key.  Deliberate deviation: a metric column
 *     declared Int64 (8 bytes) is summed in int64; one declared Int32 keeps the
 *     reference's wrapping int32 sum.
 *
 * Compiled twice: against oracle/svm_port_runtime.h (the restatement) and,
 * by oracle/build_ref.sh, against the reference's own com/cpp headers.
 */
#include SVM_ORACLE_RUNTIME

#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>

typedef int (*svmo_fn)(int, BulkVector, BulkVector, uint64);

namespace {

struct Object {
  int ncols = 0;
  int types[MaxColumnNum];
  uint64 sizes[MaxColumnNum];
  std::vector<Bulk*> bulks;
};

uint64 page_align(uint64 n) { return (n + PageSize - 1) / PageSize * PageSize; }

/* object/object.cpp:55-95 (RamObject::NewBulk), host memory. */
Bulk* new_bulk(Object* o, uint64 id, uint64 max_tuple_count) {
  Bulk* b = new Bulk();
  for (int c = 0; c < o->ncols; c++) b->schema_.AddColumn(o->types[c], o->sizes[c]);
  b->id_ = id;
  b->max_tuple_count_ = max_tuple_count;
  uint64 cap = 0;
  for (int c = 0; c < o->ncols; c++) {
    b->SetColumnPos(c, cap);
    cap += page_align(max_tuple_count * o->sizes[c]);
  }
  if (cap < KB) cap = KB;
  void* mem = nullptr;
  if (posix_memalign(&mem, 4 * KB, cap) != 0) {
    delete b;
    return nullptr;
  }
  memset(mem, 0, cap);
  b->Init(mem, cap);
  return b;
}

void free_bulk(Bulk* b) {
  free(b->buffer_);
  delete b;
}

/* com/cpp/com.hpp:168-174 (BuildHashTable): every slot empty, then rows
 * inserted in row order; a row that finds no free slot in 10 steps is left out. */
void build_hash_table(int* tab, unsigned n, unsigned key_sz, int* ht, unsigned ht_sz) {
  for (unsigned s = 0; s < ht_sz; s++) ht[s] = -1;
  for (unsigned r = 0; r < n; r++) InsertHashTable<int>(tab, (int)r, key_sz, ht, ht_sz);
}

struct Row {
  int key[3];
  long long m[3];
};

/* core/pipeline.cu:360-472 (ReduceTask), CPU branch: rows 0..n-1 of `b` hold
 * key columns then metric columns; sums are written back in key order. */
int reduce_bulk(Bulk* b, Object* o, int key_num, int metric_num) {
  if (key_num == 0) {
    b->tuple_count_ = 1;
    return 0;
  }
  if (key_num > 3 || metric_num < 1 || metric_num > 3) return -1;
  uint64 n = b->tuple_count_;
  std::vector<Row> rows(n);
  for (uint64 i = 0; i < n; i++) {
    for (int k = 0; k < key_num; k++) rows[i].key[k] = ((int*)b->column_buf_[k])[i];
    for (int m = 0; m < metric_num; m++) {
      int c = key_num + m;
      rows[i].m[m] = o->sizes[c] == 8 ? ((long long*)b->column_buf_[c])[i]
                                      : (long long)((int*)b->column_buf_[c])[i];
    }
  }
  std::stable_sort(rows.begin(), rows.end(), [key_num](const Row& a, const Row& z) {
    for (int k = 0; k < key_num; k++)
      if (a.key[k] != z.key[k]) return a.key[k] < z.key[k];
    return false;
  });
  uint64 g = 0;
  for (uint64 i = 0; i < n; i++) {
    bool same = g > 0;
    for (int k = 0; same && k < key_num; k++) same = rows[g - 1].key[k] == rows[i].key[k];
    if (same) {
      for (int m = 0; m < metric_num; m++) {
        if (o->sizes[key_num + m] == 8)
          rows[g - 1].m[m] = (long long)((unsigned long long)rows[g - 1].m[m] + (unsigned long long)rows[i].m[m]);
        else
          rows[g - 1].m[m] = (int)((unsigned)rows[g - 1].m[m] + (unsigned)rows[i].m[m]);
      }
    } else {
      rows[g++] = rows[i];
    }
  }
  for (uint64 i = 0; i < g; i++) {
    for (int k = 0; k < key_num; k++) ((int*)b->column_buf_[k])[i] = rows[i].key[k];
    for (int m = 0; m < metric_num; m++) {
      int c = key_num + m;
      if (o->sizes[c] == 8)
        ((long long*)b->column_buf_[c])[i] = rows[i].m[m];
      else
        ((int*)b->column_buf_[c])[i] = (int)rows[i].m[m];
    }
  }
  b->tuple_count_ = g;
  return 0;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

void* svmo_object_new(int ncols, const int* types, const unsigned long long* sizes) {
  if (ncols <= 0 || ncols > (int)MaxColumnNum) return nullptr;
  Object* o = new Object();
  o->ncols = ncols;
  for (int c = 0; c < ncols; c++) {
    o->types[c] = types[c];
    o->sizes[c] = sizes[c];
  }
  return o;
}

void svmo_object_free(void* p) {
  Object* o = (Object*)p;
  if (!o) return;
  for (Bulk* b : o->bulks) free_bulk(b);
  delete o;
}

int svmo_object_add_bulk(void* p, unsigned long long max_tuple_count, unsigned long long tuple_count) {
  Object* o = (Object*)p;
  Bulk* b = new_bulk(o, o->bulks.size(), max_tuple_count);
  if (!b) return -1;
  b->tuple_count_ = tuple_count;
  o->bulks.push_back(b);
  return (int)o->bulks.size() - 1;
}

int svmo_object_nbulks(void* p) { return (int)((Object*)p)->bulks.size(); }

void* svmo_bulk_column(void* p, int b, int c) { return ((Object*)p)->bulks[b]->column_buf_[c]; }

unsigned long long svmo_bulk_tuple_count(void* p, int b) { return ((Object*)p)->bulks[b]->tuple_count_; }

/* Runs one pipeline; returns its sink object, or NULL with *status < 0. */
void* svmo_run_pipeline(void* fnp, void* src, int nref, void** refs, int njoin, const int* join_obj,
                        const int* join_col, int out_ncols, const int* out_types,
                        const unsigned long long* out_sizes, unsigned long long tuple_per_bulk,
                        int is_reduce, int key_num, int metric_num, int threads, double* open_ms,
                        double* compute_ms, int* status) {
  svmo_fn fn = (svmo_fn)fnp;
  Object* source = (Object*)src;
  *status = 0;
  if (nref + 1 > (int)MaxBulkInputNum) {
    *status = -2;
    return nullptr;
  }
  /* core/pipeline.cu:82-137 (Open): tables over bulk 0 of each joined object. */
  auto t0 = std::chrono::steady_clock::now();
  for (int j = 0; j < njoin; j++) {
    int obj = join_obj[j];
    if (obj < 1 || obj > nref) {
      *status = -3;
      return nullptr;
    }
    Object* r = (Object*)refs[obj - 1];
    if (r->bulks.empty() || r->sizes[join_col[j]] != 4) {
      *status = -4;
      return nullptr;
    }
    Bulk* b = r->bulks[0];
    build_hash_table((int*)b->column_buf_[join_col[j]], (unsigned)b->tuple_count_, 4,
                     (int*)b->column_buf_[r->ncols - 1], (unsigned)(HashRate * b->max_tuple_count_));
  }
  *open_ms = ms_since(t0);

  /* core/pipeline.cu:139-254 (Run), CPU branch. */
  Object* sink = (Object*)svmo_object_new(out_ncols, out_types, out_sizes);
  size_t ntask = source->bulks.size();
  for (size_t i = 0; i < ntask; i++) {
    if (svmo_object_add_bulk(sink, tuple_per_bulk, 0) < 0) {
      svmo_object_free(sink);
      *status = -5;
      return nullptr;
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  std::atomic<size_t> next(0);
  std::atomic<int> bad(0);
  auto worker = [&]() {
    for (;;) {
      size_t i = next.fetch_add(1);
      if (i >= ntask) return;
      /* core/pipeline.cu:262-344 (TransformTask). */
      BulkVector in(source->bulks[i]);
      for (int r = 0; r < nref; r++) in.AddBulk(((Object*)refs[r])->bulks[0]);
      Bulk* ob = sink->bulks[i];
      BulkVector out(ob);
      ob->tuple_count_ = (uint64)fn((int)i, in, out, in.GetTupleCount());
      if (is_reduce && reduce_bulk(ob, sink, key_num, metric_num) != 0) bad.store(1);
    }
  };
  int nt = threads > 0 ? threads : 1;
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; t++) pool.emplace_back(worker);
  for (auto& th : pool) th.join();
  *compute_ms = ms_since(t1);
  if (bad.load()) {
    svmo_object_free(sink);
    *status = -6;
    return nullptr;
  }
  return sink;
}

}  /* extern "C" */
