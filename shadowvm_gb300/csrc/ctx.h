// Host-side state of one data-plane context: the device object store, the
// dimension-table cache, scratch memory and profiling.  Mirrors the reference's
// ObjectStore (object/store.cpp:13-91), RamObject bulks (object/object.cpp:55-95)
// and the service's cached_obj map (service/service.hpp:92), with every column
// resident in HBM.
#pragma once

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/svm_capi.h"
#include "svm_internal.h"

namespace svm {

struct Ctx;

// A device allocation charged to the context's HBM budget.
struct DevBuf {
  Ctx* ctx = nullptr;
  void* p = nullptr;
  size_t bytes = 0;
  bool owned = true;  // false: p is the caller's memory (a host-resident object's column)
  ~DevBuf();
};
using DevBufPtr = std::shared_ptr<DevBuf>;

struct ColStats {
  bool valid = false;
  int32_t min = 0, max = 0;
};

// The distinct values of a String column (fixed width, as the reference's
// ValType String, com/svm.proto:62-72), sorted by memcmp: the column stores
// each row's int32 code, the value's position here.  Sorted codes keep the
// values a StrCmp prefix comparison accepts contiguous.
struct StrDict {
  int width = 0;              // bytes per stored value
  uint32_t count = 0;
  std::vector<char> bytes;    // count x width
  const char* value(uint32_t k) const { return bytes.data() + (size_t)k * width; }
};
using StrDictPtr = std::shared_ptr<const StrDict>;

// A String column of an object: its declared width (the reference's
// val_size: a value is its dictionary bytes followed by NULs up to it), its
// dictionary, and -- once a ReduceBy has used it as a key -- the derived
// int32 column holding each row's rank among the distinct Hash values
// (cpu-runtime.hpp:68-74) and the Hash value of each rank.
struct StrCol {
  int width = 0;
  StrDictPtr dict;
  int rank_col = -1;
  std::vector<int32_t> rank_hash;
};

// A columnar object.  Columns are int32 or int64; each column's storage is
// padded to a multiple of 64 rows (+64 rows) so the scan's 16-byte group loads
// never leave the allocation.  A view shares its base object's storage.
struct Object {
  std::string id;
  unsigned long long version = 0;
  int ncols = 0;
  std::vector<int> types;
  unsigned long long nrows = 0;
  unsigned long long row0 = 0;                // rows skipped in the base storage (views)
  std::vector<DevBufPtr> storage;             // base allocation per column
  // Columns in the caller's page-locked host memory (svm_object_put_host),
  // read in place: only the fused scan of a reduce pipeline takes such an
  // object (as its fact table), copying the columns its filters read and
  // gathering the others at the surviving rows.
  bool host = false;
  // A host-resident object's whole-column device copies, made when a column's
  // statistics are needed (its values cross the host link once); a scan of
  // the object reuses them instead of copying those rows again.
  std::map<int, DevBufPtr> dev_copy;
  // The reference keeps objects as bulks of tuple_per_bulk rows and joins only
  // against bulk 0 of a joined object (core/pipeline.cu:91,295).
  bool has_bulks = false;
  unsigned long long bulk0_rows = 0;
  // Rows of the object this one was filtered from (a dimension pipeline's
  // source); estimates how selective a join against it is.
  unsigned long long source_rows = 0;
  std::vector<ColStats> stats;
  // String columns (types[c] == SVM_STRING: storage holds int32 codes).
  // Derived columns (hash ranks) follow the ncols visible ones in types and
  // storage.
  std::map<int, StrCol> strs;

  bool is_string(int c) const { return c >= 0 && c < (int)types.size() && types[c] == SVM_STRING; }
  char* base(int c) const { return (char*)storage[c]->p; }
  size_t elem(int c) const { return types[c] == SVM_INT64 ? 8 : 4; }
  char* col(int c) const { return base(c) + row0 * elem(c); }
};
using ObjectPtr = std::shared_ptr<Object>;

// A built dimension table plus what the planner needs to know about it.
struct DimTable {
  DimDesc desc{};
  DevBufPtr words;
  unsigned long long live = 0;                // rows inserted
  unsigned long long rows_considered = 0;     // rows of the object the build looked at
  std::vector<int> pay_cols;                  // object columns behind desc.pay[]
  std::vector<int32_t> pay_min, pay_max;      // over inserted rows
  int32_t key_min = 0, key_max = 0;
  size_t bytes() const { return words ? words->bytes : 0; }
};
using DimTablePtr = std::shared_ptr<DimTable>;

// A merged probe table of the batch path, kept while its source tables live.
struct MergedTable {
  DevBufPtr buf;
  std::vector<DimTablePtr> srcs;
  unsigned long long stamp = 0;
};

// A page-locked host block from the context's pool (see Ctx::pinned_take).
struct PinnedBlock {
  void* p = nullptr;
  size_t bytes = 0;
};

struct ProfEvent {
  int cls;
  cudaEvent_t a, b;
};

struct Ctx {
  svm_config cfg{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::recursive_mutex mu;
  std::string err;
  size_t in_use = 0;                          // bytes of live allocations
  // Freed blocks kept for reuse (all work runs on `stream`, so a block handed
  // out again is only written after earlier work on it).  Keyed by size
  // class; charged to the budget until trimmed.
  std::multimap<size_t, void*> pool;
  size_t pooled = 0;
  // Pinned host staging for bulk reads (grows, kept).
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
  // Page-locked blocks of folds in flight come from this pool and return to
  // it (cudaFreeHost would synchronise the device); freed at destroy.
  std::vector<PinnedBlock> pinned_pool;
  svm_status pinned_take(size_t bytes, PinnedBlock* out);
  void pinned_give(PinnedBlock* b);
  // Copy streams for large host-to-device uploads (created on first use).
  static constexpr int kCopyStreams = 4;
  cudaStream_t copy_stream[kCopyStreams] = {};
  cudaEvent_t copy_event[kCopyStreams + 1] = {};
  unsigned long long next_version = 1;
  std::map<std::string, ObjectPtr> objects;
  std::map<std::string, DimTablePtr> dim_cache;
  std::map<std::string, MergedTable> merged_cache;
  unsigned long long merged_stamp = 0;
  // Dense tables that held another value than a fellow table of their merged
  // probe group at a key present in both: they keep a payload field of their
  // own in later merges (entries die with their table).
  std::map<const DimTable*, std::weak_ptr<DimTable>> no_share;
  bool share_refused(const DimTablePtr& t) const {
    auto f = no_share.find(t.get());
    return f != no_share.end() && f->second.lock() == t;
  }
  // Hash-rank columns of String code columns, one per (code storage,
  // dictionary, width), over the storage's whole extent so that every view
  // of an object shares it; holds the code storage alive (and unreusable).
  struct RankCol {
    DevBufPtr codes, ranks;
    std::vector<int32_t> hash_of_rank;
  };
  std::map<std::tuple<const void*, const void*, int>, RankCol> rank_cache;
  // A launch configuration of the fused scan: ring depth, small tables
  // staged in shared memory, adjacent L2 probes exchanged at this step (or
  // -1), and rows per consumer lane of the kernel compiled for the plan's
  // shape (0: the interpreted kernel).
  struct StarLaunch {
    int nst = 2;
    bool staged = true;
    int swap = -1;
    int rows = 0;
    int minb = 0;   // compiled kernel: the blocks per SM it is compiled for
    int list = 3;   // compiled kernel: the step after which later steps run over a row list (3: none;
                    // 4: after step 0, steps 1 and 2 in one pass)
  };
  // Pinned launch choices (svm_pin_launch): kernel rows per lane (-1: any,
  // 0: the interpreted kernel, 4 or 8: the compiled one), the blocks per SM
  // the compiled kernel is built for (0: any), ring stages (0: any), tables
  // staged (-1: any).  A pin narrows the candidates; the rule or
  // the tuner picks among those left.
  int pin_rows = -1, pin_minb = 0, pin_stages = 0, pin_staged = -1;
  // Pinned row-list step of the compiled kernel (svm_pin_list_after; -1: any).
  int pin_list = -1;
  // Pinned merged-batch launch choices (svm_pin_batch_launch): consumer warps
  // (0: any, 28 or 24) and ring stages (0: any).
  int pin_batch_cw = 0, pin_batch_stages = 0;
  // Tuned merged-batch launches: batch shape -> (consumer warps, ring stages).
  std::map<std::string, std::pair<int, int>> batch_tune;
  // Planned fact pipelines by content and the versions of the objects they
  // read (pipeline.cpp); forget_plans drops the plans that read `o`.
  std::shared_ptr<void> plan_cache;
  void forget_plans(const Object* o);
  // Tuned star launches: plan shape -> the fastest configuration measured.
  std::map<std::string, StarLaunch> star_tune;
  std::string last_launch;                    // the last fused scan's configuration, as text
  void purge_rank_cache();  // entries whose code storage no object uses any more
  int* d_error = nullptr;                     // device error word
  // Test hook (svm_test_device_wait): the fused scan's mbarrier poll limit
  // (0 = default) and whether its copy warp issues no copies.
  uint32_t wait_polls = 0;
  int stall_copies = 0;
  // Grow-only scratch arena, carved per operation.
  DevBufPtr scratch;
  size_t scratch_used = 0;
  // Profiling.
  bool profiling = false;
  std::vector<ProfEvent> pending;
  std::vector<cudaEvent_t> event_pool;
  unsigned long long prof_launches[SVM_K_COUNT] = {};
  double prof_ms[SVM_K_COUNT] = {};

  svm_status fail(svm_status s, const std::string& m) {
    err = m;
    return s;
  }
  svm_status cuda_fail(cudaError_t e, const char* what);

  // Allocation charged to the budget (zero-filled when `zero`).
  svm_status alloc(size_t bytes, DevBufPtr* out, bool zero = false);
  void release(void* p, size_t bytes);        // a DevBuf's block: back to the pool or freed
  svm_status pinned_reserve(size_t bytes);
  // Enqueues a host-to-device copy ordered after earlier work on `stream`
  // and before later work on it; copies of 64 MB and more go in pieces over
  // the copy streams so that several copy engines work at once.
  svm_status upload(void* dst, const void* src, size_t bytes);
  void trim_pool(size_t keep);                // frees pooled blocks until at most `keep` bytes stay
  // Scratch: reset() then take() pieces; valid until the next reset().
  void scratch_reset() { scratch_used = 0; }
  svm_status scratch_take(size_t bytes, void** out);
  svm_status scratch_reserve(size_t bytes);

  // Stores object `id`, forgetting the plans that read the object it replaces.
  void put_object(const std::string& id, ObjectPtr o) {
    auto it = objects.find(id);
    if (it != objects.end()) {
      forget_plans(it->second.get());
      it->second = std::move(o);
    } else {
      objects.emplace(id, std::move(o));
    }
  }

  ObjectPtr find(const std::string& id) {
    auto it = objects.find(id);
    return it == objects.end() ? nullptr : it->second;
  }
  svm_status column_stats(const ObjectPtr& o, int c, ColStats* out);

  void prof_begin(int cls, cudaEvent_t* a);
  void prof_end(int cls, cudaEvent_t a);
  void prof_collect();
};

// The status and message for a kernel's error word (a DevError code).
inline svm_status device_error_status(int code, const char** msg) {
  switch (code) {
    case DERR_DIV0: *msg = "integer division by zero in an expression"; return SVM_E_DEVICE;
    case DERR_HASH_FULL: *msg = "dimension hash table overflow"; return SVM_E_DEVICE;
    case DERR_KEY_RANGE: *msg = "group key outside its computed range"; return SVM_E_DEVICE;
    case DERR_TIMEOUT: *msg = "a bounded device wait gave up (the kernel exited early)"; return SVM_E_TIMEOUT;
    case DERR_LOAD_ITEM: *msg = "an item longer than 4095 bytes"; return SVM_E_INVALID_ARG;
    default: *msg = "the kernel reported an error"; return SVM_E_DEVICE;
  }
}

// The allocation-free scan's static scratch, looked up for x->device
// (kern_noalloc.cu); svm_init calls it once per context.
svm_status noalloc_prepare(Ctx* x);

// Pipelines (pipeline.cpp).
// Folds: batch_begin enqueues a batch and returns an opaque fold without
// waiting for its device work; batch_wait completes it (results stored as
// objects, optionally copied to `host` in svm_objects_read's layout) and
// frees it; batch_discard frees a fold that will not be waited for.
svm_status batch_begin(Ctx* x, int n, const svm_pipeline* p, int want_host, void** fold);
svm_status batch_wait(Ctx* x, void* fold, void* host, unsigned long long cap, unsigned long long* nrows_out,
                      unsigned long long* needed);
void batch_discard(Ctx* x, void* fold);
void fold_sync(void* fold);  // waits for the fold's device work (no context state touched)
svm_status run_pipeline(Ctx* ctx, const svm_pipeline* p);
svm_status run_batch(Ctx* ctx, int n, const svm_pipeline* p);
svm_status pipeline_footprint(Ctx* ctx, const svm_pipeline* p, unsigned long long* bytes);

}  // namespace svm

struct svm_ctx {
  svm::Ctx impl;
};
