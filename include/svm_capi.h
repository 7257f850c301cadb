/*
 * svm_capi.h -- C ABI of the GB300 data plane for ShadowVM's query hot path:
 * fused fact-table filter -> dimension hash-table build/probe -> group-by
 * aggregate over columnar int32 tables, on one GPU (sm_103a).
 *
 * Plain C: opaque handles, pointers and sizes, no C++ or torch types.  Every
 * call returns an svm_status; on failure svm_last_error() describes it.
 * A context is used by one host thread at a time (the library serialises
 * calls on a context with an internal mutex).
 *
 * What each entry point stands in for in the reference (paths are relative to
 * the ShadowVM source tree):
 *   svm_init / svm_destroy        ObjectStore ctor (object/store.cpp:13-36) + ResMgr::Init
 *                                 (core/resource.cu:35-47) + ShadowVMService::Init (service/service.cu:17-21)
 *   svm_object_*                  ObjectStore Create/Get/Destroy (object/store.cpp:49-91), RamObject
 *                                 bulks (object/object.cpp:55-95), Object::To(DeviceMem) (object/object.cpp:194-294)
 *   svm_run_pipeline              ShadowVMService::RunPipelineCMD (service/service.cu:25-63) ->
 *                                 PipelineTest::Run (test/test.hpp:122-146) -> Pipeline ctor/Open/Run
 *                                 (core/pipeline.cu:11-254) -> Query::Next (core/operator.cpp:121-187) ->
 *                                 the generated per-row loop (codegen/template.cpp:61-89) ->
 *                                 ReduceTask (core/pipeline.cu:360-472); result cached by pipeline
 *                                 id like ShadowVMService::cached_obj (service/service.hpp:92)
 *   svm_run_batch                 no counterpart: many RunPipelineCMD calls folded into one launch
 *   svm_batch_begin/wait/release  no counterpart: the same, enqueued without waiting (folds in flight)
 *   svm_pipeline_footprint        no counterpart: device bytes a pipeline needs (served admission)
 *   svm_object_load_text          Loader::Host (core/operator.cpp:24-48): delimited text -> columns
 *   svm_object_put_columns        RamObject bulks with String columns (ValType String, com/svm.proto:62-72;
 *                                 StrCmp / Hash / StrCopy of com/cpp/cpu-runtime.hpp:37-77 act on them)
 */
#ifndef SVM_CAPI_H_
#define SVM_CAPI_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SVM_ABI_VERSION 1

typedef enum svm_status {
  SVM_OK = 0,
  SVM_E_INVALID_ARG = 1,  /* malformed pipeline, bad id/column, wrong sizes */
  SVM_E_UNSUPPORTED = 2,  /* outside the supported expression/operator set; no fallback runs */
  SVM_E_OOM_BUDGET = 3,   /* the HBM budget (svm_config.hbm_budget_bytes) would be exceeded */
  SVM_E_TIMEOUT = 4,      /* a bounded device wait gave up */
  SVM_E_CUDA = 5,         /* a CUDA runtime call failed */
  SVM_E_NOT_FOUND = 6,    /* unknown object / pipeline id (the RPC's CANCELLED case) */
  SVM_E_DEVICE = 7        /* a kernel reported an error (e.g. integer division by zero) */
} svm_status;

/* Value types: the numbering of ValType in com/svm.proto:62-72. */
enum { SVM_BYTE = 0, SVM_INT16 = 1, SVM_INT32 = 2, SVM_INT64 = 3, SVM_FLOAT16 = 4,
       SVM_FLOAT32 = 5, SVM_FLOAT64 = 6, SVM_STRING = 7, SVM_TENSOR = 8 };

/* Operator types: OperatorInfo.Type in com/svm.proto:102-111. */
enum { SVM_OP_SOURCE = 0, SVM_OP_LOADER = 1, SVM_OP_FILTER = 2, SVM_OP_MAP = 3,
       SVM_OP_REDUCEBY = 4, SVM_OP_SORTBY = 5, SVM_OP_JOINWITH = 6, SVM_OP_SINK = 7 };

/* Join semantics.
 * SVM_JOIN_REF_COMPAT: exactly the reference's CPU path.  A joined object
 *   contributes only its first bulk (rows that came from the first
 *   tuple_per_bulk source rows; core/pipeline.cu:91,295), and a dimension
 *   row the reference's 10-step capped linear-probing table
 *   (com/cpp/cpu-runtime.hpp:80-91, HashRate x tuple_per_bulk slots) fails to
 *   insert is never matched.
 * SVM_JOIN_EXACT: every dimension row is joinable.
 * In both modes a key present more than once matches its first row, as the
 * reference's Probe does (cpu-runtime.hpp:125-138). */
enum { SVM_JOIN_REF_COMPAT = 0, SVM_JOIN_EXACT = 1 };

typedef struct svm_config {
  int device;                        /* CUDA device ordinal */
  unsigned long long hbm_budget_bytes; /* device bytes the context may hold; 0 = no limit */
  unsigned long long tuple_per_bulk; /* the reference's bulk size, Context::tuple_per_bulk_
                                        (com/cpp/com.cu:13), default 2,000,000 */
  int join_mode;                     /* SVM_JOIN_REF_COMPAT (default) or SVM_JOIN_EXACT */
  int hash_char_signed;              /* 1 (default): hash key bytes as signed char, as the
                                        x86 reference does; 0: unsigned (aarch64 build) */
  int batch_policy;                  /* svm_run_batch: SVM_BATCH_AUTO (default) picks the cheaper
                                        of one shared launch and per-query launches by a cost
                                        model; SVM_BATCH_ALWAYS / SVM_BATCH_NEVER force one */
  int autotune;                      /* 1 (default): the first run of each query shape times the
                                        fitting launch configurations (ring depth, shared-memory
                                        table placement) and keeps the fastest; 0: a fixed rule */
} svm_config;

enum { SVM_BATCH_AUTO = 0, SVM_BATCH_ALWAYS = 1, SVM_BATCH_NEVER = 2 };

typedef struct svm_ctx svm_ctx;

/* ---- context ------------------------------------------------------------ */
void svm_config_default(svm_config* cfg);
svm_status svm_init(const svm_config* cfg, svm_ctx** out);
void svm_destroy(svm_ctx* ctx);
const char* svm_last_error(const svm_ctx* ctx);
int svm_abi_version(void);
/* The cudaStream_t every library kernel of this context is launched on. */
void* svm_stream(svm_ctx* ctx);
/* Device bytes currently held by the context (objects, tables, scratch). */
unsigned long long svm_bytes_in_use(const svm_ctx* ctx);

typedef struct svm_column_desc { /* ColumnInfo (svm.proto:73-79) */
  int type;                      /* SVM_INT32, SVM_INT64, SVM_STRING ... */
  long long val_size;
} svm_column_desc;

/* ---- object store (device-resident int32/int64 columns) ------------------ */
/* Create object `id` with `ncols` columns of `nrows` rows each.  types[c] is
 * SVM_INT32 or SVM_INT64.  columns[c] points at nrows values in host memory
 * (copied to the device) or, with columns_on_device != 0, in device memory
 * (copied device to device).  columns == NULL leaves the columns zeroed.
 * Replaces an existing object of the same id. */
svm_status svm_object_put(svm_ctx* ctx, const char* id, int ncols, const int* types,
                          unsigned long long nrows, const void* const* columns,
                          int columns_on_device);
/* A fact table left in the caller's page-locked host memory (cudaHostAlloc /
 * cudaHostRegister; anything else is SVM_E_INVALID_ARG), Int32 / Int64
 * columns, read in place: the reference keeps its fact bulks in mapped
 * pinned host memory too (object/object.cpp:194-294, SharedMem).  A reduce
 * pipeline's scan copies to the device only the rows and columns its filter
 * steps read, and gathers the other columns it needs from host memory at the
 * rows that survive.  The buffers must stay valid and unchanged while the
 * object exists.  Only a reduce pipeline's source may be such an object
 * (run alone, not batched); joins, Map pipelines, reads, generation and
 * device pointers of it are SVM_E_UNSUPPORTED.  A NULL column is absent (a
 * pipeline that reads it fails). */
svm_status svm_object_put_host(svm_ctx* ctx, const char* id, int ncols, const int* types,
                               unsigned long long nrows, const void* const* columns);
/* As svm_object_put, with each column described by {type, val_size}:
 * SVM_INT32 / SVM_INT64 as above, or SVM_STRING of val_size bytes per value
 * (the reference's fixed-width char[val_size] String column, com/svm.proto:
 * 62-72): columns[c] points at nrows x val_size bytes.  A String column is
 * dictionary-encoded (distinct values sorted bytewise, an int32 code per row
 * on the device); StrCmp predicates, ReduceBy keys (the reference's
 * Hash(value, val_size)) and Map copies work on the codes. */
svm_status svm_object_put_columns(svm_ctx* ctx, const char* id, int ncols, const svm_column_desc* cols,
                                  unsigned long long nrows, const void* const* columns,
                                  int columns_on_device);
/* Fill column `col` of an existing int32 object on the device with the seeded
 * counter-based generator: value(i) = lo + ((mix(seed, stream, row0 + i) >> 32)
 * * (hi - lo + 1)) >> 32 (splitmix64 output function), i.e. rows row0.. of an
 * unbounded synthetic table.  With `lookup` non-NULL the drawn value v in
 * [lo, hi] is replaced by lookup[v - lo] (lookup in host memory, hi - lo + 1
 * entries). */
svm_status svm_object_gen_uniform(svm_ctx* ctx, const char* id, int col, unsigned long long seed,
                                  unsigned long long stream, unsigned long long row0, int lo, int hi,
                                  const int* lookup);
/* Zero-copy view: rows [row0, row0 + nrows) of object `base` as object `id`. */
svm_status svm_object_view(svm_ctx* ctx, const char* id, const char* base,
                           unsigned long long row0, unsigned long long nrows);
svm_status svm_object_info(svm_ctx* ctx, const char* id, int* ncols, unsigned long long* nrows);
svm_status svm_object_types(svm_ctx* ctx, const char* id, int* types, int max_cols);
/* Type and width (val_size: 4 / 8, or a String column's bytes per value) of each column. */
svm_status svm_object_columns(svm_ctx* ctx, const char* id, svm_column_desc* cols, int max_cols);
/* Copy rows [row0, row0 + n) of column `col` to host memory (4 or 8 bytes per
 * value; val_size bytes per value for a String column, NUL-padded). */
svm_status svm_object_read(svm_ctx* ctx, const char* id, int col, unsigned long long row0,
                           unsigned long long n, void* host_out);
/* Device address of column `col` (valid until the object is dropped/replaced). */
svm_status svm_object_device_ptr(svm_ctx* ctx, const char* id, int col, void** dptr);
/* Parses delimited text into a new object, on the device: the reference's
 * Loader operator (Loader::Host, core/operator.cpp:24-48, items converted by
 * GetValueOfItemBySwitch, com/cpp/com.cu:33-44), e.g. SSB's "a|b|c|\n"
 * lines with col_delim '|' and row_delim '\n'.  A field is stored when a
 * column delimiter ends it (the text after a line's last column delimiter is
 * dropped); rows are counted by row delimiters; Int32 fields convert as
 * atoi, Int64 as atol (strtol, clamped on overflow).  Fields past column
 * ncols - 1 are ignored and columns a row does not reach are 0 (the
 * reference leaves both undefined).  Columns must be SVM_INT32 or
 * SVM_INT64; an item longer than 4095 bytes is SVM_E_INVALID_ARG.  `text`
 * is host memory, or device memory with on_device = 1. */
svm_status svm_object_load_text(svm_ctx* ctx, const char* id, int ncols, const int* types, const char* text,
                                unsigned long long bytes, int on_device, char col_delim, char row_delim,
                                unsigned long long* nrows_out);

/* Several whole objects to host memory in one device pass (one gather kernel,
 * one copy, one synchronisation).  For each object in order and each of its
 * columns in order, the column's rows are written to `host` starting at an
 * 8-byte-aligned offset (int32 columns take 4 bytes a row, int64 8).
 * nrows_out[k] gets object k's row count and *needed the total bytes; with
 * host == NULL only those are returned.  No counterpart in the reference (its
 * wire has no result fetch); the served loop reads a fold's results with it. */
svm_status svm_objects_read(svm_ctx* ctx, int n, const char* const* ids, void* host, unsigned long long cap,
                            unsigned long long* nrows_out, unsigned long long* needed);

svm_status svm_object_drop(svm_ctx* ctx, const char* id);

/* ---- pipelines (PipelineInfo, com/svm.proto:101-144) ---------------------- */
typedef struct svm_arg {
  const char* key;   /* OperatorInfo.args key: predication, select, lkey, rkey, dim, metric ... */
  const char* value;
} svm_arg;

typedef struct svm_operator {    /* OperatorInfo (svm.proto:101-123) */
  int type;                      /* SVM_OP_* */
  int nargs;
  const svm_arg* args;
  int ncols;                     /* output ObjectInfo's column_list */
  const svm_column_desc* output;
} svm_operator;

typedef struct svm_pipeline {    /* PipelineInfo (svm.proto:137-144) */
  const char* id;
  int nops;
  const svm_operator* ops;
  int npre;
  const char* const* pre_pipeline_id; /* [0] = source object, [1..] = joined objects */
} svm_pipeline;

/* Run one pipeline and store its output as object `pipe->id`.
 *   Source/Filter/Map/Sink            -> filtered, projected, row-order-preserving
 *                                        copy (the dimension-side pipelines)
 *   Source/Filter/JoinWith.../ReduceBy/Sink -> fused scan/probe/aggregate; output
 *                                        rows are the groups sorted by key:
 *                                        key columns (int32) then one column
 *                                        per metric, int64 when the Sink
 *                                        declares Int64, else wrapped to int32.
 * A missing pre_pipeline_id object returns SVM_E_NOT_FOUND. */
svm_status svm_run_pipeline(svm_ctx* ctx, const svm_pipeline* pipe);

/* Run n reduce pipelines as one batched persistent launch (shared scan of the
 * resident fact columns, per-query predicates, probes and aggregate slots).
 * Every output is stored as in svm_run_pipeline.  The result of each pipeline
 * equals its result from svm_run_pipeline. */
svm_status svm_run_batch(svm_ctx* ctx, int n, const svm_pipeline* pipes);

/* Folds in flight (no counterpart in the reference, whose service runs one
 * synchronous RPC at a time, service/service.cu:25-63).  svm_batch_begin
 * plans `n` pipelines like svm_run_batch and enqueues their device work
 * without waiting for it: reduce pipelines over one fact table go into
 * batched launches whose result store holds every group the queries can
 * produce, so no host step is needed between the launches and the results.
 * Map pipelines, reduce pipelines the batch kernel does not take, and ones
 * the cost model runs alone complete inside the call.  With host_results
 * != 0 every result is also copied, behind the fold's work, into page-locked
 * staging.  While a fold's work runs, the caller may plan and begin the next
 * fold (the device runs them in order on the context's stream).
 * svm_batch_wait blocks until the fold's device work is done (without
 * holding the context, so other calls proceed meanwhile), stores every
 * result as object `id` as svm_run_batch does, and reports each pipeline's
 * row count (nrows_out[i], input order) and the bytes of the host copy
 * (*needed; 0 without host_results).  svm_batch_release copies the staged
 * results to `host` (when not NULL; svm_objects_read's layout: for each
 * pipeline in input order, each column's rows from an 8-byte-aligned
 * offset) and frees the fold; every fold must be released, also one whose
 * wait failed.  The objects a fold reads must not be replaced until its
 * wait returns.  A fold never times launch configurations (with autotune,
 * svm_run_batch does, the first time it meets a batch shape): it takes the
 * one cached for its batch shape, else the rule. */
typedef struct svm_fold svm_fold;
svm_status svm_batch_begin(svm_ctx* ctx, int n, const svm_pipeline* pipes, int host_results, svm_fold** out);
svm_status svm_batch_wait(svm_ctx* ctx, svm_fold* fold, unsigned long long* nrows_out, unsigned long long* needed);
svm_status svm_batch_release(svm_ctx* ctx, svm_fold* fold, void* host, unsigned long long cap);

/* Device bytes that running `pipe` needs beyond what is resident (group
 * slots, finalize scratch and the largest possible result), for admission by
 * HBM footprint.  Plans the pipeline; dimension tables it joins are built and
 * cached as svm_run_pipeline would.  No counterpart in the reference (it has
 * no admission control, service/service.cu:25-63). */
svm_status svm_pipeline_footprint(svm_ctx* ctx, const svm_pipeline* pipe, unsigned long long* bytes);

/* ---- allocation-free scan ---------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory on their query path: a host runtime that owns all device memory
 * through its own pool, a thread that must not take the implicit device-wide
 * synchronisation of cudaMalloc/cudaFree, or code that issues work while other
 * streams must not be disturbed.  Every other entry point here allocates
 * (object storage, dimension tables, the context's scratch arena); this one
 * does not.
 *
 * It runs the same fused scan kernel as svm_run_pipeline, restricted to range
 * filters on the given columns, dense group keys on those columns and
 * SVM_METRIC_* metrics, over caller-owned device columns, and writes the
 * non-empty groups sorted by key -- the rows svm_run_pipeline stores for the
 * equivalent Filter/ReduceBy pipeline with Int64 metrics -- into
 * caller-owned device buffers.  Its scratch (group slots, compaction flags
 * and positions, the error word) is one static device array of
 * SVM_NOALLOC_SCRATCH_WORDS 64-bit words (1 MiB) that every GPU which loads
 * the library holds until the process exits; a query whose groups need more
 * is rejected with SVM_E_INVALID_ARG.  The array is shared by all calls and
 * keeps the last call's contents; each call clears what must start at zero.
 * Calls whose work overlaps on the GPU (two host threads, or two contexts on
 * one device) race on it: serialise them.  svm_init looks the array up
 * (cudaGetSymbolAddress, with the context's device current; under lazy
 * module loading that is when the driver places the array), so query calls
 * only read the cached address; were it missing, the first call would look
 * it up itself, and that call should then come before any stream capture.
 * Errors: a key outside [key_min, key_max] is SVM_E_DEVICE, a device wait
 * that gave up SVM_E_TIMEOUT (both reported before the row count is
 * compared with max_rows); more groups than max_rows, or max_rows 0 for a
 * query without keys, is SVM_E_INVALID_ARG.  The call is synchronous on the
 * context's stream.
 *
 * Inputs: cols[c] int32 device pointers, 16-byte aligned, readable up to
 * nrows rounded up to a multiple of 4.  Outputs: key_out[k] (int32) and
 * sum_out[m] (int64) device arrays of max_rows entries; *nrows_out (host) is
 * the number of rows written (1 when there are no keys and nrows > 0). */
#define SVM_NOALLOC_SCRATCH_WORDS (1u << 17)
enum { SVM_METRIC_COL = 0, SVM_METRIC_ADD = 1, SVM_METRIC_SUB = 2, SVM_METRIC_MUL = 3 };

typedef struct svm_noalloc_scan {
  int ncols;
  const int32_t* const* cols;
  unsigned long long nrows;
  int nranges;                 /* keep rows with range_lo[i] <= cols[range_col[i]] <= range_hi[i] */
  const int* range_col;
  const int* range_lo;
  const int* range_hi;
  int nkeys;                   /* 0..3 group keys; every value lies in [key_min, key_max] */
  const int* key_col;
  const int* key_min;
  const int* key_max;
  int nmetrics;                /* 1..3: metric_op applied to cols[metric_a] (and cols[metric_b]) */
  const int* metric_op;
  const int* metric_a;
  const int* metric_b;
} svm_noalloc_scan;

svm_status svm_scan_aggregate_noalloc(svm_ctx* ctx, const svm_noalloc_scan* q, int32_t* const* key_out,
                                      long long* const* sum_out, unsigned long long max_rows,
                                      unsigned long long* nrows_out);

/* Narrows the fused scan's launch configurations for the context's later
 * queries: rows_per_lane -1 (any), 0 (the interpreted kernel) or 4 / 8 (the
 * kernel compiled for the plan's shape, with that many rows per consumer
 * lane); blocks_per_sm 0 (any) or 2..4 (the compiled kernel built for that
 * many resident blocks per SM: 3 or 4 with 4 rows per lane, 2 with 8);
 * ring_stages 0 (any) or 2..4; tables_staged -1 (any), 0 (small dimension
 * tables probed in L2) or 1 (staged in shared memory).  The rule, or with
 * svm_config.autotune the tuner, picks among the configurations left; a
 * query none fits returns SVM_E_UNSUPPORTED.  Every configuration computes
 * the same result.  No counterpart in the reference (its launch is fixed at
 * 1024 threads a block, com/cpp/com.cu:19-20). */
svm_status svm_pin_launch(svm_ctx* ctx, int rows_per_lane, int blocks_per_sm, int ring_stages, int tables_staged);

/* Narrows, in the same way, the compiled kernel's row-list form:
 * list_after -1 (any), 0..2 (after that filter step each warp's live rows
 * become a list and the later steps run over the list only), 3 (every step
 * runs over all rows, predicated) or 4 (a list after step 0, then steps 1
 * and 2 over it in one pass, both lookups in flight together).  Only some
 * plan shapes have the list forms compiled.  No counterpart in the
 * reference. */
svm_status svm_pin_list_after(svm_ctx* ctx, int list_after);

/* The same for the merged batch kernel of svm_run_batch / svm_batch_begin:
 * consumer_warps 0 (any), 28 or 24 of its 32 warps (the others look rows
 * up in the merged tables and issue the bulk copies), ring_stages 0 (any)
 * or 2..4 (at most the depth at which every descriptor of a launch still
 * fits).  With autotuning, the first launch of each batch shape times the
 * candidates left and keeps the fastest.  No counterpart in the reference. */
svm_status svm_pin_batch_launch(svm_ctx* ctx, int consumer_warps, int ring_stages);

/* The launch configuration of the context's last fused scan (the kernel
 * compiled for the plan's shape or the interpreted one, rows per consumer
 * lane, ring stages, table placement, the steps in order, grid and shared
 * memory) or merged batch launch (warp split, ring stages, queries per
 * launch), as a JSON object in `buf` (cut to cap - 1 bytes, NUL-terminated;
 * empty before the first scan).  No counterpart in the reference. */
svm_status svm_last_launch(svm_ctx* ctx, char* buf, unsigned long long cap);

/* ---- test hook ----------------------------------------------------------------
 * No counterpart in the reference.  Every wait of the fused scan kernel on an
 * mbarrier (the copy warp waiting for a free stage, a consumer warp waiting
 * for its tile) gives up after a number of polls, raises SVM_E_TIMEOUT and
 * exits, instead of hanging the GPU.  This sets that limit for the context's
 * later scans (wait_polls; 0 restores the default of 2^22 polls) and, with
 * stall_copies != 0, makes the copy warp issue no copies, so that every
 * consumer wait runs out: tests use it to check that the timeout is reported
 * and that the context stays usable afterwards. */
svm_status svm_test_device_wait(svm_ctx* ctx, unsigned int wait_polls, int stall_copies);

/* ---- profiling -------------------------------------------------------------- */
/* With profiling on, the library brackets each of its kernel launches with
 * CUDA events on its stream.  svm_profile_read reports, for kernel class k
 * (SVM_K_*), the number of launches and the summed event time in ms since the
 * last reset. */
enum { SVM_K_STAR = 0, SVM_K_SELECT = 1, SVM_K_BUILD = 2, SVM_K_FINALIZE = 3, SVM_K_BATCH = 4,
       SVM_K_OTHER = 5, SVM_K_LOAD = 6 /* text Loader parse */, SVM_K_COUNT = 7 };
svm_status svm_profile_enable(svm_ctx* ctx, int on);
svm_status svm_profile_reset(svm_ctx* ctx);
svm_status svm_profile_read(svm_ctx* ctx, int kernel_class, unsigned long long* launches,
                            double* total_ms);
/* Number of CUDA kernels this library has launched in the process so far. */
unsigned long long svm_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif /* SVM_CAPI_H_ */
