// Host-callable launchers for the library's CUDA kernels.  Every launcher
// enqueues on `stream` and returns the launch's cudaError_t; none synchronizes.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "svm_internal.h"

namespace svm {

// SM count of the current device (cached per device).
int num_sms();
// Raises `fn`'s dynamic shared-memory limit to `bytes` on the current device
// (once per device and kernel; thread-safe).
cudaError_t allow_dynamic_smem(const void* fn, int bytes);
// Process-wide count of kernel launches (every <<<>>> site calls this).
void note_launch(int n = 1);
unsigned long long launches_total();

// ---- utilities (kern_util.cu)
cudaError_t launch_gen_uniform(int32_t* out, unsigned long long n, unsigned long long seed,
                               unsigned long long stream_id, unsigned long long row0, int lo, int hi,
                               const int32_t* lookup, cudaStream_t s);
// min/max of n int32 values into out[0] (min) out[1] (max); out must be preset
// to {INT_MAX, INT_MIN}.
cudaError_t launch_minmax(const int32_t* in, unsigned long long n, int32_t* out, cudaStream_t s);
// Exclusive prefix sum of n uint32 values into n+1 uint64 values (out[n] = total).
// `tmp` needs scan_tmp_words(n) uint64 words.
size_t scan_tmp_words(unsigned long long n);
cudaError_t launch_exclusive_scan(const uint32_t* in, unsigned long long n, unsigned long long* out,
                                  unsigned long long* tmp, cudaStream_t s);
// Inclusive running maximum of n int32 values (in place allowed).
cudaError_t launch_inclusive_max(const int32_t* in, unsigned long long n, int32_t* out,
                                 int32_t* tmp, cudaStream_t s);
size_t max_tmp_words(unsigned long long n);

// Copies `words` 32-bit words from `src` to dst + dst_word for every segment.
struct Segment {
  const uint32_t* src;
  unsigned long long dst_word;
  unsigned long long words;
};
cudaError_t launch_gather_segments(const Segment* segs, int nseg, uint32_t* dst, cudaStream_t s);
// flags[codes[i]] = 1 for i < n (flags zeroed by the caller; every code indexes flags).
cudaError_t launch_mark_codes(const int32_t* codes, unsigned long long n, uint32_t* flags, cudaStream_t s);
// out[i] = lut[in[i]] for i < n (in == out allowed); every in[i] indexes lut.
cudaError_t launch_lut_gather(const int32_t* in, unsigned long long n, const int32_t* lut, int32_t* out,
                              cudaStream_t s);

// ---- select pipelines (kern_dim.cu)
// Pass 1: per-tile counts of rows passing the conjuncts; pass 2: order-preserving write.
unsigned long long select_tiles(long long nrows);
cudaError_t launch_select_count(const SelectParams& p, cudaStream_t s);
cudaError_t launch_select_write(const SelectParams& p, cudaStream_t s);

// ---- dimension tables (kern_dim.cu)
struct BuildInput {
  const int32_t* key;               // key column, rows [0, n)
  long long n;
  int npay;
  const int32_t* pay[kMaxKeys + 2 * kMaxMetrics];
  const uint8_t* dropped;           // rows to leave out (may be null)
};

// Reference-table emulation: marks in `dropped` (n bytes, zeroed by the call)
// every row the sequential 10-step capped insert over ht_size slots
// (com/cpp/com.hpp:168-174, cpu-runtime.hpp:80-91) leaves out.
// `scratch` must hold refcompat_scratch_bytes(n, ht_size) bytes.
size_t refcompat_scratch_bytes(long long n, unsigned ht_size);
cudaError_t launch_refcompat(const int32_t* key, long long n, unsigned ht_size, int signed_char,
                             uint8_t* dropped, void* scratch, cudaStream_t s);

// Stats of the rows that will be inserted: out[0..1] key min/max, out[2+2f..3+2f]
// payload f min/max, out[2+2*npay] = number of rows inserted (as int32 bit pattern).
cudaError_t launch_build_stats(const BuildInput& in, int32_t* out, cudaStream_t s);

// Dense table: `owner` (span int32, scratch) and `words` (table_words) are
// written; rows collide on a key -> the lowest row wins.
cudaError_t launch_build_dense(const BuildInput& in, const DimDesc& d, int32_t* owner,
                               uint32_t* words, cudaStream_t s);
// Hash table: `slots` (cap uint64, scratch) then `words` (2*cap).
cudaError_t launch_build_hash(const BuildInput& in, const DimDesc& d, unsigned long long* slots,
                              uint32_t* words, int* error, cudaStream_t s);

// ---- fused star query (kern_star.cu)
cudaError_t launch_star(const StarParams& p, int grid, int block, size_t smem, cudaStream_t s);
int star_block_size();
int star_blocks_per_sm(const StarParams& p, size_t smem);
int star_grid_size(const StarParams& p, size_t smem);
size_t star_smem_bytes(const StarParams& p);
// The fused scan compiled per plan shape (kern_star_plan.cu): available for
// plans of at most four steps (ranges and dense-table probes), no bytecode,
// and an instantiated shape; rows_per_lane 4 (for 3 or 4 blocks per SM) or
// 8 (for 2 blocks per SM), min_blocks the blocks per SM it is compiled for,
// list_after the step after which the later steps run over a list of the
// warp's live rows (3: none do; 4: after step 0, with steps 1 and 2 in one
// pass over the list).
int star_plan_code(const StarParams& p, int k);  // step k's code (-1: not compilable)
bool star_plan_available(const StarParams& p, int rows_per_lane, int min_blocks, int list_after);
size_t star_plan_smem_bytes(const StarParams& p, int rows_per_lane);
int star_plan_blocks_per_sm(const StarParams& p, int rows_per_lane, int min_blocks, int list_after, size_t smem);
int star_plan_grid_size(const StarParams& p, int rows_per_lane, int min_blocks, int list_after, size_t smem);
cudaError_t launch_star_plan(const StarParams& p, int rows_per_lane, int min_blocks, int list_after, int grid,
                             size_t smem, cudaStream_t s);
// Compact non-empty groups in key order: writes keys (nkeys int32 columns),
// metric columns (int64 or int32 per `wide`), and out_count.
cudaError_t launch_finalize_dense(const StarParams& p, int32_t* const* key_out, void* const* met_out,
                                  const int* wide, unsigned long long* flags_tmp,
                                  unsigned long long* scan_tmp, unsigned long long* out_count,
                                  cudaStream_t s);

// ---- batched star queries (kern_star.cu)
struct BatchOut {
  int32_t* key[kMaxKeys];
  long long* sum[kMaxMetrics];
};
size_t batch_smem_bytes(const BatchParams& b);
int batch_grid_size(const BatchParams& b, size_t smem);
cudaError_t launch_batch(const BatchParams& b, int grid, size_t smem, cudaStream_t s);
// out == nullptr: flags (one per group of every query) and their exclusive
// scan into pos (total + 1 entries); else write each flagged group's keys and
// sums at pos into `out`.
// out[i] = pos[Q[i].group_off] (the first result row of query i), out[nq] = pos[total].
cudaError_t launch_batch_bounds(const BatchQuery* Q, int nq, const unsigned long long* pos, unsigned long long total,
                                unsigned long long* out, cudaStream_t s);
cudaError_t launch_batch_finalize(const BatchQuery* Q, int nq, const unsigned long long* slots,
                                  unsigned long long total, uint32_t* flags, unsigned long long* pos,
                                  unsigned long long* scan_tmp, const BatchOut* out, cudaStream_t s);

// ---- text loader (kern_load.cu)
struct LoadPos {                    // a chunk's rows and trailing fields (scan element)
  unsigned long long rows;
  unsigned int cols;
  unsigned int has;                 // the chunk holds a row delimiter
};
constexpr int kLoadMaxCols = 64;
struct LoadOut {
  int ncols;
  unsigned long long nrows;
  void* col[kLoadMaxCols];
  uint8_t wide[kLoadMaxCols];       // 1: int64 column
};
size_t load_chunks(unsigned long long bytes);
size_t load_scratch_entries(unsigned long long bytes);  // LoadPos entries
// Chunk summaries and their exclusive scan into `scratch` (text: `bytes`
// bytes of device memory, any alignment).
cudaError_t launch_load_index(const uint8_t* text, unsigned long long bytes, char cd, char rd, LoadPos* scratch,
                              cudaStream_t s);
const LoadPos* load_total(const LoadPos* scratch, unsigned long long bytes);  // rows = row delimiters
cudaError_t launch_load_parse(const uint8_t* text, unsigned long long bytes, char cd, char rd,
                              const LoadPos* scratch, const LoadOut& out, int* error, cudaStream_t s);

// ---- merged-probe batch (kern_mbatch.cu)
cudaError_t launch_merge_build(const MergeBuild& m, uint32_t* out, cudaStream_t s);
size_t mbatch_smem_bytes(const BatchParams& b);
int mbatch_grid_size(const BatchParams& b, size_t smem);  // 0: the block does not fit an SM
void mbatch_attributes(int* regs, int* max_threads, size_t* static_smem);
cudaError_t launch_mbatch(const BatchParams& b, int grid, size_t smem, cudaStream_t s);

}  // namespace svm
