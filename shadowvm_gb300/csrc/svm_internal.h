// Internal definitions shared by the host planner (C++) and the kernels (CUDA).
// Everything that crosses into a kernel is a plain struct passed by value.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace svm {

// ---------------------------------------------------------------- limits
constexpr int kMaxSteps = 8;       // fact columns one fused scan touches
constexpr int kMaxDims = 4;        // joined objects per query (join_index[8] in the reference)
constexpr int kMaxKeys = 3;        // ReduceTask handles 0..3 keys (core/pipeline.cu:373-471)
constexpr int kMaxMetrics = 3;     // ... and 1..3 metrics
constexpr int kMaxProg = 48;       // bytecode ops per expression
constexpr int kMaxPost = 4;        // residual predicates evaluated after the steps
constexpr int kSmemTableBytes = 64 * 1024;  // dimension tables staged in shared memory per block
constexpr int kSmemAggBytes = 64 * 1024;    // per-block group table in shared memory
constexpr int kHashRate = 5;       // com/cpp/define.hpp:29

// ---------------------------------------------------------------- device errors
// Error codes a kernel may raise in its error word (StarParams::error,
// SelectParams::error, ...); the first one raised is kept.
enum DevError : int { DERR_NONE = 0, DERR_DIV0 = 1, DERR_HASH_FULL = 2, DERR_KEY_RANGE = 3,
                      DERR_TIMEOUT = 4, DERR_LOAD_ITEM = 5 };

// ---------------------------------------------------------------- expressions
// Stack-machine bytecode for int32 C expressions (wrapping arithmetic, C
// truncating division, comparisons yield 0/1, && || short-circuit).
enum ExprOp : uint8_t {
  X_OPND = 0,   // push operand[arg]
  X_CONST,      // push constant[arg]
  X_NEG, X_NOT, X_BNOT,
  X_ADD, X_SUB, X_MUL, X_DIV, X_MOD, X_SHL, X_SHR,
  X_LT, X_LE, X_GT, X_GE, X_EQ, X_NE, X_BAND, X_BXOR, X_BOR,
  X_NORM,       // top = (top != 0)
  X_JZ_KEEP,    // if top == 0: jump to arg (keep the 0) else pop
  X_JNZ_ONE,    // if top != 0: top = 1, jump to arg; else pop
  X_JZ_POP,     // pop; if it was 0 jump to arg
  X_JMP,
};

struct Prog {
  uint8_t n;                 // ops
  uint8_t op[kMaxProg];
  uint8_t arg[kMaxProg];
  int32_t konst[16];
};

// Operand reference: a fact column (staged column slot) or a payload field of
// a probed dimension.
struct Operand {
  int8_t slot;     // field < 0: staged fact column slot; else dimension index
  int8_t field;    // -1: fact value; >= 0: payload field of dimension `slot`
};

// ---------------------------------------------------------------- dimension tables
enum TableLayout : int { LAYOUT_DENSE = 0, LAYOUT_HASH = 1 };

// A built dimension table.  DENSE: entry for key k at bit offset
// (k - key_min) * entry_bits of `words`; bit 0 of the entry is "present",
// payload fields follow.  HASH: `cap` slots of {int key, uint32 payload word}
// (payload word bit 0 = present), linear probing from mix32(key) & (cap - 1).
struct PayloadField {
  const int32_t* col;  // non-null: value = col[(entry >> shift) & mask] (row-index payload)
  int32_t min;         // else:     value = min + ((entry >> shift) & mask)
  uint8_t shift;
  uint8_t bits;
};

struct DimDesc {
  int layout;
  const uint32_t* words;     // global table
  int smem_word_off;         // >= 0: staged into shared memory at this word offset
  int entry_bits;            // DENSE: 1,2,4,8,16,32
  int32_t key_min;
  uint32_t span;             // DENSE: key range; HASH: capacity (power of two)
  uint32_t table_words;      // 32-bit words
  int npay;
  PayloadField pay[kMaxKeys + 2 * kMaxMetrics];
};

__host__ __device__ inline uint32_t mix32(uint32_t x) {
  // murmur3 fmix32 (Appleby, public domain)
  x ^= x >> 16; x *= 0x85ebca6bu; x ^= x >> 13; x *= 0xc2b2ae35u; x ^= x >> 16;
  return x;
}

// ---------------------------------------------------------------- fused star query
enum StepKind : int { STEP_RANGE = 0, STEP_PROBE = 1, STEP_MPROBE = 2 };

struct Step {
  int kind;
  int col;          // staged fact column slot (index into StarParams::cols)
  int32_t lo, hi;   // keep lo <= v <= hi (PROBE steps too; full range = no check)
  int dim;          // STEP_PROBE: dimension index
  // STEP_PROBE: the probed table, copied from dims[dim] so a step needs no
  // second indirection.
  int layout;
  int smem_word_off;
  const uint32_t* words;
  int32_t key_min;
  uint32_t span;
  int entry_bits;
  // 1: evaluate the next step in the same pass (its lookups in flight with
  // this step's), set by the planner for consecutive global-table probes.
  int fuse_next;
  // STEP_MPROBE (merged batch): the table's entry sits at bit `mbit` of merged
  // probe word `mword`; `col` < 0 when no key range is folded in.
  int mword, mbit;
};

// A value the aggregation reads: a staged fact column, or a payload field of a
// probed dimension (bit-packed, or a row index into `col`), plus `base`:
//   fact:   v = fact[slot] + base
//   packed: v = ((pw[dim] >> shift) & mask) + base
//   gather: v = col[(pw[dim] >> shift) & mask] + base
struct Extract {
  int dim;          // -1: fact column `slot`
  int slot;
  uint32_t shift, mask;
  int32_t base;
  const int32_t* col;
};

// The scan streams every fact column the query reads through a ring of
// shared-memory stages: tiles of kTileRows rows, one bulk copy per column.
constexpr int kConsumerWarps = 8;
constexpr int kWarpRows = 32 * 4;                     // 4 rows per consumer lane
constexpr int kTileRows = kConsumerWarps * kWarpRows;
constexpr int kStages = 4;                            // at most; StarParams::nstages in use

enum MetricForm : int { MF_OPND = 0, MF_ADD = 1, MF_SUB = 2, MF_MUL = 3, MF_PROG = 4 };

struct Metric {
  int form;
  Operand a, b;     // MF_OPND uses a; binary forms use a (op) b
  Extract xa, xb;   // the same operands, flattened (base = payload min)
  Prog prog;        // MF_PROG: operands index StarParams::opnds
};

enum AggMode : int { AGG_SCALAR = 0, AGG_DENSE_SMEM = 1, AGG_DENSE_GLOBAL = 2, AGG_HASH_GLOBAL = 3 };

struct StarParams {
  const int32_t* cols[kMaxSteps];   // fact column base pointers (row 0 of the base allocation)
  int ncols;                        // staged columns (slots 0 .. ncols-1 of cols)
  int host_late;                    // 1: the late columns are in page-locked host memory (plain loads)
  int nlate;                        // late columns, slots ncols .. ncols+nlate-1: never staged; a
                                    // surviving row's value is read from global memory (compiled scan)
  int nstages;                      // ring depth (2..kStages)
  long long row_begin, row_end;     // rows [row_begin, row_end) of the base columns
  int nsteps;
  Step steps[kMaxSteps];
  int ndims;
  DimDesc dims[kMaxDims];
  int npost;                        // residual predicates (bytecode over opnds)
  Prog post[kMaxPost];
  int nopnd;
  Operand opnds[16];                // operand table for bytecode programs
  int nkeys;
  Operand keys[kMaxKeys];
  int32_t kmin[kMaxKeys];
  uint32_t krange[kMaxKeys];
  unsigned long long kstride[kMaxKeys];
  Extract kx[kMaxKeys];             // key q's offset in its range: extract with base folded in
  int nmetrics;
  Metric metrics[kMaxMetrics];
  int agg;
  unsigned long long ngroups;       // dense: product of ranges; hash: capacity
  unsigned long long* sums;         // [nmetrics][ngroups] int64 (two's complement)
  unsigned long long* counts;       // [ngroups]
  unsigned long long* hkeys;        // AGG_HASH_GLOBAL: packed keys per slot (~0 = empty)
  int smem_table_words;             // words of dimension tables staged in shared memory
  int* error;                       // device error word (division by zero, hash overflow)
  // Bounded waits: polls of an mbarrier before the kernel gives up with
  // DERR_TIMEOUT (0: the default, 2^22).  stall_copies != 0 (a test hook)
  // makes the copy warp issue nothing, so every consumer wait runs out.
  uint32_t wait_polls;
  int stall_copies;
  // Deferred aggregation (plans without bytecode): a surviving row's operand
  // words -- the probe words and fact values its keys and metrics read -- are
  // appended to a per-warp buffer and aggregated 32 rows at a time.
  int agg_words;                    // words per buffered row; 0 = aggregate in place
  int8_t agg_src[kMaxDims + kMaxSteps];  // word k: probe word of dim d (0..3), fact slot 8 + s, or
                                         // kAggRowWord: the row's index in the base columns
  int8_t agg_step[kMaxDims + kMaxSteps]; // word k: index of the step probing that dim, or fact slot 8 + s
  Extract kx_e[kMaxKeys], xa_e[kMaxMetrics], xb_e[kMaxMetrics];  // the extractors over those words
};

// ---------------------------------------------------------------- batched star queries
// Many fact pipelines over one resident fact table in one persistent launch:
// the union of their fact columns is streamed once, and every query whose row
// range covers a tile runs its own steps and aggregation on the staged tile.
constexpr int kMaxBatchCols = 12;

// Merged probe tables (batch mode).  The dense tables that a batch's queries
// probe with the same fact column are concatenated entry by entry: for key k
// the merged table holds `words` 32-bit words; word 0 starts with the present
// bits of the group's tables (table i of the group at bit i), and each table's
// payload bits sit at a fixed word and bit after them.  One lookup per row and
// group then serves every query of the batch that probes any of those tables.
constexpr int kMaxProbeGroups = 8;
constexpr int kMaxMergedWords = 16;   // merged words per row over all groups
constexpr int kMBatchWarps = 28;      // consumer warps of the merged batch kernel (the rule's split)

struct ProbeGroup {
  int col;                  // union fact column slot of the key
  int words;                // 1..8 words per key
  int32_t key_min;
  uint32_t span;
  int word_off;             // first merged word of the group in the per-row layout
  const uint32_t* table;    // span * words
};

struct MergeSrc {           // one dense table placed into a merged table
  const uint32_t* words;
  int32_t key_min;
  uint32_t span;
  int entry_bits;
  int present_bit;          // in word 0
  int pay_word, pay_bit;    // the entry's payload (entry >> 1) ...
  int pay_bits;             // ... of this many bits (0: none)
  int shared;               // 1: the payload goes to the group's shared field as payload + val_off
  int32_t val_off;
};

constexpr int kMaxMergeSrcs = 32;
struct MergeBuild {
  int32_t key_min;
  uint32_t span;
  int words;
  int nsrc;
  unsigned int* conflict;   // bit i: source i disagreed with the shared field at a key
  MergeSrc src[kMaxMergeSrcs];
};

// The merged kernel's own compact query descriptor, held in shared memory
// for the whole launch.  Probe steps are bit tests against per-tile row
// bitmaps of the merged tables' present bits (table slots 0..63); range
// steps test staged fact values.
constexpr int kMaxMergedTables = 64;
constexpr int kMaxMRanges = 6;
constexpr int kMaxGatherCols = 15;

struct MExtract {       // 12 bytes
  int8_t src;           // -1: fact column `slot`; else the group's first merged word
  uint8_t slot;         // fact column slot, or the word within the group's entry
  uint8_t shift;
  uint8_t sg;           // merged: words per row (low 4 bits); gather column + 1 (high 4 bits, 0 = none)
  uint32_t mask;
  int32_t base;         // value = field (or gcol[field]) + base
};

struct MQuery {         // 240 bytes
  long long row_begin, row_end;
  unsigned long long slot_off;
  uint32_t ngroups;
  uint32_t gmask;                   // probe groups whose words it reads
  uint8_t nprobe, nrange, nkeys, nmetrics;
  uint8_t mform[kMaxMetrics];
  uint8_t pad0;
  uint8_t probe_tab[kMaxSteps];
  uint8_t range_col[kMaxMRanges];
  uint8_t pad1[2];
  int32_t range_lo[kMaxMRanges], range_hi[kMaxMRanges];
  uint32_t krange[kMaxKeys], kstride[kMaxKeys];
  MExtract kx[kMaxKeys], xa[kMaxMetrics], xb[kMaxMetrics];
  uint32_t pad2;
};

struct BatchQuery {                 // in device memory, one per query
  long long row_begin, row_end;     // base rows this query reads
  int nsteps;
  Step steps[kMaxSteps];            // col = union column slot; tables in global memory
  int nkeys;
  Extract kx[kMaxKeys];
  int32_t kmin[kMaxKeys];
  uint32_t krange[kMaxKeys];
  uint32_t kstride[kMaxKeys];
  int nmetrics;
  int mform[kMaxMetrics];
  Extract xa[kMaxMetrics], xb[kMaxMetrics];
  unsigned long long ngroups;
  unsigned long long slot_off;      // sums at slots + slot_off, counts after nmetrics * ngroups
  unsigned long long group_off;     // this query's first group in the batch's group numbering
  uint32_t gmask;                   // merged probe groups the query reads
};

struct BatchParams {
  const int32_t* cols[kMaxBatchCols];
  int ncols;
  int nstages;
  long long row_begin, row_end;     // union of the queries' ranges (base rows)
  const BatchQuery* queries;
  int nqueries;
  unsigned long long* slots;
  unsigned long long* tile_counter; // zeroed before the launch
  int* error;
  int nprobe;                       // merged batch kernel: probe groups
  ProbeGroup probe[kMaxProbeGroups];
  int nmwords;                      // merged words per row
  const MQuery* mq;                 // merged kernel: descriptors (nqueries)
  int gtab0[kMaxProbeGroups + 1];   // group g's tables are slots [gtab0[g], gtab0[g + 1]), in present-bit order
  const int32_t* gcol[kMaxGatherCols];  // row-index payload columns (MExtract::sg high bits)
  int cwarps;                       // merged kernel: consumer warps of the 32 (28 or 24; 0 = 28)
};

// Fills the flattened copies (Step table fields, Extract descriptors) from the
// structured plan; called on the host once the plan is complete.
// Aggregation word code of a surviving row's index (late columns gather by it).
constexpr int kAggRowWord = 16;

inline Extract make_extract(const StarParams& P, Operand o, int32_t adjust) {
  Extract x{};
  if (o.field < 0 && o.slot >= P.ncols) {
    // A late column: gathered from global memory by the row word (the
    // buffered-row extractor makes dim the row word's index).
    x.dim = -2;
    x.slot = o.slot;
    x.shift = 0;
    x.mask = 0xFFFFFFFFu;
    x.col = P.cols[o.slot];
    x.base = adjust;
    return x;
  }
  if (o.field < 0) {
    x.dim = -1;
    x.slot = o.slot;
    x.base = adjust;
    return x;
  }
  const PayloadField& f = P.dims[o.slot].pay[o.field];
  x.dim = o.slot;
  x.slot = 0;
  x.shift = f.bits ? f.shift : 0u;
  x.mask = f.bits >= 32 ? 0xFFFFFFFFu : (1u << f.bits) - 1u;
  x.col = f.col;
  x.base = (int32_t)((uint32_t)(f.col ? 0 : f.min) + (uint32_t)adjust);
  return x;
}

// Late materialisation (compiled scan only): fact columns that no filter
// step reads -- only the surviving rows' keys and metrics -- are not
// staged; they move behind the staged slots (nlate of them) and each
// survivor's value is read from global memory by its row index.  Call before
// flatten_plan, on a plan whose columns are all staged.
inline void apply_late_columns(StarParams& P) {
  bool by_step[kMaxSteps] = {};
  for (int k = 0; k < P.nsteps; k++) by_step[P.steps[k].col] = true;
  if (P.npost > 0 || P.row_end >= (1ll << 32)) return;  // residual programs read staged operands; row words are 32-bit
  int order[kMaxSteps], remap[kMaxSteps], n = 0;
  for (int c = 0; c < P.ncols; c++)
    if (by_step[c]) order[n++] = c;
  const int staged = n;
  for (int c = 0; c < P.ncols; c++)
    if (!by_step[c]) order[n++] = c;
  if (staged == P.ncols || staged == 0) return;
  const int32_t* cols[kMaxSteps];
  for (int i = 0; i < P.ncols; i++) {
    remap[order[i]] = i;
    cols[i] = P.cols[order[i]];
  }
  for (int i = 0; i < P.ncols; i++) P.cols[i] = cols[i];
  for (int k = 0; k < P.nsteps; k++) P.steps[k].col = remap[P.steps[k].col];
  auto fix = [&](Operand& o) {
    if (o.field < 0) o.slot = (int8_t)remap[o.slot];
  };
  for (int q = 0; q < P.nkeys; q++) fix(P.keys[q]);
  for (int m = 0; m < P.nmetrics; m++) {
    fix(P.metrics[m].a);
    if (P.metrics[m].form != MF_OPND) fix(P.metrics[m].b);
  }
  for (int i = 0; i < P.nopnd; i++) fix(P.opnds[i]);
  P.nlate = P.ncols - staged;
  P.ncols = staged;
}

inline void flatten_plan(StarParams& P) {
  for (int k = 0; k < P.nsteps; k++) {
    Step& st = P.steps[k];
    st.fuse_next = 0;
    if (st.kind != STEP_PROBE) continue;
    const DimDesc& D = P.dims[st.dim];
    st.layout = D.layout;
    st.smem_word_off = D.smem_word_off;
    st.words = D.words;
    st.key_min = D.key_min;
    st.span = D.span;
    st.entry_bits = D.entry_bits;
  }
  // Issuing two consecutive global-table probes together (one round trip
  // instead of two) measured slower on the 600 M-row star query, both over
  // selection vectors (5.2 vs 4.2 ms) and predicated per row (5.05 vs 4.67
  // ms): the second probe then runs for every row the first would have
  // removed.  Steps run one after another; fuse_next stays 0.
  for (int q = 0; q < P.nkeys; q++) P.kx[q] = make_extract(P, P.keys[q], (int32_t)(0u - (uint32_t)P.kmin[q]));
  bool prog = P.npost > 0;
  for (int m = 0; m < P.nmetrics; m++) {
    Metric& M = P.metrics[m];
    if (M.form == MF_PROG) {
      prog = true;
      continue;
    }
    M.xa = make_extract(P, M.a, 0);
    if (M.form != MF_OPND) M.xb = make_extract(P, M.b, 0);
  }
  // The buffered row's words: first the table entry of every probe step
  // whose entries carry a payload, in step order (the compiled kernel copies
  // these with compile-time word indices), then each further dim or fact
  // slot an extractor reads.
  P.agg_words = 0;
  if (prog) return;
  for (int s = 0; s < P.nsteps; s++) {
    const Step& st = P.steps[s];
    if (st.kind != STEP_PROBE || st.entry_bits <= 1) continue;
    int k = 0;
    while (k < P.agg_words && P.agg_src[k] != st.dim) k++;
    if (k == P.agg_words) P.agg_src[P.agg_words++] = (int8_t)st.dim;
  }
  auto word_of = [&](Extract x) {
    const int8_t code = (int8_t)(x.dim >= 0 ? x.dim : x.dim == -2 ? kAggRowWord : 8 + x.slot);
    int k = 0;
    while (k < P.agg_words && P.agg_src[k] != code) k++;
    if (k == P.agg_words) P.agg_src[P.agg_words++] = code;
    if (x.dim >= 0 || x.dim == -2)
      x.dim = k;
    else
      x.slot = k;
    return x;
  };
  for (int q = 0; q < P.nkeys; q++) P.kx_e[q] = word_of(P.kx[q]);
  for (int m = 0; m < P.nmetrics; m++) {
    const Metric& M = P.metrics[m];
    P.xa_e[m] = word_of(M.xa);
    if (M.form != MF_OPND) P.xb_e[m] = word_of(M.xb);
  }
  for (int k = 0; k < P.agg_words; k++) {
    const int code = P.agg_src[k];
    P.agg_step[k] = (int8_t)code;
    if (code < 8)
      for (int s = 0; s < P.nsteps; s++)
        if (P.steps[s].kind == STEP_PROBE && P.steps[s].dim == code) P.agg_step[k] = (int8_t)s;
  }
}

// ---------------------------------------------------------------- select (Map) pipelines
// Operands 0..ncols_in-1 are source columns; with joins, operands
// ncols_in..nopnd-1 are payload fields of the joined tables (dop[k]: table
// and field), read once every join of the row has matched.
struct SelectParams {
  const int32_t* cols[16];
  int ncols_in;
  int nopnd;                        // ncols_in + joined payload operands
  Operand dop[16];                  // operand ncols_in + k: {table, payload field}
  int ndims;                        // joins, probed in order after the conjuncts
  DimDesc dims[kMaxDims];
  int join_opnd[kMaxDims];          // operand holding join d's key (a source column)
  long long nrows;
  int npred;                        // conjunct programs over input columns (operand = column)
  Prog pred[4];
  int nout;
  Prog proj[16];                    // one program per output column
  int32_t* out[16];
  const unsigned long long* tile_offset;  // exclusive prefix of per-tile pass counts
  unsigned int* tile_count;
  unsigned long long* bulk0_count;  // passing rows among source rows [0, bulk0_rows)
  long long bulk0_rows;
  int* error;
};

}  // namespace svm
