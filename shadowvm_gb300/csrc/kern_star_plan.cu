// The fused scan compiled per plan shape.
//
// The interpreted scan (kern_star.cu) takes each filter step's kind, table
// layout, placement and entry width from its parameters at run time, so every
// step of every tile pays for the branches, the loads of those fields and
// entry arithmetic with a variable width.  The reference generates one kernel
// per pipeline instead, with the filter, join and reduce blocks spliced in as
// code (codegen/template.cpp:77-89 filled by codegen/codegen.cpp:100-229) and
// compiled at run time.  Here the same specialisation is done ahead of time:
// a plan's shape -- up to four steps, each a range test or a dense-table probe
// in shared memory or in L2 with its entry width, the aggregation mode and the
// rows each consumer lane owns -- is a template instantiation, and the
// planner's run-time values (column slots, bounds, key minimum, span, table
// addresses, payload fields) are read from the kernel parameters at
// compile-time offsets, which the compiler turns into constant-bank operands.
// A plan with another shape runs the interpreted kernel.
//
// Data movement and aggregation are the interpreted kernel's: a producer
// warp streams the tile's fact columns into a ring of shared-memory stages
// with 1-D bulk copies (completion on mbarriers, every wait bounded), eight
// consumer warps filter their rows step by step, predicated on the rows still
// live, and the survivors' operand words are buffered per warp and aggregated
// 32 rows at a time into shared-memory or global int64 slots.
//
// Rows per lane (4 or 8) set how many independent probe loads a lane has in
// flight per step, and the blocks each SM is to hold (the register budget
// the compiler gets) set how many warps wait on those loads at once.  Lane L
// owns rows 4L..4L+3 of each 128-row slice of its warp's rows, so every
// column read is one conflict-free 16-byte shared-memory load per slice.
// The entries kept for the aggregation are stored in the narrowest of 8-,
// 16- and 32-bit words that holds every probed table's entries; with 8-bit
// words the four-dimension star join's block fits three to an SM.
#include "kern_star_plan.cuh"

namespace svm {

using namespace plan;

namespace {

// Shapes the planner produces for the star-schema workloads, each with its
// small tables staged in shared memory and probed in L2:
//   date join + two fact ranges, SUM        [range, range, date(1-bit)]
//   date + part join, GROUP BY (year, brand) [part(8-bit), date(4-bit)]
//   date + customer + supplier join, GROUP BY three payloads
//                                            [date(4-bit), customer(4-bit), supplier(4-bit)]
const PlanEntry kPlans[] = {
    SVM_PLAN_R(AGG_SCALAR, R_, R_, smem(0), SC_NONE),
    SVM_PLAN_R(AGG_SCALAR, R_, R_, l2(0), SC_NONE),
    SVM_PLAN_R(AGG_DENSE_SMEM, l2(3), smem(2), SC_NONE, SC_NONE),
    SVM_PLAN_R(AGG_DENSE_SMEM, l2(3), l2(2), SC_NONE, SC_NONE),
    SVM_PLAN_R(AGG_DENSE_SMEM, smem(2), l2(2), l2(2), SC_NONE),
    SVM_PLAN_R(AGG_DENSE_SMEM, l2(2), l2(2), l2(2), SC_NONE),
};

}  // namespace

// The shapes of the batched query mix's queries run alone: the date join,
// the date + part join and the star join with a fact-side range on a fourth
// column in each place the planner may put it (kern_star_plan_mix.cu,
// kern_star_plan_mix2.cu; two files so that they compile in parallel).
extern const PlanEntry kPlansMix1[];
extern const int kPlansMix1Count;
extern const PlanEntry kPlansMix2[];
extern const int kPlansMix2Count;
// The date + part shapes with a presence prefilter (kern_star_plan_mix3.cu).
extern const PlanEntry kPlansMix3[];
extern const int kPlansMix3Count;
// Shapes whose later steps run over a list of the live rows
// (kern_star_plan_list.cu).
extern const PlanEntry kPlansList[];
extern const int kPlansListCount;

namespace {

int log2_exact(int v) {
  int b = 0;
  while ((1 << b) < v) b++;
  return (1 << b) == v ? b : -1;
}

bool plan_is_compilable(const StarParams& p) {
  if (p.nsteps > 4 || p.agg_words <= 0 || p.npost > 0) return false;
  if (p.agg != AGG_SCALAR && p.agg != AGG_DENSE_SMEM && p.agg != AGG_DENSE_GLOBAL) return false;
  for (int m = 0; m < p.nmetrics; m++)
    if (p.metrics[m].form == MF_PROG) return false;
  return true;
}

const PlanEntry* find_plan(const StarParams& p, int rows, int minb, int list_after) {
  if (!plan_is_compilable(p)) return nullptr;
  int code[4];
  for (int k = 0; k < 4; k++) {
    code[k] = star_plan_code(p, k);
    if (code[k] < 0) return nullptr;
  }
  auto match = [&](const PlanEntry& e) {
    return e.agg == p.agg && e.rows == rows && e.minb == minb && e.list_after == list_after &&
           e.s[0] == code[0] && e.s[1] == code[1] && e.s[2] == code[2] && e.s[3] == code[3];
  };
  for (const PlanEntry& e : kPlans)
    if (match(e)) return &e;
  for (int i = 0; i < kPlansMix1Count; i++)
    if (match(kPlansMix1[i])) return &kPlansMix1[i];
  for (int i = 0; i < kPlansMix2Count; i++)
    if (match(kPlansMix2[i])) return &kPlansMix2[i];
  for (int i = 0; i < kPlansMix3Count; i++)
    if (match(kPlansMix3[i])) return &kPlansMix3[i];
  for (int i = 0; i < kPlansListCount; i++)
    if (match(kPlansList[i])) return &kPlansList[i];
  return nullptr;
}

}  // namespace

int star_plan_code(const StarParams& p, int k) {
  if (k >= p.nsteps) return SC_NONE;
  const Step& st = p.steps[k];
  if (st.kind == STEP_RANGE) return SC_RANGE;
  if (st.kind != STEP_PROBE || st.layout != LAYOUT_DENSE) return -1;
  const int lg = log2_exact(st.entry_bits);
  if (lg < 0 || lg > 5) return -1;
  const bool ranged = !(st.lo == INT_MIN && st.hi == INT_MAX);
  return (st.smem_word_off >= 0 ? SC_SMEM : SC_L2) | lg << 2 | (ranged ? 32 : 0);
}

bool star_plan_available(const StarParams& p, int rows_per_lane, int min_blocks, int list_after) {
  return find_plan(p, rows_per_lane, min_blocks, list_after) != nullptr;
}

size_t star_plan_smem_bytes(const StarParams& p, int rows_per_lane) {
  const size_t tr = (size_t)kConsumerWarps * plan_warp_rows(rows_per_lane);
  int bits = 0;
  for (int k = 0; k < p.nsteps; k++)
    if (p.steps[k].kind == STEP_PROBE && p.steps[k].entry_bits > bits) bits = p.steps[k].entry_bits;
  size_t b = (size_t)p.nstages * p.ncols * tr * 4;
  b += plan_list_bytes(p.ndims, rows_per_lane, plan_entry_bytes(bits)) * kConsumerWarps;
  b += (size_t)((p.smem_table_words + 3) & ~3) * 4;
  if (p.agg == AGG_DENSE_SMEM) b += (size_t)p.ngroups * (8 * p.nmetrics + 4);
  b = (b + 15) & ~size_t(15);
  b += (size_t)kConsumerWarps * kAggCap * p.agg_words * 4;
  return b;
}

int star_plan_blocks_per_sm(const StarParams& p, int rows_per_lane, int min_blocks, int list_after, size_t smem) {
  const PlanEntry* e = find_plan(p, rows_per_lane, min_blocks, list_after);
  if (!e) return 0;
  if (allow_dynamic_smem(e->fn, 210 * 1024) != cudaSuccess) return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, e->fn, kStarThreads, smem) != cudaSuccess) return 0;
  return per_sm;
}

int star_plan_grid_size(const StarParams& p, int rows_per_lane, int min_blocks, int list_after, size_t smem) {
  int per_sm = star_plan_blocks_per_sm(p, rows_per_lane, min_blocks, list_after, smem);
  if (per_sm < 1) per_sm = 1;
  const long long tr = (long long)kConsumerWarps * plan_warp_rows(rows_per_lane);
  long long tiles = (p.row_end - (p.row_begin & ~3ll) + tr - 1) / tr;
  const long long cap = (long long)num_sms() * per_sm;
  if (tiles < 1) tiles = 1;
  return (int)(tiles < cap ? tiles : cap);
}

cudaError_t launch_star_plan(const StarParams& p, int rows_per_lane, int min_blocks, int list_after, int grid,
                             size_t smem, cudaStream_t s) {
  const PlanEntry* e = find_plan(p, rows_per_lane, min_blocks, list_after);
  if (!e) return cudaErrorInvalidValue;
  note_launch();
  void* args[] = {const_cast<StarParams*>(&p)};
  return cudaLaunchKernel(e->fn, dim3(grid), dim3(kStarThreads), args, smem, s);
}

}  // namespace svm
