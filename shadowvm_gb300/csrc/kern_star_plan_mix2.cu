// Compiled scan shapes of the batched query mix, run one query per launch:
// the four-dimension star join with a fact-side price range before the date
// probe, between it and the L2 probes, or last, with the date table staged
// in shared memory or probed in L2.
#include "kern_star_plan.cuh"

namespace svm {
using namespace plan;

extern const PlanEntry kPlansMix2[] = {
    SVM_PLAN_RL(AGG_DENSE_SMEM, R_, smem(2), l2(2), l2(2)),
    SVM_PLAN_RL(AGG_DENSE_SMEM, smem(2), R_, l2(2), l2(2)),
    SVM_PLAN_RL(AGG_DENSE_SMEM, smem(2), l2(2), l2(2), R_),
    SVM_PLAN_RL(AGG_DENSE_SMEM, R_, l2(2), l2(2), l2(2)),
    SVM_PLAN_RL(AGG_DENSE_SMEM, l2(2), R_, l2(2), l2(2)),
    SVM_PLAN_RL(AGG_DENSE_SMEM, l2(2), l2(2), l2(2), R_),
};
extern const int kPlansMix2Count = (int)(sizeof(kPlansMix2) / sizeof(kPlansMix2[0]));

}  // namespace svm
