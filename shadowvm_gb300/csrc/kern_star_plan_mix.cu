// Compiled scan shapes of the batched query mix, run one query per launch:
// the date join with a fact-side price range (three ranges and the date
// table, the price range before or after the date probe) and the date + part
// join with a price range (before or after the part probe), each with the
// small tables staged in shared memory and probed in L2.
#include "kern_star_plan.cuh"

namespace svm {
using namespace plan;

extern const PlanEntry kPlansMix1[] = {
    SVM_PLAN_RL(AGG_SCALAR, R_, R_, R_, smem(0)),
    SVM_PLAN_RL(AGG_SCALAR, R_, R_, smem(0), R_),
    SVM_PLAN_RL(AGG_SCALAR, R_, R_, R_, l2(0)),
    SVM_PLAN_RL(AGG_SCALAR, R_, R_, l2(0), R_),
    SVM_PLAN_RL(AGG_DENSE_SMEM, R_, l2(3), smem(2), SC_NONE),
    SVM_PLAN_RL(AGG_DENSE_SMEM, l2(3), R_, smem(2), SC_NONE),
    SVM_PLAN_RL(AGG_DENSE_SMEM, R_, l2(3), l2(2), SC_NONE),
    SVM_PLAN_RL(AGG_DENSE_SMEM, l2(3), R_, l2(2), SC_NONE),
};
extern const int kPlansMix1Count = (int)(sizeof(kPlansMix1) / sizeof(kPlansMix1[0]));

}  // namespace svm
