// Compiled scan shapes with a presence prefilter: the date + part join whose
// part probe (one-byte entries, 4 % of the keys present) is preceded by a
// one-bit table over the same keys, with the payload probe last -- alone,
// and with the query mix's price range before or after the bit probe; the
// bit and date tables staged in shared memory or probed in L2.
#include "kern_star_plan.cuh"

namespace svm {
using namespace plan;

extern const PlanEntry kPlansMix3[] = {
    SVM_PLAN_RL(AGG_DENSE_SMEM, l2(0), smem(2), l2(3), SC_NONE),
    SVM_PLAN_RL(AGG_DENSE_SMEM, smem(0), smem(2), l2(3), SC_NONE),
    SVM_PLAN_RL(AGG_DENSE_SMEM, l2(0), l2(2), l2(3), SC_NONE),
    SVM_PLAN_RL(AGG_DENSE_SMEM, R_, l2(0), smem(2), l2(3)),
    SVM_PLAN_RL(AGG_DENSE_SMEM, l2(0), R_, smem(2), l2(3)),
    SVM_PLAN_RL(AGG_DENSE_SMEM, R_, smem(0), smem(2), l2(3)),
    SVM_PLAN_RL(AGG_DENSE_SMEM, smem(0), R_, smem(2), l2(3)),
    SVM_PLAN_RL(AGG_DENSE_SMEM, R_, l2(0), l2(2), l2(3)),
    SVM_PLAN_RL(AGG_DENSE_SMEM, l2(0), R_, l2(2), l2(3)),
};
extern const int kPlansMix3Count = (int)(sizeof(kPlansMix3) / sizeof(kPlansMix3[0]));

}  // namespace svm
