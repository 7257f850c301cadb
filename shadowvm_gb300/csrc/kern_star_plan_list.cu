// Compiled scans whose later filter steps run over a list of the warp's live
// rows (kern_star_plan.cuh, plan_list_step): after a selective first step
// the rows that remain are few, and a predicated step would still spend its
// instructions on every row.  The launch tuner times these against the
// predicated form of the same shape.
#include "kern_star_plan.cuh"

namespace svm {

using namespace plan;

extern const PlanEntry kPlansList[] = {
    // date join + two fact ranges, SUM: list after the first or second range
    SVM_PLAN_LIST(AGG_SCALAR, 0, R_, R_, l2(0), SC_NONE),
    SVM_PLAN_LIST(AGG_SCALAR, 1, R_, R_, l2(0), SC_NONE),
    SVM_PLAN_LIST(AGG_SCALAR, 0, R_, R_, smem(0), SC_NONE),
    SVM_PLAN_LIST(AGG_SCALAR, 1, R_, R_, smem(0), SC_NONE),
    // date + part join, the part probe first
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 0, l2(3), smem(2), SC_NONE, SC_NONE),
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 0, l2(3), l2(2), SC_NONE, SC_NONE),
    // date + part join with the part presence prefilter first, the date and
    // part probes in one pass over the list (the list after step 0 alone is
    // registered with the shape, kern_star_plan_mix3.cu)
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 4, l2(0), l2(2), l2(3), SC_NONE),
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 4, l2(0), smem(2), l2(3), SC_NONE),
    // the star join: date, customer, supplier
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 0, l2(2), l2(2), l2(2), SC_NONE),
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 1, l2(2), l2(2), l2(2), SC_NONE),
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 0, smem(2), l2(2), l2(2), SC_NONE),
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 1, smem(2), l2(2), l2(2), SC_NONE),
    // the star join with the customer and supplier probes in one pass
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 4, l2(2), l2(2), l2(2), SC_NONE),
    SVM_PLAN_LIST(AGG_DENSE_SMEM, 4, smem(2), l2(2), l2(2), SC_NONE),
};
extern const int kPlansListCount = (int)(sizeof(kPlansList) / sizeof(kPlansList[0]));

}  // namespace svm
