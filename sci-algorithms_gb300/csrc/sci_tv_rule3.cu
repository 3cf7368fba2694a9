// Chambolle-pipeline passes of MATLAB-twin update rule 3 (see sci_tv.cuh:
// RULE_CHAM_ITV = 1, RULE_CHAM_ATV = 2, RULE_CLIP = 3).
#include "sci_tv.cuh"

namespace sci {
namespace tv {

void launch_rule3(const Pass &P, int SG, bool pin, bool final_pass, cudaStream_t s) {
    launch_rule_impl<3>(P, SG, pin, final_pass, s);
}

}  // namespace tv
}  // namespace sci
