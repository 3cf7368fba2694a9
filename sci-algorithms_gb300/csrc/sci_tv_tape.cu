// Chambolle TV pass kernels that also write their tape (p_k of every dual
// update and the intermediate u_k): the forward TV of the differentiable
// unrolled solver keeps the tape, so its reverse pass reads it instead of
// recomputing it.  One pass (1 to 4 dual updates), no stop test, lag-1
// pipeline.  See sci_tv.cuh.
#include "sci_tv.cuh"

namespace sci {
namespace tv {

template <int CPL>
static void launch_tape_cpl(const Pass &P, int SG, unsigned g, cudaStream_t s) {
    switch (SG) {
        case 1: k_tv_main<1, false, true, CPL, 1, 0, RULE_SKIMAGE, true><<<g, WPB * 32, 0, s>>>(P); break;
        case 2: k_tv_main<2, false, true, CPL, 1, 0, RULE_SKIMAGE, true><<<g, WPB * 32, 0, s>>>(P); break;
        case 3: k_tv_main<3, false, true, CPL, 1, 0, RULE_SKIMAGE, true><<<g, WPB * 32, 0, s>>>(P); break;
        default: k_tv_main<4, false, true, CPL, 1, 0, RULE_SKIMAGE, true><<<g, WPB * 32, 0, s>>>(P); break;
    }
}

void launch_tape(const Pass &P, int SG, cudaStream_t s) {
    const unsigned g = pass_blocks(P);
    if (P.cpl == 2) launch_tape_cpl<2>(P, SG, g, s);
    else launch_tape_cpl<4>(P, SG, g, s);
}

}  // namespace tv
}  // namespace sci
