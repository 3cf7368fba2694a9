// Chambolle TV pass kernels with 4 dual updates per pass, 4 columns per lane
// (n_iter_max = 5 in one pass; the 4-update passes of longer runs).
// See sci_tv.cuh.
#include "sci_tv.cuh"

namespace sci {
namespace tv {

void launch_main4_c4(const Pass &P, bool pin, bool final_pass, cudaStream_t s) {
    const unsigned g = pass_blocks(P);
    // without a residual output the kernel is compiled without its code
    if (!pin && final_pass && !P.resid)
        k_tv_main<4, false, true, 4, 1, 0, RULE_SKIMAGE, false, false><<<g, WPB * 32, 0, s>>>(P);
    else if (!pin && final_pass) k_tv_main<4, false, true, 4><<<g, WPB * 32, 0, s>>>(P);
    else if (!pin) k_tv_main<4, false, false, 4><<<g, WPB * 32, 0, s>>>(P);
    else if (final_pass) k_tv_main<4, true, true, 4><<<g, WPB * 32, 0, s>>>(P);
    else k_tv_main<4, true, false, 4><<<g, WPB * 32, 0, s>>>(P);
}

}  // namespace tv
}  // namespace sci
