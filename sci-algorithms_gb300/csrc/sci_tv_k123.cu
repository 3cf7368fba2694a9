// Chambolle TV pass kernels with 1-3 dual updates (n_iter_max = 2..4, and
// the last pass of longer runs).  See sci_tv.cuh.
#include "sci_tv.cuh"

namespace sci {
namespace tv {

void launch_main123(const Pass &P, int SG, bool pin, cudaStream_t s) {
    const unsigned g = pass_blocks(P);
    switch (SG * 2 + (pin ? 1 : 0)) {
        case 2: k_tv_main<1, false, true><<<g, WPB * 32, 0, s>>>(P); break;
        case 3: k_tv_main<1, true, true><<<g, WPB * 32, 0, s>>>(P); break;
        case 4: k_tv_main<2, false, true><<<g, WPB * 32, 0, s>>>(P); break;
        case 5: k_tv_main<2, true, true><<<g, WPB * 32, 0, s>>>(P); break;
        case 6: k_tv_main<3, false, true><<<g, WPB * 32, 0, s>>>(P); break;
        default: k_tv_main<3, true, true><<<g, WPB * 32, 0, s>>>(P); break;
    }
}

}  // namespace tv
}  // namespace sci
