// Chambolle TV pass kernels that apply the GAP projection while loading
// their input (single pass, 4 columns per lane).  See sci_tv.cuh.
#include "sci_tv.cuh"

namespace sci {
namespace tv {

void launch_main_proj(const Pass &P, int SG, cudaStream_t s) {
    const unsigned g = pass_blocks(P);
    switch (SG) {
        case 1: k_tv_main<1, false, true, 4, 1, 1><<<g, WPB * 32, 0, s>>>(P); break;
        case 2: k_tv_main<2, false, true, 4, 1, 1><<<g, WPB * 32, 0, s>>>(P); break;
        case 3: k_tv_main<3, false, true, 4, 1, 1><<<g, WPB * 32, 0, s>>>(P); break;
        default: k_tv_main<4, false, true, 4, 1, 1><<<g, WPB * 32, 0, s>>>(P); break;
    }
}

void launch_fixup_proj(const Pass &P, cudaStream_t s) {
    k_tv_fixup<false, 4, 1><<<pass_blocks(P), WPB * 32, 0, s>>>(P);
}

}  // namespace tv
}  // namespace sci
