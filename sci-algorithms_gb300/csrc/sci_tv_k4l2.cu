// Chambolle TV pass kernels, 4 dual updates per pass, lag-2 pipeline (the
// stages of a step are independent).  See sci_tv.cuh.
#include "sci_tv.cuh"

namespace sci {
namespace tv {

void launch_main4_lag2(const Pass &P, bool pin, bool final_pass, cudaStream_t s) {
    const unsigned g = pass_blocks(P);
    if (P.cpl == 2) {
        if (!pin && final_pass) k_tv_main<4, false, true, 2, 2><<<g, WPB * 32, 0, s>>>(P);
        else if (!pin) k_tv_main<4, false, false, 2, 2><<<g, WPB * 32, 0, s>>>(P);
        else if (final_pass) k_tv_main<4, true, true, 2, 2><<<g, WPB * 32, 0, s>>>(P);
        else k_tv_main<4, true, false, 2, 2><<<g, WPB * 32, 0, s>>>(P);
    } else {
        if (!pin && final_pass) k_tv_main<4, false, true, 4, 2><<<g, WPB * 32, 0, s>>>(P);
        else if (!pin) k_tv_main<4, false, false, 4, 2><<<g, WPB * 32, 0, s>>>(P);
        else if (final_pass) k_tv_main<4, true, true, 4, 2><<<g, WPB * 32, 0, s>>>(P);
        else k_tv_main<4, true, false, 4, 2><<<g, WPB * 32, 0, s>>>(P);
    }
}

}  // namespace tv
}  // namespace sci
