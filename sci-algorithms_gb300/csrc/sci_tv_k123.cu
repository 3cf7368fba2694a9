// Chambolle TV pass kernels with 1-3 dual updates (n_iter_max = 2..4, and
// the last pass of longer runs).  See sci_tv.cuh.
#include "sci_tv.cuh"

namespace sci {
namespace tv {

template <int CPL>
static void launch(const Pass &P, int SG, bool pin, cudaStream_t s) {
    const unsigned g = pass_blocks(P);
    switch (SG * 2 + (pin ? 1 : 0)) {
        case 2: k_tv_main<1, false, true, CPL><<<g, WPB * 32, 0, s>>>(P); break;
        case 3: k_tv_main<1, true, true, CPL><<<g, WPB * 32, 0, s>>>(P); break;
        case 4: k_tv_main<2, false, true, CPL><<<g, WPB * 32, 0, s>>>(P); break;
        case 5: k_tv_main<2, true, true, CPL><<<g, WPB * 32, 0, s>>>(P); break;
        case 6: k_tv_main<3, false, true, CPL><<<g, WPB * 32, 0, s>>>(P); break;
        default: k_tv_main<3, true, true, CPL><<<g, WPB * 32, 0, s>>>(P); break;
    }
}

void launch_main123(const Pass &P, int SG, bool pin, cudaStream_t s) {
    if (P.cpl == 2) launch<2>(P, SG, pin, s);
    else launch<4>(P, SG, pin, s);
}

}  // namespace tv
}  // namespace sci
