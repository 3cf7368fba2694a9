// Stop-test ("fixup") launches of the Chambolle TV passes.  See sci_tv.cuh.
#include "sci_tv.cuh"

namespace sci {
namespace tv {

void launch_fixup(const Pass &P, bool pin, cudaStream_t s) {
    const unsigned g = pass_blocks(P);
    if (pin) k_tv_fixup<true><<<g, WPB * 32, 0, s>>>(P);
    else k_tv_fixup<false><<<g, WPB * 32, 0, s>>>(P);
}

}  // namespace tv
}  // namespace sci
