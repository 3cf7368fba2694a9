// Launch helpers of the register-lean TV pass, instantiated per column
// width in sci_tv_slim.cu (4 columns per lane) and sci_tv_slim2.cu (2).
#pragma once
#include <mutex>

#include "sci_tv_slim.cuh"

namespace sci {
namespace tv {
namespace slim {

// Resident blocks per SM the registers of the main kernel are sized for,
// by default (n_iter_max = 5 also builds the alternatives SCI_SLIM_MINB
// picks: 3 or 4 for 4 columns per lane, 5, 6 or 7 for 2).
template <int CPL>
struct MinB {
    static constexpr int def = CPL == 4 ? 4 : 6;
};

template <int CPL, int MINB, int PROJ>
const void *main_kernel(int SG) {
    switch (SG) {
        case 1: return reinterpret_cast<const void *>(&k_tv_slim<1, CPL, MinB<CPL>::def, PROJ>);
        case 2: return reinterpret_cast<const void *>(&k_tv_slim<2, CPL, MinB<CPL>::def, PROJ>);
        case 3: return reinterpret_cast<const void *>(&k_tv_slim<3, CPL, MinB<CPL>::def, PROJ>);
        default: return reinterpret_cast<const void *>(&k_tv_slim<4, CPL, MINB, PROJ>);
    }
}

template <int CPL, int MINB, int PROJ>
void launch_main(const Pass &P, int SG, cudaStream_t s, int form = 1) {
    const unsigned g = pass_blocks(P);
    constexpr int D = MinB<CPL>::def;
    const dim3 b(WPB * 32);
    cudaError_t e;
    switch (SG) {
        case 1: e = launch_dep(k_tv_slim<1, CPL, D, PROJ>, dim3(g), b, 0, s, P); break;
        case 2: e = launch_dep(k_tv_slim<2, CPL, D, PROJ>, dim3(g), b, 0, s, P); break;
        case 3: e = launch_dep(k_tv_slim<3, CPL, D, PROJ>, dim3(g), b, 0, s, P); break;
        default:
            if (form) e = launch_dep(k_tv_slim<4, CPL, MINB, PROJ, 1>, dim3(g), b, 0, s, P);
            else e = launch_dep(k_tv_slim<4, CPL, MINB, PROJ, 0>, dim3(g), b, 0, s, P);
            break;
    }
    (void)e;  // reported by the caller's cudaGetLastError
}

// Resident blocks per SM of a kernel, queried once; minb if the query fails.
inline int resident(const void *k, int minb) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, WPB * 32, 0) != cudaSuccess ||
        n <= 0) {
        cudaGetLastError();
        n = minb;
    }
    return n;
}

}  // namespace slim
}  // namespace tv
}  // namespace sci
