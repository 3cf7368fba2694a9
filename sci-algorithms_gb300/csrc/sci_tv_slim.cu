// Launchers of the register-lean Chambolle TV pass (sci_tv_slim.cuh).
#include <mutex>

#include "sci_tv_slim.cuh"

namespace sci {
namespace tv {

template <int MINB>
static void launch_minb(const Pass &P, int SG, cudaStream_t s) {
    const unsigned g = pass_blocks(P);
    switch (SG) {
        case 1: slim::k_tv_slim<1, MINB><<<g, WPB * 32, 0, s>>>(P); break;
        case 2: slim::k_tv_slim<2, MINB><<<g, WPB * 32, 0, s>>>(P); break;
        case 3: slim::k_tv_slim<3, MINB><<<g, WPB * 32, 0, s>>>(P); break;
        default: slim::k_tv_slim<4, MINB><<<g, WPB * 32, 0, s>>>(P); break;
    }
}

void launch_slim(const Pass &P, int SG, int minb, cudaStream_t s) {
    if (minb == 3) launch_minb<3>(P, SG, s);
    else launch_minb<4>(P, SG, s);
}

void launch_slim_fix(const Pass &P, int minb, cudaStream_t s) {
    if (minb == 3) slim::k_tv_slim_fix<3><<<pass_blocks(P), WPB * 32, 0, s>>>(P);
    else slim::k_tv_slim_fix<4><<<pass_blocks(P), WPB * 32, 0, s>>>(P);
}

template <int MINB>
static const void *kernel_of(int SG) {
    switch (SG) {
        case 1: return reinterpret_cast<const void *>(&slim::k_tv_slim<1, MINB>);
        case 2: return reinterpret_cast<const void *>(&slim::k_tv_slim<2, MINB>);
        case 3: return reinterpret_cast<const void *>(&slim::k_tv_slim<3, MINB>);
        default: return reinterpret_cast<const void *>(&slim::k_tv_slim<4, MINB>);
    }
}

// Queried once per (SG, minb) on the current device; the grid sizing
// falls back to minb blocks per SM if the query fails.
int slim_resident_blocks(int SG, int minb) {
    static std::mutex mu;
    static int cache[2][5] = {};
    const int mi = minb == 3 ? 0 : 1;
    SG = SG < 1 ? 1 : (SG > 4 ? 4 : SG);
    std::lock_guard<std::mutex> lock(mu);
    int &v = cache[mi][SG];
    if (v == 0) {
        int n = 0;
        const void *k = minb == 3 ? kernel_of<3>(SG) : kernel_of<4>(SG);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, WPB * 32, 0) != cudaSuccess ||
            n <= 0) {
            cudaGetLastError();
            n = minb;
        }
        v = n;
    }
    return v;
}

}  // namespace tv
}  // namespace sci
