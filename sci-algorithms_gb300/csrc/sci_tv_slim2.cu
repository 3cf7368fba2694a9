// Register-lean TV pass (sci_tv_slim.cuh), 2 columns per lane.
#include "sci_tv_slim_launch.cuh"

namespace sci {
namespace tv {

void launch_slim2(const Pass &P, int SG, int minb, int proj, cudaStream_t s) {
    using namespace slim;
    if (proj == 3) return launch_main<2, 6, 3>(P, SG, s);
    switch (minb) {
        case 5:
            if (proj) launch_main<2, 5, 1>(P, SG, s);
            else launch_main<2, 5, 0>(P, SG, s);
            break;
        case 7:
            if (proj) launch_main<2, 7, 1>(P, SG, s);
            else launch_main<2, 7, 0>(P, SG, s);
            break;
        default:
            if (proj) launch_main<2, 6, 1>(P, SG, s);
            else launch_main<2, 6, 0>(P, SG, s);
            break;
    }
}

void launch_slim2_fix(const Pass &P, int proj, cudaStream_t s) {
    using namespace slim;
    constexpr int D = MinB<2>::def;
    if (proj == 3) (void)launch_dep(k_tv_slim_fix<2, D, 3>, dim3(pass_blocks(P)), dim3(WPB * 32), 0, s, P);
    else if (proj) (void)launch_dep(k_tv_slim_fix<2, D, 1>, dim3(pass_blocks(P)), dim3(WPB * 32), 0, s, P);
    else (void)launch_dep(k_tv_slim_fix<2, D, 0>, dim3(pass_blocks(P)), dim3(WPB * 32), 0, s, P);
}

int slim2_resident_blocks(int SG, int minb, int proj) {
    using namespace slim;
    static std::mutex mu;
    static int cache[3][4][5] = {};
    SG = SG < 1 ? 1 : (SG > 4 ? 4 : SG);
    const int mi = proj == 3 ? 1 : (minb == 5 ? 0 : (minb == 7 ? 2 : 1));
    std::lock_guard<std::mutex> lock(mu);
    int &v = cache[mi][proj & 3][SG];
    if (v == 0) {
        const void *k;
        if (proj == 3) k = main_kernel<2, 6, 3>(SG);
        else if (mi == 0) k = proj ? main_kernel<2, 5, 1>(SG) : main_kernel<2, 5, 0>(SG);
        else if (mi == 2) k = proj ? main_kernel<2, 7, 1>(SG) : main_kernel<2, 7, 0>(SG);
        else k = proj ? main_kernel<2, 6, 1>(SG) : main_kernel<2, 6, 0>(SG);
        v = resident(k, mi == 0 ? 5 : (mi == 2 ? 7 : 6));
    }
    return v;
}

}  // namespace tv
}  // namespace sci
