// Register-lean TV pass (sci_tv_slim.cuh), 4 columns per lane; the host
// entry points for both column widths.
#include <cstdlib>

#include "sci_tv_slim_launch.cuh"

namespace sci {
namespace tv {

void launch_slim2(const Pass &P, int SG, int minb, int proj, cudaStream_t s);  // sci_tv_slim2.cu
void launch_slim2_fix(const Pass &P, int proj, cudaStream_t s);
int slim2_resident_blocks(int SG, int minb, int proj);

// proj: 0 none, 1 the GAP projection on load, 3 also the t output (the
// default register budget only)
void launch_slim(const Pass &P, int SG, int minb, int proj, cudaStream_t s) {
    using namespace slim;
    if (P.cpl == 2) return launch_slim2(P, SG, minb, proj, s);
    // SCI_TV_FORM=0: the dual field held as p instead of 4 p (n_iter_max =
    // 5, 4 columns per lane at 128 registers).  Measured at 2048 x 2048 x
    // 24: 0.3197 ms as p, 0.3165 ms as 4 p (GAP-TV 2201 vs 2231 iter/s).
    const char *e = getenv("SCI_TV_FORM");
    const int form = (e && atoi(e) == 0) ? 0 : 1;
    if (proj == 3) {
        launch_main<4, 4, 3>(P, SG, s, form);
    } else if (minb == 3) {
        if (proj) launch_main<4, 3, 1>(P, SG, s);
        else launch_main<4, 3, 0>(P, SG, s);
    } else {
        if (proj) launch_main<4, 4, 1>(P, SG, s, form);
        else launch_main<4, 4, 0>(P, SG, s, form);
    }
}

void launch_slim_fix(const Pass &P, int proj, cudaStream_t s) {
    using namespace slim;
    if (P.cpl == 2) return launch_slim2_fix(P, proj, s);
    constexpr int D = MinB<4>::def;
    if (proj == 3) (void)launch_dep(k_tv_slim_fix<4, D, 3>, dim3(pass_blocks(P)), dim3(WPB * 32), 0, s, P);
    else if (proj) (void)launch_dep(k_tv_slim_fix<4, D, 1>, dim3(pass_blocks(P)), dim3(WPB * 32), 0, s, P);
    else (void)launch_dep(k_tv_slim_fix<4, D, 0>, dim3(pass_blocks(P)), dim3(WPB * 32), 0, s, P);
}

int slim_resident_blocks(int cpl, int SG, int minb, int proj) {
    using namespace slim;
    if (cpl == 2) return slim2_resident_blocks(SG, minb, proj);
    static std::mutex mu;
    static int cache[2][4][5] = {};
    SG = SG < 1 ? 1 : (SG > 4 ? 4 : SG);
    const int mi = (minb == 3 && proj != 3) ? 0 : 1;
    std::lock_guard<std::mutex> lock(mu);
    int &v = cache[mi][proj & 3][SG];
    if (v == 0) {
        const void *k = proj == 3 ? main_kernel<4, 4, 3>(SG)
                        : mi == 0 ? (proj ? main_kernel<4, 3, 1>(SG) : main_kernel<4, 3, 0>(SG))
                                  : (proj ? main_kernel<4, 4, 1>(SG) : main_kernel<4, 4, 0>(SG));
        v = resident(k, mi == 0 ? 3 : 4);
    }
    return v;
}

}  // namespace tv
}  // namespace sci
