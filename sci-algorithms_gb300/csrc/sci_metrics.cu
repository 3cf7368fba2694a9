// Per-frame PSNR and SSIM of a reconstructed stack against the ground truth
// in one pass: the diagnostics the drivers report per coded-frame block
// (compare_psnr / compare_ssim with data_range = 1, PnP_SCI/python/
// pnp_sci_algo.py:702-705, joint_pnp_sci_algo.py, scikit-image 0.16).
//
// SSIM (Wang et al. 2004, scikit-image's defaults): 7 x 7 uniform windows,
// sample covariance (N / (N - 1)), K1 = 0.01, K2 = 0.03, averaged over the
// frame cropped by 3 pixels.  Every window of the cropped region lies inside
// the frame, so the border extension of the uniform filter never enters the
// mean.  A block stages a (TY + 6) x (TX + 6) tile of both frames in shared
// memory; each thread forms its window's means, then the centred second
// moments sum((x - mx)^2), sum((y - my)^2), sum((x - mx)(y - my)) (equal to
// N (E[x^2] - mx^2) etc. without their cancellation), and the SSIM value;
// per-block float64 partial sums go to per-frame float64 totals.  The same
// pass sums (x - y)^2 over the whole frame for the PSNR.
#include "sci_common.cuh"

namespace sci {
namespace {

constexpr int TX = 32, TY = 8, R = 3, WIN = 2 * R + 1;

__global__ void __launch_bounds__(TX * TY) k_frame_metrics(const float *__restrict__ a,
                                                          const float *__restrict__ b, int H,
                                                          int W, double C1, double C2,
                                                          double *__restrict__ sqerr,
                                                          double *__restrict__ ssim_sum) {
    __shared__ float xa[TY + 2 * R][TX + 2 * R + 1], xb[TY + 2 * R][TX + 2 * R + 1];
    __shared__ double red[2][TX * TY / 32];
    const int64_t fo = (int64_t)blockIdx.z * H * W;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;  // tile of window centres
    const int tid = threadIdx.y * TX + threadIdx.x;
    // stage the tile and its 3-pixel apron (clamped loads; clamped cells are
    // only read by centres outside the cropped region, which are skipped)
    for (int c = tid; c < (TY + 2 * R) * (TX + 2 * R); c += TX * TY) {
        const int ly = c / (TX + 2 * R), lx = c - ly * (TX + 2 * R);
        const int i = min(max(y0 + ly - R, 0), H - 1), j = min(max(x0 + lx - R, 0), W - 1);
        xa[ly][lx] = a[fo + (int64_t)i * W + j];
        xb[ly][lx] = b[fo + (int64_t)i * W + j];
    }
    __syncthreads();
    const int i = y0 + threadIdx.y, j = x0 + threadIdx.x;
    double se = 0.0, ss = 0.0;
    if (i < H && j < W) {
        const double d = (double)xa[threadIdx.y + R][threadIdx.x + R] -
                         (double)xb[threadIdx.y + R][threadIdx.x + R];
        se = d * d;
        if (i >= R && i < H - R && j >= R && j < W - R) {
            float sx = 0.f, sy = 0.f;
#pragma unroll
            for (int u = 0; u < WIN; ++u)
#pragma unroll
                for (int v = 0; v < WIN; ++v) {
                    sx += xa[threadIdx.y + u][threadIdx.x + v];
                    sy += xb[threadIdx.y + u][threadIdx.x + v];
                }
            const float mx = sx * (1.f / (WIN * WIN)), my = sy * (1.f / (WIN * WIN));
            float vxx = 0.f, vyy = 0.f, vxy = 0.f;
#pragma unroll
            for (int u = 0; u < WIN; ++u)
#pragma unroll
                for (int v = 0; v < WIN; ++v) {
                    const float dx = xa[threadIdx.y + u][threadIdx.x + v] - mx;
                    const float dy = xb[threadIdx.y + u][threadIdx.x + v] - my;
                    vxx = fmaf(dx, dx, vxx);
                    vyy = fmaf(dy, dy, vyy);
                    vxy = fmaf(dx, dy, vxy);
                }
            // sample covariance: divide by N - 1
            const double inv = 1.0 / (WIN * WIN - 1);
            const double Vx = vxx * inv, Vy = vyy * inv, Vxy = vxy * inv;
            const double Mx = mx, My = my;
            ss = ((2.0 * Mx * My + C1) * (2.0 * Vxy + C2)) /
                 ((Mx * Mx + My * My + C1) * (Vx + Vy + C2));
        }
    }
    // block sums (fixed order within the block; float64 atomics across blocks)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_xor_sync(0xffffffffu, se, o);
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
    }
    if ((tid & 31) == 0) {
        red[0][tid >> 5] = se;
        red[1][tid >> 5] = ss;
    }
    __syncthreads();
    if (tid == 0) {
        double a0 = 0.0, a1 = 0.0;
        for (int w = 0; w < TX * TY / 32; ++w) {
            a0 += red[0][w];
            a1 += red[1][w];
        }
        atomicAdd(sqerr + blockIdx.z, a0);
        atomicAdd(ssim_sum + blockIdx.z, a1);
    }
}

}  // namespace
}  // namespace sci

using namespace sci;

extern "C" int sci_frame_metrics(const float *orig, const float *x, int64_t nframes, int64_t H,
                                 int64_t W, double data_range, double *sqerr, double *ssim_sum,
                                 void *stream) {
    SCI_CHECK_ARG(orig && x && sqerr && ssim_sum, "sci_frame_metrics: null pointer");
    SCI_CHECK_ARG(nframes >= 1 && nframes <= 65535 && H >= WIN && W >= WIN && H <= (1 << 24) &&
                      W <= (1 << 24),
                  "sci_frame_metrics: frames must be at least 7 x 7 (nframes <= 65535)");
    SCI_CHECK_ARG(data_range > 0.0, "sci_frame_metrics: data_range must be > 0");
    const cudaStream_t s = as_stream(stream);
    SCI_CUDA(cudaMemsetAsync(sqerr, 0, sizeof(double) * (size_t)nframes, s));
    SCI_CUDA(cudaMemsetAsync(ssim_sum, 0, sizeof(double) * (size_t)nframes, s));
    const double C1 = (0.01 * data_range) * (0.01 * data_range);
    const double C2 = (0.03 * data_range) * (0.03 * data_range);
    const dim3 g((unsigned)((W + TX - 1) / TX), (unsigned)((H + TY - 1) / TY), (unsigned)nframes);
    k_frame_metrics<<<g, dim3(TX, TY), 0, s>>>(orig, x, (int)H, (int)W, C1, C2, sqerr, ssim_sum);
    SCI_LAUNCHED("k_frame_metrics");
    return SCI_OK;
}
