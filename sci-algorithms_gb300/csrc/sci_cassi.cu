// Spectral (CASSI) forward model: a single coded aperture followed by a
// dispersion that shifts band b by `step * b` pixels along W onto a detector
// of width Wd = W + step (L - 1).
//
//   y[h, w + step b] += phi[h, w] x_b[h, w]          (forward, detector H x Wd)
//   x_b[h, w]         = phi[h, w] r[h, w + step b]   (adjoint)
//   Phi_sum[h, w']    = sum_b phi[h, w' - step b]^2  (zeros replaced by 1)
//
// The reference's Python path has no spectral operator; its MATLAB CASSI
// test uses the same model with a pre-shifted 3-D mask and
// Phisum = sum(mask.^2, 3) (DeSCI/test_desci_cassi.m:58-62).  The GAP
// projection is the video one (pnp_sci_algo.py:640-645) with these
// operators: one detector-grid kernel (A, y1 update, residual) and one
// cube-grid kernel (x += lambda At(r)).
#include <algorithm>
#include <cstdlib>
#include <string>

#include "sci_common.cuh"
#include "sci_graph.cuh"

namespace sci {

namespace {

inline dim3 grid1(int64_t n, int t) {
    int64_t b = (n + t - 1) / t;
    if (b > (int64_t)kSMs * 16) b = (int64_t)kSMs * 16;
    return dim3((unsigned)(b < 1 ? 1 : b));
}

// first/last band hitting detector column wd
__device__ __forceinline__ void band_range(int wd, int W, int L, int step, int &b0, int &b1) {
    // need 0 <= wd - step b <= W - 1
    b0 = (wd - (W - 1) + step - 1) / step;
    if (wd - (W - 1) <= 0) b0 = 0;
    b1 = wd / step;
    if (b1 > L - 1) b1 = L - 1;
}

__global__ void k_cassi_A(const float *__restrict__ x, const float *__restrict__ phi,
                          float *__restrict__ y, int L, int H, int W, int step) {
    const int Wd = W + step * (L - 1);
    const int64_t hw = (int64_t)H * W, n = (int64_t)H * Wd;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int h = (int)(i / Wd), wd = (int)(i - (int64_t)h * Wd);
        int b0, b1;
        band_range(wd, W, L, step, b0, b1);
        float s = 0.f;
        for (int b = b0; b <= b1; ++b) {
            const int64_t p = (int64_t)h * W + (wd - step * b);
            s = fmaf(__ldg(x + b * hw + p), __ldg(phi + p), s);
        }
        y[i] = s;
    }
}

__global__ void k_cassi_At(const float *__restrict__ y, const float *__restrict__ phi,
                           float *__restrict__ x, int L, int H, int W, int step) {
    const int Wd = W + step * (L - 1);
    const int64_t hw = (int64_t)H * W, n = (int64_t)L * hw;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(i / hw);
        const int64_t p = i - (int64_t)b * hw;
        const int h = (int)(p / W), w = (int)(p - (int64_t)h * W);
        x[i] = __ldg(phi + p) * __ldg(y + (int64_t)h * Wd + w + step * b);
    }
}

__global__ void k_cassi_phisum(const float *__restrict__ phi, float *__restrict__ ps, int L,
                               int H, int W, int step, int guard) {
    const int Wd = W + step * (L - 1);
    const int64_t n = (int64_t)H * Wd;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int h = (int)(i / Wd), wd = (int)(i - (int64_t)h * Wd);
        int b0, b1;
        band_range(wd, W, L, step, b0, b1);
        float s = 0.f;
        for (int b = b0; b <= b1; ++b) {
            const float m = __ldg(phi + (int64_t)h * W + (wd - step * b));
            s = fmaf(m, m, s);
        }
        if (guard && s == 0.f) s = 1.f;
        ps[i] = s;
    }
}

// detector grid: yb = A(x); ACC: y1 += y - yb, r = (y1 - yb)/ps; else r = (y - yb)/ps
template <bool ACC>
__global__ void k_cassi_resid(const float *__restrict__ x, const float *__restrict__ phi,
                              const float *__restrict__ y, float *__restrict__ y1,
                              const float *__restrict__ ps, float *__restrict__ r, int L, int H,
                              int W, int step) {
    const int Wd = W + step * (L - 1);
    const int64_t hw = (int64_t)H * W, n = (int64_t)H * Wd;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int h = (int)(i / Wd), wd = (int)(i - (int64_t)h * Wd);
        int b0, b1;
        band_range(wd, W, L, step, b0, b1);
        float s = 0.f;
        for (int b = b0; b <= b1; ++b) {
            const int64_t p = (int64_t)h * W + (wd - step * b);
            s = fmaf(__ldg(x + b * hw + p), __ldg(phi + p), s);
        }
        if (ACC) {
            const float t = y1[i] + (y[i] - s);
            y1[i] = t;
            r[i] = __fdiv_rn(t - s, ps[i]);
        } else {
            r[i] = __fdiv_rn(y[i] - s, ps[i]);
        }
    }
}

// cube grid: x_out_b = x_b + lambda (r[h, w + step b] phi[h, w])
__global__ void k_cassi_update(const float *__restrict__ x, const float *__restrict__ phi,
                               const float *__restrict__ r, float *__restrict__ xo, float lam,
                               int L, int H, int W, int step) {
    const int Wd = W + step * (L - 1);
    const int64_t hw = (int64_t)H * W, n = (int64_t)L * hw;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(i / hw);
        const int64_t p = i - (int64_t)b * hw;
        const int h = (int)(p / W), w = (int)(p - (int64_t)h * W);
        const float rv = __ldg(r + (int64_t)h * Wd + w + step * b);
        xo[i] = fmaf(lam, rv * __ldg(phi + p), __ldg(x + i));
    }
}

// The projection of one iteration with a detector row per block: the
// row's residual r (detector grid, k_cassi_resid's arithmetic) into shared
// memory, then x_out_b = x_b + lambda (r[h, w + step b] phi[h, w]) for every
// band of that row (k_cassi_update's arithmetic) -- one launch, and r never
// leaves the chip.  Needs Wd floats of shared memory.
template <bool ACC>
__global__ void __launch_bounds__(1024) k_cassi_proj_rows(
    const float *__restrict__ x, const float *__restrict__ phi, const float *__restrict__ y,
    float *__restrict__ y1, const float *__restrict__ ps, float *__restrict__ xo, float lam,
    int L, int H, int W, int step, double *__restrict__ zero, int nzero) {
    extern __shared__ float rs[];
    grid_dep_wait();
    if (blockIdx.x == 0)  // the next TV pass's stop-test sums
        for (int i = threadIdx.x; i < nzero; i += blockDim.x) zero[i] = 0.0;
    const int Wd = W + step * (L - 1);
    const int64_t hw = (int64_t)H * W;
    for (int h = blockIdx.x; h < H; h += gridDim.x) {
        for (int wd = threadIdx.x; wd < Wd; wd += blockDim.x) {
            const int64_t i = (int64_t)h * Wd + wd;
            int b0, b1;
            band_range(wd, W, L, step, b0, b1);
            float s = 0.f;
            for (int b = b0; b <= b1; ++b) {
                const int64_t p = (int64_t)h * W + (wd - step * b);
                s = fmaf(__ldg(x + b * hw + p), __ldg(phi + p), s);
            }
            if (ACC) {
                const float t = y1[i] + (y[i] - s);
                y1[i] = t;
                rs[wd] = __fdiv_rn(t - s, ps[i]);
            } else {
                rs[wd] = __fdiv_rn(y[i] - s, ps[i]);
            }
        }
        __syncthreads();
        for (int e = threadIdx.x; e < L * W; e += blockDim.x) {
            const int b = e / W, w = e - b * W;
            const int64_t p = (int64_t)h * W + w;
            xo[b * hw + p] = fmaf(lam, rs[w + step * b] * __ldg(phi + p), __ldg(x + b * hw + p));
        }
        __syncthreads();
    }
}

constexpr size_t kRowSmemMax = 48 * 1024;  // default dynamic shared memory limit

// Projection form (SCI_CASSI_ROWS; bitwise the same result): 1, the
// default, the row-fused kernel; 0 the detector-grid and cube-grid kernel
// pair.
bool rows_enabled() {
    const char *e = getenv("SCI_CASSI_ROWS");
    return !(e && atoi(e) == 0);
}

// Threads per row of the row-fused kernel (SCI_CASSI_ROWT overrides).
// Measured on 256 x 256 x 28 (80 iterations, graph): 128 threads 3.71 ms
// per solve, 256 3.19, 512 3.03, 1024 3.03 -- the kernel is latency-bound
// (about 14 us of arithmetic-light work per launch), and wider rows
// shorten each thread's chain.
int row_threads() {
    if (const char *e = getenv("SCI_CASSI_ROWT")) {
        const int v = atoi(e);
        if (v == 128 || v == 256 || v == 512 || v == 1024) return v;
    }
    return 512;
}

int check(int64_t L, int64_t H, int64_t W, int step) {
    SCI_CHECK_ARG(L >= 1 && H >= 1 && W >= 1 && step >= 1, "cassi: invalid sizes or step");
    SCI_CHECK_ARG(L <= 4096 && H * (W + step * (L - 1)) < (int64_t(1) << 40) && W < (1 << 30),
                  "cassi: sizes too large");
    return SCI_OK;
}

}  // namespace

int tv_launch_flags(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
                    int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
                    void *workspace, size_t ws_bytes, cudaStream_t s, int force_R, int flags);
double *tv_clear_region(int64_t nf, int64_t H, int64_t W, int K, void *workspace, int *words);
size_t tv_workspace_bytes(int64_t nf, int64_t H, int64_t W, int K);

static size_t r256(size_t b) { return (b + 255) & ~size_t(255); }

static size_t cassi_ws(int64_t L, int64_t H, int64_t W, int step, int K, char *base,
                       float **y1, float **r, float **xp, void **tv, size_t *tvb) {
    const size_t nd = (size_t)(H * (W + step * (L - 1))), n = (size_t)(L * H * W);
    const size_t o1 = 0, o2 = o1 + r256(4 * nd), o3 = o2 + r256(4 * nd), o4 = o3 + r256(4 * n);
    const size_t t = tv_workspace_bytes(L, H, W, K);
    if (base) {
        *y1 = reinterpret_cast<float *>(base + o1);
        *r = reinterpret_cast<float *>(base + o2);
        *xp = reinterpret_cast<float *>(base + o3);
        *tv = base + o4;
        *tvb = t;
    }
    return o4 + r256(t);
}

}  // namespace sci

using namespace sci;

extern "C" {

int sci_cassi_A(const float *x, const float *phi, float *y, int64_t L, int64_t H, int64_t W,
                int step, void *stream) {
    if (int e = check(L, H, W, step)) return e;
    SCI_CHECK_ARG(x && phi && y, "sci_cassi_A: null pointer");
    k_cassi_A<<<grid1(H * (W + step * (L - 1)), 256), 256, 0, as_stream(stream)>>>(
        x, phi, y, (int)L, (int)H, (int)W, step);
    SCI_LAUNCHED("k_cassi_A");
    return SCI_OK;
}

int sci_cassi_At(const float *y, const float *phi, float *x, int64_t L, int64_t H, int64_t W,
                 int step, void *stream) {
    if (int e = check(L, H, W, step)) return e;
    SCI_CHECK_ARG(x && phi && y, "sci_cassi_At: null pointer");
    k_cassi_At<<<grid1(L * H * W, 256), 256, 0, as_stream(stream)>>>(y, phi, x, (int)L, (int)H,
                                                                      (int)W, step);
    SCI_LAUNCHED("k_cassi_At");
    return SCI_OK;
}

int sci_cassi_phisum(const float *phi, float *phisum, int64_t L, int64_t H, int64_t W, int step,
                     int guard_zero, void *stream) {
    if (int e = check(L, H, W, step)) return e;
    SCI_CHECK_ARG(phi && phisum, "sci_cassi_phisum: null pointer");
    k_cassi_phisum<<<grid1(H * (W + step * (L - 1)), 256), 256, 0, as_stream(stream)>>>(
        phi, phisum, (int)L, (int)H, (int)W, step, guard_zero);
    SCI_LAUNCHED("k_cassi_phisum");
    return SCI_OK;
}

int sci_cassi_workspace_bytes(int64_t L, int64_t H, int64_t W, int step, int tv_iter_max,
                              size_t *bytes) {
    if (int e = check(L, H, W, step)) return e;
    SCI_CHECK_ARG(bytes && tv_iter_max >= 1, "sci_cassi_workspace_bytes: bad argument");
    *bytes = cassi_ws(L, H, W, step, tv_iter_max, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr);
    return SCI_OK;
}

int sci_cassi_gap_tv(const float *y, const float *phi, const float *phisum, const float *x0,
                     float *x_out, int64_t L, int64_t H, int64_t W, int step,
                     const sci_solve_opts *o, void *workspace, size_t workspace_bytes,
                     void *stream) {
    if (int e = check(L, H, W, step)) return e;
    SCI_CHECK_ARG(o && y && phi && phisum && x0 && x_out, "sci_cassi_gap_tv: null pointer");
    SCI_CHECK_ARG(o->iters >= 0 && o->tv_iter_max >= 1 && (o->iters == 0 || (o->lambdas && o->weights)),
                  "sci_cassi_gap_tv: bad options");
    const size_t need = cassi_ws(L, H, W, step, o->tv_iter_max, nullptr, nullptr, nullptr,
                                 nullptr, nullptr, nullptr);
    SCI_CHECK_ARG(workspace && workspace_bytes >= need,
                  "sci_cassi_gap_tv: workspace of %zu bytes needed, got %zu", need,
                  workspace_bytes);
    float *y1, *r, *xp;
    void *tv;
    size_t tvb;
    cassi_ws(L, H, W, step, o->tv_iter_max, static_cast<char *>(workspace), &y1, &r, &xp, &tv,
             &tvb);
    const int64_t n = L * H * W, nd = H * (W + step * (L - 1));
    const size_t row_smem = sizeof(float) * (size_t)(W + step * (L - 1));
    const bool rows = row_smem <= kRowSmemMax && rows_enabled();
    const int rt = row_threads();
    // the row-fused projection also clears the TV pass's stop-test sums, so
    // that the TV kernel follows it directly (flags 4)
    int nzero = 0;
    double *zero = rows ? tv_clear_region(L, H, W, o->tv_iter_max, tv, &nzero) : nullptr;
    auto enqueue = [&](cudaStream_t s) -> int {
        if (x0 != x_out) SCI_CUDA(cudaMemcpyAsync(x_out, x0, 4 * n, cudaMemcpyDeviceToDevice, s));
        if (o->accelerate) SCI_CUDA(cudaMemsetAsync(y1, 0, 4 * nd, s));
        if (o->sqerr) SCI_CUDA(cudaMemsetAsync(o->sqerr, 0, sizeof(double) * o->iters, s));
        for (int it = 0; it < o->iters; ++it) {
            SCI_CHECK_ARG(o->weights[it] > 0.f, "sci_cassi_gap_tv: tv_weight must be > 0");
            if (rows) {
                const unsigned g = (unsigned)std::min<int64_t>(H, (int64_t)kSMs * 8);
                if (o->accelerate)
                    SCI_CUDA(launch_dep(k_cassi_proj_rows<true>, dim3(g), dim3(rt), row_smem, s,
                                        x_out, phi, y, y1, phisum, xp, o->lambdas[it], (int)L,
                                        (int)H, (int)W, step, zero, nzero));
                else
                    SCI_CUDA(launch_dep(k_cassi_proj_rows<false>, dim3(g), dim3(rt), row_smem, s,
                                        x_out, phi, y, y1, phisum, xp, o->lambdas[it], (int)L,
                                        (int)H, (int)W, step, zero, nzero));
                SCI_LAUNCHED("k_cassi_proj_rows");
            } else {
                if (o->accelerate)
                    k_cassi_resid<true><<<grid1(nd, 256), 256, 0, s>>>(
                        x_out, phi, y, y1, phisum, r, (int)L, (int)H, (int)W, step);
                else
                    k_cassi_resid<false><<<grid1(nd, 256), 256, 0, s>>>(
                        x_out, phi, y, y1, phisum, r, (int)L, (int)H, (int)W, step);
                SCI_LAUNCHED("k_cassi_resid");
                k_cassi_update<<<grid1(n, 256), 256, 0, s>>>(x_out, phi, r, xp, o->lambdas[it],
                                                             (int)L, (int)H, (int)W, step);
                SCI_LAUNCHED("k_cassi_update");
            }
            int e = tv_launch_flags(xp, x_out, nullptr, L, H, W, H * W, o->weights[it], o->eps,
                                    o->tv_iter_max,
                                    o->tv_steps ? o->tv_steps + (int64_t)it * L : nullptr,
                                    nullptr, tv, tvb, s, 0, rows ? 4 : 0);
            if (e) return e;
            if (o->orig && o->sqerr) {
                e = sci_sqerr_accum(o->orig, x_out, n, o->sqerr + it, s);
                if (e) return e;
            }
        }
        return SCI_OK;
    };
    cudaStream_t s = as_stream(stream);
    if (!o->use_graph || o->iters == 0) return enqueue(s);
    std::string key;
    key_append(key, y, phi, phisum, x0, x_out, L, H, W, step, workspace, o->iters,
               o->tv_iter_max, o->eps, o->accelerate, o->orig, o->sqerr, o->tv_steps);
    key.append(reinterpret_cast<const char *>(o->lambdas), sizeof(float) * o->iters);
    key.append(reinterpret_cast<const char *>(o->weights), sizeof(float) * o->iters);
    return run_graph("cassi graph capture", key, s, enqueue);
}

}  // extern "C"
