// Differentiable unrolled GAP-TV: forward with outer-iterate checkpoints and
// a hand-written reverse pass.
//
// Model (a batch of N scenes sharing one learnable mask):
//   Phi = sigmoid(logits) (B x H x W), Phi_sum = sum_b Phi_b,
//   y_n = A(x_true_n), x^0 = At(y / Phi_sum),
//   for k < K (GAP with acceleration, pnp_sci_algo.py:641-643):
//     yb = A(x^k); y1 += y - yb; q = (y1 - yb) / Phi_sum;
//     v^k = x^k + lambda_k At(q);   x^{k+1} = TV(v^k)   (fixed T Chambolle
//     steps, no stop test: the stop rule is not differentiable)
//   loss = mean (x^K - x_true)^2.
// The forward keeps x^k and y1^k; the reverse pass recomputes each TV call
// from v^k with a step-by-step tape (u_k, p_{k+1}) and runs its adjoint:
//   p_{k+1} = (p_k - tau g_k) r_k,  r_k = 1 / (1 + (tau/w) n_k),  n_k = |g_k|,
//   gbar_k = -tau r_k pbar_{k+1} - (tau/w) r_k (g_k / n_k) <pbar_{k+1}, p_{k+1}>
//            (0 for the second term where n_k = 0: the safe-norm convention),
//   ubar_k = -div gbar_k,  fbar += ubar_k,  pbar_k = r_k pbar_{k+1} + grad ubar_k.
// then the adjoint of the projection (including d/dPhi through A, At and
// Phi_sum, and d/dlambda_k), and finally of the measurement and x^0.
#include <list>
#include <mutex>
#include <string>

#include "sci_common.cuh"

namespace sci {

int tv_launch_flags(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
                    int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
                    void *workspace, size_t ws_bytes, cudaStream_t s, int force_R, int flags);
size_t tv_workspace_bytes(int64_t nf, int64_t H, int64_t W, int K);

namespace unr {

constexpr int kNoStop = 1;  // tv_launch_flags: run all steps, no stop test

inline dim3 grid1(int64_t n, int t) {
    int64_t b = (n + t - 1) / t;
    if (b > (int64_t)kSMs * 16) b = (int64_t)kSMs * 16;
    return dim3((unsigned)(b < 1 ? 1 : b));
}

#define GRID_LOOP(i, n)                                                          \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n);    \
         i += (int64_t)gridDim.x * blockDim.x)

// ------------------------------------------------------------- forward
__global__ void k_mask(const float *__restrict__ logits, float *__restrict__ phi,
                       float *__restrict__ ps, int B, int64_t hw) {
    GRID_LOOP(p, hw) {
        float s = 0.f;
        for (int b = 0; b < B; ++b) {
            const float m = 1.f / (1.f + expf(-logits[b * hw + p]));
            phi[b * hw + p] = m;
            s += m;
        }
        ps[p] = s;
    }
}

// y_n = A(x_true_n); x^0_n = At(y_n / Phi_sum)
__global__ void k_meas_x0(const float *__restrict__ xt, const float *__restrict__ phi,
                          const float *__restrict__ ps, float *__restrict__ y,
                          float *__restrict__ x0, int N, int B, int64_t hw) {
    GRID_LOOP(i, (int64_t)N * hw) {
        const int n = (int)(i / hw);
        const int64_t p = i - (int64_t)n * hw;
        const float *xn = xt + (int64_t)n * B * hw;
        float s = 0.f;
        for (int b = 0; b < B; ++b) s = fmaf(xn[b * hw + p], phi[b * hw + p], s);
        y[i] = s;
        const float s0 = s / ps[p];
        float *x0n = x0 + (int64_t)n * B * hw;
        for (int b = 0; b < B; ++b) x0n[b * hw + p] = phi[b * hw + p] * s0;
    }
}

// yb = A(x); y1 = y1_prev + (y - yb); v = x + lambda (phi (y1 - yb)/Phi_sum)
__global__ void k_proj_fwd(const float *__restrict__ x, const float *__restrict__ phi,
                           const float *__restrict__ ps, const float *__restrict__ y,
                           const float *__restrict__ y1_prev, float *__restrict__ y1,
                           float *__restrict__ v, const float *__restrict__ lambdas, int k,
                           int N, int B, int64_t hw) {
    const float lam = lambdas[k];
    GRID_LOOP(i, (int64_t)N * hw) {
        const int n = (int)(i / hw);
        const int64_t p = i - (int64_t)n * hw;
        const float *xn = x + (int64_t)n * B * hw;
        float yb = 0.f;
        for (int b = 0; b < B; ++b) yb = fmaf(xn[b * hw + p], phi[b * hw + p], yb);
        const float t = (y1_prev ? y1_prev[i] : 0.f) + (y[i] - yb);
        y1[i] = t;
        const float q = (t - yb) / ps[p];
        float *vn = v + (int64_t)n * B * hw;
        for (int b = 0; b < B; ++b) vn[b * hw + p] = fmaf(lam, q * phi[b * hw + p], xn[b * hw + p]);
    }
}

__global__ void k_mse(const float *__restrict__ a, const float *__restrict__ b,
                      float *__restrict__ grad, float gscale, int64_t n, double *out) {
    double acc = 0.0;
    GRID_LOOP(i, n) {
        const float d = a[i] - b[i];
        acc += (double)d * d;
        if (grad) grad[i] = gscale * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && out) atomicAdd(out, acc);
}

// ------------------------------------------------------- TV tape (recompute)
// p_{k+1} from u_k and p_k (p_k = nullptr: p_0 = 0)
__global__ void k_tape_p(const float *__restrict__ u, const float *__restrict__ pin,
                         float *__restrict__ pout, int64_t nf, int H, int W, float tau,
                         float tw) {
    const int64_t hw = (int64_t)H * W;
    GRID_LOOP(i, nf * hw) {
        const int64_t f = i / hw, p = i - f * hw;
        const int r = (int)(p / W), c = (int)(p - (int64_t)r * W);
        const float *uf = u + f * hw;
        const float uc = uf[p];
        const float gr = (r + 1 < H) ? uf[p + W] - uc : 0.f;
        const float gc = (c + 1 < W) ? uf[p + 1] - uc : 0.f;
        const float nrm = sqrt_approx(fmaf(gr, gr, gc * gc));
        const float ri = rcp_approx(fmaf(tw, nrm, 1.f));
        const float qr = pin ? pin[f * 2 * hw + p] : 0.f;
        const float qc = pin ? pin[f * 2 * hw + hw + p] : 0.f;
        pout[f * 2 * hw + p] = fmaf(-tau, gr, qr) * ri;
        pout[f * 2 * hw + hw + p] = fmaf(-tau, gc, qc) * ri;
    }
}

// u = f - div p
__global__ void k_tape_u(const float *__restrict__ fsrc, const float *__restrict__ pp,
                         float *__restrict__ u, int64_t nf, int H, int W) {
    const int64_t hw = (int64_t)H * W;
    GRID_LOOP(i, nf * hw) {
        const int64_t f = i / hw, p = i - f * hw;
        const int r = (int)(p / W), c = (int)(p - (int64_t)r * W);
        const float *pr = pp + f * 2 * hw, *pc = pr + hw;
        const float up = r > 0 ? pr[p - W] : 0.f;
        const float lf = c > 0 ? pc[p - 1] : 0.f;
        const float d = ((pr[p] + pc[p]) - up) - lf;
        u[i] = fsrc[i] - d;
    }
}

// ---------------------------------------------------------- TV adjoint
// fbar = ubar; pbar = grad ubar  (u_T = f - div p_T)
__global__ void k_tvb_init(const float *__restrict__ ub, float *__restrict__ fb,
                           float *__restrict__ pb, int64_t nf, int H, int W) {
    const int64_t hw = (int64_t)H * W;
    GRID_LOOP(i, nf * hw) {
        const int64_t f = i / hw, p = i - f * hw;
        const int r = (int)(p / W), c = (int)(p - (int64_t)r * W);
        const float v = ub[i];
        fb[i] = v;
        pb[f * 2 * hw + p] = (r + 1 < H) ? ub[i + W] - v : 0.f;
        pb[f * 2 * hw + hw + p] = (c + 1 < W) ? ub[i + 1] - v : 0.f;
    }
}

// gbar_k from u_k (g_k, n_k, r_k), p_{k+1} and pbar_{k+1}
__global__ void k_tvb_g(const float *__restrict__ u, const float *__restrict__ pnext,
                        const float *__restrict__ pb, float *__restrict__ gb, int64_t nf, int H,
                        int W, float tau, float tw) {
    const int64_t hw = (int64_t)H * W;
    GRID_LOOP(i, nf * hw) {
        const int64_t f = i / hw, p = i - f * hw;
        const int r = (int)(p / W), c = (int)(p - (int64_t)r * W);
        const float *uf = u + f * hw;
        const float uc = uf[p];
        const bool hr = r + 1 < H, hc = c + 1 < W;
        const float gr = hr ? uf[p + W] - uc : 0.f;
        const float gc = hc ? uf[p + 1] - uc : 0.f;
        const float nrm = sqrt_approx(fmaf(gr, gr, gc * gc));
        const float ri = rcp_approx(fmaf(tw, nrm, 1.f));
        const int64_t o = f * 2 * hw + p;
        const float br = pb[o], bc = pb[o + hw];
        const float dot = br * pnext[o] + bc * pnext[o + hw];
        const float coef = nrm > 0.f ? -tw * ri * dot / nrm : 0.f;
        gb[o] = hr ? fmaf(-tau * ri, br, coef * gr) : 0.f;
        gb[o + hw] = hc ? fmaf(-tau * ri, bc, coef * gc) : 0.f;
    }
}

__device__ __forceinline__ float neg_div(const float *gr, const float *gc, int64_t p, int r, int c,
                                         int W) {
    const float up = r > 0 ? gr[p - W] : 0.f;
    const float lf = c > 0 ? gc[p - 1] : 0.f;
    return -(((gr[p] + gc[p]) - up) - lf);
}

// ubar_k = -div gbar_k; fbar += ubar_k; (k >= 1) pbar_k = r_k pbar_{k+1} + grad ubar_k
__global__ void k_tvb_u(const float *__restrict__ gb, const float *__restrict__ u,
                        const float *__restrict__ pb_in, float *__restrict__ pb_out,
                        float *__restrict__ fb, int64_t nf, int H, int W, float tw) {
    const int64_t hw = (int64_t)H * W;
    GRID_LOOP(i, nf * hw) {
        const int64_t f = i / hw, p = i - f * hw;
        const int r = (int)(p / W), c = (int)(p - (int64_t)r * W);
        const float *gr = gb + f * 2 * hw, *gc = gr + hw;
        const float ub = neg_div(gr, gc, p, r, c, W);
        fb[i] += ub;
        if (pb_out) {
            const float *uf = u + f * hw;
            const float uc = uf[p];
            const bool hr = r + 1 < H, hc = c + 1 < W;
            const float g1 = hr ? uf[p + W] - uc : 0.f;
            const float g2 = hc ? uf[p + 1] - uc : 0.f;
            const float ri = rcp_approx(fmaf(tw, sqrt_approx(fmaf(g1, g1, g2 * g2)), 1.f));
            const float ubr = hr ? neg_div(gr, gc, p + W, r + 1, c, W) - ub : 0.f;
            const float ubc = hc ? neg_div(gr, gc, p + 1, r, c + 1, W) - ub : 0.f;
            const int64_t o = f * 2 * hw + p;
            pb_out[o] = fmaf(ri, pb_in[o], ubr);
            pb_out[o + hw] = fmaf(ri, pb_in[o + hw], ubc);
        }
    }
}

// --------------------------------------------------- projection adjoint
// One thread per pixel, looping over the N items; accumulates dPhi, dPhi_sum
// and d lambda_k, carries dy1 and dy, and writes xbar^k.
__global__ void k_proj_bwd(const float *__restrict__ vb, const float *__restrict__ x,
                           const float *__restrict__ phi, const float *__restrict__ ps,
                           const float *__restrict__ y1, const float *__restrict__ lambdas, int k,
                           float *__restrict__ y1c, float *__restrict__ ybar,
                           float *__restrict__ phib, float *__restrict__ psb,
                           double *__restrict__ lamb, float *__restrict__ xb, int N, int B,
                           int64_t hw) {
    const float lam = lambdas[k];
    double lacc = 0.0;
    GRID_LOOP(p, hw) {
        const float s = ps[p];
        float psacc = 0.f;
        for (int n = 0; n < N; ++n) {
            const float *xn = x + (int64_t)n * B * hw;
            const float *vn = vb + (int64_t)n * B * hw;
            float yb = 0.f, pv = 0.f;
            for (int b = 0; b < B; ++b) {
                const float m = phi[b * hw + p];
                yb = fmaf(xn[b * hw + p], m, yb);
                pv = fmaf(vn[b * hw + p], m, pv);
            }
            const int64_t i = (int64_t)n * hw + p;
            const float q = (y1[i] - yb) / s;
            lacc += (double)pv * q;
            const float qb = lam * pv;
            const float y1t = y1c[i] + qb / s;
            psacc -= qb * q / s;
            const float ybb = -qb / s - y1t;
            ybar[i] += y1t;
            y1c[i] = y1t;
            float *xbn = xb + (int64_t)n * B * hw;
            for (int b = 0; b < B; ++b) {
                const float m = phi[b * hw + p];
                const float v = vn[b * hw + p];
                xbn[b * hw + p] = fmaf(m, ybb, v);
                phib[b * hw + p] += fmaf(q * lam, v, xn[b * hw + p] * ybb);
            }
        }
        psb[p] += psacc;
    }
    for (int o = 16; o > 0; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(lamb + k, lacc);
}

// Adjoint of x^0 = At(y / Phi_sum), y = A(x_true), Phi_sum = sum Phi_b and
// Phi = sigmoid(logits): writes dlogits.
__global__ void k_init_bwd(const float *__restrict__ x0b, const float *__restrict__ xt,
                           const float *__restrict__ phi, const float *__restrict__ ps,
                           const float *__restrict__ y, const float *__restrict__ ybar,
                           float *__restrict__ phib, const float *__restrict__ psb,
                           float *__restrict__ glog, float gscale, int N, int B, int64_t hw) {
    GRID_LOOP(p, hw) {
        const float s = ps[p];
        float psacc = psb[p];
        for (int n = 0; n < N; ++n) {
            const int64_t i = (int64_t)n * hw + p;
            const float *xbn = x0b + (int64_t)n * B * hw;
            const float *xtn = xt + (int64_t)n * B * hw;
            const float s0 = y[i] / s;
            float s0b = 0.f;
            for (int b = 0; b < B; ++b) s0b = fmaf(phi[b * hw + p], xbn[b * hw + p], s0b);
            const float yt = ybar[i] + s0b / s;
            psacc -= s0b * s0 / s;
            for (int b = 0; b < B; ++b)
                phib[b * hw + p] += fmaf(s0, xbn[b * hw + p], xtn[b * hw + p] * yt);
        }
        for (int b = 0; b < B; ++b) {
            const float m = phi[b * hw + p];
            glog[b * hw + p] = gscale * (phib[b * hw + p] + psacc) * m * (1.f - m);
        }
    }
}

struct Ws {
    float *phi, *ps, *y, *X, *Y1, *V;          // forward
    float *tu, *tp;                            // tape: u_1..u_{T-1}, p_1..p_{T-1}
    float *pb0, *pb1, *gb, *fb, *xb, *y1c, *ybar, *phib, *psb;  // reverse
    double *loss;
    void *tv;
    size_t tv_bytes;
};

size_t layout(int64_t N, int64_t B, int64_t H, int64_t W, int K, int T, Ws *w, char *base) {
    const size_t hw = (size_t)(H * W), nbhw = (size_t)(N * B) * hw, nhw = (size_t)N * hw;
    const int U = T - 1;
    size_t off = 0;
    auto take = [&](size_t floats) {
        size_t o = off;
        off += (floats * 4 + 255) & ~size_t(255);
        return o;
    };
    const size_t o_phi = take(B * hw), o_ps = take(hw), o_y = take(nhw);
    const size_t o_X = take((K + 1) * nbhw), o_Y1 = take((size_t)K * nhw), o_V = take(nbhw);
    const size_t o_tu = take((size_t)(U > 1 ? U - 1 : 1) * nbhw), o_tp = take((size_t)U * 2 * nbhw);
    const size_t o_pb0 = take(2 * nbhw), o_pb1 = take(2 * nbhw), o_gb = take(2 * nbhw);
    const size_t o_fb = take(nbhw), o_xb = take(nbhw), o_y1c = take(nhw), o_ybar = take(nhw);
    const size_t o_phib = take(B * hw), o_psb = take(hw), o_loss = take(4);
    const size_t tvb = tv_workspace_bytes(N * B, H, W, T);
    const size_t o_tv = off;
    off += (tvb + 255) & ~size_t(255);
    if (w) {
        auto F = [&](size_t o) { return reinterpret_cast<float *>(base + o); };
        w->phi = F(o_phi); w->ps = F(o_ps); w->y = F(o_y); w->X = F(o_X); w->Y1 = F(o_Y1);
        w->V = F(o_V); w->tu = F(o_tu); w->tp = F(o_tp); w->pb0 = F(o_pb0); w->pb1 = F(o_pb1);
        w->gb = F(o_gb); w->fb = F(o_fb); w->xb = F(o_xb); w->y1c = F(o_y1c);
        w->ybar = F(o_ybar); w->phib = F(o_phib); w->psb = F(o_psb);
        w->loss = reinterpret_cast<double *>(base + o_loss);
        w->tv = base + o_tv;
        w->tv_bytes = tvb;
    }
    return off;
}

int check(int64_t N, int64_t B, int64_t H, int64_t W, int K, int T, float weight) {
    SCI_CHECK_ARG(N >= 1 && B >= 1 && H >= 1 && W >= 1 && K >= 1, "unrolled: invalid sizes");
    SCI_CHECK_ARG(T >= 2 && T <= 5, "unrolled: tv_iters must be in [2, 5] (got %d)", T);
    SCI_CHECK_ARG(weight > 0.f, "unrolled: tv_weight must be > 0");
    return SCI_OK;
}

// forward: fills the checkpoints; loss (device double) = mean sq. error
int forward(const float *logits, const float *lambdas, const float *xt, int64_t N, int64_t B,
            int64_t H, int64_t W, int K, int T, float weight, Ws &w, cudaStream_t s) {
    const int64_t hw = H * W, nbhw = N * B * hw;
    const dim3 g = grid1(N * hw, 256);
    k_mask<<<grid1(hw, 256), 256, 0, s>>>(logits, w.phi, w.ps, (int)B, hw);
    k_meas_x0<<<g, 256, 0, s>>>(xt, w.phi, w.ps, w.y, w.X, (int)N, (int)B, hw);
    SCI_LAUNCHED("k_meas_x0");
    for (int k = 0; k < K; ++k) {
        k_proj_fwd<<<g, 256, 0, s>>>(w.X + k * nbhw, w.phi, w.ps, w.y,
                                     k ? w.Y1 + (k - 1) * N * hw : nullptr, w.Y1 + k * N * hw,
                                     w.V, lambdas, k, (int)N, (int)B, hw);
        SCI_LAUNCHED("k_proj_fwd");
        int e = tv_launch_flags(w.V, w.X + (k + 1) * nbhw, nullptr, N * B, H, W, hw, weight,
                                0.f, T, nullptr, nullptr, w.tv, w.tv_bytes, s, 0, kNoStop);
        if (e) return e;
    }
    SCI_CUDA(cudaMemsetAsync(w.loss, 0, sizeof(double), s));
    k_mse<<<grid1(nbhw, 256), 256, 0, s>>>(w.X + K * nbhw, xt, nullptr, 0.f, nbhw, w.loss);
    SCI_LAUNCHED("k_mse");
    return SCI_OK;
}

// Cached CUDA graphs of whole forward / reverse passes (keyed by every
// argument): the reverse pass is ~20 launches per outer iteration.
struct GraphCache {
    std::mutex mu;
    std::list<std::pair<std::string, cudaGraphExec_t>> e;
};
GraphCache &cache() {
    static GraphCache c;
    return c;
}

template <typename F>
int run_graph(const std::string &key, cudaStream_t s, F enqueue) {
    GraphCache &gc = cache();
    {
        std::lock_guard<std::mutex> lk(gc.mu);
        for (auto &kv : gc.e)
            if (kv.first == key) {
                SCI_CUDA(cudaGraphLaunch(kv.second, s));
                return SCI_OK;
            }
    }
    cudaStream_t cs;
    SCI_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaError_t ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = SCI_OK;
    if (ce == cudaSuccess) rc = enqueue(cs);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce2 = (ce == cudaSuccess) ? cudaStreamEndCapture(cs, &graph) : ce;
    cudaStreamDestroy(cs);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (ce2 != cudaSuccess) return cuda_status(ce2, "unrolled graph capture");
    cudaGraphExec_t exec = nullptr;
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return cuda_status(ce, "cudaGraphInstantiate");
    {
        std::lock_guard<std::mutex> lk(gc.mu);
        gc.e.emplace_front(key, exec);
        while (gc.e.size() > 8) {
            cudaGraphExecDestroy(gc.e.back().second);
            gc.e.pop_back();
        }
    }
    SCI_CUDA(cudaGraphLaunch(exec, s));
    return SCI_OK;
}

template <typename... T>
std::string make_key(const T &...v) {
    std::string k;
    (k.append(reinterpret_cast<const char *>(&v), sizeof(T)), ...);
    return k;
}

}  // namespace unr
}  // namespace sci

using namespace sci;
using namespace sci::unr;

extern "C" {

int sci_unrolled_workspace_bytes(int64_t N, int64_t B, int64_t H, int64_t W, int K, int tv_iters,
                                 size_t *bytes) {
    SCI_CHECK_ARG(bytes, "null bytes");
    if (int e = check(N, B, H, W, K, tv_iters, 1.f)) return e;
    *bytes = layout(N, B, H, W, K, tv_iters, nullptr, nullptr);
    return SCI_OK;
}

int sci_unrolled_fwd(const float *logits, const float *lambdas, const float *x_true, int64_t N,
                     int64_t B, int64_t H, int64_t W, int K, int tv_iters, float tv_weight,
                     double *loss, float *x_out, void *workspace, size_t workspace_bytes,
                     void *stream) {
    if (int e = check(N, B, H, W, K, tv_iters, tv_weight)) return e;
    SCI_CHECK_ARG(logits && lambdas && x_true, "sci_unrolled_fwd: null pointer");
    const size_t need = layout(N, B, H, W, K, tv_iters, nullptr, nullptr);
    SCI_CHECK_ARG(workspace && workspace_bytes >= need,
                  "sci_unrolled_fwd: workspace of %zu bytes needed, got %zu", need,
                  workspace_bytes);
    Ws w;
    layout(N, B, H, W, K, tv_iters, &w, static_cast<char *>(workspace));
    const int64_t nbhw = N * B * H * W;
    auto body = [&](cudaStream_t s) -> int {
        if (int e = forward(logits, lambdas, x_true, N, B, H, W, K, tv_iters, tv_weight, w, s))
            return e;
        if (loss)
            SCI_CUDA(cudaMemcpyAsync(loss, w.loss, sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (x_out)
            SCI_CUDA(cudaMemcpyAsync(x_out, w.X + (int64_t)K * nbhw, 4 * nbhw,
                                     cudaMemcpyDeviceToDevice, s));
        return SCI_OK;
    };
    const std::string key = make_key(1, logits, lambdas, x_true, N, B, H, W, K, tv_iters,
                                     tv_weight, loss, x_out, workspace);
    return run_graph(key, as_stream(stream), body);
}

int sci_unrolled_bwd(const float *logits, const float *lambdas, const float *x_true, int64_t N,
                     int64_t B, int64_t H, int64_t W, int K, int tv_iters, float tv_weight,
                     float grad_loss, float *grad_logits, double *grad_lambdas,
                     void *workspace, size_t workspace_bytes, void *stream) {
    if (int e = check(N, B, H, W, K, tv_iters, tv_weight)) return e;
    SCI_CHECK_ARG(logits && lambdas && x_true && grad_logits && grad_lambdas,
                  "sci_unrolled_bwd: null pointer");
    const size_t need = layout(N, B, H, W, K, tv_iters, nullptr, nullptr);
    SCI_CHECK_ARG(workspace && workspace_bytes >= need,
                  "sci_unrolled_bwd: workspace of %zu bytes needed, got %zu", need,
                  workspace_bytes);
    Ws w;
    layout(N, B, H, W, K, tv_iters, &w, static_cast<char *>(workspace));
    const std::string key = make_key(2, logits, lambdas, x_true, N, B, H, W, K, tv_iters,
                                     tv_weight, grad_loss, grad_logits, grad_lambdas, workspace);
    return run_graph(key, as_stream(stream), [&](cudaStream_t s) -> int {
    // The checkpoints of the preceding sci_unrolled_fwd call on this
    // workspace (same arguments) are used as they are.
    const int64_t hw = H * W, nbhw = N * B * hw, nhw = N * hw, nf = N * B;
    const int T = tv_iters, U = T - 1;
    const float tau = 0.25f, tw = 0.25f / tv_weight;
    const dim3 g = grid1(nbhw, 256), gp = grid1(hw, 128);
    // dL/dx^K = grad_loss * 2 (x^K - x_true) / numel
    k_mse<<<g, 256, 0, s>>>(w.X + (int64_t)K * nbhw, x_true, w.xb,
                            2.f * grad_loss / (float)nbhw, nbhw, nullptr);
    SCI_LAUNCHED("k_mse");
    SCI_CUDA(cudaMemsetAsync(w.y1c, 0, 4 * nhw, s));
    SCI_CUDA(cudaMemsetAsync(w.ybar, 0, 4 * nhw, s));
    SCI_CUDA(cudaMemsetAsync(w.phib, 0, 4 * B * hw, s));
    SCI_CUDA(cudaMemsetAsync(w.psb, 0, 4 * hw, s));
    SCI_CUDA(cudaMemsetAsync(grad_lambdas, 0, sizeof(double) * K, s));
    for (int k = K - 1; k >= 0; --k) {
        // recompute v^k and the TV tape
        k_proj_fwd<<<grid1(nhw, 256), 256, 0, s>>>(
            w.X + k * nbhw, w.phi, w.ps, w.y, k ? w.Y1 + (k - 1) * nhw : nullptr,
            w.Y1 + k * nhw, w.V, lambdas, k, (int)N, (int)B, hw);
        const float *u_prev = w.V;  // u_0 = f = v^k
        for (int j = 0; j < U; ++j) {
            float *pj = w.tp + (int64_t)j * 2 * nbhw;  // p_{j+1}
            k_tape_p<<<g, 256, 0, s>>>(u_prev, j ? w.tp + (int64_t)(j - 1) * 2 * nbhw : nullptr,
                                       pj, nf, (int)H, (int)W, tau, tw);
            if (j + 1 < U) {
                float *uj = w.tu + (int64_t)j * nbhw;  // u_{j+1}
                k_tape_u<<<g, 256, 0, s>>>(w.V, pj, uj, nf, (int)H, (int)W);
                u_prev = uj;
            }
        }
        SCI_LAUNCHED("tv tape");
        // TV adjoint: fbar = d/dv^k
        k_tvb_init<<<g, 256, 0, s>>>(w.xb, w.fb, w.pb0, nf, (int)H, (int)W);
        float *pb_in = w.pb0, *pb_out = w.pb1;
        for (int j = U - 1; j >= 0; --j) {
            const float *uj = j == 0 ? w.V : w.tu + (int64_t)(j - 1) * nbhw;  // u_j
            k_tvb_g<<<g, 256, 0, s>>>(uj, w.tp + (int64_t)j * 2 * nbhw, pb_in, w.gb, nf, (int)H,
                                      (int)W, tau, tw);
            k_tvb_u<<<g, 256, 0, s>>>(w.gb, uj, pb_in, j ? pb_out : nullptr, w.fb, nf, (int)H,
                                      (int)W, tw);
            float *t = pb_in;
            pb_in = pb_out;
            pb_out = t;
        }
        SCI_LAUNCHED("tv adjoint");
        // projection adjoint: xbar^k
        k_proj_bwd<<<gp, 128, 0, s>>>(w.fb, w.X + k * nbhw, w.phi, w.ps, w.Y1 + k * nhw,
                                       lambdas, k, w.y1c, w.ybar, w.phib, w.psb, grad_lambdas,
                                       w.xb, (int)N, (int)B, hw);
        SCI_LAUNCHED("k_proj_bwd");
    }
    k_init_bwd<<<gp, 128, 0, s>>>(w.xb, x_true, w.phi, w.ps, w.y, w.ybar, w.phib, w.psb,
                                  grad_logits, 1.f, (int)N, (int)B, hw);
    SCI_LAUNCHED("k_init_bwd");
    return SCI_OK;
    });
}

}  // extern "C"
