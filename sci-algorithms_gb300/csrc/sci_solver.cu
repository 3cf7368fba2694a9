// GAP-TV / ADMM-TV iteration loops (PnP_SCI/python/pnp_sci_algo.py:536-706
// and :708-864 for denoiser='tv') as a native runtime: the whole loop is
// enqueued on one stream -- per iteration one fused projection kernel, one
// TV pass and its stop-test launch -- and, with use_graph, captured once into
// a CUDA graph that is cached per argument set and replayed with a single
// launch.
#include <cstring>
#include <string>
#include <utility>

#include "sci_common.cuh"
#include "sci_graph.cuh"

namespace sci {

int tv_launch(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
              int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
              void *workspace, size_t ws_bytes, cudaStream_t s, int force_R);
size_t tv_workspace_bytes(int64_t nf, int64_t H, int64_t W, int K);
int tv_launch_impl(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
                   int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
                   void *workspace, size_t ws_bytes, cudaStream_t s, int force_R, int flags,
                   const uint32_t *proj_bits, const float *proj_c, float proj_lam);
bool tv_proj_supported(int64_t nf, int64_t W, int K);
int tvx_launch(int kind, const float *f, float *u, float *resid, int64_t nf, int64_t H,
               int64_t W, float lam, int iters, int *steps, void *ws, size_t ws_bytes,
               cudaStream_t s);
size_t tvx_workspace_bytes(int kind, int64_t nf, int64_t H, int64_t W, int iters);
int launch_proj_admm_tma(const float *th, const float *bb, const uint32_t *bits, const float *y,
                         const float *phisum, float *v, float *xo, float lam, float gamma, int B,
                         int64_t hw, cudaStream_t s, bool b_from_v, double *rn);
int proj_gap_rn(const float *x, const float *phi, const uint32_t *mask_bits, const float *y,
                float *y1, const float *phisum, float *x_out, float lambda, int accelerate,
                int64_t B, int64_t H, int64_t W, void *stream, double *rn);
int gap_residual_rn(const float *x, const float *phi, const uint32_t *mask_bits,
                    const float *y, float *y1, const float *phisum, float *c,
                    int accelerate, int64_t B, int64_t H, int64_t W, void *stream, double *rn,
                    double *zero, int nzero);
double *tv_clear_region(int64_t nf, int64_t H, int64_t W, int K, void *workspace, int *words);
int admm_residual_rn(const float *t, const uint32_t *mask_bits, const float *y,
                     const float *phisum, float *r_new, float *x_out, float lambda, float gamma,
                     int first, int64_t B, int64_t H, int64_t W, void *stream, double *rn,
                     double *zero, int nzero);
int tv_launch_tout(const float *f, float *u, int64_t nf, int64_t H, int64_t W, int64_t fs,
                   float weight, float eps, int K, int *steps, void *workspace, size_t ws_bytes,
                   cudaStream_t s, int flags, const uint32_t *proj_bits, const float *proj_c,
                   float proj_lam, float *tout);
int proj_admm_rn(const float *theta, const float *b, const float *phi,
                 const uint32_t *mask_bits, const float *y, const float *phisum, float *v,
                 float *x_out, float lambda, float gamma, int64_t B, int64_t H, int64_t W,
                 void *stream, double *rn);

namespace {

struct SolverWs {
    float *y1, *xp, *c, *theta, *v, *b0, *b1;
    void *tv;
    size_t tv_bytes;
};

size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

// tvm: 0 = scikit-image Chambolle (K steps with the stop test), 1..8 = the
// MATLAB denoisers of sci_tv_matlab (K iterations).
size_t solver_layout(bool admm, int64_t B, int64_t H, int64_t W, int K, int tvm, SolverWs *w,
                     char *base) {
    const size_t hw = (size_t)(H * W), n = (size_t)B * hw;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += round256(bytes);
        return o;
    };
    size_t oy1 = 0, oxp = 0, oc = 0, oth = 0, ov = 0, ob0 = 0, ob1 = 0;
    if (!admm) {
        oy1 = take(sizeof(float) * hw);
        oxp = take(sizeof(float) * n);
        oc = take(sizeof(float) * hw);
    } else {
        oth = take(sizeof(float) * n);
        ov = take(sizeof(float) * n);
        ob0 = take(sizeof(float) * n);
        ob1 = take(sizeof(float) * n);
    }
    const size_t tvb =
        tvm ? tvx_workspace_bytes(tvm, B, H, W, K) : tv_workspace_bytes(B, H, W, K);
    const size_t otv = take(tvb);
    if (w) {
        w->y1 = admm ? nullptr : reinterpret_cast<float *>(base + oy1);
        w->xp = admm ? nullptr : reinterpret_cast<float *>(base + oxp);
        w->c = admm ? nullptr : reinterpret_cast<float *>(base + oc);
        w->theta = admm ? reinterpret_cast<float *>(base + oth) : nullptr;
        w->v = admm ? reinterpret_cast<float *>(base + ov) : nullptr;
        w->b0 = admm ? reinterpret_cast<float *>(base + ob0) : nullptr;
        w->b1 = admm ? reinterpret_cast<float *>(base + ob1) : nullptr;
        w->tv = base + otv;
        w->tv_bytes = tvb;
    }
    return off;
}

template <typename T>
void put_bytes(std::string &k, const T &v) {
    k.append(reinterpret_cast<const char *>(&v), sizeof(T));
}

struct Args {
    bool admm;
    const float *y, *phi;
    const uint32_t *bits;
    const float *phisum, *x0;
    float *x_out;
    int64_t B, H, W;
    sci_solve_opts o;
    void *ws;
    size_t ws_bytes;

    std::string key() const {
        std::string k;
        put_bytes(k, admm);
        put_bytes(k, y);
        put_bytes(k, phi);
        put_bytes(k, bits);
        put_bytes(k, phisum);
        put_bytes(k, x0);
        put_bytes(k, x_out);
        put_bytes(k, B);
        put_bytes(k, H);
        put_bytes(k, W);
        put_bytes(k, o.iters);
        put_bytes(k, o.tv_iter_max);
        put_bytes(k, o.eps);
        put_bytes(k, o.tvm);
        put_bytes(k, o.accelerate);
        put_bytes(k, o.gamma);
        put_bytes(k, o.orig);
        put_bytes(k, o.sqerr);
        put_bytes(k, o.tv_steps);
        put_bytes(k, o.resid_norm);
        put_bytes(k, ws);
        k.append(reinterpret_cast<const char *>(o.lambdas), sizeof(float) * o.iters);
        k.append(reinterpret_cast<const char *>(o.weights), sizeof(float) * o.iters);
        put_bytes(k, o.gammas != nullptr);
        if (o.gammas) k.append(reinterpret_cast<const char *>(o.gammas), sizeof(float) * o.iters);
        return k;
    }
};

// Enqueues the whole solve on stream s.
int enqueue(const Args &a, cudaStream_t s) {
    const sci_solve_opts &o = a.o;
    const int64_t B = a.B, H = a.H, W = a.W, hw = H * W, n = B * hw;
    const int K = o.tv_iter_max;
    SolverWs w;
    solver_layout(a.admm, B, H, W, K, o.tvm, &w, static_cast<char *>(a.ws));
    // the denoising step of iteration `it` (pnp_sci_algo.py:650, :812-813;
    // MATLAB twin: gapdenoise.m:92-112, whose Chambolle files take 1/tvweight)
    auto denoise = [&](const float *in, float *out, float *resid, int it) -> int {
        int *steps = o.tv_steps ? o.tv_steps + (int64_t)it * B : nullptr;
        if (o.tvm) {
            const bool inv = o.tvm == 3 || o.tvm == 5 || o.tvm == 7;
            const float lam = inv ? 1.0f / o.weights[it] : o.weights[it];
            return tvx_launch(o.tvm, in, out, resid, B, H, W, lam, K, steps, w.tv, w.tv_bytes,
                              s);
        }
        return tv_launch(in, out, resid, B, H, W, hw, o.weights[it], o.eps, K, steps, nullptr,
                         w.tv, w.tv_bytes, s, 0);
    };
    if (o.sqerr) SCI_CUDA(cudaMemsetAsync(o.sqerr, 0, sizeof(double) * o.iters, s));
    if (o.resid_norm) SCI_CUDA(cudaMemsetAsync(o.resid_norm, 0, sizeof(double) * o.iters, s));
    // FP64 ||r||^2 of iteration `it`'s projection residual (nullable)
    auto rn = [&](int it) { return o.resid_norm ? o.resid_norm + it : nullptr; };
    const bool aligned = ((reinterpret_cast<uintptr_t>(a.x0) | reinterpret_cast<uintptr_t>(a.x_out) |
                           reinterpret_cast<uintptr_t>(a.y) | reinterpret_cast<uintptr_t>(a.phisum) |
                           reinterpret_cast<uintptr_t>(a.bits)) & 15u) == 0;
    if (!a.admm && !o.tvm && a.bits && aligned && hw % 4 == 0 && tv_proj_supported(B, W, K)) {
        // Fused iteration: a read-only pass forms the residual map c (and
        // y1); the TV kernel applies x + lambda (c phi_b) while it loads x.
        // x ping-pongs between x_out and xp; start so the last iterate
        // lands in x_out.
        float *X[2] = {a.x_out, w.xp};
        const int start = o.iters & 1;
        if (a.x0 != X[start])
            SCI_CUDA(cudaMemcpyAsync(X[start], a.x0, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        if (o.accelerate) SCI_CUDA(cudaMemsetAsync(w.y1, 0, sizeof(float) * hw, s));
        // the residual pass also clears the TV pass's stop-test sums, so
        // that the TV kernel follows it directly (flags 4)
        int nzero = 0;
        double *zero = tv_clear_region(B, H, W, K, w.tv, &nzero);
        for (int it = 0; it < o.iters; ++it) {
            const float *cur = X[(start + it) & 1];
            float *nxt = X[(start + it + 1) & 1];
            int e = gap_residual_rn(cur, nullptr, a.bits, a.y, w.y1, a.phisum, w.c,
                                    o.accelerate, B, H, W, s, rn(it), zero, nzero);
            if (e) return e;
            e = tv_launch_impl(cur, nxt, nullptr, B, H, W, hw, o.weights[it], o.eps, K,
                               o.tv_steps ? o.tv_steps + (int64_t)it * B : nullptr, nullptr, w.tv,
                               w.tv_bytes, s, 0, 4, a.bits, w.c, o.lambdas[it]);
            if (e) return e;
            if (o.orig && o.sqerr) {
                e = sci_sqerr_accum(o.orig, nxt, n, o.sqerr + it, s);
                if (e) return e;
            }
        }
        return SCI_OK;
    }
    if (!a.admm) {
        // gap_denoise: x = x0; y1 = 0  (pnp_sci_algo.py:633-635)
        if (a.x0 != a.x_out)
            SCI_CUDA(cudaMemcpyAsync(a.x_out, a.x0, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        if (o.accelerate) SCI_CUDA(cudaMemsetAsync(w.y1, 0, sizeof(float) * hw, s));
        for (int it = 0; it < o.iters; ++it) {
            int e = proj_gap_rn(a.x_out, a.phi, a.bits, a.y, w.y1, a.phisum, w.xp,
                                o.lambdas[it], o.accelerate, B, H, W, s, rn(it));
            if (e) return e;
            e = denoise(w.xp, a.x_out, nullptr, it);
            if (e) return e;
            if (o.orig && o.sqerr) {
                e = sci_sqerr_accum(o.orig, a.x_out, n, o.sqerr + it, s);
                if (e) return e;
            }
        }
        return SCI_OK;
    }
    // admm_denoise: theta = x0, b = 0  (pnp_sci_algo.py:800-802)
    SCI_CUDA(cudaMemcpyAsync(w.theta, a.x0, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    const char *af = getenv("SCI_ADMM_FUSED");
    if (!o.tvm && a.bits && aligned && hw % 4 == 0 && tv_proj_supported(B, W, K) &&
        !(af && af[0] == '0')) {
        // Fused iteration: a read-only pass forms the residual map r_k from
        // t_k = theta_k + b_k; the TV kernel applies theta_k + lambda_k
        // (r_k phi_b) = x - b while it loads theta_k and stores theta_{k+1}
        // and t_{k+1} = theta_{k+1} + (theta_{k+1} - v_k).  theta ping-pongs
        // between w.theta and w.b0; t lives in w.v, the map in w.b1.
        float *T[2] = {w.theta, w.b0};
        float *tb = w.v, *R = w.b1;
        int nzero = 0;
        double *zero = tv_clear_region(B, H, W, K, w.tv, &nzero);
        for (int it = 0; it < o.iters; ++it) {
            const bool want_x = (it == o.iters - 1) || (o.orig && o.sqerr);
            const float gamma = o.gammas ? o.gammas[it] : o.gamma;
            float *cur = T[it & 1], *nxt = T[(it + 1) & 1];
            int e = admm_residual_rn(it ? tb : cur, a.bits, a.y, a.phisum, R,
                                     want_x ? a.x_out : nullptr, o.lambdas[it], gamma, it == 0, B,
                                     H, W, s, rn(it), zero, nzero);
            if (e) return e;
            e = tv_launch_tout(cur, nxt, B, H, W, hw, o.weights[it], o.eps, K,
                               o.tv_steps ? o.tv_steps + (int64_t)it * B : nullptr, w.tv,
                               w.tv_bytes, s, 4, a.bits, R, o.lambdas[it], tb);
            if (e) return e;
            if (o.orig && o.sqerr) {
                e = sci_sqerr_accum(o.orig, a.x_out, n, o.sqerr + it, s);
                if (e) return e;
            }
        }
        return SCI_OK;
    }
    const char *bv = getenv("SCI_ADMM_B_FROM_V");
    if (a.bits && aligned && hw % 4 == 0 && B <= 32 && !(bv && bv[0] == '0')) {
        // b = b - (x - theta) = theta - v (pnp_sci_algo.py:836) is the TV's
        // residual: the next projection forms it from theta and the TV input
        // v, so the TV pass writes no residual (20N instead of 24N bytes per
        // iteration, the same values bit for bit).  v ping-pongs between b0
        // and b1; v_{-1} = theta_0 gives b_0 = 0.
        SCI_CUDA(cudaMemcpyAsync(w.b1, a.x0, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        float *vprev = w.b1, *vcur = w.b0;
        for (int it = 0; it < o.iters; ++it) {
            const bool want_x = (it == o.iters - 1) || (o.orig && o.sqerr);
            const float gamma = o.gammas ? o.gammas[it] : o.gamma;
            int e = launch_proj_admm_tma(w.theta, vprev, a.bits, a.y, a.phisum, vcur,
                                         want_x ? a.x_out : nullptr, o.lambdas[it], gamma,
                                         (int)B, hw, s, true, rn(it));
            if (e) return e;
            e = denoise(vcur, w.theta, nullptr, it);
            if (e) return e;
            if (o.orig && o.sqerr) {
                e = sci_sqerr_accum(o.orig, a.x_out, n, o.sqerr + it, s);
                if (e) return e;
            }
            std::swap(vprev, vcur);
        }
        return SCI_OK;
    }
    SCI_CUDA(cudaMemsetAsync(w.b0, 0, sizeof(float) * n, s));
    float *bcur = w.b0, *bnext = w.b1;
    for (int it = 0; it < o.iters; ++it) {
        const bool want_x = (it == o.iters - 1) || (o.orig && o.sqerr);
        const float gamma = o.gammas ? o.gammas[it] : o.gamma;
        int e = proj_admm_rn(w.theta, bcur, a.phi, a.bits, a.y, a.phisum, w.v,
                             want_x ? a.x_out : nullptr, o.lambdas[it], gamma, B, H, W, s,
                             rn(it));
        if (e) return e;
        // theta = TV(x - b);  b = b - (x - theta) = theta - v
        e = denoise(w.v, w.theta, bnext, it);
        if (e) return e;
        if (o.orig && o.sqerr) {
            e = sci_sqerr_accum(o.orig, a.x_out, n, o.sqerr + it, s);
            if (e) return e;
        }
        std::swap(bcur, bnext);
    }
    return SCI_OK;
}

int solve(const Args &a, void *stream) {
    const sci_solve_opts &o = a.o;
    SCI_CHECK_ARG(a.B >= 1 && a.H >= 1 && a.W >= 1, "solver: invalid sizes");
    SCI_CHECK_ARG(a.y && a.phisum && a.x0 && a.x_out && (a.phi || a.bits),
                  "solver: null pointer");
    SCI_CHECK_ARG(!a.bits || a.B <= 32, "solver: packed mask needs B <= 32");
    SCI_CHECK_ARG(o.iters >= 0 && o.tv_iter_max >= 1, "solver: iters >= 0, tv_iter_max >= 1");
    SCI_CHECK_ARG(o.iters == 0 || (o.lambdas && o.weights), "solver: schedules missing");
    for (int i = 0; i < o.iters; ++i)
        SCI_CHECK_ARG(o.weights[i] > 0.f, "solver: tv_weight[%d] = %g must be > 0", i,
                      (double)o.weights[i]);
    SCI_CHECK_ARG(o.tvm >= 0 && o.tvm <= 8, "solver: tvm must be 0..8 (got %d)", o.tvm);
    SCI_CHECK_ARG(!o.tvm || (a.H >= 2 && a.W >= 2), "solver: the MATLAB TVs need H, W >= 2");
    const size_t need =
        solver_layout(a.admm, a.B, a.H, a.W, o.tv_iter_max, o.tvm, nullptr, nullptr);
    SCI_CHECK_ARG(a.ws && a.ws_bytes >= need, "solver: workspace of %zu bytes needed, got %zu",
                  need, a.ws_bytes);
    cudaStream_t s = as_stream(stream);
    if (o.iters == 0) {
        if (a.x0 != a.x_out)
            SCI_CUDA(cudaMemcpyAsync(a.x_out, a.x0, sizeof(float) * a.B * a.H * a.W,
                                     cudaMemcpyDeviceToDevice, s));
        return SCI_OK;
    }
    if (!o.use_graph) return enqueue(a, s);

    return run_graph("solver graph capture", a.key(), s,
                     [&](cudaStream_t cs) { return enqueue(a, cs); });
}

}  // namespace
}  // namespace sci

using namespace sci;

extern "C" {

int sci_solver_workspace_bytes(int64_t B, int64_t H, int64_t W, const sci_solve_opts *opts,
                               size_t *bytes) {
    SCI_CHECK_ARG(opts && bytes && B >= 1 && H >= 1 && W >= 1 && opts->tv_iter_max >= 1 &&
                      opts->tvm >= 0 && opts->tvm <= 8,
                  "sci_solver_workspace_bytes: bad argument");
    const int t = opts->tvm;
    const size_t g = solver_layout(false, B, H, W, opts->tv_iter_max, t, nullptr, nullptr);
    const size_t a = solver_layout(true, B, H, W, opts->tv_iter_max, t, nullptr, nullptr);
    *bytes = g > a ? g : a;
    return SCI_OK;
}

int sci_gap_tv(const float *y, const float *phi, const uint32_t *mask_bits, const float *phisum,
               const float *x0, float *x_out, int64_t B, int64_t H, int64_t W,
               const sci_solve_opts *opts, void *workspace, size_t workspace_bytes,
               void *stream) {
    SCI_CHECK_ARG(opts, "sci_gap_tv: opts is NULL");
    Args a{false, y, phi, mask_bits, phisum, x0, x_out, B, H, W, *opts, workspace,
           workspace_bytes};
    return solve(a, stream);
}

int sci_admm_tv(const float *y, const float *phi, const uint32_t *mask_bits, const float *phisum,
                const float *x0, float *x_out, int64_t B, int64_t H, int64_t W,
                const sci_solve_opts *opts, void *workspace, size_t workspace_bytes,
                void *stream) {
    SCI_CHECK_ARG(opts, "sci_admm_tv: opts is NULL");
    Args a{true, y, phi, mask_bits, phisum, x0, x_out, B, H, W, *opts, workspace,
           workspace_bytes};
    return solve(a, stream);
}

}  // extern "C"
