// The MATLAB twin's TV denoisers (the tvm switch of
// PnP_SCI/matlab/algorithms/gapdenoise.m:92-112) on the planar frame stack.
//
//   kind 1 ATV_ClipA   TV_denoising.m             clipped dual steps, x0 = mean of h/v
//   kind 2 ATV_ClipB   TV_denoising_clip_LB.m     x0 = y0 - dht(zh) - dvt(zv), clip at lambda
//   kind 3 ATV_cham    tvdenoise_cham_ATV2D.m     Chambolle, duals projected on [-1, 1]
//   kind 4 ATV_FGP     fgp_denoise_ATV2D.m        fast gradient projection, [-1, 1]
//   kind 5 ITV2D_cham  tvdenoise_cham_ITV2D.m     Chambolle, dt = 1/8, per-frame norm
//   kind 6 ITV2D_FGP   fgp_denoise_ITV2D.m        fast gradient projection, per-frame norm
//   kind 7 ITV3D_cham  tvdenoise_cham_ITV3D.m     Chambolle, dt = 1/4, norm over all frames
//   kind 8 ITV3D_FGP   fgp_denoise_ITV3D.m        fast gradient projection, norm over frames
//
// MATLAB sees a one-frame stack as a 2-D image, and two files take another
// branch for it: ClipB then runs ClipA's update and ATV_cham the isotropic
// per-frame update.  The host maps those cases to kinds 1 and 5.
//
// Design.  The clip files and the per-frame Chambolle files are the same
// shape of recurrence as the scikit-image TV (u = f - c div p, a dual
// update from the forward differences of u), so kinds 1, 2, 3 and 5 run on
// the temporally blocked TV pipeline (sci_tv.cuh, RULE_CLIP /
// RULE_CHAM_ATV / RULE_CHAM_ITV): the stack crosses HBM once per 4 dual
// updates.  The FGP files (two dual fields and a momentum) and ITV3D_cham
// (a norm summed over all frames of a pixel) run one kernel per iteration
// over the stack, one thread per pixel (kinds 7 and 8: per pixel position,
// looping over the frames); a thread recomputes the few primal values its
// dual update needs from the neighbouring duals (served by L1).  The last
// dual update of the FGP loop does not reach the returned value and is not
// computed.
#include <cmath>
#include <utility>

#include "sci_common.cuh"
#include "sci_tv.cuh"

namespace sci {

int tv_launch_rule(int rule, const float *f, float *u, float *resid, int64_t nf, int64_t H,
                   int64_t W, int updates, float tau, float tw, float c1, float c2, int *steps,
                   void *workspace, size_t ws_bytes, cudaStream_t s);
size_t tv_workspace_bytes(int64_t nf, int64_t H, int64_t W, int K);

namespace tvx {

enum Kind {
    CLIP_A = 1, CLIP_B = 2, CHAM_ATV = 3, FGP_ATV = 4,
    CHAM_ITV2D = 5, FGP_ITV2D = 6, CHAM_ITV3D = 7, FGP_ITV3D = 8
};

struct Geo {
    int H, W;
    int64_t hw;
};

// -------------------------------------------------------- Chambolle family
// divp = p1 - p1(:,il) + p2 - p2(iu,:): no p at the first column / row.
__device__ __forceinline__ float cham_divp(const float *p1, const float *p2, const Geo &g, int i,
                                           int j) {
    const int64_t p = (int64_t)i * g.W + j;
    const float a = p1[p], l = j > 0 ? p1[p - 1] : a;
    const float b = p2[p], t = i > 0 ? p2[p - g.W] : b;
    return ((a - l) + b) - t;
}

// Frame-coupled kernels (ITV3D): a block covers 32 pixels of one row with
// FL frame lanes (threadIdx.y); lane l handles frames l, l+FL, ... (at most
// FMAX per lane, kept in registers), the per-pixel sum over frames is
// reduced in shared memory in a fixed order, then every lane updates its
// frames.
constexpr int FL = 8, FMAX = 4;  // frame lanes; frames per lane (nf <= 32)

__device__ __forceinline__ float lane_reduce(float v, float (*red)[32]) {
    red[threadIdx.y][threadIdx.x] = v;
    __syncthreads();
    float s = 0.f;
#pragma unroll
    for (int l = 0; l < FL; ++l) s += red[l][threadIdx.x];
    __syncthreads();
    return s;
}

// ITV3D: denom = 1 + dt sqrt(sum over frames of z1^2 + z2^2).  A block
// owns a strip of 32 columns and RB rows and walks down it: per row it
// loads p1, p2 and f of the next row once (the left neighbour of p1 and
// the right neighbour of z come by shuffle; lanes 0 and 31 load the strip's
// halo columns), reduces the norm over the frames in shared memory and
// writes the updated duals of the row.
#ifndef SCI_ITV3D_RB
#define SCI_ITV3D_RB 16
#endif
constexpr int RB = SCI_ITV3D_RB;  // rows per block

__global__ void __launch_bounds__(32 * FL) k_cham_update_coupled(
    const float *__restrict__ f, const float *__restrict__ p1, const float *__restrict__ p2,
    float *__restrict__ q1, float *__restrict__ q2, Geo g, int nf, float lam, float dt,
    int first) {
    __shared__ float red[FL][32];
    const int lane = threadIdx.x;
    const int x0 = blockIdx.x * 32, j = x0 + lane;
    const int i0 = blockIdx.y * RB, i1 = min(i0 + RB, g.H);
    const bool in = j < g.W;
    const int jc = in ? j : g.W - 1;           // a valid column for the loads
    const bool right = x0 + 32 < g.W;          // the strip has a right halo column
    const int jr = right ? x0 + 32 : jc;
    // z at (i, col) from p1(i, col), p1(i, col-1), p2(i, col), p2(i-1, col), f
    auto zval = [&](float a, float al, float b, float bu, float fv) {
        return (((a - al) + b) - bu) - fv * lam;
    };
    float zc[FMAX], zr[FMAX], p1c[FMAX], p2c[FMAX], p2r[FMAX];
#pragma unroll
    for (int t = 0; t < FMAX; ++t) {  // row i0
        const int b = threadIdx.y + t * FL;
        zc[t] = zr[t] = p1c[t] = p2c[t] = p2r[t] = 0.f;
        if (b >= nf) continue;
        const int64_t fo = (int64_t)b * g.hw;
        const int64_t o = fo + (int64_t)i0 * g.W;
        if (first) {
            zc[t] = -f[o + jc] * lam;
            if (lane == 31 && right) zr[t] = -f[o + jr] * lam;
            continue;
        }
        const float a = p1[o + jc], bb = p2[o + jc];
        const float al = (jc > 0) ? p1[o + jc - 1] : a;
        const float bu = (i0 > 0) ? p2[o - g.W + jc] : bb;
        zc[t] = zval(a, al, bb, bu, f[o + jc]);
        p1c[t] = a;
        p2c[t] = bb;
        if (lane == 31 && right) {
            const float ar = p1[o + jr], br = p2[o + jr];
            const float bur = (i0 > 0) ? p2[o - g.W + jr] : br;
            zr[t] = zval(ar, p1[o + jr - 1], br, bur, f[o + jr]);
            p2r[t] = br;
        }
    }
    for (int i = i0; i < i1; ++i) {
        const bool lastrow = i + 1 >= g.H;
        float z1[FMAX], z2[FMAX], zn[FMAX], p1n[FMAX], p2n[FMAX], zrn[FMAX], p2rn[FMAX];
        float s = 0.f;
        // every load of row i + 1 first, by all lanes alike (lanes that are
        // not at the strip's edge load their own column for the halo
        // values, an L1 hit), so that one memory latency covers the row
        const int jl = (lane == 0 && x0 > 0) ? x0 - 1 : jc;  // left p1
        const int jh = (lane == 31) ? jr : jc;               // right halo column
        float la[FMAX], lb[FMAX], lf[FMAX], ll[FMAX], ra[FMAX], rb[FMAX], rf[FMAX];
#pragma unroll
        for (int t = 0; t < FMAX; ++t) {
            const int b = threadIdx.y + t * FL;
            la[t] = lb[t] = lf[t] = ll[t] = ra[t] = rb[t] = rf[t] = 0.f;
            if (b >= nf || lastrow) continue;
            const int64_t o = (int64_t)b * g.hw + (int64_t)(i + 1) * g.W;
            lf[t] = f[o + jc];
            rf[t] = f[o + jh];
            if (!first) {
                la[t] = p1[o + jc];
                lb[t] = p2[o + jc];
                ll[t] = p1[o + jl];
                ra[t] = p1[o + jh];
                rb[t] = p2[o + jh];
            }
        }
#pragma unroll
        for (int t = 0; t < FMAX; ++t) {
            const int b = threadIdx.y + t * FL;
            // right neighbour of z in this row (all lanes shuffle)
            float zright = __shfl_down_sync(0xffffffffu, zc[t], 1);
            if (lane == 31) zright = zr[t];
            const float a = la[t];
            float al = __shfl_up_sync(0xffffffffu, a, 1);
            zn[t] = p1n[t] = p2n[t] = zrn[t] = p2rn[t] = 0.f;
            z1[t] = z2[t] = 0.f;
            if (b >= nf) continue;
            if (!lastrow) {  // row i + 1
                if (first) {
                    zn[t] = -lf[t] * lam;
                    if (lane == 31 && right) zrn[t] = -rf[t] * lam;
                } else {
                    const float bb = lb[t];
                    if (lane == 0) al = (x0 > 0) ? ll[t] : a;
                    if (jc == 0) al = a;  // MATLAB: no p1 at the first column
                    zn[t] = zval(a, al, bb, p2c[t], lf[t]);
                    p1n[t] = a;
                    p2n[t] = bb;
                    if (lane == 31 && right) {
                        zrn[t] = zval(ra[t], a, rb[t], p2r[t], rf[t]);
                        p2rn[t] = rb[t];
                    }
                }
            }
            z1[t] = (j < g.W - 1) ? zright - zc[t] : 0.f;
            z2[t] = lastrow ? 0.f : zn[t] - zc[t];
            s += z1[t] * z1[t] + z2[t] * z2[t];
        }
        red[threadIdx.y][lane] = s;
        __syncthreads();
        float tot = 0.f;
#pragma unroll
        for (int l = 0; l < FL; ++l) tot += red[l][lane];
        __syncthreads();
        const float denom = 1.f + dt * sqrtf(tot);
#pragma unroll
        for (int t = 0; t < FMAX; ++t) {
            const int b = threadIdx.y + t * FL;
            if (b < nf && in) {
                const int64_t q = (int64_t)b * g.hw + (int64_t)i * g.W + j;
                q1[q] = (p1c[t] + dt * z1[t]) / denom;
                q2[q] = (p2c[t] + dt * z2[t]) / denom;
            }
            zc[t] = zn[t];
            p1c[t] = p1n[t];
            p2c[t] = p2n[t];
            zr[t] = zrn[t];
            p2r[t] = p2rn[t];
        }
    }
}

__global__ void k_cham_out(const float *__restrict__ f, const float *__restrict__ p1,
                           const float *__restrict__ p2, float *__restrict__ u,
                           float *__restrict__ resid, Geo g, float lam) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.H || j >= g.W) return;
    const int64_t fo = (int64_t)blockIdx.z * g.hw;
    const int64_t p = (int64_t)i * g.W + j;
    const float x = f[fo + p] - cham_divp(p1 + fo, p2 + fo, g, i, j) / lam;
    u[fo + p] = x;
    if (resid) resid[fo + p] = x - f[fo + p];
}

// ------------------------------------------------------------ FGP family
// Lforward(R) at (i, j): R1 valid for i <= H-2, R2 for j <= W-2.
__device__ __forceinline__ float fgp_L(const float *r1, const float *r2, const Geo &g, int i,
                                       int j) {
    const int64_t p = (int64_t)i * g.W + j;
    float v = (i < g.H - 1) ? r1[p] : 0.f;
    if (j < g.W - 1) v = v + r2[p];
    if (i > 0) v = v - r1[p - g.W];
    if (j > 0) v = v - r2[p - 1];
    return v;
}

// One FGP step at (i, j): D = Xobs - lam L(R) at (i,j), (i+1,j), (i,j+1);
// P = R + Ltrans(D) / (8 lam).  Returns the unprojected components.
__device__ __forceinline__ void fgp_step(const float *xo, const float *r1, const float *r2,
                                         const Geo &g, int i, int j, float lam, float c,
                                         bool first, float &P1, float &P2) {
    const int64_t p = (int64_t)i * g.W + j;
    auto D = [&](int ii, int jj, int64_t q) {
        return first ? xo[q] : xo[q] - lam * fgp_L(r1, r2, g, ii, jj);
    };
    const float d = D(i, j, p);
    const float a = first ? 0.f : r1[p], b = first ? 0.f : r2[p];
    P1 = (i < g.H - 1) ? a + c * (d - D(i + 1, j, p + g.W)) : 0.f;
    P2 = (j < g.W - 1) ? b + c * (d - D(i, j + 1, p + 1)) : 0.f;
}

template <int KIND>
__global__ void k_fgp_update(const float *__restrict__ xo, float *__restrict__ P1,
                             float *__restrict__ P2, const float *__restrict__ r1,
                             const float *__restrict__ r2, float *__restrict__ s1,
                             float *__restrict__ s2, Geo g, float lam, float c, float mom,
                             int first) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.H || j >= g.W) return;
    const int64_t fo = (int64_t)blockIdx.z * g.hw;
    xo += fo, P1 += fo, P2 += fo, r1 += fo, r2 += fo, s1 += fo, s2 += fo;
    const int64_t p = (int64_t)i * g.W + j;
    float a, b;
    fgp_step(xo, r1, r2, g, i, j, lam, c, first != 0, a, b);
    if (KIND == FGP_ATV) {
        a = a / fmaxf(fabsf(a), 1.f);
        b = b / fmaxf(fabsf(b), 1.f);
    } else {
        const float A = sqrtf(fmaxf(a * a + b * b, 1.f));
        a = a / A;
        b = b / A;
    }
    const float o1 = first ? 0.f : P1[p], o2 = first ? 0.f : P2[p];
    P1[p] = a;
    P2[p] = b;
    s1[p] = a + mom * (a - o1);
    s2[p] = b + mom * (b - o2);
}

__global__ void __launch_bounds__(32 * FL) k_fgp_update_coupled(
    const float *__restrict__ xo, float *__restrict__ P1, float *__restrict__ P2,
    const float *__restrict__ r1, const float *__restrict__ r2, float *__restrict__ s1,
    float *__restrict__ s2, Geo g, int nf, float lam, float c, float mom, int first) {
    __shared__ float red[FL][32];
    const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y;
    const bool in = j < g.W;
    const int64_t p = (int64_t)i * g.W + j;
    float a[FMAX], b2[FMAX], s = 0.f;
#pragma unroll
    for (int t = 0; t < FMAX; ++t) {
        const int b = threadIdx.y + t * FL;
        a[t] = b2[t] = 0.f;
        if (in && b < nf) {
            const int64_t fo = (int64_t)b * g.hw;
            fgp_step(xo + fo, r1 + fo, r2 + fo, g, i, j, lam, c, first != 0, a[t], b2[t]);
            s += a[t] * a[t] + b2[t] * b2[t];
        }
    }
    const float A = sqrtf(fmaxf(lane_reduce(s, red), 1.f));
#pragma unroll
    for (int t = 0; t < FMAX; ++t) {
        const int b = threadIdx.y + t * FL;
        if (in && b < nf) {
            const int64_t q = (int64_t)b * g.hw + p;
            const float u1 = a[t] / A, u2 = b2[t] / A;
            const float o1 = first ? 0.f : P1[q], o2 = first ? 0.f : P2[q];
            P1[q] = u1;
            P2[q] = u2;
            s1[q] = u1 + mom * (u1 - o1);
            s2[q] = u2 + mom * (u2 - o2);
        }
    }
}

__global__ void k_fgp_out(const float *__restrict__ xo, const float *__restrict__ r1,
                          const float *__restrict__ r2, float *__restrict__ u,
                          float *__restrict__ resid, Geo g, float lam, int first) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.H || j >= g.W) return;
    const int64_t fo = (int64_t)blockIdx.z * g.hw;
    const int64_t p = (int64_t)i * g.W + j;
    const float x = first ? xo[fo + p] : xo[fo + p] - lam * fgp_L(r1 + fo, r2 + fo, g, i, j);
    u[fo + p] = x;
    if (resid) resid[fo + p] = x - xo[fo + p];
}

__global__ void k_fill(int *a, int v, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

// Kinds run on the TV pipeline, and its update rule.
bool on_pipeline(int kind) {
    return kind == CLIP_A || kind == CLIP_B || kind == CHAM_ATV || kind == CHAM_ITV2D;
}

}  // namespace tvx

// Workspace of kind `kind` run with at most `iters` iterations (the
// pipeline kinds carry p through the workspace when they need more than 4
// dual updates).
size_t tvx_workspace_bytes(int kind, int64_t nf, int64_t H, int64_t W, int iters) {
    using namespace tvx;
    if (on_pipeline(kind)) return tv_workspace_bytes(nf, H, W, iters + 1);
    const int planes = (kind == FGP_ATV || kind == FGP_ITV2D || kind == FGP_ITV3D) ? 6 : 4;
    return sizeof(float) * (size_t)planes * (size_t)(nf * H * W);
}

// kind 1..8 as above; lambda and iters are the denoiser's own parameters
// (gapdenoise.m passes tvweight or 1/tvweight, and 5 or 2 iterations).
int tvx_launch(int kind, const float *f, float *u, float *resid, int64_t nf, int64_t H,
               int64_t W, float lam, int iters, int *steps, void *ws, size_t ws_bytes,
               cudaStream_t s) {
    using namespace tvx;
    SCI_CHECK_ARG(kind >= CLIP_A && kind <= FGP_ITV3D, "tv_matlab: unknown kind %d", kind);
    SCI_CHECK_ARG(f && u && f != u && nf >= 1 && H >= 2 && W >= 2 && iters >= 1,
                  "tv_matlab: bad arguments (H, W >= 2, iters >= 1, f != u)");
    SCI_CHECK_ARG(nf <= 65535 && H <= 65535 && W <= (1 << 24), "tv_matlab: sizes too large");
    SCI_CHECK_ARG(nf <= FL * FMAX || (kind != CHAM_ITV3D && kind != FGP_ITV3D),
                  "tv_matlab: the ITV3D kinds take at most %d frames", FL * FMAX);
    SCI_CHECK_ARG(lam > 0.f, "tv_matlab: lambda must be > 0");
    const size_t need = tvx_workspace_bytes(kind, nf, H, W, iters);
    SCI_CHECK_ARG(ws && ws_bytes >= need, "tv_matlab: workspace of %zu bytes needed, got %zu",
                  need, ws_bytes);
    // one frame: MATLAB's 2-D branches
    if (nf == 1 && kind == CLIP_B) kind = CLIP_A;
    if (nf == 1 && kind == CHAM_ATV) kind = CHAM_ITV2D;
    const int64_t hw = H * W, n = nf * hw;
    Geo g{(int)H, (int)W, hw};
    const dim3 blk(32, 8);
    const dim3 grd((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8), (unsigned)nf);
    // frame-coupled kernels: 32 pixels x FL frame lanes per block; FGP one
    // row per block, Chambolle RB rows per block
    const dim3 blkc(32, FL);
    const dim3 grdc((unsigned)((W + 31) / 32), (unsigned)H, 1);
    const dim3 grds((unsigned)((W + 31) / 32), (unsigned)((H + RB - 1) / RB), 1);
    float *w0 = static_cast<float *>(ws);
    float *a1 = w0, *a2 = w0 + n, *b1 = w0 + 2 * n, *b2 = w0 + 3 * n;
    if (steps) {
        k_fill<<<(unsigned)((nf + 255) / 256), 256, 0, s>>>(steps, iters, (int)nf);
        SCI_LAUNCHED("k_fill");
    }
    switch (kind) {
        case CLIP_A:
        case CLIP_B:
            // TV_denoising.m:23-33 / TV_denoising_clip_LB.m:23-34: x0 of the
            // last iteration sees iters-1 dual updates; 1/alpha = 1/5
            return tv_launch_rule(tv::RULE_CLIP, f, u, resid, nf, H, W, iters - 1, 0.2f, 0.f,
                                  kind == CLIP_A ? lam / 2 : lam, kind == CLIP_A ? 0.5f : 1.f,
                                  nullptr, ws, ws_bytes, s);
        case CHAM_ITV2D:
            // tvdenoise_cham_ITV2D.m:62-93: every iteration's update is live
            return tv_launch_rule(tv::RULE_CHAM_ITV, f, u, resid, nf, H, W, iters, 0.125f,
                                  0.125f * lam, 0.f, 0.f, nullptr, ws, ws_bytes, s);
        case CHAM_ATV:
            // tvdenoise_cham_ATV2D.m:72-88
            return tv_launch_rule(tv::RULE_CHAM_ATV, f, u, resid, nf, H, W, iters, 0.125f, 0.f,
                                  lam, 0.f, nullptr, ws, ws_bytes, s);
        case CHAM_ITV3D: {
            // tvdenoise_cham_ITV3D.m:74-91
            const float dt = 0.25f;
            float *p1 = a1, *p2 = a2, *q1 = b1, *q2 = b2;
            for (int it = 0; it < iters; ++it) {
                k_cham_update_coupled<<<grds, blkc, 0, s>>>(f, p1, p2, q1, q2, g, (int)nf, lam,
                                                            dt, it == 0);
                SCI_LAUNCHED("k_cham_update_coupled");
                std::swap(p1, q1);
                std::swap(p2, q2);
            }
            k_cham_out<<<grd, blk, 0, s>>>(f, p1, p2, u, resid, g, lam);
            SCI_LAUNCHED("k_cham_out");
            return SCI_OK;
        }
        default: {
            // fgp_denoise_*.m:73-131: the step size 1/(8 lambda) and the
            // momentum (t_k - 1) / t_{k+1} with t_1 = 1
            float *P1 = a1, *P2 = a2, *r1 = b1, *r2 = b2;
            float *s1 = w0 + 4 * n, *s2 = w0 + 5 * n;
            const float c = (float)(1.0 / (8.0 * (double)lam));
            double tk = 1.0;
            for (int it = 0; it + 1 < iters; ++it) {
                const double tkp1 = (1.0 + std::sqrt(1.0 + 4.0 * tk * tk)) / 2.0;
                const float mom = (float)((tk - 1.0) / tkp1);
                const int first = it == 0;
                if (kind == FGP_ITV3D)
                    k_fgp_update_coupled<<<grdc, blkc, 0, s>>>(f, P1, P2, r1, r2, s1, s2, g,
                                                               (int)nf, lam, c, mom, first);
                else if (kind == FGP_ATV)
                    k_fgp_update<FGP_ATV><<<grd, blk, 0, s>>>(f, P1, P2, r1, r2, s1, s2, g, lam,
                                                              c, mom, first);
                else
                    k_fgp_update<FGP_ITV2D><<<grd, blk, 0, s>>>(f, P1, P2, r1, r2, s1, s2, g,
                                                                lam, c, mom, first);
                SCI_LAUNCHED("k_fgp_update");
                std::swap(r1, s1);
                std::swap(r2, s2);
                tk = tkp1;
            }
            k_fgp_out<<<grd, blk, 0, s>>>(f, r1, r2, u, resid, g, lam, iters == 1);
            SCI_LAUNCHED("k_fgp_out");
            return SCI_OK;
        }
    }
}

}  // namespace sci

extern "C" {

int sci_tv_matlab_workspace_bytes(int kind, int64_t nframes, int64_t H, int64_t W, int iters,
                                  size_t *bytes) {
    SCI_CHECK_ARG(bytes && kind >= 1 && kind <= 8 && nframes >= 1 && H >= 1 && W >= 1 &&
                      iters >= 1,
                  "sci_tv_matlab_workspace_bytes: bad argument");
    *bytes = sci::tvx_workspace_bytes(kind, nframes, H, W, iters);
    return SCI_OK;
}

int sci_tv_matlab(int kind, const float *f, float *u, int64_t nframes, int64_t H, int64_t W,
                  float lambda, int iters, void *workspace, size_t workspace_bytes,
                  void *stream) {
    return sci::tvx_launch(kind, f, u, nullptr, nframes, H, W, lambda, iters, nullptr, workspace,
                           workspace_bytes, sci::as_stream(stream));
}

}  // extern "C"
