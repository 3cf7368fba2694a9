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
// Design: one kernel per iteration over the whole stack, one thread per
// pixel (kinds 7 and 8: one thread per pixel position, looping over the
// frames for the coupled norm).  A thread recomputes the few primal values
// its dual update needs from the neighbouring duals (served by L1), so an
// iteration reads the input and the duals once and writes the duals once.
// The last dual update of the FGP loop and of the clip loops does not reach
// the returned value and is not computed.
#include <cmath>
#include <utility>

#include "sci_common.cuh"

namespace sci {
namespace tvx {

enum Kind {
    CLIP_A = 1, CLIP_B = 2, CHAM_ATV = 3, FGP_ATV = 4,
    CHAM_ITV2D = 5, FGP_ITV2D = 6, CHAM_ITV3D = 7, FGP_ITV3D = 8
};

struct Geo {
    int H, W;
    int64_t hw;
};

__device__ __forceinline__ float clipv(float v, float c) {
    // sign(v) .* min(|v|, c)
    return v > 0.f ? fminf(v, c) : (v < 0.f ? -fminf(-v, c) : 0.f);
}

// ------------------------------------------------------------ clip family
// x0 at (i, j) from y0 and the duals zh (valid j <= W-2), zv (i <= H-2):
// dht(zh)_j = -zh_0 (j = 0), -(zh_j - zh_{j-1}), zh_{W-2} (j = W-1).
template <int KIND>
__device__ __forceinline__ float clip_x0(const float *f, const float *zh, const float *zv,
                                         const Geo &g, int i, int j) {
    const int64_t p = (int64_t)i * g.W + j;
    const float dht = (j == 0) ? -zh[p] : (j == g.W - 1 ? zh[p - 1] : -(zh[p] - zh[p - 1]));
    const float dvt = (i == 0) ? -zv[p] : (i == g.H - 1 ? zv[p - g.W] : -(zv[p] - zv[p - g.W]));
    const float y0 = f[p];
    if (KIND == CLIP_A) return ((y0 - dht) + (y0 - dvt)) * 0.5f;  // (x0h + x0v)./2
    return (y0 - dht) - dvt;
}

template <int KIND>
__global__ void k_clip_update(const float *__restrict__ f, const float *__restrict__ zh,
                              const float *__restrict__ zv, float *__restrict__ zh2,
                              float *__restrict__ zv2, Geo g, float bound) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.H || j >= g.W) return;
    const int64_t fo = (int64_t)blockIdx.z * g.hw;
    f += fo, zh += fo, zv += fo, zh2 += fo, zv2 += fo;
    const float x = clip_x0<KIND>(f, zh, zv, g, i, j);
    const int64_t p = (int64_t)i * g.W + j;
    const float ia = 1.f / 5.f;  // 1/alpha
    if (j < g.W - 1) {
        const float xr = clip_x0<KIND>(f, zh, zv, g, i, j + 1);
        zh2[p] = clipv(zh[p] + ia * (xr - x), bound);
    }
    if (i < g.H - 1) {
        const float xd = clip_x0<KIND>(f, zh, zv, g, i + 1, j);
        zv2[p] = clipv(zv[p] + ia * (xd - x), bound);
    }
}

template <int KIND>
__global__ void k_clip_out(const float *__restrict__ f, const float *__restrict__ zh,
                           const float *__restrict__ zv, float *__restrict__ u,
                           float *__restrict__ resid, Geo g) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.H || j >= g.W) return;
    const int64_t fo = (int64_t)blockIdx.z * g.hw;
    const int64_t p = (int64_t)i * g.W + j;
    const float x = clip_x0<KIND>(f + fo, zh + fo, zv + fo, g, i, j);
    u[fo + p] = x;
    if (resid) resid[fo + p] = x - f[fo + p];
}

// -------------------------------------------------------- Chambolle family
// divp = p1 - p1(:,il) + p2 - p2(iu,:): no p at the first column / row.
__device__ __forceinline__ float cham_divp(const float *p1, const float *p2, const Geo &g, int i,
                                           int j) {
    const int64_t p = (int64_t)i * g.W + j;
    const float a = p1[p], l = j > 0 ? p1[p - 1] : a;
    const float b = p2[p], t = i > 0 ? p2[p - g.W] : b;
    return ((a - l) + b) - t;
}

// z = divp - f lambda and its forward differences z1 (along W), z2 (along H),
// 0 at the last column / row.
__device__ __forceinline__ void cham_grad(const float *f, const float *p1, const float *p2,
                                          const Geo &g, int i, int j, float lam, bool first,
                                          float &z1, float &z2) {
    const int64_t p = (int64_t)i * g.W + j;
    auto zat = [&](int ii, int jj, int64_t q) {
        const float d = first ? 0.f : cham_divp(p1, p2, g, ii, jj);
        return d - f[q] * lam;
    };
    const float z = zat(i, j, p);
    z1 = (j < g.W - 1) ? zat(i, j + 1, p + 1) - z : 0.f;
    z2 = (i < g.H - 1) ? zat(i + 1, j, p + g.W) - z : 0.f;
}

template <int KIND>
__global__ void k_cham_update(const float *__restrict__ f, const float *__restrict__ p1,
                              const float *__restrict__ p2, float *__restrict__ q1,
                              float *__restrict__ q2, Geo g, float lam, float dt, int first) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.H || j >= g.W) return;
    const int64_t fo = (int64_t)blockIdx.z * g.hw;
    f += fo, p1 += fo, p2 += fo, q1 += fo, q2 += fo;
    const int64_t p = (int64_t)i * g.W + j;
    float z1, z2;
    cham_grad(f, p1, p2, g, i, j, lam, first != 0, z1, z2);
    const float a = first ? 0.f : p1[p], b = first ? 0.f : p2[p];
    if (KIND == CHAM_ATV) {
        const float t1 = a + dt * z1, t2 = b + dt * z2;
        q1[p] = t1 / fmaxf(1.f, fabsf(t1));
        q2[p] = t2 / fmaxf(1.f, fabsf(t2));
    } else {
        const float denom = 1.f + dt * sqrtf(z1 * z1 + z2 * z2);
        q1[p] = (a + dt * z1) / denom;
        q2[p] = (b + dt * z2) / denom;
    }
}

// ITV3D: denom = 1 + dt sqrt(sum over frames of z1^2 + z2^2), one thread
// per pixel position.
__global__ void k_cham_update_coupled(const float *__restrict__ f, const float *__restrict__ p1,
                                      const float *__restrict__ p2, float *__restrict__ q1,
                                      float *__restrict__ q2, Geo g, int nf, float lam, float dt,
                                      int first) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.H || j >= g.W) return;
    const int64_t p = (int64_t)i * g.W + j;
    float s = 0.f;
    for (int b = 0; b < nf; ++b) {
        const int64_t fo = (int64_t)b * g.hw;
        float z1, z2;
        cham_grad(f + fo, p1 + fo, p2 + fo, g, i, j, lam, first != 0, z1, z2);
        s += z1 * z1 + z2 * z2;
    }
    const float denom = 1.f + dt * sqrtf(s);
    for (int b = 0; b < nf; ++b) {
        const int64_t fo = (int64_t)b * g.hw;
        float z1, z2;
        cham_grad(f + fo, p1 + fo, p2 + fo, g, i, j, lam, first != 0, z1, z2);
        const float a = first ? 0.f : p1[fo + p], c = first ? 0.f : p2[fo + p];
        q1[fo + p] = (a + dt * z1) / denom;
        q2[fo + p] = (c + dt * z2) / denom;
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

__global__ void k_fgp_update_coupled(const float *__restrict__ xo, float *__restrict__ P1,
                                     float *__restrict__ P2, const float *__restrict__ r1,
                                     const float *__restrict__ r2, float *__restrict__ s1,
                                     float *__restrict__ s2, Geo g, int nf, float lam, float c,
                                     float mom, int first) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.H || j >= g.W) return;
    const int64_t p = (int64_t)i * g.W + j;
    float s = 0.f;
    for (int b = 0; b < nf; ++b) {
        const int64_t fo = (int64_t)b * g.hw;
        float a, c2;
        fgp_step(xo + fo, r1 + fo, r2 + fo, g, i, j, lam, c, first != 0, a, c2);
        s += a * a + c2 * c2;
    }
    const float A = sqrtf(fmaxf(s, 1.f));
    for (int b = 0; b < nf; ++b) {
        const int64_t fo = (int64_t)b * g.hw;
        float a, c2;
        fgp_step(xo + fo, r1 + fo, r2 + fo, g, i, j, lam, c, first != 0, a, c2);
        a = a / A;
        c2 = c2 / A;
        const float o1 = first ? 0.f : P1[fo + p], o2 = first ? 0.f : P2[fo + p];
        P1[fo + p] = a;
        P2[fo + p] = c2;
        s1[fo + p] = a + mom * (a - o1);
        s2[fo + p] = c2 + mom * (c2 - o2);
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

int planes(int kind) {
    switch (kind) {
        case FGP_ATV: case FGP_ITV2D: case FGP_ITV3D: return 6;
        default: return 4;
    }
}

}  // namespace tvx

size_t tvx_workspace_bytes(int kind, int64_t nf, int64_t H, int64_t W) {
    return sizeof(float) * (size_t)tvx::planes(kind) * (size_t)(nf * H * W);
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
    SCI_CHECK_ARG(nf <= 65535 && H <= (1 << 24) && W <= (1 << 24), "tv_matlab: sizes too large");
    SCI_CHECK_ARG(lam > 0.f, "tv_matlab: lambda must be > 0");
    const size_t need = tvx_workspace_bytes(kind, nf, H, W);
    SCI_CHECK_ARG(ws && ws_bytes >= need, "tv_matlab: workspace of %zu bytes needed, got %zu",
                  need, ws_bytes);
    // one frame: MATLAB's 2-D branches
    if (nf == 1 && kind == CLIP_B) kind = CLIP_A;
    if (nf == 1 && kind == CHAM_ATV) kind = CHAM_ITV2D;
    const int64_t hw = H * W, n = nf * hw;
    Geo g{(int)H, (int)W, hw};
    const dim3 blk(32, 8);
    const dim3 grd((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8), (unsigned)nf);
    const dim3 grd1((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8), 1);
    float *w0 = static_cast<float *>(ws);
    float *a1 = w0, *a2 = w0 + n, *b1 = w0 + 2 * n, *b2 = w0 + 3 * n;
    if (steps) {
        k_fill<<<(unsigned)((nf + 255) / 256), 256, 0, s>>>(steps, iters, (int)nf);
        SCI_LAUNCHED("k_fill");
    }
    switch (kind) {
        case CLIP_A:
        case CLIP_B: {
            // TV_denoising.m:23-33 / TV_denoising_clip_LB.m:23-34
            const float bound = kind == CLIP_A ? lam / 2 : lam;
            SCI_CUDA(cudaMemsetAsync(a1, 0, sizeof(float) * 2 * n, s));
            float *zh = a1, *zv = a2, *zh2 = b1, *zv2 = b2;
            for (int it = 0; it + 1 < iters; ++it) {
                if (kind == CLIP_A)
                    k_clip_update<CLIP_A><<<grd, blk, 0, s>>>(f, zh, zv, zh2, zv2, g, bound);
                else
                    k_clip_update<CLIP_B><<<grd, blk, 0, s>>>(f, zh, zv, zh2, zv2, g, bound);
                SCI_LAUNCHED("k_clip_update");
                std::swap(zh, zh2);
                std::swap(zv, zv2);
            }
            if (kind == CLIP_A) k_clip_out<CLIP_A><<<grd, blk, 0, s>>>(f, zh, zv, u, resid, g);
            else k_clip_out<CLIP_B><<<grd, blk, 0, s>>>(f, zh, zv, u, resid, g);
            SCI_LAUNCHED("k_clip_out");
            return SCI_OK;
        }
        case CHAM_ATV:
        case CHAM_ITV2D:
        case CHAM_ITV3D: {
            // tvdenoise_cham_*.m:62-93
            const float dt = kind == CHAM_ITV3D ? 0.25f : 0.125f;
            float *p1 = a1, *p2 = a2, *q1 = b1, *q2 = b2;
            for (int it = 0; it < iters; ++it) {
                const int first = it == 0;
                if (kind == CHAM_ITV3D)
                    k_cham_update_coupled<<<grd1, blk, 0, s>>>(f, p1, p2, q1, q2, g, (int)nf, lam,
                                                               dt, first);
                else if (kind == CHAM_ATV)
                    k_cham_update<CHAM_ATV><<<grd, blk, 0, s>>>(f, p1, p2, q1, q2, g, lam, dt,
                                                                first);
                else
                    k_cham_update<CHAM_ITV2D><<<grd, blk, 0, s>>>(f, p1, p2, q1, q2, g, lam, dt,
                                                                  first);
                SCI_LAUNCHED("k_cham_update");
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
                    k_fgp_update_coupled<<<grd1, blk, 0, s>>>(f, P1, P2, r1, r2, s1, s2, g,
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

int sci_tv_matlab_workspace_bytes(int kind, int64_t nframes, int64_t H, int64_t W,
                                  size_t *bytes) {
    SCI_CHECK_ARG(bytes && kind >= 1 && kind <= 8 && nframes >= 1 && H >= 1 && W >= 1,
                  "sci_tv_matlab_workspace_bytes: bad argument");
    *bytes = sci::tvx_workspace_bytes(kind, nframes, H, W);
    return SCI_OK;
}

int sci_tv_matlab(int kind, const float *f, float *u, int64_t nframes, int64_t H, int64_t W,
                  float lambda, int iters, void *workspace, size_t workspace_bytes,
                  void *stream) {
    return sci::tvx_launch(kind, f, u, nullptr, nframes, H, W, lambda, iters, nullptr, workspace,
                           workspace_bytes, sci::as_stream(stream));
}

}  // extern "C"
