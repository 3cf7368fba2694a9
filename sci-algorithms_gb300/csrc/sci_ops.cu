// Mask operators and fused projections (the A_/At_ plug-in and the GAP/ADMM
// Euclidean projection of PnP_SCI/python/pnp_sci_algo.py).
//
// Layout: frame stacks are planar B x H x W (W fastest); 2-D maps are H x W.
// Every kernel streams the stack once per pass with 16-byte loads along W
// (one thread = 4 consecutive pixels of all B frames).  These kernels are
// HBM-bound: one pass reads x and the mask once and writes the result once;
// the second sweep over the frames inside the projection is served by L1/L2.
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "sci_common.cuh"

namespace sci {

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

int cuda_status(cudaError_t e, const char *what) {
    set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    return SCI_ERR_CUDA;
}

bool pdl_enabled() {
    const char *e = getenv("SCI_PDL");
    return !(e && atoi(e) == 0);
}

// Sweep direction of the residual passes of the fused iterations.  The TV
// pass walks its row chunks top to bottom, so the last rows it wrote are
// the ones still in L2 when the residual pass starts; a residual pass that
// walks bottom to top reads them there, and ends on the top rows, which
// the next TV pass reads first.  SCI_RESID_REV=0 keeps top to bottom.
static int resid_rev() {
    static const int v = [] {
        const char *e = getenv("SCI_RESID_REV");
        return (e && atoi(e) == 0) ? 0 : 1;
    }();
    return v;
}

int launch_proj_gap_tma(const float *x, const uint32_t *bits, const float *y, float *y1,
                        const float *phisum, float *xo, float lam, bool acc, int B, int64_t hw,
                        cudaStream_t s, double *rn);
int launch_proj_admm_tma(const float *th, const float *bb, const uint32_t *bits, const float *y,
                         const float *phisum, float *v, float *xo, float lam, float gamma, int B,
                         int64_t hw, cudaStream_t s, bool b_from_v, double *rn);

// Grid for a grid-stride loop over `n` work units of one thread each.
static inline dim3 grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)kSMs * 16;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return dim3((unsigned)b);
}

// --------------------------------------------------------- mask helpers
// MODE 0: float mask phi[b][p];  MODE 1: packed bits word[p], bit b.
template <int MODE>
struct Mask;
template <>
struct Mask<0> {
    const float *phi;
    int64_t hw;
    __device__ __forceinline__ float4 at4(int b, int64_t p, uint4) const {
        return ldg4(phi + (int64_t)b * hw + p);
    }
    __device__ __forceinline__ float at1(int b, int64_t p, uint32_t) const {
        return __ldg(phi + (int64_t)b * hw + p);
    }
    __device__ __forceinline__ uint4 word4(int64_t) const { return make_uint4(0, 0, 0, 0); }
    __device__ __forceinline__ uint32_t word1(int64_t) const { return 0u; }
};
template <>
struct Mask<1> {
    const uint32_t *bits;
    int64_t hw;
    __device__ __forceinline__ static float bit(uint32_t w, int b) {
        return ((w >> b) & 1u) ? 1.0f : 0.0f;
    }
    __device__ __forceinline__ float4 at4(int b, int64_t, uint4 w) const {
        return make_float4(bit(w.x, b), bit(w.y, b), bit(w.z, b), bit(w.w, b));
    }
    __device__ __forceinline__ float at1(int b, int64_t, uint32_t w) const { return bit(w, b); }
    __device__ __forceinline__ uint4 word4(int64_t p) const {
        return __ldg(reinterpret_cast<const uint4 *>(bits + p));
    }
    __device__ __forceinline__ uint32_t word1(int64_t p) const { return __ldg(bits + p); }
};

// ------------------------------------------------------------------- A_
__global__ void k_A_vec(const float *__restrict__ x, const float *__restrict__ phi,
                        float *__restrict__ y, int B, int64_t hw) {
    const int64_t n4 = hw >> 2;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = q << 2;
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
        for (int b = 0; b < B; ++b) {
            const float4 a = ldg4(x + b * hw + p), m = ldg4(phi + b * hw + p);
            s.x = fmaf(a.x, m.x, s.x);
            s.y = fmaf(a.y, m.y, s.y);
            s.z = fmaf(a.z, m.z, s.z);
            s.w = fmaf(a.w, m.w, s.w);
        }
        st4(y + p, s);
    }
}
__global__ void k_A_scalar(const float *__restrict__ x, const float *__restrict__ phi,
                           float *__restrict__ y, int B, int64_t hw) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < hw;
         p += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < B; ++b) s = fmaf(__ldg(x + b * hw + p), __ldg(phi + b * hw + p), s);
        y[p] = s;
    }
}

// ------------------------------------------------------------------ At_
__global__ void k_At_vec(const float *__restrict__ y, const float *__restrict__ phi,
                         float *__restrict__ x, int B, int64_t hw) {
    const int64_t n4 = hw >> 2;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = q << 2;
        const float4 v = ldg4(y + p);
#pragma unroll 4
        for (int b = 0; b < B; ++b) {
            const float4 m = ldg4(phi + b * hw + p);
            st4(x + b * hw + p, make_float4(v.x * m.x, v.y * m.y, v.z * m.z, v.w * m.w));
        }
    }
}
__global__ void k_At_scalar(const float *__restrict__ y, const float *__restrict__ phi,
                            float *__restrict__ x, int B, int64_t hw) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < hw;
         p += (int64_t)gridDim.x * blockDim.x) {
        const float v = y[p];
        for (int b = 0; b < B; ++b) x[b * hw + p] = v * __ldg(phi + b * hw + p);
    }
}

// -------------------------------------------------------------- Phi_sum
__global__ void k_phisum(const float *__restrict__ phi, float *__restrict__ s, int B,
                         int64_t hw, int guard) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < hw;
         p += (int64_t)gridDim.x * blockDim.x) {
        float a = 0.f;
        for (int b = 0; b < B; ++b) a += __ldg(phi + b * hw + p);
        if (guard && a == 0.f) a = 1.f;
        s[p] = a;
    }
}

// ------------------------------------------------------------ pack mask
__global__ void k_pack(const float *__restrict__ phi, uint32_t *__restrict__ bits,
                       int *__restrict__ flag, int B, int64_t hw) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < hw;
         p += (int64_t)gridDim.x * blockDim.x) {
        uint32_t w = 0;
        bool bad = false;
        for (int b = 0; b < B; ++b) {
            const float m = __ldg(phi + b * hw + p);
            if (m == 1.f) w |= (1u << b);
            else if (m != 0.f) bad = true;
        }
        bits[p] = w;
        if (bad) *flag = 1;
    }
}

// ------------------------------------------------------ GAP projection
// yb = sum_b phi_b x_b; ACC: y1 += y - yb, r = (y1 - yb)/phisum;
// else r = (y - yb)/phisum; x_out_b = x_b + lambda * (r * phi_b).
template <int MODE, bool ACC>
__global__ void __launch_bounds__(256) k_proj_gap_vec(
    const float *__restrict__ x, Mask<MODE> M, const float *__restrict__ y,
    float *__restrict__ y1, const float *__restrict__ phisum, float *__restrict__ xo,
    float lam, int B, int64_t hw, double *__restrict__ rn) {
    const int64_t n4 = hw >> 2;
    double racc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = q << 2;
        const uint4 w = M.word4(p);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
        for (int b = 0; b < B; ++b) {
            const float4 a = ldg4(x + b * hw + p), m = M.at4(b, p, w);
            s.x = fmaf(a.x, m.x, s.x);
            s.y = fmaf(a.y, m.y, s.y);
            s.z = fmaf(a.z, m.z, s.z);
            s.w = fmaf(a.w, m.w, s.w);
        }
        const float4 yv = ldg4(y + p), ps = ldg4(phisum + p);
        float4 r;
        if (ACC) {
            float4 t = ldg4(y1 + p);
            t.x = t.x + (yv.x - s.x);
            t.y = t.y + (yv.y - s.y);
            t.z = t.z + (yv.z - s.z);
            t.w = t.w + (yv.w - s.w);
            st4(y1 + p, t);
            r = make_float4(__fdiv_rn(t.x - s.x, ps.x), __fdiv_rn(t.y - s.y, ps.y),
                            __fdiv_rn(t.z - s.z, ps.z), __fdiv_rn(t.w - s.w, ps.w));
        } else {
            r = make_float4(__fdiv_rn(yv.x - s.x, ps.x), __fdiv_rn(yv.y - s.y, ps.y),
                            __fdiv_rn(yv.z - s.z, ps.z), __fdiv_rn(yv.w - s.w, ps.w));
        }
        if (rn) rn_add4(racc, r);
#pragma unroll 4
        for (int b = 0; b < B; ++b) {
            const float4 a = ldg4(x + b * hw + p), m = M.at4(b, p, w);
            st4_cs(xo + b * hw + p,
                   make_float4(fmaf(lam, r.x * m.x, a.x), fmaf(lam, r.y * m.y, a.y),
                               fmaf(lam, r.z * m.z, a.z), fmaf(lam, r.w * m.w, a.w)));
        }
    }
    if (rn) rn_flush(racc, rn);
}

template <int MODE, bool ACC>
__global__ void k_proj_gap_scalar(const float *__restrict__ x, Mask<MODE> M,
                                  const float *__restrict__ y, float *__restrict__ y1,
                                  const float *__restrict__ phisum, float *__restrict__ xo,
                                  float lam, int B, int64_t hw, double *__restrict__ rn) {
    double racc = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < hw;
         p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t w = M.word1(p);
        float s = 0.f;
        for (int b = 0; b < B; ++b) s = fmaf(__ldg(x + b * hw + p), M.at1(b, p, w), s);
        float r;
        if (ACC) {
            const float t = y1[p] + (y[p] - s);
            y1[p] = t;
            r = __fdiv_rn(t - s, phisum[p]);
        } else {
            r = __fdiv_rn(y[p] - s, phisum[p]);
        }
        if (rn) rn_add1(racc, r);
        for (int b = 0; b < B; ++b)
            xo[b * hw + p] = fmaf(lam, r * M.at1(b, p, w), __ldg(x + b * hw + p));
    }
    if (rn) rn_flush(racc, rn);
}

// --------------------------------------- register-resident projections
// One pass over HBM: a thread holds the B values of its pixels in registers
// between forming yb and writing the update (the two-sweep kernels above
// re-read x, and under the streaming load the second sweep misses L2).
// BMAX >= B is the unrolled register capacity.
// GAP projection staging each thread's B values of x in shared memory
// (slot [b][thread], bank-conflict free) between the A(x) sum and the
// update, so x crosses HBM once while registers stay low.
template <int MODE, bool ACC>
__global__ void __launch_bounds__(256) k_proj_gap_smem(
    const float *__restrict__ x, Mask<MODE> M, const float *__restrict__ y,
    float *__restrict__ y1, const float *__restrict__ phisum, float *__restrict__ xo,
    float lam, int B, int64_t hw, double *__restrict__ rn) {
    extern __shared__ float xs[];  // [B][blockDim.x]
    const int t = threadIdx.x, nt = blockDim.x;
    double racc = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < hw;
         p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t w = M.word1(p);
        float s = 0.f;
#pragma unroll 8
        for (int b = 0; b < B; ++b) {
            const float v = __ldg(x + b * hw + p);
            xs[b * nt + t] = v;
            s = fmaf(v, M.at1(b, p, w), s);
        }
        const float yv = __ldg(y + p), ps = __ldg(phisum + p);
        float r;
        if (ACC) {
            const float tt = y1[p] + (yv - s);
            y1[p] = tt;
            r = __fdiv_rn(tt - s, ps);
        } else {
            r = __fdiv_rn(yv - s, ps);
        }
        if (rn) rn_add1(racc, r);
#pragma unroll 8
        for (int b = 0; b < B; ++b)
            __stcs(xo + b * hw + p, fmaf(lam, r * M.at1(b, p, w), xs[b * nt + t]));
    }
    if (rn) rn_flush(racc, rn);
}

// ADMM projection staging t = theta + b and b in shared memory (slots
// [b][thread]), one HBM pass over theta and b.
template <int MODE>
__global__ void __launch_bounds__(128) k_proj_admm_smem(
    const float *__restrict__ th, const float *__restrict__ bb, Mask<MODE> M,
    const float *__restrict__ y, const float *__restrict__ phisum, float *__restrict__ v,
    float *__restrict__ xo, float lam, float gamma, int B, int64_t hw, double *__restrict__ rn) {
    extern __shared__ float st[];  // [2][B][blockDim.x]: t, b
    const int t = threadIdx.x, nt = blockDim.x;
    float *ts = st, *bs = st + B * nt;
    double racc = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < hw;
         p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t w = M.word1(p);
        float s = 0.f;
#pragma unroll 8
        for (int b = 0; b < B; ++b) {
            const float bv = __ldg(bb + b * hw + p);
            const float tv = __ldg(th + b * hw + p) + bv;
            ts[b * nt + t] = tv;
            bs[b * nt + t] = bv;
            s = fmaf(tv, M.at1(b, p, w), s);
        }
        const float r = __fdiv_rn(__ldg(y + p) - s, __ldg(phisum + p) + gamma);
        if (rn) rn_add1(racc, r);
#pragma unroll 8
        for (int b = 0; b < B; ++b) {
            const float xv = fmaf(lam, r * M.at1(b, p, w), ts[b * nt + t]);
            if (xo) xo[b * hw + p] = xv;
            __stcs(v + b * hw + p, xv - bs[b * nt + t]);
        }
    }
    if (rn) rn_flush(racc, rn);
}

template <int MODE, bool ACC>
static void launch_gap_smem(const float *x, Mask<MODE> M, const float *y, float *y1,
                            const float *ps, float *xo, float lam, int B, int64_t hw,
                            cudaStream_t s, double *rn) {
    const size_t smem = sizeof(float) * (size_t)B * 256;  // <= 32 KB for B <= 32
    k_proj_gap_smem<MODE, ACC><<<grid_for(hw, 256), 256, smem, s>>>(x, M, y, y1, ps, xo, lam, B,
                                                                    hw, rn);
}

template <int MODE>
static void launch_admm_smem(const float *th, const float *bb, Mask<MODE> M, const float *y,
                             const float *ps, float *v, float *xo, float lam, float gamma, int B,
                             int64_t hw, cudaStream_t s, double *rn) {
    // 128 threads: 2 * B * 128 floats <= 32 KB of shared memory for B <= 32
    const size_t smem = sizeof(float) * 2 * (size_t)B * 128;
    k_proj_admm_smem<MODE><<<grid_for(hw, 128), 128, smem, s>>>(th, bb, M, y, ps, v, xo, lam,
                                                                gamma, B, hw, rn);
}

// ------------------------------------------- GAP residual map (fused path)
// yb = sum_b phi_b x_b; ACC: y1 += y - yb, c = (y1 - yb)/phisum; else
// c = (y - yb)/phisum.  The x update x + lambda (c phi_b) is applied by the
// TV kernel while it loads x (same arithmetic as k_proj_gap).
template <int MODE, bool ACC>
__global__ void __launch_bounds__(256) k_gap_resid_vec(
    const float *__restrict__ x, Mask<MODE> M, const float *__restrict__ y,
    float *__restrict__ y1, const float *__restrict__ phisum, float *__restrict__ c, int B,
    int64_t hw, double *__restrict__ rn, double *__restrict__ zero, int nzero, int rev) {
    grid_dep_wait();
    if (blockIdx.x == 0)  // the next TV pass's stop-test sums
        for (int i = threadIdx.x; i < nzero; i += blockDim.x) zero[i] = 0.0;
    const int64_t n4 = hw >> 2;
    double racc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = (rev ? n4 - 1 - q : q) << 2;  // rev: bottom rows first
        const uint4 w = M.word4(p);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
        for (int b = 0; b < B; ++b) {
            const float4 a = ldg4(x + b * hw + p), m = M.at4(b, p, w);
            s.x = fmaf(a.x, m.x, s.x);
            s.y = fmaf(a.y, m.y, s.y);
            s.z = fmaf(a.z, m.z, s.z);
            s.w = fmaf(a.w, m.w, s.w);
        }
        const float4 yv = ldg4(y + p), ps = ldg4(phisum + p);
        float4 r;
        if (ACC) {
            float4 t = ldg4(y1 + p);
            t.x = t.x + (yv.x - s.x);
            t.y = t.y + (yv.y - s.y);
            t.z = t.z + (yv.z - s.z);
            t.w = t.w + (yv.w - s.w);
            st4(y1 + p, t);
            r = make_float4(__fdiv_rn(t.x - s.x, ps.x), __fdiv_rn(t.y - s.y, ps.y),
                            __fdiv_rn(t.z - s.z, ps.z), __fdiv_rn(t.w - s.w, ps.w));
        } else {
            r = make_float4(__fdiv_rn(yv.x - s.x, ps.x), __fdiv_rn(yv.y - s.y, ps.y),
                            __fdiv_rn(yv.z - s.z, ps.z), __fdiv_rn(yv.w - s.w, ps.w));
        }
        if (rn) rn_add4(racc, r);
        st4(c + p, r);
    }
    if (rn) rn_flush(racc, rn);
}

// ------------------------------------------ ADMM residual map (fused path)
// The ADMM iteration (pnp_sci_algo.py:808-836) with the projection applied
// by the TV kernel while it loads theta: the TV input of iteration k is
// v_k = theta_k + lambda_k (r_k phi_b) (= x - b), its output theta_{k+1},
// and b_{k+1} = b_k - (x_k - theta_{k+1}) = theta_{k+1} - v_k; the TV pass
// also stores t = theta_{k+1} + b_{k+1} (PROJ 3 of the lean pass).  This
// pass reads t (t = theta_0 + 0 at the first iteration), forms
// yb = sum_b phi_b t_b and r_{k+1} = (y - yb) / (phisum + gamma).  With xo
// it also writes x = t + lambda (r phi_b) of every frame (a second sweep).
template <bool FIRST, bool WANT_X>
__global__ void __launch_bounds__(256) k_admm_resid_vec(
    const float *__restrict__ tp, Mask<1> M, const float *__restrict__ y,
    const float *__restrict__ phisum, float *__restrict__ rnew, float *__restrict__ xo, float lam,
    float gamma, int B, int64_t hw, double *__restrict__ rn, double *__restrict__ zero,
    int nzero, int rev) {
    grid_dep_wait();
    if (blockIdx.x == 0)  // the next TV pass's stop-test sums
        for (int i = threadIdx.x; i < nzero; i += blockDim.x) zero[i] = 0.0;
    auto tload = [&](int64_t o) {
        const float4 a = ldg4(tp + o);
        return FIRST ? make_float4(a.x + 0.f, a.y + 0.f, a.z + 0.f, a.w + 0.f) : a;
    };
    const int64_t n4 = hw >> 2;
    double racc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = (rev ? n4 - 1 - q : q) << 2;
        const uint4 w = M.word4(p);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
        for (int b = 0; b < B; ++b) {
            const float4 m = M.at4(b, p, w);
            const float4 t = tload(b * hw + p);
            s.x = fmaf(t.x, m.x, s.x);
            s.y = fmaf(t.y, m.y, s.y);
            s.z = fmaf(t.z, m.z, s.z);
            s.w = fmaf(t.w, m.w, s.w);
        }
        const float4 yv = ldg4(y + p), ps = ldg4(phisum + p);
        const float4 r = make_float4(__fdiv_rn(yv.x - s.x, ps.x + gamma),
                                     __fdiv_rn(yv.y - s.y, ps.y + gamma),
                                     __fdiv_rn(yv.z - s.z, ps.z + gamma),
                                     __fdiv_rn(yv.w - s.w, ps.w + gamma));
        if (rn) rn_add4(racc, r);
        st4(rnew + p, r);
        if (WANT_X) {
#pragma unroll 4
            for (int b = 0; b < B; ++b) {
                const float4 m = M.at4(b, p, w);
                const float4 t = tload(b * hw + p);
                st4(xo + b * hw + p,
                    make_float4(fmaf(lam, r.x * m.x, t.x), fmaf(lam, r.y * m.y, t.y),
                                fmaf(lam, r.z * m.z, t.z), fmaf(lam, r.w * m.w, t.w)));
            }
        }
    }
    if (rn) rn_flush(racc, rn);
}

// ----------------------------------------------------- ADMM projection
// t = theta + b; yb = A(t); x = t + lambda*(r*phi), r = (y-yb)/(phisum+gamma);
// v = x - b.  x written only when xo != nullptr.
template <int MODE>
__global__ void __launch_bounds__(256) k_proj_admm_vec(
    const float *__restrict__ th, const float *__restrict__ bb, Mask<MODE> M,
    const float *__restrict__ y, const float *__restrict__ phisum, float *__restrict__ v,
    float *__restrict__ xo, float lam, float gamma, int B, int64_t hw, double *__restrict__ rn) {
    const int64_t n4 = hw >> 2;
    double racc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = q << 2;
        const uint4 w = M.word4(p);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
        for (int b = 0; b < B; ++b) {
            const float4 a = ldg4(th + b * hw + p), c = ldg4(bb + b * hw + p);
            const float4 m = M.at4(b, p, w);
            s.x = fmaf(a.x + c.x, m.x, s.x);
            s.y = fmaf(a.y + c.y, m.y, s.y);
            s.z = fmaf(a.z + c.z, m.z, s.z);
            s.w = fmaf(a.w + c.w, m.w, s.w);
        }
        const float4 yv = ldg4(y + p), ps = ldg4(phisum + p);
        const float4 r = make_float4(__fdiv_rn(yv.x - s.x, ps.x + gamma),
                                     __fdiv_rn(yv.y - s.y, ps.y + gamma),
                                     __fdiv_rn(yv.z - s.z, ps.z + gamma),
                                     __fdiv_rn(yv.w - s.w, ps.w + gamma));
        if (rn) rn_add4(racc, r);
#pragma unroll 4
        for (int b = 0; b < B; ++b) {
            const float4 a = ldg4(th + b * hw + p), c = ldg4(bb + b * hw + p);
            const float4 m = M.at4(b, p, w);
            const float4 xv = make_float4(fmaf(lam, r.x * m.x, a.x + c.x),
                                          fmaf(lam, r.y * m.y, a.y + c.y),
                                          fmaf(lam, r.z * m.z, a.z + c.z),
                                          fmaf(lam, r.w * m.w, a.w + c.w));
            if (xo) st4(xo + b * hw + p, xv);
            st4_cs(v + b * hw + p,
                   make_float4(xv.x - c.x, xv.y - c.y, xv.z - c.z, xv.w - c.w));
        }
    }
    if (rn) rn_flush(racc, rn);
}

template <int MODE>
__global__ void k_proj_admm_scalar(const float *__restrict__ th, const float *__restrict__ bb,
                                   Mask<MODE> M, const float *__restrict__ y,
                                   const float *__restrict__ phisum, float *__restrict__ v,
                                   float *__restrict__ xo, float lam, float gamma, int B,
                                   int64_t hw, double *__restrict__ rn) {
    double racc = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < hw;
         p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t w = M.word1(p);
        float s = 0.f;
        for (int b = 0; b < B; ++b)
            s = fmaf(__ldg(th + b * hw + p) + __ldg(bb + b * hw + p), M.at1(b, p, w), s);
        const float r = __fdiv_rn(y[p] - s, phisum[p] + gamma);
        if (rn) rn_add1(racc, r);
        for (int b = 0; b < B; ++b) {
            const float t = __ldg(th + b * hw + p) + __ldg(bb + b * hw + p);
            const float xv = fmaf(lam, r * M.at1(b, p, w), t);
            if (xo) xo[b * hw + p] = xv;
            v[b * hw + p] = xv - __ldg(bb + b * hw + p);
        }
    }
    if (rn) rn_flush(racc, rn);
}

// ------------------------------------------------------- squared error
__global__ void k_sqerr(const float *__restrict__ a, const float *__restrict__ b, int64_t n,
                        double *out) {
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double d = (double)a[i] - (double)b[i];
        acc += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double red[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = acc;
    __syncthreads();
    if (wid == 0) {
        acc = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) atomicAdd(out, acc);
    }
}

static int check_dims(int64_t B, int64_t H, int64_t W) {
    SCI_CHECK_ARG(B >= 1 && H >= 1 && W >= 1, "invalid sizes B=%lld H=%lld W=%lld",
                  (long long)B, (long long)H, (long long)W);
    SCI_CHECK_ARG(B <= (1 << 20) && H * W <= (int64_t(1) << 40), "sizes too large");
    return SCI_OK;
}

static bool vec_ok(int64_t hw, std::initializer_list<const void *> ptrs) {
    if (hw & 3) return false;
    for (const void *p : ptrs)
        if (p && !aligned16(p)) return false;
    return true;
}

// Projection entry points with an optional FP64 ||r||^2 accumulator `rn`
// (the C ABI's functions pass none; the native solver loops pass the
// iteration's slot).
int proj_gap_rn(const float *x, const float *phi, const uint32_t *mask_bits, const float *y,
                 float *y1, const float *phisum, float *x_out, float lambda, int accelerate,
                 int64_t B, int64_t H, int64_t W, void *stream, double *rn) {
    if (int e = check_dims(B, H, W)) return e;
    SCI_CHECK_ARG(x && y && phisum && x_out && (phi || mask_bits),
                  "sci_proj_gap: null pointer");
    SCI_CHECK_ARG(!accelerate || y1, "sci_proj_gap: accelerate needs y1");
    SCI_CHECK_ARG(!mask_bits || B <= 32, "sci_proj_gap: packed mask needs B <= 32");
    SCI_CHECK_ARG(x != x_out, "sci_proj_gap: x and x_out must not alias");
    const int64_t hw = H * W;
    cudaStream_t s = as_stream(stream);
    const bool vec = vec_ok(hw, {x, phi, mask_bits, y, y1, phisum, x_out});
    const int Bi = (int)B;
#define LAUNCH_GAP(MODE, M)                                                                 \
    do {                                                                                    \
        if (vec) {                                                                          \
            if (accelerate)                                                                 \
                k_proj_gap_vec<MODE, true><<<grid_for(hw / 4, 256), 256, 0, s>>>(           \
                    x, M, y, y1, phisum, x_out, lambda, Bi, hw, rn);                        \
            else                                                                            \
                k_proj_gap_vec<MODE, false><<<grid_for(hw / 4, 256), 256, 0, s>>>(          \
                    x, M, y, y1, phisum, x_out, lambda, Bi, hw, rn);                        \
        } else {                                                                            \
            if (accelerate)                                                                 \
                k_proj_gap_scalar<MODE, true><<<grid_for(hw, 256), 256, 0, s>>>(            \
                    x, M, y, y1, phisum, x_out, lambda, Bi, hw, rn);                        \
            else                                                                            \
                k_proj_gap_scalar<MODE, false><<<grid_for(hw, 256), 256, 0, s>>>(           \
                    x, M, y, y1, phisum, x_out, lambda, Bi, hw, rn);                        \
        }                                                                                   \
    } while (0)
    const char *tma = getenv("SCI_PROJ_TMA");
    if (mask_bits && !(tma && atoi(tma) == 0)) {
        // bulk-copy staged kernel; SCI_ERR_UNSUPPORTED: alignment or B
        const int e = launch_proj_gap_tma(x, mask_bits, y, y1, phisum, x_out, lambda,
                                          accelerate != 0, Bi, hw, s, rn);
        if (e != SCI_ERR_UNSUPPORTED) return e;
    }
    if (mask_bits) {
        Mask<1> M{mask_bits, hw};
        if (accelerate)
            launch_gap_smem<1, true>(x, M, y, y1, phisum, x_out, lambda, Bi, hw, s, rn);
        else
            launch_gap_smem<1, false>(x, M, y, y1, phisum, x_out, lambda, Bi, hw, s, rn);
    } else {
        Mask<0> M{phi, hw};
        LAUNCH_GAP(0, M);
    }
#undef LAUNCH_GAP
    SCI_LAUNCHED("k_proj_gap");
    return SCI_OK;
}

int gap_residual_rn(const float *x, const float *phi, const uint32_t *mask_bits,
                     const float *y, float *y1, const float *phisum, float *c,
                     int accelerate, int64_t B, int64_t H, int64_t W, void *stream, double *rn,
                     double *zero, int nzero) {
    if (int e = check_dims(B, H, W)) return e;
    SCI_CHECK_ARG(x && y && phisum && c && (phi || mask_bits), "sci_gap_residual: null pointer");
    SCI_CHECK_ARG(!accelerate || y1, "sci_gap_residual: accelerate needs y1");
    SCI_CHECK_ARG(!mask_bits || B <= 32, "sci_gap_residual: packed mask needs B <= 32");
    const int64_t hw = H * W;
    SCI_CHECK_ARG(vec_ok(hw, {x, phi, mask_bits, y, y1, phisum, c}),
                  "sci_gap_residual: needs H*W %% 4 == 0 and 16-byte aligned buffers");
    cudaStream_t s = as_stream(stream);
    const dim3 g = grid_for(hw / 4, 256);
    if (mask_bits) {
        Mask<1> M{mask_bits, hw};
        if (accelerate) SCI_CUDA(launch_dep(k_gap_resid_vec<1, true>, g, dim3(256), 0, s, x, M, y, y1,
                                        phisum, c, (int)B, hw, rn, zero, nzero, resid_rev()));
        else SCI_CUDA(launch_dep(k_gap_resid_vec<1, false>, g, dim3(256), 0, s, x, M, y, y1,
                                        phisum, c, (int)B, hw, rn, zero, nzero, resid_rev()));
    } else {
        Mask<0> M{phi, hw};
        if (accelerate) SCI_CUDA(launch_dep(k_gap_resid_vec<0, true>, g, dim3(256), 0, s, x, M, y, y1,
                                        phisum, c, (int)B, hw, rn, zero, nzero, resid_rev()));
        else SCI_CUDA(launch_dep(k_gap_resid_vec<0, false>, g, dim3(256), 0, s, x, M, y, y1,
                                        phisum, c, (int)B, hw, rn, zero, nzero, resid_rev()));
    }
    SCI_LAUNCHED("k_gap_resid");
    return SCI_OK;
}

// The fused ADMM iteration's residual pass (k_admm_resid_vec): packed
// mask, H*W % 4 == 0, 16-byte aligned planes.  t: theta + b of every frame
// (theta_0 at the first iteration, `first`).
int admm_residual_rn(const float *t, const uint32_t *mask_bits, const float *y,
                     const float *phisum, float *r_new, float *x_out, float lambda, float gamma,
                     int first, int64_t B, int64_t H, int64_t W, void *stream, double *rn,
                     double *zero, int nzero) {
    if (int e = check_dims(B, H, W)) return e;
    SCI_CHECK_ARG(t && y && phisum && r_new && mask_bits, "admm residual: null pointer");
    SCI_CHECK_ARG(B <= 32, "admm residual: packed mask needs B <= 32");
    const int64_t hw = H * W;
    SCI_CHECK_ARG(vec_ok(hw, {t, mask_bits, y, phisum, r_new, x_out}),
                  "admm residual: needs H*W %% 4 == 0 and 16-byte aligned buffers");
    cudaStream_t s = as_stream(stream);
    const dim3 g = grid_for(hw / 4, 256);
    Mask<1> M{mask_bits, hw};
#define SCI_ADMM_RESID(F, X)                                                                  \
    SCI_CUDA(launch_dep(k_admm_resid_vec<F, X>, g, dim3(256), 0, s, t, M, y, phisum, r_new,   \
                        x_out, lambda, gamma, (int)B, hw, rn, zero, nzero, resid_rev()))
    if (first) {
        if (x_out) SCI_ADMM_RESID(true, true);
        else SCI_ADMM_RESID(true, false);
    } else {
        if (x_out) SCI_ADMM_RESID(false, true);
        else SCI_ADMM_RESID(false, false);
    }
#undef SCI_ADMM_RESID
    SCI_LAUNCHED("k_admm_resid");
    return SCI_OK;
}

int proj_admm_rn(const float *theta, const float *b, const float *phi,
                  const uint32_t *mask_bits, const float *y, const float *phisum, float *v,
                  float *x_out, float lambda, float gamma, int64_t B, int64_t H, int64_t W,
                  void *stream, double *rn) {
    if (int e = check_dims(B, H, W)) return e;
    SCI_CHECK_ARG(theta && b && y && phisum && v && (phi || mask_bits),
                  "sci_proj_admm: null pointer");
    SCI_CHECK_ARG(!mask_bits || B <= 32, "sci_proj_admm: packed mask needs B <= 32");
    SCI_CHECK_ARG(v != theta && v != b && x_out != theta && x_out != b,
                  "sci_proj_admm: outputs must not alias inputs");
    const int64_t hw = H * W;
    cudaStream_t s = as_stream(stream);
    const bool vec = vec_ok(hw, {theta, b, phi, mask_bits, y, phisum, v, x_out});
    const int Bi = (int)B;
    const char *tma = getenv("SCI_PROJ_TMA");
    if (mask_bits && !(tma && atoi(tma) == 0)) {
        // bulk-copy staged kernel; SCI_ERR_UNSUPPORTED: alignment or B
        const int e = launch_proj_admm_tma(theta, b, mask_bits, y, phisum, v, x_out, lambda,
                                           gamma, Bi, hw, s, false, rn);
        if (e != SCI_ERR_UNSUPPORTED) return e;
    }
    if (mask_bits) {
        Mask<1> M{mask_bits, hw};
        launch_admm_smem<1>(theta, b, M, y, phisum, v, x_out, lambda, gamma, Bi, hw, s, rn);
    } else {
        Mask<0> M{phi, hw};
        if (vec)
            k_proj_admm_vec<0><<<grid_for(hw / 4, 256), 256, 0, s>>>(theta, b, M, y, phisum, v,
                                                                     x_out, lambda, gamma, Bi, hw,
                                                                     rn);
        else
            k_proj_admm_scalar<0><<<grid_for(hw, 256), 256, 0, s>>>(theta, b, M, y, phisum, v,
                                                                    x_out, lambda, gamma, Bi, hw,
                                                                    rn);
    }
    SCI_LAUNCHED("k_proj_admm");
    return SCI_OK;
}

}  // namespace sci

using namespace sci;

extern "C" {

int sci_version(void) { return 100; }

int sci_last_error(char *buf, size_t n) {
    const std::string &s = g_last_error;
    if (buf && n) {
        size_t k = s.size() < n - 1 ? s.size() : n - 1;
        memcpy(buf, s.data(), k);
        buf[k] = 0;
    }
    return (int)s.size();
}

int sci_A(const float *x, const float *phi, float *y, int64_t B, int64_t H, int64_t W,
          void *stream) {
    if (int e = check_dims(B, H, W)) return e;
    SCI_CHECK_ARG(x && phi && y, "sci_A: null pointer");
    const int64_t hw = H * W;
    cudaStream_t s = as_stream(stream);
    if (vec_ok(hw, {x, phi, y}))
        k_A_vec<<<grid_for(hw / 4, 256), 256, 0, s>>>(x, phi, y, (int)B, hw);
    else
        k_A_scalar<<<grid_for(hw, 256), 256, 0, s>>>(x, phi, y, (int)B, hw);
    SCI_LAUNCHED("k_A");
    return SCI_OK;
}

int sci_At(const float *y, const float *phi, float *x, int64_t B, int64_t H, int64_t W,
           void *stream) {
    if (int e = check_dims(B, H, W)) return e;
    SCI_CHECK_ARG(x && phi && y, "sci_At: null pointer");
    const int64_t hw = H * W;
    cudaStream_t s = as_stream(stream);
    if (vec_ok(hw, {x, phi, y}))
        k_At_vec<<<grid_for(hw / 4, 256), 256, 0, s>>>(y, phi, x, (int)B, hw);
    else
        k_At_scalar<<<grid_for(hw, 256), 256, 0, s>>>(y, phi, x, (int)B, hw);
    SCI_LAUNCHED("k_At");
    return SCI_OK;
}

int sci_phisum(const float *phi, float *phisum, int64_t B, int64_t H, int64_t W,
               int guard_zero, void *stream) {
    if (int e = check_dims(B, H, W)) return e;
    SCI_CHECK_ARG(phi && phisum, "sci_phisum: null pointer");
    const int64_t hw = H * W;
    k_phisum<<<grid_for(hw, 256), 256, 0, as_stream(stream)>>>(phi, phisum, (int)B, hw,
                                                                guard_zero);
    SCI_LAUNCHED("k_phisum");
    return SCI_OK;
}

int sci_pack_mask(const float *phi, uint32_t *bits, int *flag, int64_t B, int64_t H,
                  int64_t W, void *stream) {
    if (int e = check_dims(B, H, W)) return e;
    SCI_CHECK_ARG(B <= 32, "sci_pack_mask: B=%lld > 32 frames", (long long)B);
    SCI_CHECK_ARG(phi && bits && flag, "sci_pack_mask: null pointer");
    const int64_t hw = H * W;
    k_pack<<<grid_for(hw, 256), 256, 0, as_stream(stream)>>>(phi, bits, flag, (int)B, hw);
    SCI_LAUNCHED("k_pack");
    return SCI_OK;
}

int sci_proj_gap(const float *x, const float *phi, const uint32_t *mask_bits, const float *y,
                 float *y1, const float *phisum, float *x_out, float lambda, int accelerate,
                 int64_t B, int64_t H, int64_t W, void *stream) {
    return sci::proj_gap_rn(x, phi, mask_bits, y, y1, phisum, x_out, lambda, accelerate, B, H,
                            W, stream, nullptr);
}

int sci_gap_residual(const float *x, const float *phi, const uint32_t *mask_bits,
                     const float *y, float *y1, const float *phisum, float *c,
                     int accelerate, int64_t B, int64_t H, int64_t W, void *stream) {
    return sci::gap_residual_rn(x, phi, mask_bits, y, y1, phisum, c, accelerate, B, H, W,
                                stream, nullptr, nullptr, 0);
}

int sci_proj_admm(const float *theta, const float *b, const float *phi,
                  const uint32_t *mask_bits, const float *y, const float *phisum, float *v,
                  float *x_out, float lambda, float gamma, int64_t B, int64_t H, int64_t W,
                  void *stream) {
    return sci::proj_admm_rn(theta, b, phi, mask_bits, y, phisum, v, x_out, lambda, gamma, B, H,
                             W, stream, nullptr);
}

int sci_sqerr_accum(const float *a, const float *b, int64_t n, double *out, void *stream) {
    SCI_CHECK_ARG(a && b && out && n >= 0, "sci_sqerr_accum: bad argument");
    if (n == 0) return SCI_OK;
    k_sqerr<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(a, b, n, out);
    SCI_LAUNCHED("k_sqerr");
    return SCI_OK;
}

}  // extern "C"
