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
// updates.  ITV3D_cham (a norm summed over all frames of a pixel) runs its
// own row pipeline with the frames of a pixel spread over the warps of a
// block: up to 5 updates and the output per pass, so the stack crosses HBM
// once per call.  The FGP files (two dual fields and a momentum) run one
// kernel per iteration over the stack, one thread per pixel (kind 8: per
// pixel position, looping over the frames); a thread recomputes the few
// primal values its dual update needs from the neighbouring duals (served
// by L1).  The last dual update of the FGP loop does not reach the
// returned value and is not computed.
#include <cmath>
#include <type_traits>
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

// ITV3D Chambolle (tvdenoise_cham_ITV3D.m:74-91), up to 5 updates and the
// output u = f - div p / lambda in one pass over the stack.  Per update,
//   z  = div p - lambda f          (div p = p1 - p1(:,il) + p2 - p2(iu,:))
//   z1 = z(:, ir) - z, z2 = z(ir, :) - z   (zero at the last column / row)
//   q  = (p + dt z) / (1 + dt sqrt(sum over frames of z1^2 + z2^2)).
// q at (i, j) reads p at (i, j-1 .. j+1) and (i-1 .. i+1, j): radius one,
// so S updates chain as a row pipeline (the lean scikit-image TV pass's
// scheme): when input row r arrives, update k produces row r - k from the
// rows of update k - 1 it keeps in registers, and the output stage forms
// u at row r - S.  A block is 32 columns (lanes) x FL frame lanes (warps);
// warp w holds frames w, w + FL, ... (NT slots); the norm over the frames
// of a pixel is reduced in shared memory, one barrier per update and row
// (the sums of consecutive rows in alternate buffers, so a warp that runs
// ahead never overwrites sums another warp still reads).
// Each update narrows the valid columns by one on either side, so a strip
// owns 32 - 2S - 1 columns; a chunk of rows starts S + 1 rows early.  f
// rows come through a per-thread cp.async ring (each lane reads back only
// the values it copied).  The first pass starts from p = 0; a run of more
// than 5 updates carries p through the workspace between passes (pin: load
// p of the input rows, out == 0: store p^S instead of u).
constexpr int IT3_RING = 8;  // f rows in the ring (>= S + 1 + prefetch distance 2)

__device__ __forceinline__ void cp4(uint32_t dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp4_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp4_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// EDGE: the strip holds column 0 or W - 1 (or columns outside the frame);
// interior strips compile without the edge selects.  The square root and
// reciprocal of the dual update are the approximate MUFU forms, and the
// output divides by lambda as a product with its reciprocal.
template <int S, int NT, bool EDGE>
__device__ __forceinline__ void itv3d_body(
    const float *__restrict__ f, const float *__restrict__ pin1, const float *__restrict__ pin2,
    float *__restrict__ u, float *__restrict__ resid, float *__restrict__ pout1,
    float *__restrict__ pout2, const Geo &g, int nf, float lam, float dt, int R, int own, int pin,
    int out, float (&ring)[IT3_RING][NT * FL][32], float (&red)[2][S][32][FL]) {
    constexpr int PF = IT3_RING - S - 1;  // rows prefetched ahead
    static_assert(S >= 1 && S <= 5 && PF >= 2, "ITV3D pass: 1..5 updates");
    static_assert((IT3_RING & (IT3_RING - 1)) == 0 && FL == 8, "ring slots by mask");
    const int lane = threadIdx.x, w = threadIdx.y;
    const int H = g.H, W = g.W;
    const int col = blockIdx.x * own - (S + 1) + lane;
    const int colc = EDGE ? min(max(col, 0), W - 1) : col;
    const bool owned = lane >= S + 1 && lane < S + 1 + own && col < W;
    const bool first_col = EDGE && col <= 0, last_col = EDGE && col >= W - 1;
    const float ilam = 1.f / lam;
    const int slot = w ^ ((lane >> 2) & (FL - 1));
    const int r0 = blockIdx.y * R, r1 = min(r0 + R, H);
    const int rs = max(0, r0 - S - 1), re = r1 - 1 + S;  // input rows rs.., last step re
    bool fv[NT];
    int64_t fo[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const int b = w + t * FL;
        fv[t] = b < nf;
        fo[t] = (int64_t)min(b, nf - 1) * g.hw + colc;
    }
    auto fetch = [&](int r) {  // f row r into its ring slot
        if (r < H && r <= re) {
#pragma unroll
            for (int t = 0; t < NT; ++t)
                cp4((uint32_t)__cvta_generic_to_shared(
                        &ring[r & (IT3_RING - 1)][w + t * FL][lane]),
                    f + fo[t] + (int64_t)r * W);
        }
        cp4_commit();
    };
    // kept per update k: p^{k-1} and z^{k-1} of the row before its input row
    float zc[S][NT], p1c[S][NT], p2c[S][NT], p2o[NT];
#pragma unroll
    for (int k = 0; k < S; ++k)
#pragma unroll
        for (int t = 0; t < NT; ++t) zc[k][t] = p1c[k][t] = p2c[k][t] = 0.f;
#pragma unroll
    for (int t = 0; t < NT; ++t) p2o[t] = 0.f;

    // One step: input row r enters, update k + 1 produces row r - k - 1,
    // the output stage row r - S.  FAST: every stage has its input and
    // output rows inside [rs, H - 1) and none is row 0 (no tests needed).
    auto step = [&](int r, auto fast) {
        constexpr bool FAST = decltype(fast)::value;
        fetch(r + PF);
        cp4_wait<PF>();
        float in1[NT], in2[NT];  // p^0 of input row r
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            in1[t] = in2[t] = 0.f;
            if (pin && (FAST || r < H)) {
                in1[t] = __ldg(pin1 + fo[t] + (int64_t)r * W);
                in2[t] = __ldg(pin2 + fo[t] + (int64_t)r * W);
            }
        }
#pragma unroll
        for (int k = 0; k < S; ++k) {  // update k + 1: input row a, output row a - 1
            const int a = r - k, b = a - 1;
            const bool vin = FAST || (a < H && a >= rs), vout = FAST || (b >= rs && b < H);
            float zin[NT];
#pragma unroll
            for (int t = 0; t < NT; ++t) zin[t] = 0.f;
            if (vin) {
#pragma unroll
                for (int t = 0; t < NT; ++t) {
                    float l = __shfl_up_sync(0xffffffffu, in1[t], 1);
                    if (first_col) l = in1[t];
                    const float up = (!FAST && a == 0) ? in2[t] : p2c[k][t];
                    const float fa = ring[a & (IT3_RING - 1)][w + t * FL][lane];
                    zin[t] = (((in1[t] - l) + in2[t]) - up) - fa * lam;
                }
            }
            if (vout) {
                float z1[NT], z2[NT], s = 0.f;
#pragma unroll
                for (int t = 0; t < NT; ++t) {
                    const float zr = __shfl_down_sync(0xffffffffu, zc[k][t], 1);
                    z1[t] = last_col ? 0.f : zr - zc[k][t];
                    z2[t] = (FAST || b < H - 1) ? zin[t] - zc[k][t] : 0.f;
                    if (fv[t]) s += z1[t] * z1[t] + z2[t] * z2[t];
                }
                float(&rs_)[FL] = red[r & 1][k][lane];
                rs_[slot] = s;
                __syncthreads();
                const float4 v0 = *reinterpret_cast<const float4 *>(&rs_[0]);
                const float4 v1 = *reinterpret_cast<const float4 *>(&rs_[4]);
                const float tot = ((((((v0.x + v0.y) + v0.z) + v0.w) + v1.x) + v1.y) + v1.z) + v1.w;
                const float rd = rcp_approx(fmaf(dt, sqrt_approx(tot), 1.f));
                // p^{k+1} of row b becomes the next update's input row
#pragma unroll
                for (int t = 0; t < NT; ++t) {
                    const float q1 = (p1c[k][t] + dt * z1[t]) * rd;
                    const float q2 = (p2c[k][t] + dt * z2[t]) * rd;
                    if (vin) {
                        zc[k][t] = zin[t];
                        p1c[k][t] = in1[t];
                        p2c[k][t] = in2[t];
                    }
                    in1[t] = q1;
                    in2[t] = q2;
                }
            } else {
#pragma unroll
                for (int t = 0; t < NT; ++t) {
                    if (vin) {
                        zc[k][t] = zin[t];
                        p1c[k][t] = in1[t];
                        p2c[k][t] = in2[t];
                    }
                    in1[t] = in2[t] = 0.f;
                }
            }
        }
        // p^S of row a = r - S
        const int a = r - S;
        if (!FAST && (a < rs || a >= H)) return;
        const bool keep = owned && a >= r0 && a < r1;
        if (!out) {
#pragma unroll
            for (int t = 0; t < NT; ++t)
                if (keep && fv[t]) {
                    pout1[fo[t] + (int64_t)a * W] = in1[t];
                    pout2[fo[t] + (int64_t)a * W] = in2[t];
                }
            return;
        }
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            float l = __shfl_up_sync(0xffffffffu, in1[t], 1);
            if (first_col) l = in1[t];
            const float up = (!FAST && a == 0) ? in2[t] : p2o[t];
            p2o[t] = in2[t];
            const float fa = ring[a & (IT3_RING - 1)][w + t * FL][lane];
            const float x = fa - (((in1[t] - l) + in2[t]) - up) * ilam;
            if (keep && fv[t]) {
                u[fo[t] + (int64_t)a * W] = x;
                if (resid) resid[fo[t] + (int64_t)a * W] = x - fa;
            }
        }
    };

#pragma unroll
    for (int q = 0; q < PF; ++q) fetch(rs + q);
    // steady rows: r in [rs + S + 1, min(H - 1, re)]
    const int fb = rs + S + 1, fe = min(H - 1, re);
    int r = rs;
    for (; r <= re && r < fb; ++r) step(r, std::false_type{});
    for (; r <= fe; ++r) step(r, std::true_type{});
    for (; r <= re; ++r) step(r, std::false_type{});
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

template <int S, int NT>
__global__ void __launch_bounds__(32 * FL, 2) k_itv3d_cham(
    const float *__restrict__ f, const float *__restrict__ pin1, const float *__restrict__ pin2,
    float *__restrict__ u, float *__restrict__ resid, float *__restrict__ pout1,
    float *__restrict__ pout2, Geo g, int nf, float lam, float dt, int R, int own, int pin,
    int out) {
    __shared__ float ring[IT3_RING][NT * FL][32];
    // per-pixel sums of the frame lanes, [row parity][update][column][lane
    // slot]: a column's FL sums are one 32-byte row, read with two vector
    // loads; the slot is the frame lane XOR (column / 4) % FL, so the FL
    // lanes' stores of one warp hit distinct banks.  Every warp adds a
    // column's slots in the same (slot) order, so all frames of a pixel see
    // the same total.
    __shared__ __align__(16) float red[2][S][32][FL];
    const int c0 = blockIdx.x * own - (S + 1);  // the strip's first column
    if (c0 >= 1 && c0 + 31 <= g.W - 2)
        itv3d_body<S, NT, false>(f, pin1, pin2, u, resid, pout1, pout2, g, nf, lam, dt, R, own,
                                 pin, out, ring, red);
    else
        itv3d_body<S, NT, true>(f, pin1, pin2, u, resid, pout1, pout2, g, nf, lam, dt, R, own,
                                pin, out, ring, red);
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

// One pass of S ITV3D updates (p_in null: p = 0; p_out null: store u).
// Row chunks are sized so the blocks fill whole waves of the resident
// blocks, counting the 2S + 1 rows every chunk recomputes.
int itv3d_pass(int S, const float *f, const float *p_in1, const float *p_in2, float *u,
               float *resid, float *p_out1, float *p_out2, const Geo &g, int nf, float lam,
               float dt, cudaStream_t s) {
    const int nt = (nf + FL - 1) / FL;
    const int own = 32 - 2 * S - 1;
    const int strips = (g.W + own - 1) / own;
    static int resident[6][5] = {};
    const void *kp = nullptr;
#define SCI_IT3_PTR(SV, NV) if (S == SV && nt == NV) kp = reinterpret_cast<const void *>(&k_itv3d_cham<SV, NV>);
#define SCI_IT3_ROW(SV) SCI_IT3_PTR(SV, 1) SCI_IT3_PTR(SV, 2) SCI_IT3_PTR(SV, 3) SCI_IT3_PTR(SV, 4)
    SCI_IT3_ROW(1) SCI_IT3_ROW(2) SCI_IT3_ROW(3) SCI_IT3_ROW(4) SCI_IT3_ROW(5)
#undef SCI_IT3_ROW
#undef SCI_IT3_PTR
    SCI_CHECK_ARG(kp != nullptr, "tv_matlab: ITV3D pass of %d updates, %d frames", S, nf);
    if (resident[S][nt - 1] == 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kp, 32 * FL, 0) !=
                cudaSuccess || per_sm <= 0) {
            cudaGetLastError();
            per_sm = 1;
        }
        resident[S][nt - 1] = per_sm * kSMs;
    }
    const int64_t slots = resident[S][nt - 1];
    int best_n = 1;
    double best = 1e300;
    for (int n = 1; n <= std::min(g.H, 256); ++n) {
        const int R = (g.H + n - 1) / n;
        const int64_t blocks = (int64_t)strips * ((g.H + R - 1) / R);
        const double t = (double)((blocks + slots - 1) / slots) * (R + 2 * S + 1);
        if (t < best - 1e-9) {
            best = t;
            best_n = n;
        }
    }
    const int R = (g.H + best_n - 1) / best_n;
    const dim3 grd((unsigned)strips, (unsigned)((g.H + R - 1) / R)), blk(32, FL);
    const int pin = p_in1 != nullptr, out = p_out1 == nullptr;
#define SCI_IT3_CASE(SV, NV)                                                                  \
    if (S == SV && nt == NV)                                                                  \
        k_itv3d_cham<SV, NV><<<grd, blk, 0, s>>>(f, p_in1, p_in2, u, resid, p_out1, p_out2, g, \
                                                 nf, lam, dt, R, own, pin, out);
#define SCI_IT3_ROW(SV) SCI_IT3_CASE(SV, 1) SCI_IT3_CASE(SV, 2) SCI_IT3_CASE(SV, 3) SCI_IT3_CASE(SV, 4)
    SCI_IT3_ROW(1) SCI_IT3_ROW(2) SCI_IT3_ROW(3) SCI_IT3_ROW(4) SCI_IT3_ROW(5)
#undef SCI_IT3_ROW
#undef SCI_IT3_CASE
    SCI_LAUNCHED("k_itv3d_cham");
    return SCI_OK;
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
    // frame-coupled FGP: 32 pixels x FL frame lanes per block, one row
    const dim3 blkc(32, FL);
    const dim3 grdc((unsigned)((W + 31) / 32), (unsigned)H, 1);
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
            // tvdenoise_cham_ITV3D.m:74-91: passes of up to 5 updates, the
            // last one forming u
            const float dt = 0.25f;
            const int npass = (iters + 4) / 5;
            const float *p_in1 = nullptr, *p_in2 = nullptr;
            float *q1 = a1, *q2 = a2;
            for (int ps = 0; ps < npass; ++ps) {
                const bool last = ps + 1 == npass;
                const int S = last ? iters - 5 * (npass - 1) : 5;
                const int e = itv3d_pass(S, f, p_in1, p_in2, u, resid, last ? nullptr : q1,
                                         last ? nullptr : q2, g, (int)nf, lam, dt, s);
                if (e) return e;
                p_in1 = q1;
                p_in2 = q2;
                std::swap(q1, b1);
                std::swap(q2, b2);
            }
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
