// Chambolle TV denoiser on sm_103a: a row-streaming, temporally blocked
// stencil pipeline.
//
// Semantics: scikit-image 0.16 denoise_tv_chambolle(f, weight, eps,
// n_iter_max) applied to each H x W frame independently (the reference calls
// it with multichannel=True on the H x W x B stack,
// PnP_SCI/python/pnp_sci_algo.py:650 and :812-813).  With tau = 1/4, p_0 = 0:
//   u_k = f - div p_k,   n_k = |grad u_k|   (forward differences, 0 at the
//   last row/column; div = backward differences with p_{-1} = 0),
//   E_k = (sum (div p_k)^2 + weight sum n_k) / (H W),
//   p_{k+1} = (p_k - tau grad u_k) / (1 + tau/weight n_k),
//   stop after step k >= 1 when |E_{k-1} - E_k| < eps E_0; the result is
//   u_k of the last executed step (u_{K-1} without an early stop).
//
// Mapping.  One warp owns a band of 128 columns (4 per lane, float4 loads
// along W) of one frame and marches down a chunk of rows.  The K-1 dual
// updates form a register pipeline: stage k (k = 1..S) handles row r-k when
// input row r arrives, computing p_k and u_k of that row from stage k-1's
// rows r-k and r-k+1.  p and div p never leave registers; horizontal
// neighbours come from warp shuffles; the band overlaps its neighbours by
// S (+1) halo columns and the chunk by S (+1) halo rows, and a stage reads
// the input row it needs back from L1.  Per pass the frame is read once and
// written once: 8 bytes per pixel of HBM traffic.
//
// Stop test.  The per-frame energies E_k need whole-frame sums, which a
// tiled pipeline sees only after every tile has finished.  The pass
// therefore runs all of its steps speculatively, accumulating per-frame
// float64 sums of (div p_k)^2 and n_k; a second launch of the same kernel
// ("fixup") evaluates the stop rule per frame in float64 and re-runs only
// the frames that would have stopped inside the pass, with the shorter step
// count.  Frames that do not stop (nearly all, for n_iter_max = 5) cost the
// fixup one read of a few doubles.
//
// More than 4 dual updates are split into passes of at most 4 that carry p
// through a workspace (p_in / p_out), with the same speculative scheme per
// pass window.
#pragma once
#include <algorithm>

#include "sci_common.cuh"

namespace sci {
namespace tv {

constexpr int CPL = 4;             // columns per lane
constexpr int BANDW = 32 * CPL;    // columns per warp band
constexpr int WPB = 4;             // warps per block
constexpr int SMAX = 4;            // dual updates per pass
constexpr unsigned FULL = 0xffffffffu;

enum { INTERIOR = 0, EDGE = 1 };  // EDGE: band touches a frame edge, or W % 4 != 0

struct Pass {
    const float *f;       // input stack  [nf][H][W] (frame stride fs)
    float *u;             // output stack (same strides)
    float *resid;         // nullable: u - f
    const float *p_in;    // nullable: [nf][2][H][W]  (pr plane, pc plane)
    float *p_out;         // nullable
    double *energy;       // [nf][K][2]: sum (div p_k)^2, sum |grad u_k|
    int *done;            // [nf]: stop index j >= 1, or -1
    int *steps;           // nullable [nf]: executed Chambolle steps
    int64_t fs;           // frame stride of f/u/resid (elements)
    int nf, H, W, K;      // frames, rows, cols, n_iter_max
    int a;                // this pass starts from p_a (p_in) and computes p_{a+1..a+S}
    float tau, tw;        // tau, tau / weight
    float weight, eps;
    int nbands, nchunks, R, own, hl, ht;
    int S;                // dual updates of this pass (geometry of the window)
    int vec;              // 1: rows are 16-byte aligned (float4 path)
};

struct V4 {
    float x, y, z, w;
};
__device__ __forceinline__ V4 v4(float4 a) { return {a.x, a.y, a.z, a.w}; }
__device__ __forceinline__ float4 f4(V4 a) { return make_float4(a.x, a.y, a.z, a.w); }
__device__ __forceinline__ V4 zero4() { return {0.f, 0.f, 0.f, 0.f}; }

template <int S>
struct St {
    V4 up[S > 0 ? S : 1];  // up[k]: u_k at stage (k+1)'s current row (k = 0..S-1)
    V4 pr[S + 1];          // pr[k]: p_k (row component) at the row of stage k+1
    V4 pc[S > 0 ? S : 1];  // pc[k]: p_k (column component) at the row of stage k+1
};

template <int MODE>
__device__ __forceinline__ V4 load_row(const float *rowp, int col, int W, bool vec) {
    if (MODE == INTERIOR) return v4(ldg4(rowp + col));
    if (vec) return (col >= 0 && col < W) ? v4(ldg4(rowp + col)) : zero4();
    V4 v;
    v.x = (col + 0 >= 0 && col + 0 < W) ? __ldg(rowp + col + 0) : 0.f;
    v.y = (col + 1 >= 0 && col + 1 < W) ? __ldg(rowp + col + 1) : 0.f;
    v.z = (col + 2 >= 0 && col + 2 < W) ? __ldg(rowp + col + 2) : 0.f;
    v.w = (col + 3 >= 0 && col + 3 < W) ? __ldg(rowp + col + 3) : 0.f;
    return v;
}

// Store the columns of this lane that the band owns.
template <int MODE>
__device__ __forceinline__ void store_row(float *rowp, int col, V4 v, bool lane_own,
                                          const V4 &mk, bool vec) {
    if (MODE == INTERIOR || vec) {
        if (lane_own) st4(rowp + col, f4(v));
    } else {
        if (mk.x != 0.f) rowp[col + 0] = v.x;
        if (mk.y != 0.f) rowp[col + 1] = v.y;
        if (mk.z != 0.f) rowp[col + 2] = v.z;
        if (mk.w != 0.f) rowp[col + 3] = v.w;
    }
}

// One pipeline step: input row r enters, stage k handles row r-k.
// GEN: rows may be outside [r0, r1) or touch the frame's first/last row.
template <int S, bool PIN, bool OUT_U, bool ENERGY, int MODE, bool GEN>
__device__ __forceinline__ void step(const Pass &P, const St<S> &in, St<S> &out, int r, int rs,
                                     int r0, int r1, int col, const float *fb, const float *pinb,
                                     float *ob, float *rb, bool lane_own, const V4 &mk,
                                     float (&en)[S > 0 ? S : 1], float (&ed)[S > 0 ? S : 1]) {
    const int H = P.H, W = P.W;
    const bool vec = P.vec != 0;
    const int64_t hw = (int64_t)H * W;
    const bool cedge = (MODE != INTERIOR);
    // per-column frame-boundary flags (edge bands only)
    const bool first_col = cedge && (col == 0);
    const bool lastx = cedge && (col + 0 == W - 1), lasty = cedge && (col + 1 == W - 1),
               lastz = cedge && (col + 2 == W - 1), lastw = cedge && (col + 3 == W - 1);

    // ---------------- stage 0: u_0 at row r
    const bool act0 = !GEN || (r < H);
    V4 ucur = act0 ? load_row<MODE>(fb + (int64_t)r * W, col, W, vec) : zero4();
    if (PIN) {
        V4 qr = act0 ? load_row<MODE>(pinb + (int64_t)r * W, col, W, vec) : zero4();
        V4 qc = act0 ? load_row<MODE>(pinb + hw + (int64_t)r * W, col, W, vec) : zero4();
        float pcl = __shfl_up_sync(FULL, qc.w, 1);
        if (first_col) pcl = 0.f;
        const V4 pu = in.pr[0];
        V4 d;
        d.x = (qr.x + qc.x) - pu.x - pcl;
        d.y = (qr.y + qc.y) - pu.y - qc.x;
        d.z = (qr.z + qc.z) - pu.z - qc.y;
        d.w = (qr.w + qc.w) - pu.w - qc.z;
        ucur.x -= d.x;
        ucur.y -= d.y;
        ucur.z -= d.z;
        ucur.w -= d.w;
        if (ENERGY && act0 && (!GEN || (r >= r0 && r < r1))) {
            if (MODE == INTERIOR)
                ed[0] += d.x * d.x + d.y * d.y + d.z * d.z + d.w * d.w;
            else
                ed[0] += mk.x * d.x * d.x + mk.y * d.y * d.y + mk.z * d.z * d.z + mk.w * d.w * d.w;
        }
        out.pr[0] = qr;
        if (S > 0) out.pc[0] = qc;
        if (S == 0 && OUT_U && act0 && (!GEN || (r >= r0 && r < r1))) {
            const int64_t ro = (int64_t)r * W;
            store_row<MODE>(ob + ro, col, ucur, lane_own, mk, vec);
            if (rb) {
                const V4 fr = load_row<MODE>(fb + ro, col, W, vec);
                store_row<MODE>(rb + ro, col, {ucur.x - fr.x, ucur.y - fr.y, ucur.z - fr.z, ucur.w - fr.w},
                                lane_own, mk, vec);
            }
        }
    }

    // ---------------- stages 1..S
#pragma unroll
    for (int k = 1; k <= S; ++k) {
        const int i = r - k;
        out.up[k - 1] = ucur;  // u_{k-1}(i+1): stage k's "current" row next step
        const bool act = !GEN || (i >= rs && i < H);
        if (!act) {
            out.pr[k] = zero4();
            if (k < S) out.pc[k] = zero4();
            ucur = zero4();
            // keep the warp converged: shuffles below are skipped uniformly
            continue;
        }
        const V4 up = in.up[k - 1];  // u_{k-1}(i)
        float uR = __shfl_down_sync(FULL, up.x, 1);
        V4 gc;
        gc.x = lastx ? 0.f : up.y - up.x;
        gc.y = lasty ? 0.f : up.z - up.y;
        gc.z = lastz ? 0.f : up.w - up.z;
        gc.w = lastw ? 0.f : uR - up.w;
        V4 gr;
        if (GEN && i == H - 1) {
            gr = zero4();
        } else {
            gr.x = ucur.x - up.x;
            gr.y = ucur.y - up.y;
            gr.z = ucur.z - up.z;
            gr.w = ucur.w - up.w;
        }
        V4 n;
        n.x = sqrt_approx(fmaf(gr.x, gr.x, gc.x * gc.x));
        n.y = sqrt_approx(fmaf(gr.y, gr.y, gc.y * gc.y));
        n.z = sqrt_approx(fmaf(gr.z, gr.z, gc.z * gc.z));
        n.w = sqrt_approx(fmaf(gr.w, gr.w, gc.w * gc.w));
        V4 ri;
        ri.x = rcp_approx(fmaf(P.tw, n.x, 1.f));
        ri.y = rcp_approx(fmaf(P.tw, n.y, 1.f));
        ri.z = rcp_approx(fmaf(P.tw, n.z, 1.f));
        ri.w = rcp_approx(fmaf(P.tw, n.w, 1.f));
        const bool p0zero = (k == 1 && !PIN);
        const V4 qr = p0zero ? zero4() : in.pr[k - 1];
        const V4 qc = p0zero ? zero4() : in.pc[k - 1];
        const float nt = -P.tau;
        V4 prn, pcn;
        prn.x = fmaf(nt, gr.x, qr.x) * ri.x;
        prn.y = fmaf(nt, gr.y, qr.y) * ri.y;
        prn.z = fmaf(nt, gr.z, qr.z) * ri.z;
        prn.w = fmaf(nt, gr.w, qr.w) * ri.w;
        pcn.x = fmaf(nt, gc.x, qc.x) * ri.x;
        pcn.y = fmaf(nt, gc.y, qc.y) * ri.y;
        pcn.z = fmaf(nt, gc.z, qc.z) * ri.z;
        pcn.w = fmaf(nt, gc.w, qc.w) * ri.w;
        out.pr[k] = prn;
        if (k < S) out.pc[k] = pcn;
        // div p_k at row i
        float pcl = __shfl_up_sync(FULL, pcn.w, 1);
        if (first_col) pcl = 0.f;
        const V4 pu = in.pr[k];  // pr_k(i-1)
        V4 d;
        d.x = (prn.x + pcn.x) - pu.x - pcl;
        d.y = (prn.y + pcn.y) - pu.y - pcn.x;
        d.z = (prn.z + pcn.z) - pu.z - pcn.y;
        d.w = (prn.w + pcn.w) - pu.w - pcn.z;
        const int64_t ro = (int64_t)i * W;
        const V4 fi = load_row<MODE>(fb + ro, col, W, vec);
        V4 uk;
        uk.x = fi.x - d.x;
        uk.y = fi.y - d.y;
        uk.z = fi.z - d.z;
        uk.w = fi.w - d.w;
        if (ENERGY && (!GEN || (i >= r0 && i < r1))) {
            if (MODE == INTERIOR) {
                en[k - 1] += (n.x + n.y) + (n.z + n.w);
                if (k < S) ed[k] += d.x * d.x + d.y * d.y + d.z * d.z + d.w * d.w;
            } else {
                en[k - 1] += mk.x * n.x + mk.y * n.y + mk.z * n.z + mk.w * n.w;
                if (k < S)
                    ed[k] += mk.x * d.x * d.x + mk.y * d.y * d.y + mk.z * d.z * d.z +
                             mk.w * d.w * d.w;
            }
        }
        if (k == S && (!GEN || (i >= r0 && i < r1))) {
            if (OUT_U) {
                store_row<MODE>(ob + ro, col, uk, lane_own, mk, vec);
                if (rb)
                    store_row<MODE>(rb + ro, col, {uk.x - fi.x, uk.y - fi.y, uk.z - fi.z, uk.w - fi.w},
                                    lane_own, mk, vec);
            } else {
                store_row<MODE>(ob + ro, col, prn, lane_own, mk, vec);
                store_row<MODE>(ob + hw + ro, col, pcn, lane_own, mk, vec);
            }
        }
        ucur = uk;
    }
}

template <int S, bool PIN, bool OUT_U, bool ENERGY, int MODE>
__device__ __forceinline__ void run(const Pass &P, int frame, int chunk, int band, int lane) {
    const int H = P.H, W = P.W;
    const int col = band * P.own - P.hl + lane * CPL;
    const int r0 = chunk * P.R, r1 = min(r0 + P.R, H);
    const int rs = max(0, r0 - P.ht);
    const int own_lo = band * P.own, own_hi = min(own_lo + P.own, W);
    const bool lane_own = (col >= own_lo) && (col + CPL <= own_hi);
    V4 mk;
    mk.x = (col + 0 >= own_lo && col + 0 < own_hi) ? 1.f : 0.f;
    mk.y = (col + 1 >= own_lo && col + 1 < own_hi) ? 1.f : 0.f;
    mk.z = (col + 2 >= own_lo && col + 2 < own_hi) ? 1.f : 0.f;
    mk.w = (col + 3 >= own_lo && col + 3 < own_hi) ? 1.f : 0.f;

    const int64_t hw = (int64_t)H * W;
    const float *fb = P.f + (int64_t)frame * P.fs;
    const float *pinb = PIN ? P.p_in + (int64_t)frame * 2 * hw : nullptr;
    float *ob = OUT_U ? P.u + (int64_t)frame * P.fs : P.p_out + (int64_t)frame * 2 * hw;
    float *rb = (OUT_U && P.resid) ? P.resid + (int64_t)frame * P.fs : nullptr;

    St<S> A, B;
#pragma unroll
    for (int k = 0; k < (S > 0 ? S : 1); ++k) {
        A.up[k] = zero4();
        A.pc[k] = zero4();
    }
#pragma unroll
    for (int k = 0; k <= S; ++k) A.pr[k] = zero4();
    float en[S > 0 ? S : 1], ed[S > 0 ? S : 1];
#pragma unroll
    for (int k = 0; k < (S > 0 ? S : 1); ++k) en[k] = ed[k] = 0.f;

    const int rlast = min(r1 - 1 + S, H - 1 + S);
    // Fast steps: every stage inside [r0, r1), away from the frame's last row.
    const int rfb = r0 + S;
    const int rfe = min((PIN || S == 0) ? r1 - 1 : r1, H - 1);
    int r = rs;
    while (r <= rlast) {
        if (r == rfb && r + 1 <= rfe) {
            for (; r + 1 <= rfe; r += 2) {
                step<S, PIN, OUT_U, ENERGY, MODE, false>(P, A, B, r, rs, r0, r1, col, fb, pinb,
                                                          ob, rb, lane_own, mk, en, ed);
                step<S, PIN, OUT_U, ENERGY, MODE, false>(P, B, A, r + 1, rs, r0, r1, col, fb,
                                                          pinb, ob, rb, lane_own, mk, en, ed);
            }
            continue;
        }
        // prologue (halo rows, first S steps) and epilogue (chunk tail, last row)
        step<S, PIN, OUT_U, ENERGY, MODE, true>(P, A, B, r, rs, r0, r1, col, fb, pinb, ob, rb,
                                                 lane_own, mk, en, ed);
        A = B;
        ++r;
    }

    if (ENERGY) {
        const float lm = (MODE == INTERIOR) ? (lane_own ? 1.f : 0.f) : 1.f;
        double *eb = P.energy + (int64_t)frame * P.K * 2;
#pragma unroll
        for (int k = 0; k < (S > 0 ? S : 1); ++k) {
            double vn = (double)(en[k] * lm), vd = (double)(ed[k] * lm);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                vn += __shfl_xor_sync(FULL, vn, o);
                vd += __shfl_xor_sync(FULL, vd, o);
            }
            if (lane == 0) {
                const int j = P.a + k;
                if (S > 0) atomicAdd(eb + 2 * j + 1, vn);
                if (k > 0 || PIN) atomicAdd(eb + 2 * j + 0, vd);
            }
        }
    }
}

template <int S, bool PIN, bool OUT_U, bool ENERGY>
__device__ __forceinline__ void run_mode(const Pass &P, int frame, int chunk, int band, int lane) {
    const int c0 = band * P.own - P.hl;
    if (P.vec && c0 >= 0 && c0 + BANDW - 1 <= P.W - 1)
        run<S, PIN, OUT_U, ENERGY, INTERIOR>(P, frame, chunk, band, lane);
    else
        run<S, PIN, OUT_U, ENERGY, EDGE>(P, frame, chunk, band, lane);
}

// Decodes a warp's work item: (frame, row chunk, column band).
__device__ __forceinline__ bool decode_item(const Pass &P, int &frame, int &chunk, int &band) {
    const int warp = threadIdx.x >> 5;
    const int64_t per_frame = (int64_t)P.nbands * P.nchunks;
    const int64_t item = (int64_t)blockIdx.x * WPB + warp;
    if (item >= per_frame * P.nf) return false;
    frame = (int)(item / per_frame);
    const int rem = (int)(item - (int64_t)frame * per_frame);
    chunk = rem / P.nbands;
    band = rem - chunk * P.nbands;
    return true;
}

// First j in this pass's window with |E_{j-1} - E_j| < eps * E_0, or -1.
__device__ __forceinline__ int find_stop(const Pass &P, int frame) {
    const int SG = P.S;
    const double *eb = P.energy + (int64_t)frame * P.K * 2;
    const double inv = 1.0 / ((double)P.H * (double)P.W);
    const double w = (double)P.weight;
    const int j0 = max(1, P.a), j1 = min(P.a + SG - 1, P.K - 2);
    if (j0 > j1) return -1;
    const double e0 = (eb[0] + w * eb[1]) * inv;
    double eprev = (eb[2 * (j0 - 1)] + w * eb[2 * (j0 - 1) + 1]) * inv;
    for (int j = j0; j <= j1; ++j) {
        const double e = (eb[2 * j] + w * eb[2 * j + 1]) * inv;
        if (fabs(eprev - e) < (double)P.eps * e0) return j;
        eprev = e;
    }
    return -1;
}

// Main launch of one pass: every frame not yet stopped runs all SG updates.
template <int SG, bool PIN, bool FINAL>
__global__ void __launch_bounds__(WPB * 32) k_tv_main(Pass P) {
    int frame, chunk, band;
    if (!decode_item(P, frame, chunk, band)) return;
    if (P.done[frame] >= 0) return;
    run_mode<SG, PIN, FINAL, true>(P, frame, chunk, band, threadIdx.x & 31);
}

// Stop-test launch of one pass: frames whose rule fires at j inside the
// window [a, a+S-1] are recomputed with j - a updates and write u_j.
template <bool PIN>
__global__ void __launch_bounds__(WPB * 32) k_tv_fixup(Pass P) {
    int frame, chunk, band;
    if (!decode_item(P, frame, chunk, band)) return;
    const int d = P.done[frame];
    if (d >= 0 && d < P.a) return;  // stopped in an earlier window
    const int j = find_stop(P, frame);
    if (j < 0) return;
    const int lane = threadIdx.x & 31;
    if (chunk == 0 && band == 0 && lane == 0) {
        P.done[frame] = j;  // every block of this frame writes the same j
        if (P.steps) P.steps[frame] = j + 1;
    }
    switch (j - P.a) {
        case 0: if constexpr (PIN) run_mode<0, PIN, true, false>(P, frame, chunk, band, lane); break;
        case 1: run_mode<1, PIN, true, false>(P, frame, chunk, band, lane); break;
        case 2: run_mode<2, PIN, true, false>(P, frame, chunk, band, lane); break;
        case 3: run_mode<3, PIN, true, false>(P, frame, chunk, band, lane); break;
        default: break;
    }
}

// Host launchers (one translation unit each, compiled in parallel).
void launch_main4(const Pass &P, bool pin, bool final_pass, cudaStream_t s);
void launch_main123(const Pass &P, int SG, bool pin, cudaStream_t s);
void launch_fixup(const Pass &P, bool pin, cudaStream_t s);

inline unsigned pass_blocks(const Pass &P) {
    const int64_t items = (int64_t)P.nbands * P.nchunks * P.nf;
    return (unsigned)((items + WPB - 1) / WPB);
}

}  // namespace tv
}  // namespace sci
