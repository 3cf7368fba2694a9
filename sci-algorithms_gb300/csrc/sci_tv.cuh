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
// Mapping.  One warp owns a band of 32*CPL columns (CPL = 2 or 4 per lane,
// vector loads along W) of one frame and marches down a chunk of rows.  The K-1 dual
// updates form a register pipeline: stage k (k = 1..S) handles row r-k when
// input row r arrives, computing p_k and u_k of that row from stage k-1's
// rows r-k and r-k+1.  p and div p never leave registers; horizontal
// neighbours come from warp shuffles; the band overlaps its neighbours by
// S (+1) halo columns and the chunk by S (+1) halo rows.  Each stage hands
// its input row down to the next stage, and the next input row is
// prefetched one step ahead.  Arithmetic on column pairs uses the packed
// f32x2 instructions.  Per pass the frame is read once and written once:
// 8 bytes per pixel of HBM traffic.
//
// Stop test.  The per-frame energies E_k need whole-frame sums, which a
// tiled pipeline sees only after every tile has finished.  The pass
// therefore runs all of its steps speculatively, accumulating per-frame
// float64 sums of (div p_k)^2 and n_k; the work item that finishes last
// (the last ticket of the launch) evaluates the stop rule per frame in
// float64, and a second launch ("fixup") re-runs only the frames that would
// have stopped inside the pass, with the shorter step count.  Frames that
// do not stop (nearly all, for n_iter_max = 5) cost the fixup one read of
// an int per work item.
//
// More than 4 dual updates are split into passes of at most 4 that carry p
// through a workspace (p_in / p_out), with the same speculative scheme per
// pass window.
#pragma once
#include <algorithm>

#include "sci_common.cuh"

namespace sci {
namespace tv {

constexpr int WPB = 4;             // warps per block
#ifndef SCI_TV_PF
#define SCI_TV_PF 2                // input prefetch distance in rows (1 or 2)
#endif
constexpr int SMAX = 4;            // dual updates per pass
constexpr unsigned FULL = 0xffffffffu;

enum { INTERIOR = 0, EDGE = 1 };  // EDGE: band touches a frame edge, or W % 4 != 0

struct Pass {
    const float *f;       // input stack  [nf][H][W] (frame stride fs)
    float *u;             // output stack (same strides)
    float *resid;         // nullable: u - f
    const float *p_in;    // nullable: [nf][2][H][W]  (pr plane, pc plane)
    float *p_out;         // nullable
    double *energy;       // [nf][K][2]: H*W*E_k in [.][k][0]; [.][k][1] stays 0
    int *done;            // [nf]: stop index j >= 1, or -1
    int *steps;           // nullable [nf]: executed Chambolle steps
    int64_t fs;           // frame stride of f/u/resid (elements)
    int nf, H, W, K;      // frames, rows, cols, n_iter_max
    int a;                // this pass starts from p_a (p_in) and computes p_{a+1..a+S}
    float tau, tw;        // tau, tau / weight
    float weight, eps;
    // Column bands (band_window): a band is a window of 32 CPL columns; the
    // middle bands own `own` columns after hl columns of left halo and
    // before hr of right halo; the first band starts at column 0 and the
    // last ends at column W - 1, so no lane works outside the frame.
    int nbands, nchunks, R, own, hl, hr, ht;
    int S;                // dual updates of this pass (geometry of the window)
    int vec;              // 1: rows are aligned for CPL-wide vector loads
    int cpl;              // columns per lane (2 or 4)
    int gpf;              // stop-test launch: blocks per frame
    int lag;              // 1: stages chained within a step; 2: independent stages
    // GAP projection applied while loading f (proj = 1): the stored stack
    // holds x and f = x + lam * (c * phi_b) with phi_b = bit `frame` of the
    // packed mask word and c the per-pixel residual map.
    int proj;
    const uint32_t *bits; // [H][W] packed binary mask
    const float *cmap;    // [H][W] (y1 - A x) / Phi_sum
    float lam;
    int frame_fast;       // work-item order: 1 = frames of one tile adjacent
    // MATLAB-twin update rules (RULE != 0; no stop test): c1 is lambda of
    // the anisotropic Chambolle projection (RULE_CHAM_ITV) or the clip
    // bound (RULE_CLIP); c2 scales div p in u = f - c2 div p (RULE_CLIP)
    float c1, c2;
    // Tape of a single-pass run (kernels with TAPE = true): every stage k
    // writes its p_k to tape_p [S][nf][2][H][W] and, for k < S, its u_k to
    // tape_u [S-1][nf][H][W] (the reverse pass of the unrolled solver).
    float *tape_p, *tape_u;
    // Stop decisions of the pass (nullable; kernels with energies): the
    // main launch's last block to finish writes stopj[frame] = the stop
    // index j in this pass's window, -1 for none, -2 for a frame stopped in
    // an earlier window; ticket counts the main launch's finished blocks
    // (zero when it starts; the last block resets it).
    int *stopj;
    unsigned *ticket;
    // Lean pass with the projection on load and the t output (PROJ 3):
    // t = u + (u - f) of every frame, same layout as u (nullable otherwise).
    float *tout;
};

// Dual update rules of the pipeline (the dual p is held as p / lambda for
// the MATLAB Chambolle files, and as -z for the clip files):
//   RULE_SKIMAGE   scikit-image: p' = (p - tau g) / (1 + tw |g|)
//   RULE_CHAM_ITV  tvdenoise_cham_ITV2D.m: the same with tau = dt,
//                  tw = dt lambda; div p takes no p at the first row /
//                  column (MATLAB's il / iu index vectors)
//   RULE_CHAM_ATV  tvdenoise_cham_ATV2D.m (stacks): t = p - tau g,
//                  p' = t / max(1, lambda |t|) per component; same div
//   RULE_CLIP      TV_denoising*.m: p' = clamp(p - tau g, -c1, c1) per
//                  component (tau = 1/alpha), u = f - c2 div p
enum { RULE_SKIMAGE = 0, RULE_CHAM_ITV = 1, RULE_CHAM_ATV = 2, RULE_CLIP = 3 };


// ------------------------------------------------------------ lane vectors
// CPL consecutive columns of one row held by a lane, as CPL/2 packed pairs.
template <int CPL>
struct Row {
    f2 q[CPL / 2];
};

template <int CPL>
__device__ __forceinline__ Row<CPL> zrow() {
    Row<CPL> r;
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j) r.q[j].v = 0ull;
    return r;
}

template <int CPL>
__device__ __forceinline__ Row<CPL> vload(const float *p) {
    Row<CPL> r;
    if (CPL == 2) {
        r.q[0].v = __ldg(reinterpret_cast<const unsigned long long *>(p));
    } else {
        const ulonglong2 t = __ldg(reinterpret_cast<const ulonglong2 *>(p));
        r.q[0].v = t.x;
        r.q[CPL / 2 - 1].v = t.y;
    }
    return r;
}

template <int CPL>
__device__ __forceinline__ void vstore(float *p, const Row<CPL> &v) {
    if (CPL == 2) {
        *reinterpret_cast<unsigned long long *>(p) = v.q[0].v;
    } else {
        ulonglong2 t;
        t.x = v.q[0].v;
        t.y = v.q[CPL / 2 - 1].v;
        *reinterpret_cast<ulonglong2 *>(p) = t;
    }
}

template <int CPL>
__device__ __forceinline__ float elem(const Row<CPL> &v, int c) {
    return (c & 1) ? hi(v.q[c >> 1]) : lo(v.q[c >> 1]);
}

// Row load with the band's bounds handling (zeros outside the frame).
template <int CPL, int MODE>
__device__ __forceinline__ Row<CPL> load_row(const float *rowp, int col, int W, bool vec) {
    if (MODE == INTERIOR) return vload<CPL>(rowp + col);
    if (vec) return (col >= 0 && col < W) ? vload<CPL>(rowp + col) : zrow<CPL>();
    Row<CPL> r;
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j) {
        const int c = col + 2 * j;
        const float a = (c >= 0 && c < W) ? __ldg(rowp + c) : 0.f;
        const float b = (c + 1 >= 0 && c + 1 < W) ? __ldg(rowp + c + 1) : 0.f;
        r.q[j] = mk2(a, b);
    }
    return r;
}

// Store the columns of this lane that the band owns.
template <int CPL, int MODE>
__device__ __forceinline__ void store_row(float *rowp, int col, const Row<CPL> &v,
                                          bool lane_own, const Row<CPL> &mk, bool vec) {
    if (MODE == INTERIOR || vec) {
        if (lane_own) vstore<CPL>(rowp + col, v);
    } else {
#pragma unroll
        for (int c = 0; c < CPL; ++c)
            if (elem<CPL>(mk, c) != 0.f) rowp[col + c] = elem<CPL>(v, c);
    }
}

// One pixel of the GAP projection x + lam (c phi_b) with phi_b = bit
// `frame` of the packed mask word w (fbit = 1 << frame): fma(lam, c, x)
// where the bit is set, x where it is not -- the value of
// fmaf(lam, c * phi_b, x) (up to the sign of a zero x), in three
// instructions instead of five.
__device__ __forceinline__ float proj_px(float lam, float c, float x, uint32_t w, uint32_t fbit) {
    return (w & fbit) ? fmaf(lam, c, x) : x;
}

// Input row of frame `frame`: the stored row, or with the GAP projection
// applied on the fly (same arithmetic as k_proj_gap: x + lam * (c * phi_b)).
template <int CPL, int MODE, int PROJ>
__device__ __forceinline__ Row<CPL> load_f(const Pass &P, const float *fb, int frame, int64_t row,
                                           int col, int W, bool vec) {
    const Row<CPL> x = load_row<CPL, MODE>(fb + row * W, col, W, vec);
    if (PROJ == 0) return x;
    const Row<CPL> c = load_row<CPL, MODE>(P.cmap + row * W, col, W, vec);
    const Row<CPL> wb =
        load_row<CPL, MODE>(reinterpret_cast<const float *>(P.bits) + row * W, col, W, vec);
    Row<CPL> f;
    const uint32_t fbit = 1u << frame;
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j)
        f.q[j] = mk2(proj_px(P.lam, lo(c.q[j]), lo(x.q[j]), __float_as_uint(lo(wb.q[j])), fbit),
                     proj_px(P.lam, hi(c.q[j]), hi(x.q[j]), __float_as_uint(hi(wb.q[j])), fbit));
    return f;
}

// Pipeline state between steps.
template <int S, int CPL>
struct St {
    Row<CPL> up[S > 0 ? S : 1];  // u_k at the row of stage k+1 (k = 0..S-1)
    Row<CPL> fv[S > 0 ? S : 1];  // f at the row of stage k+1
    Row<CPL> pr[S + 1];          // p_k (row component) at the row of stage k+1
    Row<CPL> pc[S > 0 ? S : 1];  // p_k (column component) at the row of stage k+1
    Row<CPL> nf, nr, nc;         // next input row: f (and p_in planes when PIN)
    Row<CPL> nf2;                // the input row after it (prefetch distance 2)
};

template <int S, int CPL>
__device__ __forceinline__ void zero_state(St<S, CPL> &A) {
#pragma unroll
    for (int k = 0; k < (S > 0 ? S : 1); ++k) {
        A.up[k] = zrow<CPL>();
        A.fv[k] = zrow<CPL>();
        A.pc[k] = zrow<CPL>();
    }
#pragma unroll
    for (int k = 0; k <= S; ++k) A.pr[k] = zrow<CPL>();
    A.nf = A.nr = A.nc = A.nf2 = zrow<CPL>();
}

// Per-lane constants of a band.
template <int CPL>
struct Lane {
    int col;           // first column of this lane
    bool lane_own;     // every column of the lane is owned by the band
    bool first_col;    // this lane holds column 0 (edge bands)
    Row<CPL> mk;       // 1 for owned columns
    Row<CPL> gmask;    // 0 at column W-1 (edge bands)
};

// div p of a row: (pr - pr_up) + (pc - pc_left), with pc_left shifted in
// from the lane on the left.
template <int CPL, int RULE = RULE_SKIMAGE>
__device__ __forceinline__ Row<CPL> divergence(const Row<CPL> &prn, const Row<CPL> &pcn,
                                               const Row<CPL> &pru, bool first_col) {
    float pcl = __shfl_up_sync(FULL, hi(pcn.q[CPL / 2 - 1]), 1);
    // column 0: scikit-image takes p_0, the MATLAB Chambolle files p_0 - p_0
    if (first_col) pcl = (RULE == RULE_CHAM_ITV || RULE == RULE_CHAM_ATV) ? lo(pcn.q[0]) : 0.f;
    Row<CPL> d;
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j) {
        const f2 left = mk2(j == 0 ? pcl : hi(pcn.q[j - 1]), lo(pcn.q[j]));
        d.q[j] = sub2(sub2(add2(prn.q[j], pcn.q[j]), pru.q[j]), left);
    }
    return d;
}

// One pipeline step: input row r enters, stage k handles row r-k.
// GEN: rows may be outside [r0, r1) or touch the frame's first/last row.
template <int S, int CPL, bool PIN, bool OUT_U, bool ENERGY, int MODE, bool GEN, int PROJ,
          int RULE = RULE_SKIMAGE, bool TAPE = false>
__device__ __forceinline__ void step(const Pass &P, const St<S, CPL> &in, St<S, CPL> &out,
                                     int r, int rs, int r0, int r1, const Lane<CPL> &L,
                                     const float *fb, const float *pinb, float *ob, float *rb,
                                     f2 (&ek)[S > 0 ? S : 1], int frame) {
    constexpr int NQ = CPL / 2;
    const int H = P.H, W = P.W;
    const bool vec = P.vec != 0;
    const int64_t hw = (int64_t)H * W;
    const f2 one2 = mk2(1.f, 1.f), tw2 = mk2(P.tw, P.tw), nt2 = mk2(-P.tau, -P.tau);
    const f2 w2 = mk2(P.weight, P.weight);

    // prefetch the input rows ahead (clamped into the frame; unused past it)
    {
        const int64_t rn = (int64_t)min(r + 1, H - 1) * W;
        if (PIN || SCI_TV_PF == 1) {
            out.nf = load_f<CPL, MODE, PROJ>(P, fb, frame, min(r + 1, H - 1), L.col, W, vec);
        } else {
            out.nf = in.nf2;
            out.nf2 = load_f<CPL, MODE, PROJ>(P, fb, frame, min(r + 2, H - 1), L.col, W, vec);
        }
        if (PIN) {
            out.nr = load_row<CPL, MODE>(pinb + rn, L.col, W, vec);
            out.nc = load_row<CPL, MODE>(pinb + hw + rn, L.col, W, vec);
        }
    }

    // ---------------- stage 0: u_0 at row r
    const bool act0 = !GEN || (r < H);
    const Row<CPL> fr = act0 ? in.nf : zrow<CPL>();
    Row<CPL> ucur = fr;
    if (PIN) {
        const Row<CPL> qr = act0 ? in.nr : zrow<CPL>();
        const Row<CPL> qc = act0 ? in.nc : zrow<CPL>();
        // row 0 (MATLAB rules): no p from the row above, p_0 - p_0
        const bool row0 = (RULE == RULE_CHAM_ITV || RULE == RULE_CHAM_ATV) && r == 0;
        const Row<CPL> d = divergence<CPL, RULE>(qr, qc, row0 ? qr : in.pr[0], L.first_col);
#pragma unroll
        for (int j = 0; j < NQ; ++j)
            ucur.q[j] = (RULE == RULE_CLIP) ? fma2(mk2(-P.c2, -P.c2), d.q[j], fr.q[j])
                                            : sub2(fr.q[j], d.q[j]);
        if (ENERGY && act0 && (!GEN || (r >= r0 && r < r1))) {
#pragma unroll
            for (int j = 0; j < NQ; ++j)
                ek[0] = (MODE == INTERIOR) ? fma2(d.q[j], d.q[j], ek[0])
                                           : fma2(mul2(L.mk.q[j], d.q[j]), d.q[j], ek[0]);
        }
        out.pr[0] = qr;
        if (S > 0) out.pc[0] = qc;
        if (S == 0 && OUT_U && act0 && (!GEN || (r >= r0 && r < r1))) {
            const int64_t ro = (int64_t)r * W;
            store_row<CPL, MODE>(ob + ro, L.col, ucur, L.lane_own, L.mk, vec);
            if (rb) {
                Row<CPL> dr;
#pragma unroll
                for (int j = 0; j < NQ; ++j) dr.q[j] = sub2(ucur.q[j], fr.q[j]);
                store_row<CPL, MODE>(rb + ro, L.col, dr, L.lane_own, L.mk, vec);
            }
        }
    }
    if (S > 0) out.fv[0] = fr;

    // ---------------- stages 1..S
#pragma unroll
    for (int k = 1; k <= S; ++k) {
        const int i = r - k;
        out.up[k - 1] = ucur;  // u_{k-1}(i+1): stage k's row in the next step
        const bool act = !GEN || (i >= rs && i < H);
        if (!act) {  // warp-uniform
            out.pr[k] = zrow<CPL>();
            if (k < S) {
                out.pc[k] = zrow<CPL>();
                out.fv[k] = zrow<CPL>();
            }
            ucur = zrow<CPL>();
            continue;
        }
        const Row<CPL> &up = in.up[k - 1];  // u_{k-1}(i)
        const Row<CPL> &fi = in.fv[k - 1];  // f(i)
        const float uR = __shfl_down_sync(FULL, lo(up.q[0]), 1);
        const bool last_row = GEN && (i == H - 1);
        Row<CPL> gr, gc, n, ri, prn, pcn;
#pragma unroll
        for (int j = 0; j < NQ; ++j) {
            const f2 right = mk2(hi(up.q[j]), j + 1 < NQ ? lo(up.q[j + 1]) : uR);
            gc.q[j] = sub2(right, up.q[j]);
            if (MODE != INTERIOR) gc.q[j] = mul2(gc.q[j], L.gmask.q[j]);
            gr.q[j] = last_row ? mk2(0.f, 0.f) : sub2(ucur.q[j], up.q[j]);
            const bool p0zero = (k == 1 && !PIN);
            const f2 qr = p0zero ? mk2(0.f, 0.f) : in.pr[k - 1].q[j];
            const f2 qc = p0zero ? mk2(0.f, 0.f) : in.pc[k - 1].q[j];
            if constexpr (RULE == RULE_SKIMAGE || RULE == RULE_CHAM_ITV) {
                const f2 s = fma2(gr.q[j], gr.q[j], mul2(gc.q[j], gc.q[j]));
                n.q[j] = mk2(sqrt_approx(lo(s)), sqrt_approx(hi(s)));
                const f2 den = fma2(tw2, n.q[j], one2);
                ri.q[j] = mk2(rcp_approx(lo(den)), rcp_approx(hi(den)));
                prn.q[j] = mul2(fma2(nt2, gr.q[j], qr), ri.q[j]);
                pcn.q[j] = mul2(fma2(nt2, gc.q[j], qc), ri.q[j]);
            } else if constexpr (RULE == RULE_CHAM_ATV) {
                const f2 tr = fma2(nt2, gr.q[j], qr), tc = fma2(nt2, gc.q[j], qc);
                const float l = P.c1;
                prn.q[j] = mk2(lo(tr) * rcp_approx(fmaxf(1.f, l * fabsf(lo(tr)))),
                               hi(tr) * rcp_approx(fmaxf(1.f, l * fabsf(hi(tr)))));
                pcn.q[j] = mk2(lo(tc) * rcp_approx(fmaxf(1.f, l * fabsf(lo(tc)))),
                               hi(tc) * rcp_approx(fmaxf(1.f, l * fabsf(hi(tc)))));
            } else {  // RULE_CLIP
                const f2 tr = fma2(nt2, gr.q[j], qr), tc = fma2(nt2, gc.q[j], qc);
                const float c = P.c1;
                prn.q[j] = mk2(fminf(fmaxf(lo(tr), -c), c), fminf(fmaxf(hi(tr), -c), c));
                pcn.q[j] = mk2(fminf(fmaxf(lo(tc), -c), c), fminf(fmaxf(hi(tc), -c), c));
            }
        }
        out.pr[k] = prn;
        if (k < S) out.pc[k] = pcn;
        // row 0 is also reached by fast steps (chunk 0, r = S)
        const bool row0 = (RULE == RULE_CHAM_ITV || RULE == RULE_CHAM_ATV) && i == 0;
        const Row<CPL> d = divergence<CPL, RULE>(prn, pcn, row0 ? prn : in.pr[k], L.first_col);
        Row<CPL> uk;
#pragma unroll
        for (int j = 0; j < NQ; ++j)
            uk.q[j] = (RULE == RULE_CLIP) ? fma2(mk2(-P.c2, -P.c2), d.q[j], fi.q[j])
                                          : sub2(fi.q[j], d.q[j]);
        if (ENERGY && (!GEN || (i >= r0 && i < r1))) {
#pragma unroll
            for (int j = 0; j < NQ; ++j) {
                if (MODE == INTERIOR) {
                    ek[k - 1] = fma2(w2, n.q[j], ek[k - 1]);
                    if (k < S) ek[k] = fma2(d.q[j], d.q[j], ek[k]);
                } else {
                    ek[k - 1] = fma2(mul2(w2, L.mk.q[j]), n.q[j], ek[k - 1]);
                    if (k < S) ek[k] = fma2(mul2(L.mk.q[j], d.q[j]), d.q[j], ek[k]);
                }
            }
        }
        if (TAPE && (!GEN || (i >= r0 && i < r1))) {
            const int64_t ro = (int64_t)i * W;
            float *tp = P.tape_p + ((int64_t)(k - 1) * P.nf + frame) * 2 * hw;
            store_row<CPL, MODE>(tp + ro, L.col, prn, L.lane_own, L.mk, vec);
            store_row<CPL, MODE>(tp + hw + ro, L.col, pcn, L.lane_own, L.mk, vec);
            if (k < S) {
                float *tu = P.tape_u + ((int64_t)(k - 1) * P.nf + frame) * hw;
                store_row<CPL, MODE>(tu + ro, L.col, uk, L.lane_own, L.mk, vec);
            }
        }
        if (k == S) {
            if (!GEN || (i >= r0 && i < r1)) {
                const int64_t ro = (int64_t)i * W;
                if (OUT_U) {
                    store_row<CPL, MODE>(ob + ro, L.col, uk, L.lane_own, L.mk, vec);
                    if (rb) {
                        Row<CPL> dr;
#pragma unroll
                        for (int j = 0; j < NQ; ++j) dr.q[j] = sub2(uk.q[j], fi.q[j]);
                        store_row<CPL, MODE>(rb + ro, L.col, dr, L.lane_own, L.mk, vec);
                    }
                } else {
                    store_row<CPL, MODE>(ob + ro, L.col, prn, L.lane_own, L.mk, vec);
                    store_row<CPL, MODE>(ob + hw + ro, L.col, pcn, L.lane_own, L.mk, vec);
                }
            }
        } else {
            out.fv[k] = fi;
        }
        ucur = uk;
    }
}

// Number of column bands of a W-wide frame for windows of `width` columns
// (band_window): one window when it covers the frame, else a first and a
// last band flush with the frame's edges and as many middle bands as the
// columns between them need.
inline int band_count(int W, int width, int hl, int hr) {
    if (W <= width) return 1;
    const int own = width - hl - hr;
    const int mid = W - 2 * width + hl + hr;
    return 2 + (mid > 0 ? (mid + own - 1) / own : 0);
}

// Band `band`'s window [c0, c0 + width) and owned columns [lo, hi).  The
// first band starts at column 0 and owns up to its right halo; middle
// bands own P.own columns each; the last band ends at column W - 1 (its
// window may reach further left than hl columns before lo, which only
// adds halo).  A frame that fits one window is band 0 alone.
__device__ __forceinline__ void band_window(const Pass &P, int band, int width, int &c0, int &lo,
                                            int &hi) {
    if (band == 0) {
        c0 = 0;
        lo = 0;
        hi = P.nbands == 1 ? P.W : width - P.hr;
    } else {
        lo = width - P.hr + (band - 1) * P.own;
        if (band == P.nbands - 1) {
            c0 = P.W - width;
            hi = P.W;
        } else {
            c0 = lo - P.hl;
            hi = lo + P.own;
        }
    }
}

// A window with frame columns on both sides: no frame edge, no column
// outside the frame.
__device__ __forceinline__ bool band_interior(const Pass &P, int c0, int width) {
    return c0 > 0 && c0 + width < P.W;
}

template <int S, int CPL, bool PIN, bool OUT_U, bool ENERGY, int MODE, int PROJ,
          int RULE = RULE_SKIMAGE, bool TAPE = false, bool RES = true>
__device__ __forceinline__ void run(const Pass &P, int frame, int chunk, int band, int lane) {
    const int H = P.H, W = P.W;
    Lane<CPL> L;
    int c0, own_lo, own_hi;
    band_window(P, band, 32 * CPL, c0, own_lo, own_hi);
    L.col = c0 + lane * CPL;
    const int r0 = chunk * P.R, r1 = min(r0 + P.R, H);
    const int rs = max(0, r0 - P.ht);
    L.lane_own = (L.col >= own_lo) && (L.col + CPL <= own_hi);
    L.first_col = (MODE != INTERIOR) && (L.col == 0);
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j) {
        const int c = L.col + 2 * j;
        L.mk.q[j] = mk2((c >= own_lo && c < own_hi) ? 1.f : 0.f,
                        (c + 1 >= own_lo && c + 1 < own_hi) ? 1.f : 0.f);
        L.gmask.q[j] = mk2(c == W - 1 ? 0.f : 1.f, c + 1 == W - 1 ? 0.f : 1.f);
    }

    const int64_t hw = (int64_t)H * W;
    const float *fb = P.f + (int64_t)frame * P.fs;
    const float *pinb = PIN ? P.p_in + (int64_t)frame * 2 * hw : nullptr;
    float *ob = OUT_U ? P.u + (int64_t)frame * P.fs : P.p_out + (int64_t)frame * 2 * hw;
    // RES = false: compiled without the residual output (P.resid is null)
    float *rb = (RES && OUT_U && P.resid) ? P.resid + (int64_t)frame * P.fs : nullptr;
    const bool vec = P.vec != 0;

    St<S, CPL> A, B;
    zero_state<S, CPL>(A);
    // ek[k]: this lane's part of H*W*E_{a+k} = sum (div p)^2 + weight sum |grad u|
    f2 ek[S > 0 ? S : 1];
#pragma unroll
    for (int k = 0; k < (S > 0 ? S : 1); ++k) ek[k].v = 0ull;
    // first input rows
    A.nf = load_f<CPL, MODE, PROJ>(P, fb, frame, rs, L.col, W, vec);
    A.nf2 = load_f<CPL, MODE, PROJ>(P, fb, frame, min(rs + 1, H - 1), L.col, W, vec);
    if (PIN) {
        A.nr = load_row<CPL, MODE>(pinb + (int64_t)rs * W, L.col, W, vec);
        A.nc = load_row<CPL, MODE>(pinb + hw + (int64_t)rs * W, L.col, W, vec);
    }

    const int rlast = min(r1 - 1 + S, H - 1 + S);
    // Fast steps: every stage inside [r0, r1), away from the frame's last row.
    const int rfb = r0 + S;
    const int rfe = min((PIN || S == 0) ? r1 - 1 : r1, H - 1);
    int r = rs;
    while (r <= rlast) {
        if (r == rfb && r + 1 <= rfe) {
            for (; r + 1 <= rfe; r += 2) {
                step<S, CPL, PIN, OUT_U, ENERGY, MODE, false, PROJ, RULE, TAPE>(
                    P, A, B, r, rs, r0, r1, L, fb, pinb, ob, rb, ek, frame);
                step<S, CPL, PIN, OUT_U, ENERGY, MODE, false, PROJ, RULE, TAPE>(
                    P, B, A, r + 1, rs, r0, r1, L, fb, pinb, ob, rb, ek, frame);
            }
            continue;
        }
        // prologue (halo rows, first S steps) and epilogue (chunk tail, last row)
        step<S, CPL, PIN, OUT_U, ENERGY, MODE, true, PROJ, RULE, TAPE>(P, A, B, r, rs, r0, r1, L,
                                                                        fb, pinb, ob, rb, ek,
                                                                        frame);
        A = B;
        ++r;
    }

    if (ENERGY) {
        const float lm = (MODE == INTERIOR) ? (L.lane_own ? 1.f : 0.f) : 1.f;
        double *eb = P.energy + (int64_t)frame * P.K * 2;
#pragma unroll
        for (int k = 0; k < (S > 0 ? S : 1); ++k) {
            double v = (double)((lo(ek[k]) + hi(ek[k])) * lm);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
            if (lane == 0) atomicAdd(eb + 2 * (P.a + k), v);
        }
        // the sums are in before the block draws its ticket (decide_stops)
        if (lane == 0 && P.ticket) __threadfence();
    }
}

// ------------------------------------------------------- lag-2 pipeline
// Stage k handles row r - 2k when input row r arrives, so it consumes only
// rows its predecessor produced in the two previous steps: the S stages of
// a step are independent of each other (S-fold instruction-level
// parallelism per warp) at the cost of a two-row history per stage.
template <int CPL>
struct Slab {
    Row<CPL> u, pr, pc, f;  // u_k, p_k (both components) and f of one row
};

template <int S, int CPL>
struct St2 {
    Slab<CPL> X1[S > 0 ? S : 1];  // newest row produced by stage k (k = 0..S-1)
    Slab<CPL> X2[S > 0 ? S : 1];  // the row before it
    Row<CPL> ps1;                 // stage S: its previous row of p_S (row component)
    Row<CPL> nf, nr, nc;          // next input row
};

template <int CPL>
__device__ __forceinline__ Slab<CPL> zslab() {
    Slab<CPL> z;
    z.u = z.pr = z.pc = z.f = zrow<CPL>();
    return z;
}

template <int S, int CPL, bool PIN, bool OUT_U, bool ENERGY, int MODE, bool GEN>
__device__ __forceinline__ void step2(const Pass &P, const St2<S, CPL> &in, St2<S, CPL> &out,
                                      int r, int rs, int r0, int r1, const Lane<CPL> &L,
                                      const float *fb, const float *pinb, float *ob, float *rb,
                                      f2 (&ek)[S > 0 ? S : 1]) {
    constexpr int NQ = CPL / 2;
    const int H = P.H, W = P.W;
    const bool vec = P.vec != 0;
    const int64_t hw = (int64_t)H * W;
    const f2 one2 = mk2(1.f, 1.f), tw2 = mk2(P.tw, P.tw), nt2 = mk2(-P.tau, -P.tau);
    const f2 w2 = mk2(P.weight, P.weight);

    {   // prefetch the next input row (clamped into the frame; unused past it)
        const int64_t rn = (int64_t)min(r + 1, H - 1) * W;
        out.nf = load_row<CPL, MODE>(fb + rn, L.col, W, vec);
        if (PIN) {
            out.nr = load_row<CPL, MODE>(pinb + rn, L.col, W, vec);
            out.nc = load_row<CPL, MODE>(pinb + hw + rn, L.col, W, vec);
        }
    }

    // ---------------- stages S..1: row i = r - 2k, inputs from earlier steps
#pragma unroll
    for (int k = S; k >= 1; --k) {
        const int i = r - 2 * k;
        const bool act = !GEN || (i >= rs && i < H);
        if (!act) {  // warp-uniform
            if (k < S) out.X1[k] = zslab<CPL>();
            else out.ps1 = zrow<CPL>();
            continue;
        }
        const Slab<CPL> &a = in.X2[k - 1];  // stage k-1, row i
        const Slab<CPL> &b = in.X1[k - 1];  // stage k-1, row i+1
        const Row<CPL> &pru = (k < S) ? in.X1[k].pr : in.ps1;  // p_k row i-1
        const float uR = __shfl_down_sync(FULL, lo(a.u.q[0]), 1);
        const bool last_row = GEN && (i == H - 1);
        Row<CPL> gr, gc, n, prn, pcn;
#pragma unroll
        for (int j = 0; j < NQ; ++j) {
            const f2 right = mk2(hi(a.u.q[j]), j + 1 < NQ ? lo(a.u.q[j + 1]) : uR);
            gc.q[j] = sub2(right, a.u.q[j]);
            if (MODE != INTERIOR) gc.q[j] = mul2(gc.q[j], L.gmask.q[j]);
            gr.q[j] = last_row ? mk2(0.f, 0.f) : sub2(b.u.q[j], a.u.q[j]);
            const f2 s2 = fma2(gr.q[j], gr.q[j], mul2(gc.q[j], gc.q[j]));
            n.q[j] = mk2(sqrt_approx(lo(s2)), sqrt_approx(hi(s2)));
            const f2 den = fma2(tw2, n.q[j], one2);
            const f2 ri = mk2(rcp_approx(lo(den)), rcp_approx(hi(den)));
            const bool p0zero = (k == 1 && !PIN);
            const f2 qr = p0zero ? mk2(0.f, 0.f) : a.pr.q[j];
            const f2 qc = p0zero ? mk2(0.f, 0.f) : a.pc.q[j];
            prn.q[j] = mul2(fma2(nt2, gr.q[j], qr), ri);
            pcn.q[j] = mul2(fma2(nt2, gc.q[j], qc), ri);
        }
        const Row<CPL> d = divergence<CPL>(prn, pcn, pru, L.first_col);
        Row<CPL> uk;
#pragma unroll
        for (int j = 0; j < NQ; ++j) uk.q[j] = sub2(a.f.q[j], d.q[j]);
        if (ENERGY && (!GEN || (i >= r0 && i < r1))) {
#pragma unroll
            for (int j = 0; j < NQ; ++j) {
                if (MODE == INTERIOR) {
                    ek[k - 1] = fma2(w2, n.q[j], ek[k - 1]);
                    if (k < S) ek[k] = fma2(d.q[j], d.q[j], ek[k]);
                } else {
                    ek[k - 1] = fma2(mul2(w2, L.mk.q[j]), n.q[j], ek[k - 1]);
                    if (k < S) ek[k] = fma2(mul2(L.mk.q[j], d.q[j]), d.q[j], ek[k]);
                }
            }
        }
        if (k == S) {
            out.ps1 = prn;
            if (!GEN || (i >= r0 && i < r1)) {
                const int64_t ro = (int64_t)i * W;
                if (OUT_U) {
                    store_row<CPL, MODE>(ob + ro, L.col, uk, L.lane_own, L.mk, vec);
                    if (rb) {
                        Row<CPL> dr;
#pragma unroll
                        for (int j = 0; j < NQ; ++j) dr.q[j] = sub2(uk.q[j], a.f.q[j]);
                        store_row<CPL, MODE>(rb + ro, L.col, dr, L.lane_own, L.mk, vec);
                    }
                } else {
                    store_row<CPL, MODE>(ob + ro, L.col, prn, L.lane_own, L.mk, vec);
                    store_row<CPL, MODE>(ob + hw + ro, L.col, pcn, L.lane_own, L.mk, vec);
                }
            }
        } else {
            Slab<CPL> o;
            o.u = uk;
            o.pr = prn;
            o.pc = pcn;
            o.f = a.f;
            out.X1[k] = o;
        }
    }
    // history shift
#pragma unroll
    for (int k = 0; k < S; ++k) out.X2[k] = in.X1[k];

    // ---------------- stage 0: u_0 at row r
    const bool act0 = !GEN || (r < H);
    const Row<CPL> fr = act0 ? in.nf : zrow<CPL>();
    Slab<CPL> o0;
    o0.u = fr;
    o0.f = fr;
    o0.pr = zrow<CPL>();
    o0.pc = zrow<CPL>();
    if (PIN) {
        const Row<CPL> qr = act0 ? in.nr : zrow<CPL>();
        const Row<CPL> qc = act0 ? in.nc : zrow<CPL>();
        const Row<CPL> &pru0 = (S > 0) ? in.X1[0].pr : in.ps1;
        const Row<CPL> d = divergence<CPL>(qr, qc, pru0, L.first_col);
#pragma unroll
        for (int j = 0; j < NQ; ++j) o0.u.q[j] = sub2(fr.q[j], d.q[j]);
        if (ENERGY && act0 && (!GEN || (r >= r0 && r < r1))) {
#pragma unroll
            for (int j = 0; j < NQ; ++j)
                ek[0] = (MODE == INTERIOR) ? fma2(d.q[j], d.q[j], ek[0])
                                           : fma2(mul2(L.mk.q[j], d.q[j]), d.q[j], ek[0]);
        }
        o0.pr = qr;
        o0.pc = qc;
        if (S == 0) {
            out.ps1 = qr;
            if (OUT_U && act0 && (!GEN || (r >= r0 && r < r1))) {
                const int64_t ro = (int64_t)r * W;
                store_row<CPL, MODE>(ob + ro, L.col, o0.u, L.lane_own, L.mk, vec);
                if (rb) {
                    Row<CPL> dr;
#pragma unroll
                    for (int j = 0; j < NQ; ++j) dr.q[j] = sub2(o0.u.q[j], fr.q[j]);
                    store_row<CPL, MODE>(rb + ro, L.col, dr, L.lane_own, L.mk, vec);
                }
            }
        }
    }
    if (S > 0) out.X1[0] = o0;
}

template <int S, int CPL, bool PIN, bool OUT_U, bool ENERGY, int MODE>
__device__ __forceinline__ void run2(const Pass &P, int frame, int chunk, int band, int lane) {
    const int H = P.H, W = P.W;
    Lane<CPL> L;
    int c0, own_lo, own_hi;
    band_window(P, band, 32 * CPL, c0, own_lo, own_hi);
    L.col = c0 + lane * CPL;
    const int r0 = chunk * P.R, r1 = min(r0 + P.R, H);
    const int rs = max(0, r0 - P.ht);
    L.lane_own = (L.col >= own_lo) && (L.col + CPL <= own_hi);
    L.first_col = (MODE != INTERIOR) && (L.col == 0);
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j) {
        const int c = L.col + 2 * j;
        L.mk.q[j] = mk2((c >= own_lo && c < own_hi) ? 1.f : 0.f,
                        (c + 1 >= own_lo && c + 1 < own_hi) ? 1.f : 0.f);
        L.gmask.q[j] = mk2(c == W - 1 ? 0.f : 1.f, c + 1 == W - 1 ? 0.f : 1.f);
    }
    const int64_t hw = (int64_t)H * W;
    const float *fb = P.f + (int64_t)frame * P.fs;
    const float *pinb = PIN ? P.p_in + (int64_t)frame * 2 * hw : nullptr;
    float *ob = OUT_U ? P.u + (int64_t)frame * P.fs : P.p_out + (int64_t)frame * 2 * hw;
    float *rb = (OUT_U && P.resid) ? P.resid + (int64_t)frame * P.fs : nullptr;
    const bool vec = P.vec != 0;

    St2<S, CPL> A, B;
#pragma unroll
    for (int k = 0; k < (S > 0 ? S : 1); ++k) A.X1[k] = A.X2[k] = zslab<CPL>();
    A.ps1 = A.nr = A.nc = zrow<CPL>();
    f2 ek[S > 0 ? S : 1];
#pragma unroll
    for (int k = 0; k < (S > 0 ? S : 1); ++k) ek[k].v = 0ull;
    A.nf = load_row<CPL, MODE>(fb + (int64_t)rs * W, L.col, W, vec);
    if (PIN) {
        A.nr = load_row<CPL, MODE>(pinb + (int64_t)rs * W, L.col, W, vec);
        A.nc = load_row<CPL, MODE>(pinb + hw + (int64_t)rs * W, L.col, W, vec);
    }
    const int rlast = min(r1 - 1 + 2 * S, H - 1 + 2 * S);
    const int rfb = r0 + 2 * S;
    const int rfe = min((PIN || S == 0) ? r1 - 1 : r1 + 1, H - 1);
    int r = rs;
    while (r <= rlast) {
        if (r == rfb && r + 1 <= rfe) {
            for (; r + 1 <= rfe; r += 2) {
                step2<S, CPL, PIN, OUT_U, ENERGY, MODE, false>(P, A, B, r, rs, r0, r1, L, fb,
                                                                pinb, ob, rb, ek);
                step2<S, CPL, PIN, OUT_U, ENERGY, MODE, false>(P, B, A, r + 1, rs, r0, r1, L, fb,
                                                                pinb, ob, rb, ek);
            }
            continue;
        }
        step2<S, CPL, PIN, OUT_U, ENERGY, MODE, true>(P, A, B, r, rs, r0, r1, L, fb, pinb, ob,
                                                       rb, ek);
        A = B;
        ++r;
    }
    if (ENERGY) {
        const float lm = (MODE == INTERIOR) ? (L.lane_own ? 1.f : 0.f) : 1.f;
        double *eb = P.energy + (int64_t)frame * P.K * 2;
#pragma unroll
        for (int k = 0; k < (S > 0 ? S : 1); ++k) {
            double v = (double)((lo(ek[k]) + hi(ek[k])) * lm);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
            if (lane == 0) atomicAdd(eb + 2 * (P.a + k), v);
        }
        // the sums are in before the block draws its ticket (decide_stops)
        if (lane == 0 && P.ticket) __threadfence();
    }
}

template <int S, int CPL, bool PIN, bool OUT_U, bool ENERGY, int LAG = 1, int PROJ = 0,
          int RULE = RULE_SKIMAGE, bool TAPE = false, bool RES = true>
__device__ __forceinline__ void run_mode(const Pass &P, int frame, int chunk, int band, int lane) {
    int c0, lo, hi;
    band_window(P, band, 32 * CPL, c0, lo, hi);
    const bool interior = P.vec && band_interior(P, c0, 32 * CPL);
    static_assert(!(TAPE && LAG == 2), "the tape is written by the lag-1 pipeline");
    if (LAG == 2) {
        if (interior) run2<S, CPL, PIN, OUT_U, ENERGY, INTERIOR>(P, frame, chunk, band, lane);
        else run2<S, CPL, PIN, OUT_U, ENERGY, EDGE>(P, frame, chunk, band, lane);
    } else {
        if (interior)
            run<S, CPL, PIN, OUT_U, ENERGY, INTERIOR, PROJ, RULE, TAPE, RES>(P, frame, chunk,
                                                                              band, lane);
        else
            run<S, CPL, PIN, OUT_U, ENERGY, EDGE, PROJ, RULE, TAPE, RES>(P, frame, chunk, band,
                                                                          lane);
    }
}

// Decodes a work item: (frame, row chunk, column band).  With frame_fast
// the frames of one tile are adjacent items (they share the tile's rows of
// the per-pixel maps in L1/L2); otherwise the bands of one frame are.
__device__ __forceinline__ bool decode_index(const Pass &P, int64_t item, int &frame, int &chunk,
                                             int &band) {
    const int64_t per_frame = (int64_t)P.nbands * P.nchunks;
    if (item >= per_frame * P.nf) return false;
    int rem;
    if (P.frame_fast) {
        const int64_t tile = item / P.nf;
        frame = (int)(item - tile * P.nf);
        rem = (int)tile;
    } else {
        frame = (int)(item / per_frame);
        rem = (int)(item - (int64_t)frame * per_frame);
    }
    chunk = rem / P.nbands;
    band = rem - chunk * P.nbands;
    return true;
}

__device__ __forceinline__ bool decode_item(const Pass &P, int &frame, int &chunk, int &band) {
    return decode_index(P, (int64_t)blockIdx.x * WPB + (threadIdx.x >> 5), frame, chunk, band);
}

// First j in this pass's window with |E_{j-1} - E_j| < eps * E_0, or -1.
// CG: read the sums from L2 (they were added by other blocks' atomics
// during the same launch).
template <bool CG = false>
__device__ __forceinline__ int find_stop(const Pass &P, int frame) {
    const int SG = P.S;
    const double *eb = P.energy + (int64_t)frame * P.K * 2;
    auto ld = [&](int i) { return CG ? __ldcg(eb + i) : eb[i]; };
    const double inv = 1.0 / ((double)P.H * (double)P.W);
    const double w = (double)P.weight;
    const int j0 = max(1, P.a), j1 = min(P.a + SG - 1, P.K - 2);
    if (j0 > j1) return -1;
    const double e0 = (ld(0) + w * ld(1)) * inv;
    double eprev = (ld(2 * (j0 - 1)) + w * ld(2 * (j0 - 1) + 1)) * inv;
    for (int j = j0; j <= j1; ++j) {
        const double e = (ld(2 * j) + w * ld(2 * j + 1)) * inv;
        if (fabs(eprev - e) < (double)P.eps * e0) return j;
        eprev = e;
    }
    return -1;
}

template <int CPL>
constexpr int min_blocks() { return CPL == 2 ? 4 : 3; }

// The main launch's last work item to finish evaluates the stop rule of
// every frame into P.stopj (a warp learns that it is the last from the
// ticket its lane 0 draws after the warp's energy sums are in; no warp
// waits), so that the stop-test launch reads one int per work item instead
// of the sums.  Every work item (warp) of the launch draws one ticket.
__device__ __forceinline__ void decide_stops(const Pass &P, int lane) {
    const unsigned items = (unsigned)((int64_t)P.nbands * P.nchunks * P.nf);
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(P.ticket, 1u);
    t = __shfl_sync(FULL, t, 0);
    if (t != items - 1) return;
    __threadfence();
    for (int f = lane; f < P.nf; f += 32) {
        const int d = P.a > 0 ? P.done[f] : -1;
        P.stopj[f] = (d >= 0 && d < P.a) ? -2 : find_stop<true>(P, f);
    }
    if (lane == 0) *P.ticket = 0u;
}

// Main launch of one pass: every frame not yet stopped runs all SG updates.
template <int SG, bool PIN, bool FINAL, int CPL, int LAG = 1, int PROJ = 0,
          int RULE = RULE_SKIMAGE, bool TAPE = false, bool RES = true>
__global__ void __launch_bounds__(WPB * 32, min_blocks<CPL>()) k_tv_main(Pass P) {
    int frame, chunk, band;
    if (!decode_item(P, frame, chunk, band)) return;
    // the MATLAB rules and the taped runs have no stop test and need no energies
    constexpr bool EN = RULE == RULE_SKIMAGE && !TAPE;
    const int lane = threadIdx.x & 31;
    if (!(PIN && P.done[frame] >= 0))  // not stopped in an earlier pass
        run_mode<SG, CPL, PIN, FINAL, EN, LAG, PROJ, RULE, TAPE, RES>(P, frame, chunk, band,
                                                                      lane);
    if constexpr (EN) {
        if (P.ticket) decide_stops(P, lane);
    }
}

// Stop-test launch of one pass over the same work items as the main launch:
// frames whose rule fires at j inside the window [a, a+S-1] are recomputed
// (by all their items at once) with j - a updates and write u_j; the other
// items exit after reading a few doubles.
template <bool PIN, int CPL, int PROJ = 0>
__global__ void __launch_bounds__(WPB * 32, min_blocks<CPL>()) k_tv_fixup(Pass P) {
    int frame, chunk, band;
    if (!decode_item(P, frame, chunk, band)) return;
    int j;
    if (P.stopj) {
        j = P.stopj[frame];  // decided by the main launch
        if (j == -2) return;  // stopped in an earlier window
    } else {
        if (PIN) {
            const int d = P.done[frame];
            if (d >= 0 && d < P.a) return;  // stopped in an earlier window
        }
        j = find_stop(P, frame);
    }
    const int lane = threadIdx.x & 31;
    const bool lead = (chunk == 0 && band == 0 && lane == 0);
    if (j < 0) {
        if (lead && P.steps && P.a + P.S == P.K - 1) P.steps[frame] = P.K;
        return;
    }
    if (lead) {
        P.done[frame] = j;  // every warp of this frame computes the same j
        if (P.steps) P.steps[frame] = j + 1;
    }
    switch (j - P.a) {
        case 0: if constexpr (PIN) run_mode<0, CPL, PIN, true, false, 1, PROJ>(P, frame, chunk, band, lane); break;
        case 1: run_mode<1, CPL, PIN, true, false, 1, PROJ>(P, frame, chunk, band, lane); break;
        case 2: run_mode<2, CPL, PIN, true, false, 1, PROJ>(P, frame, chunk, band, lane); break;
        case 3: run_mode<3, CPL, PIN, true, false, 1, PROJ>(P, frame, chunk, band, lane); break;
        default: break;
    }
}

// Host launchers (one translation unit each, compiled in parallel).
void launch_main4_c4(const Pass &P, bool pin, bool final_pass, cudaStream_t s);
void launch_main4_c2(const Pass &P, bool pin, bool final_pass, cudaStream_t s);
void launch_main4_lag2(const Pass &P, bool pin, bool final_pass, cudaStream_t s);
void launch_main_proj(const Pass &P, int SG, cudaStream_t s);
void launch_fixup_proj(const Pass &P, cudaStream_t s);
void launch_main123(const Pass &P, int SG, bool pin, cudaStream_t s);
void launch_tape(const Pass &P, int SG, cudaStream_t s);  // sci_tv_tape.cu
void launch_rule1(const Pass &P, int SG, bool pin, bool final_pass, cudaStream_t s);
void launch_rule2(const Pass &P, int SG, bool pin, bool final_pass, cudaStream_t s);
void launch_rule3(const Pass &P, int SG, bool pin, bool final_pass, cudaStream_t s);

// Main kernels of one MATLAB-rule pass (4 columns per lane, no stop test).
template <int RULE>
void launch_rule_impl(const Pass &P, int SG, bool pin, bool final_pass, cudaStream_t s) {
    const unsigned g = (unsigned)(((int64_t)P.nbands * P.nchunks * P.nf + WPB - 1) / WPB);
    const unsigned T = WPB * 32;
#define SCI_RULE_CASE(SGV)                                                            \
    case SGV:                                                                         \
        if (!pin && final_pass) k_tv_main<SGV, false, true, 4, 1, 0, RULE><<<g, T, 0, s>>>(P); \
        else if (pin && final_pass) k_tv_main<SGV, true, true, 4, 1, 0, RULE><<<g, T, 0, s>>>(P); \
        break;
    switch (SG) {
        SCI_RULE_CASE(1)
        SCI_RULE_CASE(2)
        SCI_RULE_CASE(3)
        default:
            if (!pin && final_pass) k_tv_main<4, false, true, 4, 1, 0, RULE><<<g, T, 0, s>>>(P);
            else if (!pin) k_tv_main<4, false, false, 4, 1, 0, RULE><<<g, T, 0, s>>>(P);
            else if (final_pass) k_tv_main<4, true, true, 4, 1, 0, RULE><<<g, T, 0, s>>>(P);
            else k_tv_main<4, true, false, 4, 1, 0, RULE><<<g, T, 0, s>>>(P);
            break;
    }
#undef SCI_RULE_CASE
}
void launch_fixup(const Pass &P, bool pin, cudaStream_t s);
// Register-lean single-pass kernels (sci_tv_slim.cu, P.cpl = 2 or 4); minb:
// the resident blocks per SM their registers are sized for (0: default);
// proj: the GAP projection applied on load.
void launch_slim(const Pass &P, int SG, int minb, int proj, cudaStream_t s);
void launch_slim_fix(const Pass &P, int proj, cudaStream_t s);
int slim_resident_blocks(int cpl, int SG, int minb, int proj);  // of the main kernel

inline unsigned pass_blocks(const Pass &P) {
    const int64_t items = (int64_t)P.nbands * P.nchunks * P.nf;
    return (unsigned)((items + WPB - 1) / WPB);
}

}  // namespace tv
}  // namespace sci
