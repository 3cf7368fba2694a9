// Chambolle TV pass, register-lean form of the row pipeline (sci_tv.cuh).
//
// Same mapping and the same arithmetic, operation for operation, as the
// generic pipeline's scikit-image rule without a p input (one pass of
// n_iter_max <= 5 steps): a warp owns a 128-column band of one frame (4
// columns per lane) and marches down a chunk of rows; stage k computes p_k
// and u_k of row r - k when input row r arrives.  What differs is where the
// values live:
//
//  * f rows.  Stage k needs f(r - k).  The generic pipeline hands f down the
//    stages in registers (16 registers and 12 register copies per step); here
//    every input row is copied by cp.async into a per-warp ring of RING rows
//    in shared memory, PF rows ahead of its use, and each stage reads its f
//    row back from the ring (a lane reads only the 16 bytes it copied itself,
//    so the per-thread cp.async.wait_group is the only synchronisation).
//    Stage 1 takes f(r - 1) = u_0(r - 1) from the state it already holds.
//  * shifted neighbours.  The one-column shifts of the forward column
//    difference and of the divergence pair values across f32x2 register
//    pairs; they are computed as scalar FP32 operations whose results land in
//    fresh pairs, instead of re-pairing shifted halves with moves.
//
// Rounding is identical to the generic pipeline (same operations in the same
// order), so the two produce bit-identical frames.
#pragma once

#include "sci_tv.cuh"

namespace sci {
namespace tv {
namespace slim {

constexpr int RING = 8;              // f rows per warp in shared memory (power of 2)
constexpr int PF = 3;                // rows copied ahead of the step that reads them
constexpr int ROWB = 32 * 16;        // bytes of one band row (4 floats per lane)
static_assert(RING >= SMAX + 1 + PF, "ring too small for the pipeline depth");

// A lane's 4 columns as two packed pairs: (c0, c1), (c2, c3).
struct R4 {
    f2 a, b;
};

__device__ __forceinline__ R4 z4() {
    R4 r;
    r.a.v = 0ull;
    r.b.v = 0ull;
    return r;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// 16-byte asynchronous copy global -> shared; bytes = 0 fills zeros.
__device__ __forceinline__ void cp16(uint32_t dst, const float *src, uint32_t bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ R4 lds(const unsigned char *ring, int row) {
    const ulonglong2 t =
        *reinterpret_cast<const ulonglong2 *>(ring + (row & (RING - 1)) * ROWB);
    R4 r;
    r.a.v = t.x;
    r.b.v = t.y;
    return r;
}

// Pipeline state between steps (no p input: p_0 = 0, u_0 = f).
template <int S>
struct SS {
    R4 up[S];      // up[k]: u_k of the row stage k+1 handles next step
    R4 pr[S + 1];  // pr[k] (k >= 1): p_k (row component) of the row stage k handled last
    R4 pc[S];      // pc[k] (1 <= k < S): p_k (column component), same row
};

template <int S>
__device__ __forceinline__ void zero_ss(SS<S> &A) {
#pragma unroll
    for (int k = 0; k < S; ++k) {
        A.up[k] = z4();
        A.pc[k] = z4();
    }
#pragma unroll
    for (int k = 0; k <= S; ++k) A.pr[k] = z4();
}

// Per-lane constants of a band.
struct SLane {
    int col;          // first column of this lane
    int colc;         // col clamped into [0, W - 4] (the address of a zero-filled copy)
    bool lane_own;    // the band owns all 4 columns of the lane
    bool first_col;   // the lane holds column 0
    R4 mk;            // 1 for owned columns (edge bands)
    R4 gmask;         // 0 at column W-1 (edge bands)
};

// One pipeline step: input row r enters, stage k handles row r - k.
// GEN: rows may lie outside [r0, r1) or touch the frame's last row.
template <int S, bool ENERGY, int MODE, bool GEN>
__device__ __forceinline__ void sstep(const Pass &P, const SS<S> &in, SS<S> &out, int r, int rs,
                                      int r0, int r1, const SLane &L, const float *fb, float *ob,
                                      const unsigned char *ring, uint32_t ring_s, uint32_t ldb,
                                      f2 (&ek)[S]) {
    const int H = P.H, W = P.W;
    const f2 one2 = mk2(1.f, 1.f), tw2 = mk2(P.tw, P.tw), nt2 = mk2(-P.tau, -P.tau);
    const f2 w2 = mk2(P.weight, P.weight);

    // copy input row r + PF into its ring slot (clamped into the frame; a
    // clamped row is never read), then wait for row r
    {
        const int rp = min(r + PF, H - 1);
        cp16(ring_s + ((r + PF) & (RING - 1)) * ROWB, fb + (int64_t)rp * W + L.colc, ldb);
        cp_commit();
        cp_wait<PF>();
    }

    // ---------------- stage 0: u_0 = f at row r
    R4 ucur = (!GEN || r < H) ? lds(ring, r) : z4();

    // ---------------- stages 1..S
#pragma unroll
    for (int k = 1; k <= S; ++k) {
        const int i = r - k;
        out.up[k - 1] = ucur;  // u_{k-1}(i+1): stage k's row in the next step
        const bool act = !GEN || (i >= rs && i < H);
        if (!act) {  // warp-uniform
            out.pr[k] = z4();
            if (k < S) out.pc[k] = z4();
            ucur = z4();
            continue;
        }
        const R4 &up = in.up[k - 1];  // u_{k-1}(i)
        // f(i): u_0(i) for stage 1, else the ring
        const R4 fi = (k == 1) ? up : lds(ring, i);
        const float uR = __shfl_down_sync(FULL, lo(up.a), 1);
        // forward column difference (one-column shift: scalar)
        float g0 = hi(up.a) - lo(up.a), g1 = lo(up.b) - hi(up.a);
        float g2 = hi(up.b) - lo(up.b), g3 = uR - hi(up.b);
        R4 gc;
        gc.a = mk2(g0, g1);
        gc.b = mk2(g2, g3);
        if (MODE != INTERIOR) {
            gc.a = mul2(gc.a, L.gmask.a);
            gc.b = mul2(gc.b, L.gmask.b);
        }
        R4 gr;
        if (GEN && i == H - 1) {
            gr = z4();
        } else {
            gr.a = sub2(ucur.a, up.a);
            gr.b = sub2(ucur.b, up.b);
        }
        R4 n, prn, pcn;
        {
            const f2 sa = fma2(gr.a, gr.a, mul2(gc.a, gc.a));
            const f2 sb = fma2(gr.b, gr.b, mul2(gc.b, gc.b));
            n.a = mk2(sqrt_approx(lo(sa)), sqrt_approx(hi(sa)));
            n.b = mk2(sqrt_approx(lo(sb)), sqrt_approx(hi(sb)));
            const f2 da = fma2(tw2, n.a, one2), db = fma2(tw2, n.b, one2);
            const f2 ra = mk2(rcp_approx(lo(da)), rcp_approx(hi(da)));
            const f2 rb = mk2(rcp_approx(lo(db)), rcp_approx(hi(db)));
            if (k == 1) {  // p_0 = 0: (0 - tau g) rounds as the product
                prn.a = mul2(mul2(nt2, gr.a), ra);
                prn.b = mul2(mul2(nt2, gr.b), rb);
                pcn.a = mul2(mul2(nt2, gc.a), ra);
                pcn.b = mul2(mul2(nt2, gc.b), rb);
            } else {
                prn.a = mul2(fma2(nt2, gr.a, in.pr[k - 1].a), ra);
                prn.b = mul2(fma2(nt2, gr.b, in.pr[k - 1].b), rb);
                pcn.a = mul2(fma2(nt2, gc.a, in.pc[k - 1].a), ra);
                pcn.b = mul2(fma2(nt2, gc.b, in.pc[k - 1].b), rb);
            }
        }
        out.pr[k] = prn;
        if (k < S) out.pc[k] = pcn;
        // divergence ((pr + pc) - pr_up) - pc_left, the left shift in scalar
        float pcl = __shfl_up_sync(FULL, hi(pcn.b), 1);
        if (MODE != INTERIOR && L.first_col) pcl = 0.f;
        const f2 ta = sub2(add2(prn.a, pcn.a), in.pr[k].a);
        const f2 tb = sub2(add2(prn.b, pcn.b), in.pr[k].b);
        R4 d;
        d.a = mk2(lo(ta) - pcl, hi(ta) - lo(pcn.a));
        d.b = mk2(lo(tb) - hi(pcn.a), hi(tb) - lo(pcn.b));
        R4 uk;
        uk.a = sub2(fi.a, d.a);
        uk.b = sub2(fi.b, d.b);
        if (ENERGY && (!GEN || (i >= r0 && i < r1))) {
            if (MODE == INTERIOR) {
                ek[k - 1] = fma2(w2, n.a, ek[k - 1]);
                if (k < S) ek[k] = fma2(d.a, d.a, ek[k]);
                ek[k - 1] = fma2(w2, n.b, ek[k - 1]);
                if (k < S) ek[k] = fma2(d.b, d.b, ek[k]);
            } else {
                ek[k - 1] = fma2(mul2(w2, L.mk.a), n.a, ek[k - 1]);
                if (k < S) ek[k] = fma2(mul2(L.mk.a, d.a), d.a, ek[k]);
                ek[k - 1] = fma2(mul2(w2, L.mk.b), n.b, ek[k - 1]);
                if (k < S) ek[k] = fma2(mul2(L.mk.b, d.b), d.b, ek[k]);
            }
        }
        if (k == S && (!GEN || (i >= r0 && i < r1)) && L.lane_own) {
            ulonglong2 t;
            t.x = uk.a.v;
            t.y = uk.b.v;
            *reinterpret_cast<ulonglong2 *>(ob + (int64_t)i * W + L.col) = t;
        }
        ucur = uk;
    }
}

// One work item: frame, row chunk, column band.  Requires rows aligned for
// 16-byte access (W % 4 == 0, 16-byte aligned base pointers).
template <int S, bool ENERGY, int MODE>
__device__ __forceinline__ void srun(const Pass &P, int frame, int chunk, int band, int lane,
                                     const unsigned char *ring, uint32_t ring_s) {
    const int H = P.H, W = P.W;
    SLane L;
    L.col = band * P.own - P.hl + lane * 4;
    const int r0 = chunk * P.R, r1 = min(r0 + P.R, H);
    const int rs = max(0, r0 - P.ht);
    const int own_lo = band * P.own, own_hi = min(own_lo + P.own, W);
    L.lane_own = (L.col >= own_lo) && (L.col + 4 <= own_hi);
    L.first_col = (MODE != INTERIOR) && (L.col == 0);
    if (MODE != INTERIOR) {
        auto m = [&](int c) { return (c >= own_lo && c < own_hi) ? 1.f : 0.f; };
        auto g = [&](int c) { return c == W - 1 ? 0.f : 1.f; };
        L.mk.a = mk2(m(L.col), m(L.col + 1));
        L.mk.b = mk2(m(L.col + 2), m(L.col + 3));
        L.gmask.a = mk2(g(L.col), g(L.col + 1));
        L.gmask.b = mk2(g(L.col + 2), g(L.col + 3));
    }
    // columns outside the frame read as zeros (W % 4 == 0: all 4 or none)
    const uint32_t ldb = (L.col >= 0 && L.col < W) ? 16u : 0u;
    L.colc = min(max(L.col, 0), W - 4);
    const float *fb = P.f + (int64_t)frame * P.fs;
    float *ob = P.u + (int64_t)frame * P.fs;

    // the first PF input rows
#pragma unroll
    for (int q = 0; q < PF; ++q) {
        const int rp = min(rs + q, H - 1);
        cp16(ring_s + ((rs + q) & (RING - 1)) * ROWB, fb + (int64_t)rp * W + L.colc, ldb);
        cp_commit();
    }

    SS<S> A, B;
    zero_ss<S>(A);
    f2 ek[S];
#pragma unroll
    for (int k = 0; k < S; ++k) ek[k].v = 0ull;

    const int rlast = min(r1 - 1 + S, H - 1 + S);
    // fast steps: every stage inside [r0, r1), away from the frame's last row
    const int rfb = r0 + S;
    const int rfe = min(r1, H - 1);
    int r = rs;
    while (r <= rlast) {
        if (r == rfb && r + 1 <= rfe) {
            for (; r + 1 <= rfe; r += 2) {
                sstep<S, ENERGY, MODE, false>(P, A, B, r, rs, r0, r1, L, fb, ob, ring, ring_s, ldb,
                                              ek);
                sstep<S, ENERGY, MODE, false>(P, B, A, r + 1, rs, r0, r1, L, fb, ob, ring, ring_s,
                                              ldb, ek);
            }
            continue;
        }
        sstep<S, ENERGY, MODE, true>(P, A, B, r, rs, r0, r1, L, fb, ob, ring, ring_s, ldb, ek);
        A = B;
        ++r;
    }
    cp_wait_all();

    if (ENERGY) {
        const float lm = (MODE == INTERIOR) ? (L.lane_own ? 1.f : 0.f) : 1.f;
        double *eb = P.energy + (int64_t)frame * P.K * 2;
#pragma unroll
        for (int k = 0; k < S; ++k) {
            double v = (double)((lo(ek[k]) + hi(ek[k])) * lm);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
            if (lane == 0) atomicAdd(eb + 2 * (P.a + k), v);
        }
        if (lane == 0 && P.ticket) __threadfence();
    }
}

template <int S, bool ENERGY>
__device__ __forceinline__ void srun_mode(const Pass &P, int frame, int chunk, int band, int lane,
                                          const unsigned char *ring, uint32_t ring_s) {
    const int c0 = band * P.own - P.hl;
    if (c0 >= 0 && c0 + 127 <= P.W - 1)
        srun<S, ENERGY, INTERIOR>(P, frame, chunk, band, lane, ring, ring_s);
    else
        srun<S, ENERGY, EDGE>(P, frame, chunk, band, lane, ring, ring_s);
}

// Main launch of a single-pass run (n_iter_max = S + 1 <= 5, no p input):
// all S dual updates of every frame, and (with a ticket) the stop decision
// by the last work item, as k_tv_main.
// MINB: resident blocks per SM the registers are sized for (3: 168 registers
// per thread, 4: 128).
template <int S, int MINB>
__global__ void __launch_bounds__(WPB * 32, MINB) k_tv_slim(Pass P) {
    __shared__ __align__(16) unsigned char rings[WPB][RING * ROWB];
    int frame, chunk, band;
    if (!decode_item(P, frame, chunk, band)) return;
    const int lane = threadIdx.x & 31;
    const unsigned char *ring = &rings[threadIdx.x >> 5][lane * 16];
    srun_mode<S, true>(P, frame, chunk, band, lane, ring, smem_u32(ring));
    if (P.ticket) decide_stops(P, lane);
}

// Stop-test launch of a single-pass run: frames whose rule fired at step j
// are recomputed with j updates (as k_tv_fixup).
template <int MINB>
__global__ void __launch_bounds__(WPB * 32, MINB) k_tv_slim_fix(Pass P) {
    __shared__ __align__(16) unsigned char rings[WPB][RING * ROWB];
    int frame, chunk, band;
    if (!decode_item(P, frame, chunk, band)) return;
    const int j = P.stopj[frame];
    const int lane = threadIdx.x & 31;
    const bool lead = (chunk == 0 && band == 0 && lane == 0);
    if (j < 0) {
        if (lead && P.steps && P.S == P.K - 1) P.steps[frame] = P.K;
        return;
    }
    if (lead) {
        P.done[frame] = j;
        if (P.steps) P.steps[frame] = j + 1;
    }
    const unsigned char *ring = &rings[threadIdx.x >> 5][lane * 16];
    const uint32_t rs = smem_u32(ring);
    switch (j) {
        case 1: srun_mode<1, false>(P, frame, chunk, band, lane, ring, rs); break;
        case 2: srun_mode<2, false>(P, frame, chunk, band, lane, ring, rs); break;
        case 3: srun_mode<3, false>(P, frame, chunk, band, lane, ring, rs); break;
        default: break;
    }
}

}  // namespace slim


}  // namespace tv
}  // namespace sci
