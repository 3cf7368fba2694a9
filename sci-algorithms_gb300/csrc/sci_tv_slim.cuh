// Chambolle TV pass, register-lean form of the row pipeline (sci_tv.cuh).
//
// Same mapping and the same arithmetic, operation for operation, as the
// generic pipeline's scikit-image rule without a p input (one pass of
// n_iter_max <= 5 steps): a warp owns a band of 32 * CPL columns of one
// frame (CPL = 2 or 4 columns per lane) and marches down a chunk of rows;
// stage k computes p_k and u_k of row r - k when input row r arrives.  What
// differs is where the values live:
//
//  * f rows.  Stage k needs f(r - k).  The generic pipeline hands f down the
//    stages in registers (4 CPL registers and their copies every step); here
//    every input row is copied by cp.async into a per-warp ring of RING rows
//    in shared memory, PF rows ahead of its use, and each stage reads its f
//    row back from the ring (a lane reads only the bytes it copied itself,
//    so the per-thread cp.async.wait_group is the only synchronisation).
//    Stage 1 takes f(r - 1) = u_0(r - 1) from the state it already holds.
//  * shifted neighbours.  The one-column shifts of the forward column
//    difference and of the divergence pair values across f32x2 register
//    pairs; they are computed as scalar FP32 operations whose results land in
//    fresh pairs, instead of re-pairing shifted halves with moves.
//
// With PROJ the GAP projection is applied as the input is loaded: the
// stored stack holds x, and f = x + lam (c phi_b) with c the per-pixel
// residual map and phi_b bit `frame` of the packed mask word; the map and
// mask rows come through two more rings, and stage 0 writes f back into the
// input ring for the later stages.  PROJ 3 is PROJ 1 that also stores
// t = u + (u - f) beside u (P.tout): in the ADMM iteration f is the TV
// input v = x - b and u the new theta, so t = theta + b of the next
// projection.
//
// Rounding is identical to the generic pipeline (same operations in the same
// order), so the two produce bit-identical frames.
#pragma once

#include "sci_tv.cuh"

namespace sci {
namespace tv {
namespace slim {

constexpr int RING = 8;              // rows per warp in each shared-memory ring (power of 2)
constexpr int PF = 3;                // rows copied ahead of the step that reads them
static_assert(RING >= SMAX + 1 + PF, "ring too small for the pipeline depth");

template <int CPL>
struct Geo {
    static constexpr int LB = 4 * CPL;     // bytes of one row of a lane
    static constexpr int ROWB = 32 * LB;   // bytes of one band row
    static constexpr int NQ = CPL / 2;     // packed pairs per lane
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Asynchronous copy of one lane's row segment global -> shared; bytes = 0
// fills zeros.
template <int CPL>
__device__ __forceinline__ void cp_row(uint32_t dst, const void *src, uint32_t bytes) {
    if (CPL == 4)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
                     "r"(bytes)
                     : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src),
                     "r"(bytes)
                     : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <int CPL>
__device__ __forceinline__ Row<CPL> lds(const unsigned char *ring, int row) {
    const unsigned char *p = ring + (row & (RING - 1)) * Geo<CPL>::ROWB;
    Row<CPL> r;
    if (CPL == 4) {
        const ulonglong2 t = *reinterpret_cast<const ulonglong2 *>(p);
        r.q[0].v = t.x;
        r.q[CPL / 2 - 1].v = t.y;
    } else {
        r.q[0].v = *reinterpret_cast<const unsigned long long *>(p);
    }
    return r;
}

template <int CPL>
__device__ __forceinline__ void sts(unsigned char *ring, int row, const Row<CPL> &v) {
    unsigned char *p = ring + (row & (RING - 1)) * Geo<CPL>::ROWB;
    if (CPL == 4) {
        ulonglong2 t;
        t.x = v.q[0].v;
        t.y = v.q[CPL / 2 - 1].v;
        *reinterpret_cast<ulonglong2 *>(p) = t;
    } else {
        *reinterpret_cast<unsigned long long *>(p) = v.q[0].v;
    }
}

// Pipeline state between steps (no p input: p_0 = 0, u_0 = f).
template <int S, int CPL>
struct SS {
    Row<CPL> up[S];      // up[k]: u_k of the row stage k+1 handles next step
    Row<CPL> pr[S + 1];  // pr[k] (k >= 1): p_k (row component) of the row stage k handled last
    Row<CPL> pc[S];      // pc[k] (1 <= k < S): p_k (column component), same row
};

template <int S, int CPL>
__device__ __forceinline__ void zero_ss(SS<S, CPL> &A) {
#pragma unroll
    for (int k = 0; k < S; ++k) {
        A.up[k] = zrow<CPL>();
        A.pc[k] = zrow<CPL>();
    }
#pragma unroll
    for (int k = 0; k <= S; ++k) A.pr[k] = zrow<CPL>();
}

// Per-lane constants of a band.
template <int CPL>
struct SLane {
    int col;            // first column of this lane
    int colc;           // col clamped into [0, W - CPL] (the address of a zero-filled copy)
    bool lane_own;      // the band owns all CPL columns of the lane
    bool first_col;     // the lane holds column 0
    Row<CPL> mk;        // 1 for owned columns (edge bands)
    Row<CPL> gmask;     // 0 at column W-1 (edge bands)
};

// Shared-memory rings of one lane: x (then f), and with PROJ the residual
// map and the packed mask words.
struct Rings {
    unsigned char *x;
    const unsigned char *c, *m;
    uint32_t xs, cs, ms;  // shared-space addresses
};

// Copies input row `row` into ring slot `slot` of every ring of the lane.
// COH (coherent): the rows may have been written earlier in the same launch
// by other SMs, so every copy goes through L2 only (cp.async.cg): with 2
// columns per lane the even lane of each pair copies both lanes' 16 bytes
// (ldb: the pair's bytes inside the frame) and sstep synchronises the warp.
template <int CPL, int PROJ, int COH = 0>
__device__ __forceinline__ void fetch(const Pass &P, const Rings &G, const float *fb, int slot,
                                      int row, int colc, uint32_t ldb) {
    const int64_t o = (int64_t)row * P.W + colc;
    const uint32_t so = (uint32_t)(slot & (RING - 1)) * Geo<CPL>::ROWB;
    if (COH && CPL == 2) {
        if ((threadIdx.x & 1) == 0) {
            cp_row<4>(G.xs + so, fb + o, ldb);
            if (PROJ) {
                cp_row<4>(G.cs + so, P.cmap + o, ldb);
                cp_row<4>(G.ms + so, P.bits + o, ldb);
            }
        }
    } else {
        cp_row<CPL>(G.xs + so, fb + o, ldb);
        if (PROJ) {
            cp_row<CPL>(G.cs + so, P.cmap + o, ldb);
            cp_row<CPL>(G.ms + so, P.bits + o, ldb);
        }
    }
    cp_commit();
}

// Stage 0 of step r: u_0 = f at row r from the input ring (with PROJ the
// projection applied, and f written back for the later stages).
template <int CPL, int PROJ>
__device__ __forceinline__ Row<CPL> stage0(const Pass &P, const Rings &G, int r, int frame) {
    constexpr int NQ = Geo<CPL>::NQ;
    Row<CPL> u = lds<CPL>(G.x, r);
    if (PROJ) {  // f = x + lam (c phi_b), as the GAP projection rounds it
        const Row<CPL> c = lds<CPL>(G.c, r);
        const Row<CPL> wb = lds<CPL>(G.m, r);
        const uint32_t fbit = 1u << frame;
#pragma unroll
        for (int j = 0; j < NQ; ++j)
            u.q[j] = mk2(proj_px(P.lam, lo(c.q[j]), lo(u.q[j]), __float_as_uint(lo(wb.q[j])), fbit),
                         proj_px(P.lam, hi(c.q[j]), hi(u.q[j]), __float_as_uint(hi(wb.q[j])), fbit));
        sts<CPL>(G.x, r, u);
    }
    return u;
}

// Stage k of step r (row i = r - k): p_k and u_k of row i from stage k-1's
// rows i (in.up[k-1], held since the last step) and i+1 (ucur, this step);
// ucur becomes u_k(i).  GEN: rows may lie outside [r0, r1) or touch the
// frame's last row.
//
// FORM 1 (the default) holds the dual field as 4 p (a power-of-two scaling,
// so every rounding is that of FORM 0 scaled): p' = (4p - g) / den needs no
// tau product, u = f - d / 4 takes it once per pixel instead, and the energy
// sums are accumulated 16-fold (their w |grad u| term with 16 w).  FORM 0
// holds p itself.
template <int S, int K, int CPL, bool ENERGY, int MODE, bool GEN, int FORM = 1, bool TOUT = false>
__device__ __forceinline__ void stage(const Pass &P, const SS<S, CPL> &in, SS<S, CPL> &out,
                                      Row<CPL> &ucur, int r, int rs, int r0, int r1,
                                      const SLane<CPL> &L, float *ob, const Rings &G,
                                      f2 (&ek)[S]) {
    constexpr int NQ = Geo<CPL>::NQ;
    const int H = P.H, W = P.W;
    const f2 one2 = mk2(1.f, 1.f), tw2 = mk2(P.tw, P.tw);
    const f2 nt2 = FORM ? mk2(-0.25f, -0.25f) : mk2(-P.tau, -P.tau);
    const f2 w2 = FORM ? mk2(16.f * P.weight, 16.f * P.weight) : mk2(P.weight, P.weight);
    const int i = r - K;
    out.up[K - 1] = ucur;  // u_{K-1}(i+1): stage K's row in the next step
    if (GEN && !(i >= rs && i < H)) {  // warp-uniform
        out.pr[K] = zrow<CPL>();
        if (K < S) out.pc[K] = zrow<CPL>();
        ucur = zrow<CPL>();
        return;
    }
    const Row<CPL> &up = in.up[K - 1];  // u_{K-1}(i)
    // f(i): u_0(i) for stage 1, else the ring
    const Row<CPL> fi = (K == 1) ? up : lds<CPL>(G.x, i);
    const float uR = __shfl_down_sync(FULL, lo(up.q[0]), 1);
    Row<CPL> gc, gr, n, prn, pcn, d, uk;
#pragma unroll
    for (int j = 0; j < NQ; ++j) {
        // forward column difference (one-column shift: scalar)
        const float nx = (j + 1 < NQ) ? lo(up.q[(j + 1) % NQ]) : uR;
        gc.q[j] = mk2(hi(up.q[j]) - lo(up.q[j]), nx - hi(up.q[j]));
        if (MODE != INTERIOR) gc.q[j] = mul2(gc.q[j], L.gmask.q[j]);
        gr.q[j] = (GEN && i == H - 1) ? mk2(0.f, 0.f) : sub2(ucur.q[j], up.q[j]);
        const f2 s = fma2(gr.q[j], gr.q[j], mul2(gc.q[j], gc.q[j]));
        n.q[j] = mk2(sqrt_approx(lo(s)), sqrt_approx(hi(s)));
        const f2 den = fma2(tw2, n.q[j], one2);
        const f2 ri = mk2(rcp_approx(lo(den)), rcp_approx(hi(den)));
        if (FORM) {  // 4 p
            if (K == 1) {
                prn.q[j] = mul2(sub2(mk2(0.f, 0.f), gr.q[j]), ri);
                pcn.q[j] = mul2(sub2(mk2(0.f, 0.f), gc.q[j]), ri);
            } else {
                prn.q[j] = mul2(sub2(in.pr[K - 1].q[j], gr.q[j]), ri);
                pcn.q[j] = mul2(sub2(in.pc[K - 1].q[j], gc.q[j]), ri);
            }
        } else if (K == 1) {  // p_0 = 0: (0 - tau g) rounds as the product
            prn.q[j] = mul2(mul2(nt2, gr.q[j]), ri);
            pcn.q[j] = mul2(mul2(nt2, gc.q[j]), ri);
        } else {
            prn.q[j] = mul2(fma2(nt2, gr.q[j], in.pr[K - 1].q[j]), ri);
            pcn.q[j] = mul2(fma2(nt2, gc.q[j], in.pc[K - 1].q[j]), ri);
        }
    }
    // divergence ((pr + pc) - pr_up) - pc_left, the left shift in scalar
    float pcl = __shfl_up_sync(FULL, hi(pcn.q[NQ - 1]), 1);
    if (MODE != INTERIOR && L.first_col) pcl = 0.f;
#pragma unroll
    for (int j = 0; j < NQ; ++j) {
        const f2 t = sub2(add2(prn.q[j], pcn.q[j]), in.pr[K].q[j]);
        const float left = (j == 0) ? pcl : hi(pcn.q[(j + NQ - 1) % NQ]);
        d.q[j] = mk2(lo(t) - left, hi(t) - lo(pcn.q[j]));
        uk.q[j] = FORM ? fma2(nt2, d.q[j], fi.q[j]) : sub2(fi.q[j], d.q[j]);
    }
    out.pr[K] = prn;
    if (K < S) out.pc[K] = pcn;
    if (ENERGY && (!GEN || (i >= r0 && i < r1))) {
#pragma unroll
        for (int j = 0; j < NQ; ++j) {
            if (MODE == INTERIOR) {
                ek[K - 1] = fma2(w2, n.q[j], ek[K - 1]);
                if (K < S) ek[K] = fma2(d.q[j], d.q[j], ek[K]);
            } else {
                ek[K - 1] = fma2(mul2(w2, L.mk.q[j]), n.q[j], ek[K - 1]);
                if (K < S) ek[K] = fma2(mul2(L.mk.q[j], d.q[j]), d.q[j], ek[K]);
            }
        }
    }
    if (K == S && (!GEN || (i >= r0 && i < r1)) && L.lane_own) {
        vstore<CPL>(ob + (int64_t)i * W + L.col, uk);
        if (TOUT) {  // t = u + (u - f), the ADMM iterate theta + b of the next residual
            Row<CPL> t;
#pragma unroll
            for (int j = 0; j < NQ; ++j) t.q[j] = add2(uk.q[j], sub2(uk.q[j], fi.q[j]));
            vstore<CPL>(P.tout + (ob - P.u) + (int64_t)i * W + L.col, t);
        }
    }
    ucur = uk;
}

// Stages K..S of one step, in order.
template <int S, int K, int CPL, bool ENERGY, int MODE, bool GEN, int FORM, bool TOUT = false>
__device__ __forceinline__ void stages(const Pass &P, const SS<S, CPL> &in, SS<S, CPL> &out,
                                       Row<CPL> &ucur, int r, int rs, int r0, int r1,
                                       const SLane<CPL> &L, float *ob, const Rings &G,
                                       f2 (&ek)[S]) {
    if constexpr (K <= S) {
        stage<S, K, CPL, ENERGY, MODE, GEN, FORM, TOUT>(P, in, out, ucur, r, rs, r0, r1, L, ob, G,
                                                        ek);
        stages<S, K + 1, CPL, ENERGY, MODE, GEN, FORM, TOUT>(P, in, out, ucur, r, rs, r0, r1, L, ob, G,
                                                       ek);
    }
}

// One pipeline step: input row r enters, stage k handles row r - k.
template <int S, int CPL, bool ENERGY, int MODE, bool GEN, int PROJ, int FORM = 1, int COH = 0>
__device__ __forceinline__ void sstep(const Pass &P, const SS<S, CPL> &in, SS<S, CPL> &out,
                                      int r, int rs, int r0, int r1, const SLane<CPL> &L,
                                      const float *fb, float *ob, const Rings &G, uint32_t ldb,
                                      int frame, f2 (&ek)[S]) {
    // copy input row r + PF into its ring slots (clamped into the frame; a
    // clamped row is never read), then wait for row r
    fetch<CPL, PROJ, COH>(P, G, fb, r + PF, min(r + PF, P.H - 1), L.colc, ldb);
    cp_wait<PF>();
    if (COH && CPL == 2) __syncwarp();  // the pair's copy was the even lane's
    Row<CPL> ucur = (!GEN || r < P.H) ? stage0<CPL, PROJ>(P, G, r, frame) : zrow<CPL>();
    stages<S, 1, CPL, ENERGY, MODE, GEN, FORM, PROJ == 3>(P, in, out, ucur, r, rs, r0, r1, L, ob, G,
                                                        ek);
}

// One work item: frame, row chunk, column band.  Requires rows aligned for
// CPL-wide access (W % CPL == 0, base pointers aligned to 4 CPL bytes).
template <int S, int CPL, bool ENERGY, int MODE, int PROJ, int FORM = 1, int COH = 0>
__device__ __forceinline__ void srun(const Pass &P, int frame, int chunk, int band, int lane,
                                     const Rings &G) {
    const int H = P.H, W = P.W;
    SLane<CPL> L;
    int c0, own_lo, own_hi;
    band_window(P, band, 32 * CPL, c0, own_lo, own_hi);
    L.col = c0 + lane * CPL;
    const int r0 = chunk * P.R, r1 = min(r0 + P.R, H);
    const int rs = max(0, r0 - P.ht);
    L.lane_own = (L.col >= own_lo) && (L.col + CPL <= own_hi);
    L.first_col = (MODE != INTERIOR) && (L.col == 0);
    if (MODE != INTERIOR) {
#pragma unroll
        for (int j = 0; j < CPL / 2; ++j) {
            const int c = L.col + 2 * j;
            L.mk.q[j] = mk2((c >= own_lo && c < own_hi) ? 1.f : 0.f,
                            (c + 1 >= own_lo && c + 1 < own_hi) ? 1.f : 0.f);
            L.gmask.q[j] = mk2(c == W - 1 ? 0.f : 1.f, c + 1 == W - 1 ? 0.f : 1.f);
        }
    }
    // columns outside the frame read as zeros (W % CPL == 0: all or none)
    uint32_t ldb = (L.col >= 0 && L.col < W) ? 4u * CPL : 0u;
    L.colc = min(max(L.col, 0), W - CPL);
    if (COH && CPL == 2) {  // a coherent pair copy: the pair's columns inside the frame
        ldb = (L.col >= 0 && L.col < W) ? 4u * (uint32_t)min(4, W - L.col) : 0u;
        L.colc = min(max(L.col, 0), W - 4);
    }
    const float *fb = P.f + (int64_t)frame * P.fs;
    float *ob = P.u + (int64_t)frame * P.fs;

    // the first PF input rows
#pragma unroll
    for (int q = 0; q < PF; ++q)
        fetch<CPL, PROJ, COH>(P, G, fb, rs + q, min(rs + q, H - 1), L.colc, ldb);

    SS<S, CPL> A, B;
    zero_ss<S, CPL>(A);
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
                sstep<S, CPL, ENERGY, MODE, false, PROJ, FORM, COH>(P, A, B, r, rs, r0, r1, L, fb, ob, G,
                                                         ldb, frame, ek);
                sstep<S, CPL, ENERGY, MODE, false, PROJ, FORM, COH>(P, B, A, r + 1, rs, r0, r1, L, fb, ob,
                                                         G, ldb, frame, ek);
            }
            continue;
        }
        sstep<S, CPL, ENERGY, MODE, true, PROJ, FORM, COH>(P, A, B, r, rs, r0, r1, L, fb, ob, G, ldb, frame,
                                                ek);
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
            if (FORM) v *= 0.0625;  // the sums were accumulated 16-fold
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
            if (lane == 0) atomicAdd(eb + 2 * (P.a + k), v);
        }
        if (lane == 0 && P.ticket) __threadfence();
    }
}

template <int S, int CPL, bool ENERGY, int PROJ, int FORM = 1, int COH = 0>
__device__ __forceinline__ void srun_mode(const Pass &P, int frame, int chunk, int band, int lane,
                                          const Rings &G) {
    int c0, lo, hi;
    band_window(P, band, 32 * CPL, c0, lo, hi);
    if (band_interior(P, c0, 32 * CPL))
        srun<S, CPL, ENERGY, INTERIOR, PROJ, FORM, COH>(P, frame, chunk, band, lane, G);
    else
        srun<S, CPL, ENERGY, EDGE, PROJ, FORM, COH>(P, frame, chunk, band, lane, G);
}

// Shared memory of a block: RING rows per warp per ring (one ring, three
// with PROJ).
template <int CPL, int PROJ>
struct Smem {
    static constexpr int bytes = WPB * RING * Geo<CPL>::ROWB * (PROJ ? 3 : 1);
};

// The rings of one lane: warp w's rings start at w * warp_bytes (by default
// its own share of Smem<CPL, PROJ>; a kernel that runs both column widths
// passes the larger share, so that a warp's rings never reach another's).
template <int CPL, int PROJ>
__device__ __forceinline__ Rings lane_rings(unsigned char *smem, int lane, int warp_bytes = 0) {
    constexpr int per = RING * Geo<CPL>::ROWB;  // one ring of one warp
    const int w = threadIdx.x >> 5;
    if (warp_bytes == 0) warp_bytes = (PROJ ? 3 : 1) * per;
    Rings G;
    G.x = smem + w * warp_bytes + lane * Geo<CPL>::LB;
    G.c = PROJ ? G.x + per : G.x;
    G.m = PROJ ? G.x + 2 * per : G.x;
    G.xs = smem_u32(G.x);
    G.cs = smem_u32(G.c);
    G.ms = smem_u32(G.m);
    return G;
}

// Main launch of a single-pass run (n_iter_max = S + 1 <= 5, no p input):
// all S dual updates of every frame, and (with a ticket) the stop decision
// by the last work item, as k_tv_main.  MINB: resident blocks per SM the
// registers are sized for.
template <int S, int CPL, int MINB, int PROJ, int FORM = 1>
__global__ void __launch_bounds__(WPB * 32, MINB) k_tv_slim(Pass P) {
    __shared__ __align__(16) unsigned char smem[Smem<CPL, PROJ>::bytes];
    grid_dep_wait();
    int frame, chunk, band;
    if (!decode_item(P, frame, chunk, band)) return;
    const int lane = threadIdx.x & 31;
    srun_mode<S, CPL, true, PROJ, FORM>(P, frame, chunk, band, lane,
                                        lane_rings<CPL, PROJ>(smem, lane));
    if (P.ticket) decide_stops(P, lane);
}

// Stop-test launch of a single-pass run: frames whose rule fired at step j
// are recomputed with j updates (as k_tv_fixup).
template <int CPL, int MINB, int PROJ>
__global__ void __launch_bounds__(WPB * 32, MINB) k_tv_slim_fix(Pass P) {
    __shared__ __align__(16) unsigned char smem[Smem<CPL, PROJ>::bytes];
    grid_dep_wait();
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
    const Rings G = lane_rings<CPL, PROJ>(smem, lane);
    switch (j) {
        case 1: srun_mode<1, CPL, false, PROJ>(P, frame, chunk, band, lane, G); break;
        case 2: srun_mode<2, CPL, false, PROJ>(P, frame, chunk, band, lane, G); break;
        case 3: srun_mode<3, CPL, false, PROJ>(P, frame, chunk, band, lane, G); break;
        default: break;
    }
}

}  // namespace slim
}  // namespace tv
}  // namespace sci
