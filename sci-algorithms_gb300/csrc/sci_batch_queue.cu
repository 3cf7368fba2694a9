// Batched uneven GAP-TV as persistent launches over a device work queue.
//
// One launch runs iterations [k0, k1) of every item of a batch.  Its tasks
// are numbered in a fixed order -- per iteration the residual tasks of all
// items (128-pixel tiles: the GAP residual map c, as the single-measurement
// solver's fused iteration forms it), then their TV tasks (one (frame, row
// chunk, column band) work item of the register-lean pipeline each, which
// applies the projection x + lam (c phi_b) as it loads x), then their
// stop-test tasks (the same work items) -- and the resident warps take the
// next number from an atomic counter until the launch's tasks are used up.
// A task waits only for tasks of its own item with smaller numbers:
//   projection of iteration k   after every stop-test task of k - 1,
//   TV pass of iteration k      after every projection task of k,
//   stop test of iteration k    after every TV task of k (whose last task
//                               decides the item's stop steps).
// Tasks are taken in number order by warps that are already running, so
// every task waited on is held by a running warp: the waits end without any
// assumption on how many blocks are resident.  An item whose projection is
// done starts its TV pass while other items still project; there is no
// grid-wide drain between the phases.  Per item, the per-pixel and per-tile
// arithmetic is that of the single-measurement solver (k_proj_gap_tma, the
// lean TV pass and its stop test), so each item's result is the same.
//
// Waits are bounded: a wait that gives up raises the launch's abort flag,
// every warp leaves at its next task, and sci_batch.cu folds the flag into
// the batch status word (bit 1).
#include "sci_batch.cuh"
#include "sci_tv_slim.cuh"

namespace sci {
namespace batch {

namespace {

constexpr int QMINB = 4;                    // resident blocks per SM the registers are sized for
enum { PH_PROJ = 0, PH_TV = 1, PH_FIX = 2 };

// The task's writes are visible before its count is.
__device__ __forceinline__ void finish(Queue *Q, int phase, int item, int lane) {
    __syncwarp();
    if (lane == 0) {
        __threadfence();
        atomicAdd(&Q->done[phase][item], 1u);
    }
}

__device__ __forceinline__ float bitf(uint32_t w, int b) { return ((w >> b) & 1u) ? 1.0f : 0.0f; }

// GAP residual map of one 128-pixel tile of item I (4 pixels per lane), the
// arithmetic of k_gap_resid_vec: yb = sum_b phi_b x_b in frame order, ACC:
// y1 += y - yb, c = (y1 - yb) / Phi_sum, else c = (y - yb) / Phi_sum, with
// x the iteration's TV input P.f.  Tile 0 also clears the energy sums the
// item's TV pass of this iteration adds to.
// x and y1 were written earlier in this launch by warps on other SMs: they
// are read at L2 (ld.global.cg), never through the non-coherent or L1
// caches, which may still hold the lines of an earlier iteration.
template <bool ACC>
__device__ __forceinline__ void resid_task(const Item &I, const tv::Pass &P, int tile, int lane) {
    if (tile == 0) {
        const int ne = P.nf * P.K * 2;
        for (int e = lane; e < ne; e += 32) P.energy[e] = 0.0;
    }
    const int64_t hw = I.hw;
    const int64_t p = (int64_t)tile * QP_T + lane * 4;
    if (p >= hw) return;  // hw % 4 == 0: all 4 pixels are inside
    const int B = I.B;
    const uint4 w = __ldg(reinterpret_cast<const uint4 *>(I.bits + p));
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 8
    for (int b = 0; b < B; ++b) {
        const float4 v = __ldcg(reinterpret_cast<const float4 *>(P.f + b * hw + p));
        s.x = fmaf(v.x, bitf(w.x, b), s.x);
        s.y = fmaf(v.y, bitf(w.y, b), s.y);
        s.z = fmaf(v.z, bitf(w.z, b), s.z);
        s.w = fmaf(v.w, bitf(w.w, b), s.w);
    }
    const float4 yv = ldg4(I.y + p), ps = ldg4(I.phisum + p);
    float4 r;
    if (ACC) {
        float4 tt = __ldcg(reinterpret_cast<const float4 *>(I.y1 + p));
        tt.x = tt.x + (yv.x - s.x);
        tt.y = tt.y + (yv.y - s.y);
        tt.z = tt.z + (yv.z - s.z);
        tt.w = tt.w + (yv.w - s.w);
        st4(I.y1 + p, tt);
        r = make_float4(__fdiv_rn(tt.x - s.x, ps.x), __fdiv_rn(tt.y - s.y, ps.y),
                        __fdiv_rn(tt.z - s.z, ps.z), __fdiv_rn(tt.w - s.w, ps.w));
    } else {
        r = make_float4(__fdiv_rn(yv.x - s.x, ps.x), __fdiv_rn(yv.y - s.y, ps.y),
                        __fdiv_rn(yv.z - s.z, ps.z), __fdiv_rn(yv.w - s.w, ps.w));
    }
    st4(I.c + p, r);
}

// The TV pass with S dual updates of one work item, or (FIX) its re-run with
// the stop index j the pass decided.
// N2: some item runs 2 columns per lane (otherwise that code is not built,
// which leaves the 4-column pipeline more registers).
template <int S, bool FIX, bool N2>
__device__ __forceinline__ void tv_task(const tv::Pass &P, int frame, int chunk, int band,
                                        int lane, const tv::slim::Rings &G4,
                                        const tv::slim::Rings &G2) {
    using namespace tv::slim;
    if (!FIX) {
        if (N2 && P.cpl == 2) srun_mode<S, 2, true, 1, 1, 1>(P, frame, chunk, band, lane, G2);
        else srun_mode<S, 4, true, 1, 1, 1>(P, frame, chunk, band, lane, G4);
        return;
    }
    const int j = __ldcg(P.stopj + frame);  // decided by another warp of this launch
    if (j < 1 || j >= S) return;
    switch (j) {
        case 1:
            if (N2 && P.cpl == 2) srun_mode<1, 2, false, 1, 1, 1>(P, frame, chunk, band, lane, G2);
            else srun_mode<1, 4, false, 1, 1, 1>(P, frame, chunk, band, lane, G4);
            break;
        case 2:
            if constexpr (S > 2) {
                if (N2 && P.cpl == 2) srun_mode<2, 2, false, 1, 1, 1>(P, frame, chunk, band, lane, G2);
                else srun_mode<2, 4, false, 1, 1, 1>(P, frame, chunk, band, lane, G4);
            }
            break;
        default:
            if constexpr (S > 3) {
                if (N2 && P.cpl == 2) srun_mode<3, 2, false, 1, 1, 1>(P, frame, chunk, band, lane, G2);
                else srun_mode<3, 4, false, 1, 1, 1>(P, frame, chunk, band, lane, G4);
            }
            break;
    }
}

// The persistent worker loop: S = tv_iter_max - 1 dual updates per TV pass.
template <int S, bool ACC, bool N2 = true>
__global__ void __launch_bounds__(tv::WPB * 32, QMINB)
    k_batch_queue(const Table *__restrict__ T, Queue *__restrict__ Q, int k0, int k1) {
    __shared__ __align__(16) unsigned char smem[tv::slim::Smem<4, 1>::bytes];
    const int lane = threadIdx.x & 31;
    // each warp's share holds its three 4-column rings (x, map, mask); the
    // 2-column rings use the first half of the same share
    constexpr int share = tv::slim::Smem<4, 1>::bytes / tv::WPB;
    const tv::slim::Rings G4 = tv::slim::lane_rings<4, 1>(smem, lane, share);
    const tv::slim::Rings G2 = tv::slim::lane_rings<2, 1>(smem, lane, share);
    const int n = T->n;
    const unsigned np = (unsigned)T->qp_prefix[n], nt = (unsigned)T->tq_prefix[n];
    const unsigned span = np + 2u * nt;
    const unsigned total = span * (unsigned)(k1 - k0);
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&Q->next, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= total) return;
        const unsigned j = t / span;  // iteration within the launch
        const unsigned rem = t - j * span;
        const int k = k0 + (int)j;
        if (rem < np) {
            const int i = find_item(T->qp_prefix, n, (int)rem);
            const unsigned ntv = (unsigned)(T->tq_prefix[i + 1] - T->tq_prefix[i]);
            if (j > 0 && !wait_count(Q, &Q->done[PH_FIX][i], j * ntv, lane)) return;
            resid_task<ACC>(T->it[i], T->it[i].tvq[k & 1], (int)rem - T->qp_prefix[i], lane);
            finish(Q, PH_PROJ, i, lane);
            continue;
        }
        const bool fix = rem >= np + nt;
        const int g = (int)(rem - np - (fix ? nt : 0u));
        const int i = find_item(T->tq_prefix, n, g);
        const unsigned need =
            fix ? (j + 1) * (unsigned)(T->tq_prefix[i + 1] - T->tq_prefix[i])
                : (j + 1) * (unsigned)(T->qp_prefix[i + 1] - T->qp_prefix[i]);
        if (!wait_count(Q, &Q->done[fix ? PH_TV : PH_PROJ][i], need, lane)) return;
        const tv::Pass &P = T->it[i].tvq[k & 1];
        int frame, chunk, band;
        tv::decode_index(P, g - T->tq_prefix[i], frame, chunk, band);
        if (!fix) {
            tv_task<S, false, N2>(P, frame, chunk, band, lane, G4, G2);
            tv::decide_stops(P, lane);
        } else {
            tv_task<S, true, N2>(P, frame, chunk, band, lane, G4, G2);
        }
        finish(Q, fix ? PH_FIX : PH_TV, i, lane);
    }
}

template <int S, bool ACC>
const void *kernel_ptr() {
    return reinterpret_cast<const void *>(&k_batch_queue<S, ACC>);
}

}  // namespace

int queue_blocks() {
    static int v = 0;
    if (v == 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel_ptr<4, true>(),
                                                          tv::WPB * 32, 0) != cudaSuccess ||
            per_sm <= 0) {
            cudaGetLastError();
            per_sm = QMINB;
        }
        v = per_sm * kSMs;
    }
    return v;
}

int queue_launch(const Table *dT, Queue *dQ, int k0, int k1, bool accelerate, int S, int blocks,
                 bool narrow, cudaStream_t s) {
#define SCI_QUEUE_CASE(SV)                                                                 \
    case SV:                                                                               \
        if (accelerate) k_batch_queue<SV, true><<<blocks, tv::WPB * 32, 0, s>>>(dT, dQ, k0, k1); \
        else k_batch_queue<SV, false><<<blocks, tv::WPB * 32, 0, s>>>(dT, dQ, k0, k1);     \
        break;
    switch (S) {
        SCI_QUEUE_CASE(1)
        SCI_QUEUE_CASE(2)
        SCI_QUEUE_CASE(3)
        default:  // n_iter_max 5: without the 2-column code when no item needs it
            if (narrow) {
                if (accelerate) k_batch_queue<4, true><<<blocks, tv::WPB * 32, 0, s>>>(dT, dQ, k0, k1);
                else k_batch_queue<4, false><<<blocks, tv::WPB * 32, 0, s>>>(dT, dQ, k0, k1);
            } else {
                if (accelerate)
                    k_batch_queue<4, true, false><<<blocks, tv::WPB * 32, 0, s>>>(dT, dQ, k0, k1);
                else
                    k_batch_queue<4, false, false><<<blocks, tv::WPB * 32, 0, s>>>(dT, dQ, k0, k1);
            }
            break;
    }
#undef SCI_QUEUE_CASE
    SCI_LAUNCHED("k_batch_queue");
    return SCI_OK;
}

}  // namespace batch
}  // namespace sci
