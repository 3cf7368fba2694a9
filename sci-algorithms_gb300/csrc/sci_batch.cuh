// Device item table of the batched uneven GAP-TV (sci_batch.cu: per-phase
// launches, autotuner and C ABI; sci_batch_queue.cu: the persistent
// work-queue launch).
#pragma once

#include "sci_tv.cuh"

namespace sci {
namespace batch {

constexpr int MAXI = 256;    // items per batch
constexpr int PROJ_T = 256;  // pixels per projection tile of the per-phase launches
constexpr int QP_T = 128;    // pixels per projection task of the work queue (one warp)

struct Item {
    tv::Pass tv;      // per-phase launches: f = xp (projected stack), u = x
    tv::Pass tvq[2];  // work queue, iterations of even / odd k: the lean pass with
                      // the projection applied on load from the residual map c,
                      // the stack ping-ponging x -> xp (even k) and xp -> x (odd
                      // k), the energies of even / odd k, the item's stop decisions
    const float *y;
    const uint32_t *bits;
    const float *phisum;
    float *x, *xp, *y1, *c;  // c: the work queue's residual map (H W)
    int B;
    int64_t hw;
    float lam;
};

struct Table {
    int n;
    int proj_prefix[MAXI + 1];  // 256-pixel tiles
    int qp_prefix[MAXI + 1];    // 128-pixel projection tasks of the work queue
    int tv_prefix[MAXI + 1];    // TV work items (one warp each) of the per-phase launches
    int tq_prefix[MAXI + 1];    // TV work items of the work queue (tvq geometry)
    Item it[MAXI];
};

// Progress of one persistent launch (zeroed before it): the task counter,
// the give-up flag of the bounded waits and per item the finished tasks of
// each phase (projection, TV pass, stop test) since the launch began.
struct Queue {
    unsigned next;
    unsigned abort;
    unsigned done[3][MAXI];
};

constexpr unsigned kWaitPolls = 1u << 22;  // polls of at most ~1 us each: a few seconds

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Lane 0 of a warp waits until *cnt >= target, at most `polls` polls with
// a growing sleep between them; false (the launch's abort flag raised) when
// the wait gave up or another warp's wait had.
__device__ __forceinline__ bool wait_count(Queue *Q, const unsigned *cnt, unsigned target,
                                           int lane, unsigned polls = kWaitPolls) {
    int ok = 1;
    if (lane == 0) {
        unsigned n = 0, ns = 32;
        while (ld_acquire(cnt) < target) {
            if (ld_acquire(&Q->abort) != 0u || ++n > polls) {
                atomicExch(&Q->abort, 1u);
                ok = 0;
                break;
            }
            __nanosleep(ns);
            if (ns < 1024) ns <<= 1;
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    // the lanes' loads after the wait are ordered after lane 0's acquire
    __syncwarp();
    return ok != 0;
}

__device__ __forceinline__ int find_item(const int *prefix, int n, int g) {
    int lo = 0, hi = n;  // prefix[lo] <= g < prefix[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (prefix[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// sci_batch_queue.cu: iterations [k0, k1) of every item in one persistent
// launch over a device work queue.  Returns a negative status on a launch
// error.
int queue_launch(const Table *dT, Queue *dQ, int k0, int k1, bool accelerate, int S, int blocks,
                 bool narrow, cudaStream_t s);  // narrow: some item runs 2 columns per lane
int queue_blocks();  // resident blocks of the persistent kernel (whole GPU)

}  // namespace batch
}  // namespace sci
