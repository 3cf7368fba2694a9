// Batched GAP-TV over many measurements of uneven sizes.
//
// The reference reconstructs coded-frame blocks one after another
// (admmdenoise_cacti's frame-block loop, PnP_SCI/python/pnp_sci_algo.py:498);
// here a batch of independent measurements (each with its own H x W x B and
// packed binary mask) advances together.  Every phase of an iteration is
// one launch over a work queue spanning all items: the GAP projection over
// 256-pixel tiles of every item, then the Chambolle TV pass over every
// item's (frame, row chunk, column band) tiles, then the stop-test launch
// over the same tiles.  Items are found from the tile index through prefix
// tables in a device-resident item table.  The whole multi-iteration loop is
// captured once into a CUDA graph and replayed.  An autotuner times the TV
// row-chunk height per distinct frame shape on the item's own data.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "sci_bulk.cuh"
#include "sci_graph.cuh"
#include "sci_batch.cuh"
#include "sci_tv.cuh"

namespace sci {

// bit 0: a bounded bulk-copy wait of the batched projection gave up
__device__ unsigned int g_batch_status;

int tv_launch(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
              int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
              void *workspace, size_t ws_bytes, cudaStream_t s, int force_R);
size_t tv_workspace_bytes(int64_t nf, int64_t H, int64_t W, int K);

namespace batch {

// x0 = At(y / Phi_sum) for every item (the start point of the GAP loop).
// Start of a solve, one pass over every item's pixels: X0, x = At(y /
// Phi_sum); Y1, the accelerated GAP's y1 = 0 (one launch instead of a
// memset node per item).
template <bool X0, bool Y1>
__global__ void __launch_bounds__(PROJ_T) k_batch_init(const Table *__restrict__ T) {
    const int g = blockIdx.x;
    if (g >= T->proj_prefix[T->n]) return;
    const int i = find_item(T->proj_prefix, T->n, g);
    const Item &I = T->it[i];
    const int64_t p = (int64_t)(g - T->proj_prefix[i]) * PROJ_T + threadIdx.x;
    if (p >= I.hw) return;
    if (Y1) I.y1[p] = 0.f;
    if (X0) {
        const uint32_t w = I.bits[p];
        const float s0 = I.y[p] / I.phisum[p];
        for (int b = 0; b < I.B; ++b) I.x[b * I.hw + p] = ((w >> b) & 1u) ? s0 : 0.f * s0;
    }
}

// GAP projection (acc: y1 += y - A x, x_p = x + lam At((y1 - A x)/Phi_sum)).
template <bool ACC>
__global__ void __launch_bounds__(PROJ_T) k_batch_proj(const Table *__restrict__ T) {
    __shared__ float xs[32 * PROJ_T];
    const int g = blockIdx.x;
    if (g >= T->proj_prefix[T->n]) return;
    const int i = find_item(T->proj_prefix, T->n, g);
    const Item &I = T->it[i];
    const int t = threadIdx.x;
    const int64_t p = (int64_t)(g - T->proj_prefix[i]) * PROJ_T + t;
    if (p >= I.hw) return;
    const int64_t hw = I.hw;
    const int B = I.B;
    const uint32_t w = __ldg(I.bits + p);
    float s = 0.f;
    for (int b = 0; b < B; ++b) {
        const float v = __ldg(I.x + b * hw + p);
        xs[b * PROJ_T + t] = v;
        s = fmaf(v, ((w >> b) & 1u) ? 1.f : 0.f, s);
    }
    const float yv = __ldg(I.y + p), ps = __ldg(I.phisum + p);
    float r;
    if (ACC) {
        const float tt = I.y1[p] + (yv - s);
        I.y1[p] = tt;
        r = __fdiv_rn(tt - s, ps);
    } else {
        r = __fdiv_rn(yv - s, ps);
    }
    for (int b = 0; b < B; ++b) {
        const float m = ((w >> b) & 1u) ? 1.f : 0.f;
        __stcs(I.xp + b * hw + p, fmaf(I.lam, r * m, xs[b * PROJ_T + t]));
    }
}

// The same projection with the tile's B rows of 256 floats staged by bulk
// copies (one mbarrier, 64 threads x 4 pixels); the default for items whose
// planes are 16-byte aligned with hw % 4 == 0 (all items of a batch, see
// check()).  Same arithmetic, bit-identical results.
template <bool ACC>
__global__ void __launch_bounds__(PROJ_T / 4) k_batch_proj_tma(const Table *__restrict__ T) {
    extern __shared__ __align__(128) float xs[];  // [B][PROJ_T]
    __shared__ __align__(8) uint64_t bar;
    const int g = blockIdx.x;
    if (g >= T->proj_prefix[T->n]) return;
    const int i = find_item(T->proj_prefix, T->n, g);
    const Item &I = T->it[i];
    const int64_t hw = I.hw;
    const int B = I.B;
    const int64_t p0 = (int64_t)(g - T->proj_prefix[i]) * PROJ_T;
    const unsigned n = (unsigned)(hw - p0 < PROJ_T ? hw - p0 : PROJ_T);
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&bar, (unsigned)B * n * 4u);
        for (int b = 0; b < B; ++b) bulk_g2s(xs + b * PROJ_T, I.x + b * hw + p0, n * 4u, &bar);
    }
    __syncthreads();  // the barrier is initialised before anyone waits on it
    const bool ok = mbar_wait(&bar, 0);
    if (__syncthreads_or(!ok)) {
        if (tid == 0) {
            atomicOr(&g_batch_status, 1u);
            mbar_wait(&bar, 0);  // let the copies land before the block ends
        }
        return;
    }
    const int q = tid * 4;
    if ((unsigned)q >= n) return;
    const int64_t p = p0 + q;
    const uint4 w4 = __ldg(reinterpret_cast<const uint4 *>(I.bits + p));
    const uint32_t wv[4] = {w4.x, w4.y, w4.z, w4.w};
    const float4 yv = ldg4(I.y + p), psv = ldg4(I.phisum + p);
    const float yy[4] = {yv.x, yv.y, yv.z, yv.w}, pp[4] = {psv.x, psv.y, psv.z, psv.w};
    float r[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float sacc = 0.f;
        for (int b = 0; b < B; ++b)
            sacc = fmaf(xs[b * PROJ_T + q + e], ((wv[e] >> b) & 1u) ? 1.f : 0.f, sacc);
        if (ACC) {
            const float tt = I.y1[p + e] + (yy[e] - sacc);
            I.y1[p + e] = tt;
            r[e] = __fdiv_rn(tt - sacc, pp[e]);
        } else {
            r[e] = __fdiv_rn(yy[e] - sacc, pp[e]);
        }
    }
    for (int b = 0; b < B; ++b) {
        const float4 xv = *reinterpret_cast<const float4 *>(xs + b * PROJ_T + q);
        float4 o;
        o.x = fmaf(I.lam, r[0] * (((wv[0] >> b) & 1u) ? 1.f : 0.f), xv.x);
        o.y = fmaf(I.lam, r[1] * (((wv[1] >> b) & 1u) ? 1.f : 0.f), xv.y);
        o.z = fmaf(I.lam, r[2] * (((wv[2] >> b) & 1u) ? 1.f : 0.f), xv.z);
        o.w = fmaf(I.lam, r[3] * (((wv[3] >> b) & 1u) ? 1.f : 0.f), xv.w);
        st4_cs(I.xp + b * hw + p, o);
    }
}

unsigned batch_device_status(bool clear) {
    unsigned v = 0;
    if (cudaMemcpyFromSymbol(&v, g_batch_status, sizeof(v)) != cudaSuccess) return 0;
    if (clear && v) {
        const unsigned z = 0;
        cudaMemcpyToSymbol(g_batch_status, &z, sizeof(z));
    }
    return v;
}

// TV pass (FIX = 0) or its stop-test launch (FIX = 1) over all items' tiles.
template <int FIX>
__global__ void __launch_bounds__(tv::WPB * 32, 3) k_batch_tv(const Table *__restrict__ T) {
    const int g = blockIdx.x * tv::WPB + (threadIdx.x >> 5);
    if (g >= T->tv_prefix[T->n]) return;  // warp-uniform
    const int i = find_item(T->tv_prefix, T->n, g);
    const tv::Pass &P = T->it[i].tv;
    int frame, chunk, band;
    if (!tv::decode_index(P, g - T->tv_prefix[i], frame, chunk, band)) return;
    const int lane = threadIdx.x & 31;
    if (!FIX) {
        switch (P.S) {
            case 1: tv::run_mode<1, 4, false, true, true>(P, frame, chunk, band, lane); break;
            case 2: tv::run_mode<2, 4, false, true, true>(P, frame, chunk, band, lane); break;
            case 3: tv::run_mode<3, 4, false, true, true>(P, frame, chunk, band, lane); break;
            default: tv::run_mode<4, 4, false, true, true>(P, frame, chunk, band, lane); break;
        }
        return;
    }
    const int j = tv::find_stop(P, frame);
    switch (j) {  // a = 0: j in [1, S-1] re-runs with j updates
        case 1: tv::run_mode<1, 4, false, true, false>(P, frame, chunk, band, lane); break;
        case 2: tv::run_mode<2, 4, false, true, false>(P, frame, chunk, band, lane); break;
        case 3: tv::run_mode<3, 4, false, true, false>(P, frame, chunk, band, lane); break;
        default: break;
    }
}

// --------------------------------------------------------------- host side
size_t r256(size_t b) { return (b + 255) & ~size_t(255); }

struct Layout {
    size_t table, xp, y1, energy, stop, queue, tvscratch, total;
    std::vector<size_t> item_xp, item_y1, item_c, item_e, item_e1, item_stop;
};

Layout layout(const sci_batch_item *items, int n, int K) {
    Layout L;
    size_t off = 0;
    L.table = off;
    off += r256(sizeof(Table));
    for (int i = 0; i < n; ++i) {
        const int64_t hw = items[i].H * items[i].W, nn = items[i].B * hw;
        L.item_xp.push_back(off);
        off += r256(4 * (size_t)nn);
        L.item_y1.push_back(off);
        off += r256(4 * (size_t)hw);
        L.item_c.push_back(off);
        off += r256(4 * (size_t)hw);
    }
    // per item the energy sums of even and odd iterations (the per-phase
    // launches use the first), then its stop decisions and ticket
    L.energy = off;
    for (int i = 0; i < n; ++i) {
        const size_t eb = r256(sizeof(double) * 2 * K * (size_t)items[i].B);
        L.item_e.push_back(off - L.energy);
        L.item_e1.push_back(off + eb - L.energy);
        off += 2 * eb;
    }
    const size_t energy_end = off;
    L.stop = off;
    for (int i = 0; i < n; ++i) {
        L.item_stop.push_back(off);
        off += r256(sizeof(int) * (size_t)items[i].B + sizeof(unsigned));
    }
    L.queue = off;
    off += r256(sizeof(Queue));
    L.tvscratch = off;
    size_t tvmax = 0;  // autotuning scratch: the largest single-item TV workspace
    for (int i = 0; i < n; ++i)
        tvmax = std::max(tvmax, tv_workspace_bytes(items[i].B, items[i].H, items[i].W, K));
    off += r256(tvmax);
    L.total = off;
    (void)energy_end;
    return L;
}

int check(const sci_batch_item *items, int n, int K) {
    SCI_CHECK_ARG(items && n >= 1 && n <= MAXI, "batch: 1..%d items (got %d)", MAXI, n);
    SCI_CHECK_ARG(K >= 2 && K <= tv::SMAX + 1, "batch: tv_iter_max must be in [2, 5]");
    for (int i = 0; i < n; ++i) {
        const sci_batch_item &it = items[i];
        SCI_CHECK_ARG(it.y && it.mask_bits && it.phisum && it.x, "batch: item %d null pointer", i);
        SCI_CHECK_ARG(it.B >= 1 && it.B <= 32 && it.H >= 1 && it.W >= 4 && it.W % 4 == 0,
                      "batch: item %d needs 1 <= B <= 32, W %% 4 == 0 (B=%lld H=%lld W=%lld)", i,
                      (long long)it.B, (long long)it.H, (long long)it.W);
        SCI_CHECK_ARG(it.tv_weight > 0.f, "batch: item %d tv_weight must be > 0", i);
        SCI_CHECK_ARG(((reinterpret_cast<uintptr_t>(it.x) | reinterpret_cast<uintptr_t>(it.y) |
                        reinterpret_cast<uintptr_t>(it.phisum)) & 15u) == 0,
                      "batch: item %d buffers must be 16-byte aligned", i);
    }
    return SCI_OK;
}

int default_R(int64_t H, int64_t W, int64_t B) {
    (void)W;
    (void)B;
    return H >= 1024 ? 256 : (H >= 256 ? 128 : 64);
}

// Builds the host copy of the device table.
void build_table(const sci_batch_item *items, int n, int K, float eps, char *ws, const Layout &L,
                 Table &T) {
    memset(&T, 0, sizeof(T));
    T.n = n;
    T.proj_prefix[0] = T.tv_prefix[0] = T.qp_prefix[0] = T.tq_prefix[0] = 0;
    for (int i = 0; i < n; ++i) {
        const sci_batch_item &s = items[i];
        Item &I = T.it[i];
        I.y = s.y;
        I.bits = s.mask_bits;
        I.phisum = s.phisum;
        I.x = s.x;
        I.xp = reinterpret_cast<float *>(ws + L.item_xp[i]);
        I.y1 = reinterpret_cast<float *>(ws + L.item_y1[i]);
        I.c = reinterpret_cast<float *>(ws + L.item_c[i]);
        I.B = (int)s.B;
        I.hw = s.H * s.W;
        I.lam = s.lambda;
        tv::Pass &P = I.tv;
        P.f = I.xp;
        P.u = s.x;
        P.energy = reinterpret_cast<double *>(ws + L.energy + L.item_e[i]);
        P.fs = I.hw;
        P.nf = (int)s.B;
        P.H = (int)s.H;
        P.W = (int)s.W;
        P.K = K;
        P.a = 0;
        P.tau = 0.25f;
        P.tw = 0.25f / s.tv_weight;
        P.weight = s.tv_weight;
        P.eps = eps;
        P.cpl = 4;
        P.S = K - 1;
        P.hl = 4;
        P.hr = 4;
        P.own = 128 - 4 - 4;
        P.ht = K - 1;
        P.nbands = tv::band_count((int)s.W, 128, P.hl, P.hr);
        P.R = s.R > 0 ? s.R : default_R(s.H, s.W, s.B);
        P.nchunks = (int)((s.H + P.R - 1) / P.R);
        P.vec = 1;
        P.lag = 1;
        P.frame_fast = 1;
        T.proj_prefix[i + 1] = T.proj_prefix[i] + (int)((I.hw + PROJ_T - 1) / PROJ_T);
        T.qp_prefix[i + 1] = T.qp_prefix[i] + (int)((I.hw + QP_T - 1) / QP_T);
        // the work-queue passes: the lean pipeline with the item's column
        // width, energies of even / odd iterations, stop decisions by ticket
        for (int par = 0; par < 2; ++par) {
            tv::Pass &Q = I.tvq[par];
            Q = P;
            // halos of 4 columns for either width: with W % 4 == 0 every
            // band window starts on a multiple of 4 columns, so that a lane
            // pair's 16-byte copies (2 columns per lane) are aligned
            const int cpl = s.cpl == 2 ? 2 : 4;
            Q.cpl = cpl;
            Q.hl = 4;
            Q.hr = 4;
            Q.own = 32 * cpl - 8;
            Q.nbands = tv::band_count((int)s.W, 32 * cpl, Q.hl, Q.hr);
            Q.energy = reinterpret_cast<double *>(ws + L.energy +
                                                  (par ? L.item_e1[i] : L.item_e[i]));
            Q.stopj = reinterpret_cast<int *>(ws + L.item_stop[i]);
            Q.ticket = reinterpret_cast<unsigned *>(ws + L.item_stop[i] + sizeof(int) * s.B);
            // the fused iteration: the TV pass loads x_k and applies
            // x_k + lam (c phi_b) (the projection's rounding), writing x_{k+1}
            Q.f = par ? I.xp : I.x;
            Q.u = par ? I.x : I.xp;
            Q.proj = 1;
            Q.bits = I.bits;
            Q.cmap = I.c;
            Q.lam = I.lam;
        }
        T.tv_prefix[i + 1] = T.tv_prefix[i] + P.nbands * P.nchunks * P.nf;
        // both parities have the same geometry
        T.tq_prefix[i + 1] =
            T.tq_prefix[i] + I.tvq[0].nbands * I.tvq[0].nchunks * I.tvq[0].nf;
    }
}

// After an odd number of work-queue iterations the last x is in xp: copy
// it into every item's x.
__global__ void __launch_bounds__(PROJ_T) k_batch_copy_x(const Table *__restrict__ T) {
    const int g = blockIdx.x;
    if (g >= T->proj_prefix[T->n]) return;
    const int i = find_item(T->proj_prefix, T->n, g);
    const Item &I = T->it[i];
    const int64_t p = (int64_t)(g - T->proj_prefix[i]) * PROJ_T + threadIdx.x;
    if (p >= I.hw) return;
    for (int b = 0; b < I.B; ++b) I.x[b * I.hw + p] = I.xp[b * I.hw + p];
}

// bit 1 of the batch status: a bounded wait of a work-queue launch gave up
__global__ void k_batch_fold(const Queue *Q) {
    if (threadIdx.x == 0 && Q->abort) atomicOr(&g_batch_status, 2u);
}

// The give-up path of the work queue's bounded waits, on purpose: one warp
// waits at most `polls` polls for a count that nothing raises, then raises
// the abort flag, which the fold turns into status bit 1.
__global__ void k_queue_wait_selftest(Queue *Q, unsigned polls) {
    wait_count(Q, &Q->done[0][0], 1u, threadIdx.x & 31, polls);
}

int queue_selftest(unsigned polls, Queue *dQ, cudaStream_t s) {
    SCI_CUDA(cudaMemsetAsync(dQ, 0, sizeof(Queue), s));
    k_queue_wait_selftest<<<1, 32, 0, s>>>(dQ, polls);
    SCI_LAUNCHED("k_queue_wait_selftest");
    k_batch_fold<<<1, 32, 0, s>>>(dQ);
    SCI_LAUNCHED("k_batch_fold");
    return SCI_OK;
}

// The work-queue form (sci_batch_queue.cu) unless SCI_BATCH_QUEUE=0.
bool queue_enabled() {
    const char *e = getenv("SCI_BATCH_QUEUE");
    return !(e && atoi(e) == 0);
}

// per_launch: iterations per persistent launch of the work queue (0: all).
int enqueue(const Table &T, Table *dT, const Layout &L, char *ws, int n, int iters, int K,
            int accelerate, int init_x0, int per_launch, cudaStream_t s) {
    const int pb = T.proj_prefix[n], tb = (T.tv_prefix[n] + tv::WPB - 1) / tv::WPB;
    if (init_x0 || accelerate) {
        if (init_x0 && accelerate) k_batch_init<true, true><<<pb, PROJ_T, 0, s>>>(dT);
        else if (init_x0) k_batch_init<true, false><<<pb, PROJ_T, 0, s>>>(dT);
        else k_batch_init<false, true><<<pb, PROJ_T, 0, s>>>(dT);
        SCI_LAUNCHED("k_batch_init");
    }
    if (queue_enabled()) {
        // the items' stop decisions and tickets: a ticket counts the TV
        // tasks of an iteration and is reset by the last one, so it starts
        // at zero once per solve
        SCI_CUDA(cudaMemsetAsync(ws + L.stop, 0, L.queue - L.stop, s));
        Queue *dQ = reinterpret_cast<Queue *>(ws + L.queue);
        const int m = per_launch > 0 ? per_launch : std::max(1, iters);
        const int blocks = queue_blocks();
        bool narrow = false;
        for (int i = 0; i < n; ++i) narrow = narrow || T.it[i].tvq[0].cpl == 2;
        for (int k0 = 0; k0 < iters; k0 += m) {
            SCI_CUDA(cudaMemsetAsync(dQ, 0, sizeof(Queue), s));
            if (int e = queue_launch(dT, dQ, k0, std::min(iters, k0 + m), accelerate != 0, K - 1,
                                     blocks, narrow, s))
                return e;
            k_batch_fold<<<1, 32, 0, s>>>(dQ);
            SCI_LAUNCHED("k_batch_fold");
        }
        if (iters & 1) {  // the last TV pass wrote xp
            k_batch_copy_x<<<pb, PROJ_T, 0, s>>>(dT);
            SCI_LAUNCHED("k_batch_copy_x");
        }
        return SCI_OK;
    }
    const size_t ebytes = L.tvscratch - L.energy;
    // bulk-copy projection unless a mask is not 16-byte aligned (the other
    // planes are checked by check(); SCI_PROJ_TMA=0 selects the plain kernel)
    int maxB = 1;
    bool bulk = true;
    for (int i = 0; i < n; ++i) {
        maxB = std::max(maxB, T.it[i].B);
        bulk = bulk && (reinterpret_cast<uintptr_t>(T.it[i].bits) & 15u) == 0;
    }
    if (const char *e = getenv("SCI_PROJ_TMA")) bulk = bulk && atoi(e) != 0;
    for (int it = 0; it < iters; ++it) {
        const size_t psm = sizeof(float) * (size_t)maxB * PROJ_T;  // <= 32 KB
        if (bulk) {
            if (accelerate) k_batch_proj_tma<true><<<pb, PROJ_T / 4, psm, s>>>(dT);
            else k_batch_proj_tma<false><<<pb, PROJ_T / 4, psm, s>>>(dT);
        } else {
            if (accelerate) k_batch_proj<true><<<pb, PROJ_T, 0, s>>>(dT);
            else k_batch_proj<false><<<pb, PROJ_T, 0, s>>>(dT);
        }
        SCI_LAUNCHED("k_batch_proj");
        SCI_CUDA(cudaMemsetAsync(ws + L.energy, 0, ebytes, s));
        k_batch_tv<0><<<tb, tv::WPB * 32, 0, s>>>(dT);
        SCI_LAUNCHED("k_batch_tv");
        if (K >= 3) {
            k_batch_tv<1><<<tb, tv::WPB * 32, 0, s>>>(dT);
            SCI_LAUNCHED("k_batch_tv fixup");
        }
    }
    return SCI_OK;
}

// The whole solve of a batch (table upload, then the loop, captured once
// into a cached CUDA graph when use_graph).
int solve(const sci_batch_item *items, int n, int iters, int tv_iter_max, float eps,
                 int accelerate, int init_x0, int use_graph, int per_launch, void *workspace,
                 size_t workspace_bytes, cudaStream_t s) {
    const Layout L = layout(items, n, tv_iter_max);
    SCI_CHECK_ARG(workspace && workspace_bytes >= L.total,
                  "batch: workspace of %zu bytes needed, got %zu", L.total, workspace_bytes);
    char *ws = static_cast<char *>(workspace);
    Table *hT = new Table;
    build_table(items, n, tv_iter_max, eps, ws, L, *hT);
    Table *dT = reinterpret_cast<Table *>(ws + L.table);
    // the table is small; a stream-ordered copy from this host struct needs
    // it to stay alive until the copy ran, so the copy is synchronous here
    cudaError_t ce = cudaStreamSynchronize(s);
    if (ce == cudaSuccess) ce = cudaMemcpy(dT, hT, sizeof(Table), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
        delete hT;
        return cuda_status(ce, "batch table upload");
    }
    int rc = SCI_OK;
    if (!use_graph) {
        rc = enqueue(*hT, dT, L, ws, n, iters, tv_iter_max, accelerate, init_x0, per_launch, s);
        delete hT;
        return rc;
    }
    std::string key(reinterpret_cast<const char *>(hT), sizeof(Table));
    key_append(key, iters, accelerate, init_x0, per_launch);
    rc = run_graph("batch graph capture", key, s, [&](cudaStream_t cs) {
        return enqueue(*hT, dT, L, ws, n, iters, tv_iter_max, accelerate, init_x0, per_launch,
                       cs);
    });
    delete hT;
    return rc;
}

}  // namespace batch
}  // namespace sci

using namespace sci;
using namespace sci::batch;

extern "C" {

int sci_batch_workspace_bytes(const sci_batch_item *items, int n, int tv_iter_max,
                              size_t *bytes) {
    if (int e = check(items, n, tv_iter_max)) return e;
    SCI_CHECK_ARG(bytes, "null bytes");
    *bytes = layout(items, n, tv_iter_max).total;
    return SCI_OK;
}

int sci_batch_autotune(sci_batch_item *items, int n, int iters, int tv_iter_max, float eps,
                       int accelerate, int *iters_per_launch, void *workspace,
                       size_t workspace_bytes, void *stream) {
    if (int e = check(items, n, tv_iter_max)) return e;
    const Layout L = layout(items, n, tv_iter_max);
    SCI_CHECK_ARG(workspace && workspace_bytes >= L.total, "batch: workspace too small");
    SCI_CHECK_ARG(iters >= 0, "batch: iters must be >= 0");
    cudaStream_t s = as_stream(stream);
    // Every candidate is timed on the batch itself -- a few iterations of its
    // own solve from x0 = At(y / Phi_sum) (overwriting x), inside the
    // persistent launch where all items share the GPU -- because a tiling
    // timed on one item alone ranks differently there (measured on the
    // 64-item uneven batch: per-shape single-item tuning 185 ms per solve,
    // the default tiling 138 ms).  Candidates: row-chunk heights of
    // 1/2, 1 and 2 times the default for each item's height (16..512 rows),
    // 4 columns per lane for every item or 2 for items at most 256 columns
    // wide; then, for the best tiling, 1, 2 or 3 iterations per launch
    // against all of them.  The choice is cached per process for the batch's
    // list of shapes.
    const int probe = std::max(1, std::min(iters, 6));
    std::string key;
    key_append(key, n, tv_iter_max, probe, accelerate);
    for (int i = 0; i < n; ++i) key_append(key, items[i].B, items[i].H, items[i].W);
    static std::mutex mu;
    static std::map<std::string, std::tuple<int, int, int>> tuned;  // scale x 2, narrow, m
    auto apply = [&](int scale2, int narrow) {
        for (int i = 0; i < n; ++i) {
            const int R = default_R(items[i].H, items[i].W, items[i].B) * scale2 / 2;
            items[i].R = std::max(16, std::min(512, R));
            items[i].cpl = (narrow && items[i].W <= 256) ? 2 : 4;
        }
    };
    {
        std::lock_guard<std::mutex> lk(mu);
        auto f = tuned.find(key);
        if (f != tuned.end()) {
            apply(std::get<0>(f->second), std::get<1>(f->second));
            if (iters_per_launch) *iters_per_launch = std::get<2>(f->second);
            return SCI_OK;
        }
    }
    cudaEvent_t e0, e1;
    SCI_CUDA(cudaEventCreate(&e0));
    SCI_CUDA(cudaEventCreate(&e1));
    int rc = SCI_OK;
    auto timed = [&](int m) -> float {  // the first run warms up
        float ms = 0.f;
        for (int rep = 0; rep <= 2; ++rep) {
            cudaEventRecord(e0, s);
            rc = solve(items, n, probe, tv_iter_max, eps, accelerate, 1, 0, m, workspace,
                       workspace_bytes, s);
            if (rc != SCI_OK) return -1.f;
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (rep > 0) ms += t;
        }
        return ms;
    };
    float best = 1e30f;
    int bs = 2, bn = 0, bm = 0;
    for (int scale2 : {2, 1, 4}) {
        for (int narrow : {0, 1}) {
            apply(scale2, narrow);
            const float ms = timed(0);
            if (ms < 0.f) break;
            if (ms < best) {
                best = ms;
                bs = scale2;
                bn = narrow;
            }
        }
        if (rc != SCI_OK) break;
    }
    apply(bs, bn);
    if (rc == SCI_OK && iters_per_launch) {
        for (int m : {1, 2, 3}) {
            if (m >= probe) continue;
            const float ms = timed(m);
            if (ms < 0.f) break;
            if (ms < best) {
                best = ms;
                bm = m;
            }
        }
        // a launch of all `probe` iterations stands for one of all iterations
        *iters_per_launch = bm;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == SCI_OK) {
        std::lock_guard<std::mutex> lk(mu);
        tuned[key] = std::make_tuple(bs, bn, bm);
    }
    return rc;
}

int sci_batch_selftest_queue_wait(unsigned int polls, void *workspace, size_t workspace_bytes,
                                  void *stream) {
    SCI_CHECK_ARG(polls >= 1 && polls <= (1u << 20), "selftest: polls in [1, 2^20]");
    SCI_CHECK_ARG(workspace && workspace_bytes >= sizeof(Queue),
                  "selftest: a workspace of %zu bytes is needed", sizeof(Queue));
    return queue_selftest(polls, static_cast<Queue *>(workspace), as_stream(stream));
}

int sci_batch_gap_tv(const sci_batch_item *items, int n, int iters, int tv_iter_max, float eps,
                     int accelerate, int init_x0, int use_graph, int iters_per_launch,
                     void *workspace, size_t workspace_bytes, void *stream) {
    if (int e = check(items, n, tv_iter_max)) return e;
    SCI_CHECK_ARG(iters >= 0, "batch: iters must be >= 0");
    SCI_CHECK_ARG(iters_per_launch >= 0, "batch: iters_per_launch must be >= 0");
    return solve(items, n, iters, tv_iter_max, eps, accelerate, init_x0, use_graph,
                 iters_per_launch, workspace, workspace_bytes, as_stream(stream));
}

}  // extern "C"
