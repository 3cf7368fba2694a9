// GAP projection with bulk-copy (TMA) staging of the frame stack.
//
// Same arithmetic as k_proj_gap_smem (PnP_SCI/python/pnp_sci_algo.py:640-645
// with a packed binary mask): per pixel yb = sum_b phi_b x_b (in frame
// order, fused multiply-adds), ACC: y1 += y - yb, r = (y1 - yb) / Phi_sum,
// else r = (y - yb) / Phi_sum; x_out_b = x_b + lambda (r phi_b).
//
// Layout and schedule.  A tile is TP consecutive pixels of all B frames:
// B rows of TP floats, each contiguous in HBM.  One thread per block issues
// the B row copies of a tile with cp.async.bulk into shared memory and
// arms an mbarrier with the byte count; the block waits on it, each thread
// reduces 4 pixels over the frames from shared memory and writes the 4
// updated pixels of every frame with 16-byte streaming stores.  Tiles are
// double-buffered (two tiles in flight per block), blocks are persistent
// (grid = resident blocks), and a buffer is refilled only after the whole
// block has finished reading it.  x is read from HBM once and x_out written
// once: 8 bytes per pixel and frame, plus 20 bytes per pixel of maps.
//
// Waits are bounded: a wait that gives up sets bit 0 of the device status
// word (sci_device_status), waits a bounded time for the block's copies in
// flight and ends the block.
#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include "sci_bulk.cuh"
#include "sci_common.cuh"

namespace sci {

__device__ unsigned int g_device_status;

namespace {

__device__ __forceinline__ float bit(uint32_t w, int b) { return ((w >> b) & 1u) ? 1.0f : 0.0f; }

// Resident blocks per SM of a persistent kernel at `threads` threads and
// `smem` bytes of dynamic shared memory, from the occupancy calculator
// (cached per kernel and size; at least 1).
int resident_blocks(const void *kern, int threads, size_t smem) {
    static std::mutex mu;
    static std::map<std::tuple<const void *, int, size_t>, int> cache;
    const auto key = std::make_tuple(kern, threads, smem);
    std::lock_guard<std::mutex> lock(mu);
    auto f = cache.find(key);
    if (f != cache.end()) return f->second;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem) != cudaSuccess ||
        n < 1) {
        cudaGetLastError();
        n = 1;
    }
    cache[key] = n;
    return n;
}

// Issues the copies of tile t into buffer `buf` (thread 0 only).  The
// per-pixel maps are read with plain loads: staging them as well (28 KB
// instead of 24 KB per block at 24 frames) measured slower, 150 vs 141 us.
template <int TP>
__device__ __forceinline__ void issue_tile(float *xs, uint64_t *bars, int buf, int64_t t,
                                           const float *x, int B, int64_t hw) {
    const int64_t p0 = t * TP;
    const int64_t rem = hw - p0;
    const unsigned n = (unsigned)(rem < TP ? rem : TP);
    float *dst = xs + (int64_t)buf * B * TP;
    mbar_expect_tx(bars + buf, (unsigned)B * n * 4u);
    for (int b = 0; b < B; ++b) bulk_g2s(dst + b * TP, x + b * hw + p0, n * 4u, bars + buf);
}

template <int TP, bool ACC>
__global__ void __launch_bounds__(TP / 4) k_proj_gap_tma(
    const float *__restrict__ x, const uint32_t *__restrict__ bits, const float *__restrict__ y,
    float *__restrict__ y1, const float *__restrict__ phisum, float *__restrict__ xo, float lam,
    int B, int64_t hw, double *__restrict__ rn) {
    extern __shared__ __align__(128) float xs[];  // [2][B][TP]
    __shared__ __align__(8) uint64_t bars[2];
    double racc = 0.0;  // FP64 partial of ||r||^2 (rn != nullptr)
    const int tid = threadIdx.x;
    const int64_t ntiles = (hw + TP - 1) / TP;
    const int64_t G = gridDim.x;
    if (tid == 0) {
        mbar_init(bars + 0, 1);
        mbar_init(bars + 1, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    const int64_t t0 = blockIdx.x;
    if (tid == 0) {
        if (t0 < ntiles) issue_tile<TP>(xs, bars, 0, t0, x, B, hw);
        if (t0 + G < ntiles) issue_tile<TP>(xs, bars, 1, t0 + G, x, B, hw);
    }
    int i = 0;
    for (int64_t t = t0; t < ntiles; t += G, ++i) {
        const int buf = i & 1;
        const unsigned parity = (unsigned)(i >> 1) & 1u;
        const bool ok = mbar_wait(bars + buf, parity);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(&g_device_status, 1u);
                // let the copies in flight land before the block's shared
                // memory is released
                mbar_wait(bars + buf, parity);
                if (t + G < ntiles) mbar_wait(bars + (buf ^ 1), (unsigned)((i + 1) >> 1) & 1u);
            }
            return;
        }
        const int64_t p0 = t * TP;
        const int q = tid * 4;
        if (p0 + q < hw) {  // hw % 4 == 0: all 4 pixels are inside
            const int64_t p = p0 + q;
            const float *xb = xs + (int64_t)buf * B * TP + q;
            const uint4 w = __ldg(reinterpret_cast<const uint4 *>(bits + p));
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
            for (int b = 0; b < B; ++b) {
                const float4 v = *reinterpret_cast<const float4 *>(xb + b * TP);
                s.x = fmaf(v.x, bit(w.x, b), s.x);
                s.y = fmaf(v.y, bit(w.y, b), s.y);
                s.z = fmaf(v.z, bit(w.z, b), s.z);
                s.w = fmaf(v.w, bit(w.w, b), s.w);
            }
            const float4 yv = ldg4(y + p), ps = ldg4(phisum + p);
            float4 r;
            if (ACC) {
                float4 tt = *reinterpret_cast<const float4 *>(y1 + p);
                tt.x = tt.x + (yv.x - s.x);
                tt.y = tt.y + (yv.y - s.y);
                tt.z = tt.z + (yv.z - s.z);
                tt.w = tt.w + (yv.w - s.w);
                st4(y1 + p, tt);
                r = make_float4(__fdiv_rn(tt.x - s.x, ps.x), __fdiv_rn(tt.y - s.y, ps.y),
                                __fdiv_rn(tt.z - s.z, ps.z), __fdiv_rn(tt.w - s.w, ps.w));
            } else {
                r = make_float4(__fdiv_rn(yv.x - s.x, ps.x), __fdiv_rn(yv.y - s.y, ps.y),
                                __fdiv_rn(yv.z - s.z, ps.z), __fdiv_rn(yv.w - s.w, ps.w));
            }
            if (rn) rn_add4(racc, r);
#pragma unroll 4
            for (int b = 0; b < B; ++b) {
                const float4 v = *reinterpret_cast<const float4 *>(xb + b * TP);
                float4 o;
                o.x = fmaf(lam, r.x * bit(w.x, b), v.x);
                o.y = fmaf(lam, r.y * bit(w.y, b), v.y);
                o.z = fmaf(lam, r.z * bit(w.z, b), v.z);
                o.w = fmaf(lam, r.w * bit(w.w, b), v.w);
                st4_cs(xo + b * hw + p, o);
            }
        }
        __syncthreads();  // every thread is done with this buffer
        if (tid == 0 && t + 2 * G < ntiles) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue_tile<TP>(xs, bars, buf, t + 2 * G, x, B, hw);
        }
    }
    if (rn) rn_flush_warp(racc, rn);
}

// ADMM projection (pnp_sci_algo.py:808-812 with a packed mask), same
// arithmetic as k_proj_admm_smem: t_b = theta_b + b_b, yb = sum_b t_b phi_b,
// r = (y - yb) / (Phi_sum + gamma), x_b = t_b + lambda (r phi_b),
// v_b = x_b - b_b; x written when WANT_X.  A tile stages theta (B rows of
// TP floats) with the same bulk copies and mbarrier scheme.
// theta rows of one ADMM tile (thread 0 only); b is read with 16-byte loads
// (twice; the second read is served by the caches).  Staging b as well
// (twice the shared memory per block) measured the same, 0.251 ms at
// 2048 x 2048 x 24.
template <int TP>
__device__ __forceinline__ void issue_theta(float *xs, uint64_t *bars, int buf, int64_t t,
                                            const float *th, int B, int64_t hw) {
    const int64_t p0 = t * TP;
    const int64_t rem = hw - p0;
    const unsigned n = (unsigned)(rem < TP ? rem : TP);
    float *dst = xs + (int64_t)buf * B * TP;
    mbar_expect_tx(bars + buf, (unsigned)B * n * 4u);
    for (int b = 0; b < B; ++b) bulk_g2s(dst + b * TP, th + b * hw + p0, n * 4u, bars + buf);
}

// Unroll of the band loops: the 16-byte loads of the second stack (b, or
// the previous TV input) are in flight together per thread.  Measured on
// the ADMM-TV solve at 2048 x 2048 x 24 (60 iterations), bitwise equal:
// unroll 4 38.9 ms, 8 37.6 ms, 12 37.0 ms, 24 36.5 ms.
#ifndef SCI_ADMM_UNROLL
#define SCI_ADMM_UNROLL 24
#endif
constexpr int kAdmmUnroll = SCI_ADMM_UNROLL;

// BFV: the multiplier comes as the previous TV input, b = theta - bb (the
// TV's residual u - f, formed here instead of stored by the TV pass).
template <int TP, bool WANT_X, bool BFV = false>
__global__ void __launch_bounds__(TP / 4) k_proj_admm_tma(
    const float *__restrict__ th, const float *__restrict__ bb, const uint32_t *__restrict__ bits,
    const float *__restrict__ y, const float *__restrict__ phisum, float *__restrict__ v,
    float *__restrict__ xo, float lam, float gamma, int B, int64_t hw, double *__restrict__ rn) {
    extern __shared__ __align__(128) float xs[];  // [2][B][TP]: theta
    __shared__ __align__(8) uint64_t bars[2];
    double racc = 0.0;  // FP64 partial of ||r||^2 (rn != nullptr)
    const int tid = threadIdx.x;
    const int64_t ntiles = (hw + TP - 1) / TP;
    const int64_t G = gridDim.x;
    if (tid == 0) {
        mbar_init(bars + 0, 1);
        mbar_init(bars + 1, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    const int64_t t0 = blockIdx.x;
    if (tid == 0) {
        if (t0 < ntiles) issue_theta<TP>(xs, bars, 0, t0, th, B, hw);
        if (t0 + G < ntiles) issue_theta<TP>(xs, bars, 1, t0 + G, th, B, hw);
    }
    int i = 0;
    for (int64_t t = t0; t < ntiles; t += G, ++i) {
        const int buf = i & 1;
        const unsigned parity = (unsigned)(i >> 1) & 1u;
        const bool ok = mbar_wait(bars + buf, parity);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(&g_device_status, 1u);
                mbar_wait(bars + buf, parity);
                if (t + G < ntiles) mbar_wait(bars + (buf ^ 1), (unsigned)((i + 1) >> 1) & 1u);
            }
            return;
        }
        const int64_t p0 = t * TP;
        const int q = tid * 4;
        if (p0 + q < hw) {
            const int64_t p = p0 + q;
            const float *tb = xs + (int64_t)buf * B * TP + q;
            auto bload = [&](int b) {
                if (!BFV) return ldg4(bb + b * hw + p);
                const float4 a = *reinterpret_cast<const float4 *>(tb + b * TP);
                const float4 f = ldg4(bb + b * hw + p);
                return make_float4(a.x - f.x, a.y - f.y, a.z - f.z, a.w - f.w);
            };
            const uint4 w = __ldg(reinterpret_cast<const uint4 *>(bits + p));
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll kAdmmUnroll
            for (int b = 0; b < B; ++b) {
                const float4 a = *reinterpret_cast<const float4 *>(tb + b * TP);
                const float4 c = bload(b);
                s.x = fmaf(a.x + c.x, bit(w.x, b), s.x);
                s.y = fmaf(a.y + c.y, bit(w.y, b), s.y);
                s.z = fmaf(a.z + c.z, bit(w.z, b), s.z);
                s.w = fmaf(a.w + c.w, bit(w.w, b), s.w);
            }
            const float4 yv = ldg4(y + p), ps = ldg4(phisum + p);
            const float4 r = make_float4(__fdiv_rn(yv.x - s.x, ps.x + gamma),
                                         __fdiv_rn(yv.y - s.y, ps.y + gamma),
                                         __fdiv_rn(yv.z - s.z, ps.z + gamma),
                                         __fdiv_rn(yv.w - s.w, ps.w + gamma));
            if (rn) rn_add4(racc, r);
#pragma unroll kAdmmUnroll
            for (int b = 0; b < B; ++b) {
                const float4 a = *reinterpret_cast<const float4 *>(tb + b * TP);
                const float4 c = bload(b);
                float4 x;
                x.x = fmaf(lam, r.x * bit(w.x, b), a.x + c.x);
                x.y = fmaf(lam, r.y * bit(w.y, b), a.y + c.y);
                x.z = fmaf(lam, r.z * bit(w.z, b), a.z + c.z);
                x.w = fmaf(lam, r.w * bit(w.w, b), a.w + c.w);
                if (WANT_X) st4(xo + b * hw + p, x);
                st4_cs(v + b * hw + p, make_float4(x.x - c.x, x.y - c.y, x.z - c.z, x.w - c.w));
            }
        }
        __syncthreads();
        if (tid == 0 && t + 2 * G < ntiles) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue_theta<TP>(xs, bars, buf, t + 2 * G, th, B, hw);
        }
    }
    if (rn) rn_flush_warp(racc, rn);
}

template <int TP>
int launch_tp(const float *x, const uint32_t *bits, const float *y, float *y1,
              const float *phisum, float *xo, float lam, bool acc, int B, int64_t hw,
              cudaStream_t s, double *rn) {
    const size_t smem = sizeof(float) * 2 * (size_t)B * TP;
    const int64_t ntiles = (hw + TP - 1) / TP;
    auto kern = acc ? k_proj_gap_tma<TP, true> : k_proj_gap_tma<TP, false>;
    // above 48 KB of dynamic shared memory needs the opt-in attribute; a
    // host-side call, also valid while the stream is being captured
    SCI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // the persistent grid: every block resident at once
    const unsigned g = (unsigned)std::min<int64_t>(
        ntiles, (int64_t)resident_blocks(reinterpret_cast<const void *>(kern), TP / 4, smem) * kSMs);
    kern<<<g, TP / 4, smem, s>>>(x, bits, y, y1, phisum, xo, lam, B, hw, rn);
    SCI_LAUNCHED("k_proj_gap_tma");
    return SCI_OK;
}

}  // namespace

// Packed mask, B <= 32, 16-byte aligned planes with hw % 4 == 0.  Returns
// SCI_OK, or a negative code when the caller must use another kernel.
int launch_proj_gap_tma(const float *x, const uint32_t *bits, const float *y, float *y1,
                        const float *phisum, float *xo, float lam, bool acc, int B, int64_t hw,
                        cudaStream_t s, double *rn) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(bits) |
                        reinterpret_cast<uintptr_t>(y) | reinterpret_cast<uintptr_t>(y1) |
                        reinterpret_cast<uintptr_t>(phisum) | reinterpret_cast<uintptr_t>(xo);
    if ((a & 15u) || hw % 4 || B < 1 || B > 32) return SCI_ERR_UNSUPPORTED;
    // pixels per tile (SCI_PROJ_TP overrides).  Measured at 2048 x 2048 x
    // 24: 128 (one warp, 24 KB, 9 blocks per SM) 141 us, 256 146 us, 512 153 us.
    const char *e = getenv("SCI_PROJ_TP");
    const int tp = e ? atoi(e) : 128;
    if (tp == 512) return launch_tp<512>(x, bits, y, y1, phisum, xo, lam, acc, B, hw, s, rn);
    if (tp == 256) return launch_tp<256>(x, bits, y, y1, phisum, xo, lam, acc, B, hw, s, rn);
    return launch_tp<128>(x, bits, y, y1, phisum, xo, lam, acc, B, hw, s, rn);
}

// ADMM projection with a packed mask (B <= 32, 16-byte aligned planes,
// hw % 4 == 0); SCI_ERR_UNSUPPORTED otherwise.  Tiles of TP pixels x B
// rows, double-buffered (24 KB at 24 frames and TP = 128).  b_from_v: bb
// is the previous TV input v and b = theta - v (bitwise the TV's residual).
int launch_proj_admm_tma(const float *th, const float *bb, const uint32_t *bits, const float *y,
                         const float *phisum, float *v, float *xo, float lam, float gamma, int B,
                         int64_t hw, cudaStream_t s, bool b_from_v, double *rn) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(th) | reinterpret_cast<uintptr_t>(bb) |
                        reinterpret_cast<uintptr_t>(bits) | reinterpret_cast<uintptr_t>(y) |
                        reinterpret_cast<uintptr_t>(phisum) | reinterpret_cast<uintptr_t>(v) |
                        reinterpret_cast<uintptr_t>(xo);
    if ((a & 15u) || hw % 4 || B < 1 || B > 32) return SCI_ERR_UNSUPPORTED;
    const char *e = getenv("SCI_PROJ_TP");
    const int tp = e ? atoi(e) : 128;
    auto go = [&](auto tpc) -> int {
        constexpr int TP = decltype(tpc)::value;
        const size_t smem = sizeof(float) * 2 * (size_t)B * TP;
        const int64_t ntiles = (hw + TP - 1) / TP;
        auto kern = b_from_v ? (xo ? k_proj_admm_tma<TP, true, true>
                                   : k_proj_admm_tma<TP, false, true>)
                             : (xo ? k_proj_admm_tma<TP, true, false>
                                   : k_proj_admm_tma<TP, false, false>);
        SCI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        const unsigned g = (unsigned)std::min<int64_t>(
            ntiles,
            (int64_t)resident_blocks(reinterpret_cast<const void *>(kern), TP / 4, smem) * kSMs);
        kern<<<g, TP / 4, smem, s>>>(th, bb, bits, y, phisum, v, xo, lam, gamma, B, hw, rn);
        SCI_LAUNCHED("k_proj_admm_tma");
        return SCI_OK;
    };
    if (tp == 256) return go(std::integral_constant<int, 256>{});
    if (tp == 64) return go(std::integral_constant<int, 64>{});
    return go(std::integral_constant<int, 128>{});
}

}  // namespace sci

namespace sci {
namespace batch {
unsigned batch_device_status(bool clear);  // sci_batch.cu
}
namespace cnn {
unsigned cnn_device_status(int clear);  // sci_cnn_tc.cu
}
namespace {

// The error path of the bounded waits, on purpose: the barrier expects 16
// bytes that no copy delivers, so every poll fails; after `polls` polls the
// kernel records the timeout in the status word and returns.  No copy is in
// flight, so nothing lands in the block's shared memory after it ends.
__global__ void k_wait_selftest(unsigned polls) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_expect_tx(&bar, 16u);
    }
    __syncthreads();
    bool ok = false;
    for (unsigned i = 0; i < polls && !ok; ++i) ok = mbar_try_wait(&bar, 0);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(&g_device_status, 1u);
}

}  // namespace

int selftest_bounded_wait(unsigned polls, cudaStream_t s) {
    SCI_CHECK_ARG(polls >= 1 && polls <= (1u << 20), "selftest: 1 <= polls <= 2^20");
    k_wait_selftest<<<1, 32, 0, s>>>(polls);
    SCI_LAUNCHED("k_wait_selftest");
    return SCI_OK;
}

}  // namespace sci

extern "C" int sci_selftest_bounded_wait(unsigned int polls, void *stream) {
    return sci::selftest_bounded_wait(polls, sci::as_stream(stream));
}

extern "C" int sci_device_status(unsigned int *status, int clear) {
    SCI_CHECK_ARG(status, "sci_device_status: null pointer");
    const unsigned int batch = sci::batch::batch_device_status(clear != 0) |
                               sci::cnn::cnn_device_status(clear);
    unsigned int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, sci::g_device_status, sizeof(v));
    if (e != cudaSuccess) return sci::cuda_status(e, "cudaMemcpyFromSymbol");
    if (clear && v) {
        const unsigned int z = 0;
        e = cudaMemcpyToSymbol(sci::g_device_status, &z, sizeof(z));
        if (e != cudaSuccess) return sci::cuda_status(e, "cudaMemcpyToSymbol");
    }
    *status = v | batch;
    return SCI_OK;
}
