// Shared helpers of the sm_103a kernels: error reporting, argument checks,
// vector loads, packed-FP32 arithmetic.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>

#include "sci_gb300.h"

namespace sci {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *what);

#define SCI_CHECK_ARG(cond, ...)                                   \
    do {                                                           \
        if (!(cond)) {                                             \
            ::sci::set_error(__VA_ARGS__);                         \
            return SCI_ERR_INVALID_ARG;                            \
        }                                                          \
    } while (0)

#define SCI_CUDA(call)                                             \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return ::sci::cuda_status(_e, #call); \
    } while (0)

#define SCI_LAUNCHED(name) SCI_CUDA(cudaGetLastError())

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs

// ------------------------------------------- programmatic dependent launch
// The iteration kernels of the solvers (residual passes, TV passes, their
// stop-test launches, the spectral projection) are launched so that a
// kernel's blocks may be scheduled while its predecessor in the stream
// drains; each of them calls grid_dep_wait() before it touches memory, which
// returns once the predecessor grid has completed and its writes are
// visible (a no-op for a normal launch).  This hides the launch gap between
// consecutive kernels.  SCI_PDL=0 launches them normally.
bool pdl_enabled();

template <typename... K, typename... A>
cudaError_t launch_dep(void (*kernel)(K...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t s, A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

__device__ __forceinline__ void grid_dep_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ------------------------------------------------------------- device side
__device__ __forceinline__ float4 ldg4(const float *p) {
    return __ldg(reinterpret_cast<const float4 *>(p));
}
__device__ __forceinline__ void st4(float *p, float4 v) {
    *reinterpret_cast<float4 *>(p) = v;
}
// streaming store (written once, not re-read by this kernel)
__device__ __forceinline__ void st4_cs(float *p, float4 v) {
    __stcs(reinterpret_cast<float4 *>(p), v);
}

__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ---- FP64 sum of squares of a projection residual ----------------------
// The projection kernels accumulate ||r||^2 of their residual map r (one
// float per pixel) when given a non-null `rn`: the squares of a thread's
// 4-pixel group are summed in FP32 and added to a per-thread FP64 partial;
// rn_flush reduces the partials of the block (warp shuffles, shared memory)
// and adds them to *rn with one FP64 atomic.  Every thread of the block
// calls rn_flush (it synchronises the block).
__device__ __forceinline__ void rn_add4(double &acc, float4 r) {
    float q = r.x * r.x;
    q = fmaf(r.y, r.y, q);
    q = fmaf(r.z, r.z, q);
    q = fmaf(r.w, r.w, q);
    acc += (double)q;
}
__device__ __forceinline__ void rn_add1(double &acc, float r) { acc += (double)(r * r); }
// Warp-level flush (one FP64 atomic per warp, no shared memory): for the
// persistent bulk-copy kernels, whose blocks are one to four warps.
__device__ __forceinline__ void rn_flush_warp(double acc, double *rn) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(rn, acc);
}
__device__ __forceinline__ void rn_flush(double acc, double *rn) {
    __shared__ double part[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) part[w] = acc;
    __syncthreads();
    if (w == 0) {
        const int nw = (int)((blockDim.x + 31) >> 5);
        double v = lane < nw ? part[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) atomicAdd(rn, v);
    }
}

// ---- packed FP32 pairs (sm_100+ f32x2 arithmetic) --------------------
// A float2 is held as one 64-bit register pair; add/sub/mul/fma on both
// halves issue as one instruction.
struct f2 {
    unsigned long long v;
};
__device__ __forceinline__ f2 mk2(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1,%2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float lo(f2 a) {
    float x, y;
    asm("mov.b64 {%0,%1}, %2;" : "=f"(x), "=f"(y) : "l"(a.v));
    (void)y;
    return x;
}
__device__ __forceinline__ float hi(f2 a) {
    float x, y;
    asm("mov.b64 {%0,%1}, %2;" : "=f"(x), "=f"(y) : "l"(a.v));
    (void)x;
    return y;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}

}  // namespace sci
