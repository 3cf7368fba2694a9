// Convolutions on the 5th-generation tensor cores (tcgen05.mma, accumulator
// in tensor memory).
//
// 1. The thin-input 3 x 3 convolution: the first layer of FastDVDnet's
// denoising block (6 input channels -> 90 features, padded to 8 -> 96;
// packages/fastdvdnet/models.py:29-43) and of FFDNet (5 -> 64,
// packages/ffdnet/models.py:37-42), where cuDNN falls back to slow kernels
// because each filter tap has only 8 input channels.  Implicit GEMM per
// tile of kM = 128 output pixels (TMEM lane m = pixel m of the tile):
//   D[m, n] = sum_k A[m, k] * B[n, k],  k = tap * 8 + c  (tap = 3 dy + dx),
// K = 9 taps x 8 bf16 channels plus one zero chunk = 80 = 5 MMAs of K 16;
// B = the N x 80 weights, staged once per block.  Both operands are K-major
// without swizzle: an 8-row x 16-byte core matrix is 128 contiguous bytes,
// with explicit byte offsets between K-adjacent core matrices (LBO) and
// between 8-row groups (SBO).  The epilogue reads D with tcgen05.ld (warp w
// owns lanes 32w..32w+31, i.e. thread t owns pixel t), adds the bias,
// applies ReLU, stages the tile's N bf16 channels in shared memory and
// writes them with bulk copies that drain while the block starts its next
// tile.  Three forms:
//   k_conv_thin_rd (the default): 128-pixel segments of a frame row; the
//     three input row segments a tile needs are bulk-copied into shared
//     memory two tiles ahead and read by the MMAs in place through
//     tap-shifted descriptors; the output stage is swizzled and written by
//     tensor stores (conflict-free 16-byte stage stores);
//   k_conv_thin_rows: the same row segments, with the im2col rows built in
//     shared memory and a pixel-major stage written by one bulk copy;
//   k_conv_thin_tc: any 128 consecutive pixels, each row's nine taps
//     gathered from global memory by cp.async.
// 56 KiB of shared memory per block gives k_conv_thin_rd 4 blocks per SM
// (4 x 128 = the SM's 512 TMEM columns); 64 / 74 KiB cap the other two
// forms at 3.
//
// 2. k_den_tail: FastDVDnet's DenBlock tail (shuffle + add, the 32 -> 32 and
// 32 -> 1 convolutions, centre - output) in one warp-specialised kernel;
// see the comments at the kernel.
//
// Every wait on an mbarrier is bounded: on timeout the block sets bit 0 of
// the CNN status word, waits once more (bounded) for the copies and MMAs in
// flight, frees its tensor memory and returns.
#include <cuda.h>  // CUtensorMap; the encoder is fetched through the runtime
#include <cuda_bf16.h>

#include <cstdlib>
#include <cstring>

#include "sci_bulk.cuh"
#include "sci_common.cuh"

namespace sci {
namespace {

__device__ unsigned int g_cnn_status;

constexpr int kM = 128;                  // output pixels per tile = TMEM lanes
constexpr int kThr = 128;                // threads per block (thread t <-> pixel t)
constexpr int kKC = 10;                  // 16-byte K chunks per row: 9 taps + 1 zero chunk
constexpr int kCore = 128;               // bytes of one core matrix (8 rows x 16 B)
constexpr int kSBO = kKC * kCore;        // bytes between 8-row groups
constexpr int kATile = (kM / 8) * kSBO;  // 20 KiB
constexpr int kTmemCols = 128;
constexpr int kSmemBytes = 64 * 1024;  // requested per block: at most 3 blocks per SM

template <int N>
struct alignas(1024) TcSmem {
    uint8_t a[kATile];
    uint8_t b[(N / 8) * kSBO];
    uint8_t stage[kM * N * 2];  // the tile's output, pixel-major (NHWC)
    float bias[N];
    uint64_t bar;
    uint32_t tmem;
};

// tcgen05 shared-memory matrix descriptor: start address, leading (K) and
// stride (M / N) byte offsets in 16-byte units, descriptor version 1 (bit
// 46), no swizzle, base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(kCore >> 4) << 16) |
           ((uint64_t)(kSBO >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D float32 (bits 4-5 = 1), A and B
// bfloat16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
template <int N>
__host__ __device__ constexpr uint32_t instr_desc() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(kM >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

// 32 consecutive float32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
        "[%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// shared -> global bulk copy (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_s2g(void *dst, const void *src, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                 "r"(smem_u32(src)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src)
                 : "memory");
}

// One im2col row (this thread's pixel p, 9 taps) of a tile into an A buffer:
// cp.async for taps inside the frame, zeros outside.
__device__ __forceinline__ void gather_row(const uint4 *__restrict__ in, uint8_t *arow,
                                           int64_t p, int64_t P, int64_t H, int64_t W) {
    if (p >= P) return;  // rows past the end keep stale data; their results are not stored
    const int64_t x = p % W, y = (p / W) % H, f = p / (W * H);
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
        const int64_t yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
        uint8_t *dst = arow + tap * kCore;
        if (yy >= 0 && yy < H && xx >= 0 && xx < W)
            cp_async16(dst, in + (f * H + yy) * W + xx);
        else
            *reinterpret_cast<uint4 *>(dst) = make_uint4(0u, 0u, 0u, 0u);
    }
}

template <int N>
__global__ void __launch_bounds__(kThr, 3)
    k_conv_thin_tc(const uint4 *__restrict__ in, const uint4 *__restrict__ wts,
                   const float *__restrict__ bias, uint4 *__restrict__ out, int64_t F,
                   int64_t H, int64_t W, int relu) {
    static_assert(N % 32 == 0 && N >= 32 && N <= 256, "N: multiple of 32 up to 256");
    static_assert(sizeof(TcSmem<N>) + 1024 <= kSmemBytes, "shared memory layout too large");
    extern __shared__ uint8_t smem_raw[];
    TcSmem<N> &s = *reinterpret_cast<TcSmem<N> *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5;

    // weights into the core-matrix layout; the zero K chunk of A
    for (int i = tid; i < N * kKC; i += kThr) {
        const int n = i / kKC, kc = i % kKC;
        *reinterpret_cast<uint4 *>(s.b + (n >> 3) * kSBO + kc * kCore + (n & 7) * 16) = wts[i];
    }
    for (int i = tid; i < N; i += kThr) s.bias[i] = bias[i];
    const int row_off = (tid >> 3) * kSBO + (tid & 7) * 16;
    *reinterpret_cast<uint4 *>(s.a + row_off + 9 * kCore) = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        mbar_init(&s.bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s.tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s.tmem;
    const uint32_t b_addr = smem_u32(s.b);
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);

    const int64_t P = F * H * W, ntiles = (P + kM - 1) / kM;
    unsigned phase = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t p = tile * kM + tid;
        gather_row(in, s.a + row_off, p, P, H, W);
        asm volatile("cp.async.wait_all;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();  // the previous tile's tcgen05.ld before the barrier
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const uint32_t a_addr = smem_u32(s.a);
#pragma unroll
            for (int kk = 0; kk < kKC / 2; ++kk)
                tc_mma(tmem, smem_desc(a_addr + kk * 2 * kCore), smem_desc(b_addr + kk * 2 * kCore),
                       instr_desc<N>(), kk > 0 ? 1u : 0u);
            tc_commit(&s.bar);
        }
        const bool ok = mbar_wait(&s.bar, phase);
        // the previous tile's bulk store must have read the staging buffer
        if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(&g_cnn_status, 1u);
            mbar_wait(&s.bar, phase);  // let the MMAs in flight finish (bounded)
            break;
        }
        phase ^= 1u;
        tc_fence_after();
        uint4 *srow = reinterpret_cast<uint4 *>(s.stage) + tid * (N / 8);
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 32) {
            uint32_t r[32];
            tc_ld32(lane_base + (uint32_t)c0, r);
            uint4 *o = srow + c0 / 8;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint32_t w4[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int j = q * 8 + e * 2;
                    float v0 = __uint_as_float(r[j]) + s.bias[c0 + j];
                    float v1 = __uint_as_float(r[j + 1]) + s.bias[c0 + j + 1];
                    if (relu) {
                        v0 = fmaxf(v0, 0.f);
                        v1 = fmaxf(v1, 0.f);
                    }
                    const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
                    w4[e] = *reinterpret_cast<const uint32_t *>(&h);
                }
                o[q] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
            }
        }
        // the staged tile -> global memory in one bulk copy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            const int64_t rows = (P - tile * kM) < kM ? (P - tile * kM) : kM;
            bulk_s2g(out + tile * kM * (N / 8), s.stage, (unsigned)(rows * N * 2));
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");  // no copy may land after the block ends
    if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
}

// Row-segment tiles: a tile is kM = 128 consecutive pixels of one frame row
// (x0 = 128 k; the last segment of a row may be shorter).  One thread
// copies the tile's three input row segments (columns x0 - 1 .. x0 + 128,
// clipped to the frame) into shared memory with bulk copies, two tiles
// ahead (double-buffered, mbarrier-completed); the block then builds the
// im2col rows from shared memory (zeros outside the frame) instead of nine
// gathers per pixel from L2.
constexpr int kRowPx = kM + 2;                 // staged pixels per input row
constexpr int kRowBuf = 3 * kRowPx * 16;       // bytes of one tile's three rows
constexpr int kSmemRows = 74 * 1024;           // 3 blocks per SM

template <int N>
struct alignas(1024) RowSmem {
    uint8_t a[kATile];
    uint8_t b[(N / 8) * kSBO];
    uint8_t stage[kM * N * 2];
    uint8_t rows[2][kRowBuf];
    float bias[N];
    uint64_t rbar[2];  // row copies of buffer 0 / 1
    uint64_t bar;      // MMA completion
    uint32_t tmem;
};

struct RowTile {
    int64_t f, y, x0;
    int nv;  // valid pixels
};

__device__ __forceinline__ RowTile row_tile(int64_t t, int64_t H, int64_t W, int64_t nseg) {
    RowTile r;
    const int64_t sg = t % nseg, fy = t / nseg;
    r.y = fy % H;
    r.f = fy / H;
    r.x0 = sg * kM;
    r.nv = (int)((W - r.x0) < kM ? (W - r.x0) : kM);
    return r;
}

// thread 0: bulk copies of tile t's input rows into rows buffer `buf`
__device__ __forceinline__ void issue_rows(const uint4 *in, uint8_t *rows, uint64_t *bar,
                                          int64_t t, int64_t H, int64_t W, int64_t nseg) {
    const RowTile r = row_tile(t, H, W, nseg);
    const int64_t c0 = r.x0 - 1 < 0 ? 0 : r.x0 - 1;
    const int64_t c1 = (r.x0 + kM + 1) < W ? (r.x0 + kM + 1) : W;  // exclusive
    unsigned bytes = 0;
    for (int dy = 0; dy < 3; ++dy) {
        const int64_t yy = r.y + dy - 1;
        if (yy >= 0 && yy < H) bytes += (unsigned)((c1 - c0) * 16);
    }
    mbar_expect_tx(bar, bytes);
    for (int dy = 0; dy < 3; ++dy) {
        const int64_t yy = r.y + dy - 1;
        if (yy < 0 || yy >= H) continue;
        uint8_t *dst = rows + dy * kRowPx * 16 + (c0 - (r.x0 - 1)) * 16;
        bulk_g2s(dst, in + (r.f * H + yy) * W + c0, (unsigned)((c1 - c0) * 16), bar);
    }
}

template <int N>
__global__ void __launch_bounds__(kThr, 3)
    k_conv_thin_rows(const uint4 *__restrict__ in, const uint4 *__restrict__ wts,
                     const float *__restrict__ bias, uint4 *__restrict__ out, int64_t F,
                     int64_t H, int64_t W, int relu) {
    static_assert(N % 32 == 0 && N >= 32 && N <= 256, "N: multiple of 32 up to 256");
    static_assert(sizeof(RowSmem<N>) + 1024 <= kSmemRows, "shared memory layout too large");
    extern __shared__ uint8_t smem_raw[];
    RowSmem<N> &s = *reinterpret_cast<RowSmem<N> *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    for (int i = tid; i < N * kKC; i += kThr) {
        const int n = i / kKC, kc = i % kKC;
        *reinterpret_cast<uint4 *>(s.b + (n >> 3) * kSBO + kc * kCore + (n & 7) * 16) = wts[i];
    }
    for (int i = tid; i < N; i += kThr) s.bias[i] = bias[i];
    uint8_t *arow = s.a + (tid >> 3) * kSBO + (tid & 7) * 16;
    *reinterpret_cast<uint4 *>(arow + 9 * kCore) = zero;
    const int64_t nseg = (W + kM - 1) / kM, ntiles = F * H * nseg;
    const int64_t G = gridDim.x;
    if (tid == 0) {
        mbar_init(&s.bar, 1);
        mbar_init(s.rbar + 0, 1);
        mbar_init(s.rbar + 1, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int64_t t0 = blockIdx.x;
        if (t0 < ntiles) issue_rows(in, s.rows[0], s.rbar + 0, t0, H, W, nseg);
        if (t0 + G < ntiles) issue_rows(in, s.rows[1], s.rbar + 1, t0 + G, H, W, nseg);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s.tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s.tmem;
    const uint32_t a_addr = smem_u32(s.a), b_addr = smem_u32(s.b);
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    unsigned phase = 0;
    int i = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += G, ++i) {
        const int buf = i & 1;
        const RowTile r = row_tile(t, H, W, nseg);
        const bool rows_ok = mbar_wait(s.rbar + buf, (unsigned)(i >> 1) & 1u);
        if (__syncthreads_or(!rows_ok)) {
            if (tid == 0) {
                atomicOr(&g_cnn_status, 1u);
                mbar_wait(s.rbar + buf, (unsigned)(i >> 1) & 1u);
                if (t + G < ntiles) mbar_wait(s.rbar + (buf ^ 1), (unsigned)((i + 1) >> 1) & 1u);
            }
            break;
        }
        // im2col row of pixel x0 + tid from the staged rows
        const uint4 *rw = reinterpret_cast<const uint4 *>(s.rows[buf]);
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int dy = tap / 3, dx = tap % 3;
            const int64_t yy = r.y + dy - 1, xx = r.x0 - 1 + tid + dx;
            const bool ok = yy >= 0 && yy < H && xx >= 0 && xx < W;
            *reinterpret_cast<uint4 *>(arow + tap * kCore) = ok ? rw[dy * kRowPx + tid + dx] : zero;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();  // the previous tile's tcgen05.ld before the barrier
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            // the rows of this buffer are consumed: refill it two tiles ahead
            if (t + 2 * G < ntiles) issue_rows(in, s.rows[buf], s.rbar + buf, t + 2 * G, H, W, nseg);
#pragma unroll
            for (int kk = 0; kk < kKC / 2; ++kk)
                tc_mma(tmem, smem_desc(a_addr + kk * 2 * kCore), smem_desc(b_addr + kk * 2 * kCore),
                       instr_desc<N>(), kk > 0 ? 1u : 0u);
            tc_commit(&s.bar);
        }
        const bool ok = mbar_wait(&s.bar, phase);
        if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(&g_cnn_status, 1u);
                mbar_wait(&s.bar, phase);
                if (t + G < ntiles) mbar_wait(s.rbar + (buf ^ 1), (unsigned)((i + 1) >> 1) & 1u);
                if (t + 2 * G < ntiles) mbar_wait(s.rbar + buf, (unsigned)((i + 2) >> 1) & 1u);
            }
            break;
        }
        phase ^= 1u;
        tc_fence_after();
        uint4 *srow = reinterpret_cast<uint4 *>(s.stage) + tid * (N / 8);
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 32) {
            uint32_t rr[32];
            tc_ld32(lane_base + (uint32_t)c0, rr);
            uint4 *o = srow + c0 / 8;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint32_t w4[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int j = q * 8 + e * 2;
                    float v0 = __uint_as_float(rr[j]) + s.bias[c0 + j];
                    float v1 = __uint_as_float(rr[j + 1]) + s.bias[c0 + j + 1];
                    if (relu) {
                        v0 = fmaxf(v0, 0.f);
                        v1 = fmaxf(v1, 0.f);
                    }
                    const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
                    w4[e] = *reinterpret_cast<const uint32_t *>(&h);
                }
                o[q] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            const int64_t p0 = (r.f * H + r.y) * W + r.x0;
            bulk_s2g(out + p0 * (N / 8), s.stage, (unsigned)(r.nv * N * 2));
        }
    }
    if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
}

// Row-segment tiles read by the tensor cores in place (k_conv_thin_rd, the
// default): the staged input rows are [row dy][pixel][8 channels], 16 bytes
// per pixel, which is the K-major core-matrix layout of an A operand whose
// rows are consecutive pixels (8 rows of 16 bytes = 128 contiguous bytes,
// 8-row groups 128 bytes apart).  Tap (dy, dx) of output pixel m is staged
// pixel m + dx of row dy, so a pair of taps is one descriptor: start at the
// first tap's pixel 0, leading byte offset = the second tap's distance
// (16 bytes within a row, or a row minus 32 bytes from dx = 2 to the next
// row's dx = 0).  The five MMAs take taps (0,1), (2,3), (4,5), (6,7) and
// (7,8), the weights of the last pair being (zero, tap 8), so no read
// leaves the tile's three rows and no im2col copy is built.  Pixels outside
// the frame are zeroed in the staged rows before the MMAs (the bulk copies
// skip them); a buffer is refilled, two tiles ahead, once its MMAs are done.
constexpr int kRowStride = kRowPx * 16;   // bytes of one staged row
constexpr int kSmemRd = 56 * 1024;        // 4 blocks per SM

template <int N>
struct alignas(1024) RdSmem {
    uint8_t b[(N / 8) * kSBO];  // weights, K chunks (tap 0..7, zero, tap 8)
    alignas(1024) uint8_t stage[kM * N * 2];
    uint8_t rows[2][kRowBuf];
    alignas(16) float bias[N];
    uint64_t rbar[2];
    uint64_t bar;
    uint32_t tmem;
};

// Output tile staged for tensor stores (TM): boxes of 64 channels (128-byte
// pixel rows, 128-byte swizzle: 16-byte chunk k of pixel t at chunk
// k ^ (t & 7)) and, when N % 64 == 32, one box of 32 channels (64-byte
// rows, 64-byte swizzle: chunk k ^ ((t >> 1) & 3)).  Either way the eight
// pixels of a quarter warp write eight different 16-byte bank groups; the
// plain pixel-major stage (N * 2 bytes per pixel) puts them on two.
template <int N>
__device__ __forceinline__ uint32_t stage_off(int kc, int t) {
    constexpr int nA = N / 64;
    if (kc < 8 * nA)
        return (uint32_t)((kc >> 3) * 16384 + t * 128 + (((kc & 7) ^ (t & 7)) << 4));
    return (uint32_t)(nA * 16384 + t * 64 + (((kc - 8 * nA) ^ ((t >> 1) & 3)) << 4));
}

__device__ __forceinline__ void tma_store3(const CUtensorMap *m, const void *src, int c, int x,
                                           int row) {
    asm volatile(
        "cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
            reinterpret_cast<uint64_t>(m)),
        "r"(c), "r"(x), "r"(row), "r"(smem_u32(src))
        : "memory");
}

// Descriptor with explicit leading / stride byte offsets (no swizzle).
__device__ __forceinline__ uint64_t smem_desc_lbo(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

template <int N, bool TM>
__global__ void __launch_bounds__(kThr, 4)
    k_conv_thin_rd(const uint4 *__restrict__ in, const uint4 *__restrict__ wts,
                   const float *__restrict__ bias, uint4 *__restrict__ out, int64_t F,
                   int64_t H, int64_t W, int relu, const __grid_constant__ CUtensorMap tm64,
                   const __grid_constant__ CUtensorMap tm32) {
    static_assert(N % 32 == 0 && N >= 32 && N <= 256, "N: multiple of 32 up to 256");
    static_assert(sizeof(RdSmem<N>) + 1024 <= kSmemRd, "shared memory layout too large");
    extern __shared__ uint8_t smem_raw[];
    RdSmem<N> &s = *reinterpret_cast<RdSmem<N> *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    // weights: chunk 8 (zeros) and chunk 9 (tap 8) change places
    for (int i = tid; i < N * kKC; i += kThr) {
        const int n = i / kKC, kc = i % kKC;
        const int dkc = kc == 8 ? 9 : (kc == 9 ? 8 : kc);
        *reinterpret_cast<uint4 *>(s.b + (n >> 3) * kSBO + dkc * kCore + (n & 7) * 16) = wts[i];
    }
    for (int i = tid; i < N; i += kThr) s.bias[i] = bias[i];
    const int64_t nseg = (W + kM - 1) / kM, ntiles = F * H * nseg;
    const int64_t G = gridDim.x;
    if (tid == 0) {
        mbar_init(&s.bar, 1);
        mbar_init(s.rbar + 0, 1);
        mbar_init(s.rbar + 1, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int64_t t0 = blockIdx.x;
        if (t0 < ntiles) issue_rows(in, s.rows[0], s.rbar + 0, t0, H, W, nseg);
        if (t0 + G < ntiles) issue_rows(in, s.rows[1], s.rbar + 1, t0 + G, H, W, nseg);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s.tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s.tmem;
    const uint32_t b_addr = smem_u32(s.b);
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    // (first tap's byte offset in the staged rows, leading byte offset) of the five MMAs
    constexpr uint32_t a_off[5] = {0u, 32u, (uint32_t)kRowStride + 16u, 2u * kRowStride,
                                   2u * kRowStride + 16u};
    constexpr uint32_t a_lbo[5] = {16u, (uint32_t)kRowStride - 32u, 16u, 16u, 16u};
    unsigned phase = 0;
    int i = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += G, ++i) {
        const int buf = i & 1;
        const RowTile r = row_tile(t, H, W, nseg);
        const bool rows_ok = mbar_wait(s.rbar + buf, (unsigned)(i >> 1) & 1u);
        if (__syncthreads_or(!rows_ok)) {
            if (tid == 0) {
                atomicOr(&g_cnn_status, 1u);
                mbar_wait(s.rbar + buf, (unsigned)(i >> 1) & 1u);
                if (t + G < ntiles) mbar_wait(s.rbar + (buf ^ 1), (unsigned)((i + 1) >> 1) & 1u);
            }
            break;
        }
        // zeros for the staged pixels outside the frame: whole rows above or
        // below it, column x0 - 1 of the first segment, columns >= W of the last
        {
            uint4 *rw = reinterpret_cast<uint4 *>(s.rows[buf]);
            const int px_hi = (int)((W - (r.x0 - 1)) < kRowPx ? (W - (r.x0 - 1)) : kRowPx);
#pragma unroll
            for (int dy = 0; dy < 3; ++dy) {
                const int64_t yy = r.y + dy - 1;
                if (yy < 0 || yy >= H) {
                    for (int px = tid; px < kRowPx; px += kThr) rw[dy * kRowPx + px] = zero;
                } else {
                    if (r.x0 == 0 && tid == 0) rw[dy * kRowPx] = zero;
                    for (int px = px_hi + tid; px < kRowPx; px += kThr) rw[dy * kRowPx + px] = zero;
                }
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();  // the previous tile's tcgen05.ld before the barrier
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const uint32_t rows_addr = smem_u32(s.rows[buf]);
#pragma unroll
            for (int kk = 0; kk < kKC / 2; ++kk)
                tc_mma(tmem, smem_desc_lbo(rows_addr + a_off[kk], a_lbo[kk], 128u),
                       smem_desc(b_addr + kk * 2 * kCore), instr_desc<N>(), kk > 0 ? 1u : 0u);
            tc_commit(&s.bar);
        }
        const bool ok = mbar_wait(&s.bar, phase);
        if (tid == 0) {
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
            // this buffer's MMAs are done: refill it two tiles ahead
            if (ok && t + 2 * G < ntiles)
                issue_rows(in, s.rows[buf], s.rbar + buf, t + 2 * G, H, W, nseg);
        }
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(&g_cnn_status, 1u);
                mbar_wait(&s.bar, phase);
                if (t + G < ntiles) mbar_wait(s.rbar + (buf ^ 1), (unsigned)((i + 1) >> 1) & 1u);
            }
            break;
        }
        phase ^= 1u;
        tc_fence_after();
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 32) {
            uint32_t rr[32];
            tc_ld32(lane_base + (uint32_t)c0, rr);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 *b4 = reinterpret_cast<const float4 *>(s.bias + c0 + q * 8);
                const float4 ba = b4[0], bb = b4[1];
                const float bv[8] = {ba.x, ba.y, ba.z, ba.w, bb.x, bb.y, bb.z, bb.w};
                uint32_t w4[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int j = q * 8 + e * 2;
                    float v0 = __uint_as_float(rr[j]) + bv[2 * e];
                    float v1 = __uint_as_float(rr[j + 1]) + bv[2 * e + 1];
                    if (relu) {
                        v0 = fmaxf(v0, 0.f);
                        v1 = fmaxf(v1, 0.f);
                    }
                    const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
                    w4[e] = *reinterpret_cast<const uint32_t *>(&h);
                }
                const int kc = c0 / 8 + q;
                const uint32_t off = TM ? stage_off<N>(kc, tid) : (uint32_t)(tid * N * 2 + kc * 16);
                *reinterpret_cast<uint4 *>(s.stage + off) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            if (TM) {
                const int row = (int)(r.f * H + r.y), x = (int)r.x0;
#pragma unroll
                for (int i = 0; i < N / 64; ++i) tma_store3(&tm64, s.stage + i * 16384, i * 64, x, row);
                if (N % 64) tma_store3(&tm32, s.stage + (N / 64) * 16384, (N / 64) * 64, x, row);
                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            } else {
                const int64_t p0 = (r.f * H + r.y) * W + r.x0;
                bulk_s2g(out + p0 * (N / 8), s.stage, (unsigned)(r.nv * N * 2));
            }
        }
    }
    if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
}

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn tensor_map_encoder() {
    static const EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// Tensor map of the NHWC bf16 output: dims (N channels, W, F H rows), box
// (bc channels, 128 pixels, 1 row), swizzle matching stage_off; pixels past
// the row end of a tile are clipped by the store.
static bool out_map(CUtensorMap *m, void *out, int64_t F, int64_t H, int64_t W, int N, int bc) {
    const EncodeTiledFn enc = tensor_map_encoder();
    if (!enc || F * H > INT32_MAX || W > INT32_MAX) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)N, (cuuint64_t)W, (cuuint64_t)(F * H)};
    const cuuint64_t strides[2] = {(cuuint64_t)N * 2, (cuuint64_t)W * (cuuint64_t)N * 2};
    const cuuint32_t box[3] = {(cuuint32_t)bc, (cuuint32_t)kM, 1u};
    const cuuint32_t es[3] = {1u, 1u, 1u};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, out, dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE,
               bc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
               CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// SCI_THIN_TMA=0: the staged tile written by one plain bulk copy (pixel-major
// stage) instead of swizzled tensor stores.
static bool thin_tma() {
    static const bool v = [] {
        const char *e = getenv("SCI_THIN_TMA");
        return !(e && atoi(e) == 0);
    }();
    return v;
}

template <int N>
int launch_rd(const void *in, const void *wts, const float *bias, void *out, int64_t F,
              int64_t H, int64_t W, int relu, cudaStream_t st) {
    const int64_t ntiles = F * H * ((W + kM - 1) / kM);
    const int64_t cap = int64_t(kSMs) * 4;
    const int grid = int(ntiles < cap ? ntiles : cap);
    CUtensorMap m64, m32;
    memset(&m64, 0, sizeof(m64));
    memset(&m32, 0, sizeof(m32));
    bool tm = thin_tma() && out_map(&m64, out, F, H, W, N, 64);
    if (tm && N % 64) tm = out_map(&m32, out, F, H, W, N, 32);
    auto go = [&](auto kern) -> int {
        SCI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemRd));
        kern<<<grid, kThr, kSmemRd, st>>>(reinterpret_cast<const uint4 *>(in),
                                          reinterpret_cast<const uint4 *>(wts), bias,
                                          reinterpret_cast<uint4 *>(out), F, H, W, relu, m64, m32);
        return SCI_OK;
    };
    const int rc = tm ? go(k_conv_thin_rd<N, true>) : go(k_conv_thin_rd<N, false>);
    if (rc != SCI_OK) return rc;
    SCI_LAUNCHED("k_conv_thin_rd");
    return SCI_OK;
}

template <int N>
int launch_rows(const void *in, const void *wts, const float *bias, void *out, int64_t F,
                int64_t H, int64_t W, int relu, cudaStream_t st) {
    const int64_t ntiles = F * H * ((W + kM - 1) / kM);
    const int64_t cap = int64_t(kSMs) * 3;
    const int grid = int(ntiles < cap ? ntiles : cap);
    SCI_CUDA(cudaFuncSetAttribute(k_conv_thin_rows<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kSmemRows));
    k_conv_thin_rows<N><<<grid, kThr, kSmemRows, st>>>(
        reinterpret_cast<const uint4 *>(in), reinterpret_cast<const uint4 *>(wts), bias,
        reinterpret_cast<uint4 *>(out), F, H, W, relu);
    SCI_LAUNCHED("k_conv_thin_rows");
    return SCI_OK;
}

template <int N>
int launch_thin(const void *in, const void *wts, const float *bias, void *out, int64_t F,
                int64_t H, int64_t W, int relu, cudaStream_t st) {
    const int64_t ntiles = (F * H * W + kM - 1) / kM;
    const int64_t cap = int64_t(kSMs) * 3;
    const int grid = int(ntiles < cap ? ntiles : cap);
    SCI_CUDA(cudaFuncSetAttribute(k_conv_thin_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kSmemBytes));
    k_conv_thin_tc<N><<<grid, kThr, kSmemBytes, st>>>(
        reinterpret_cast<const uint4 *>(in), reinterpret_cast<const uint4 *>(wts), bias,
        reinterpret_cast<uint4 *>(out), F, H, W, relu);
    SCI_LAUNCHED("k_conv_thin_tc");
    return SCI_OK;
}

// ------------------------------------------------------- DenBlock tail
// FastDVDnet's DenBlock after its last upsampling convolution, one pass per
// column strip of a frame (packages/fastdvdnet/models.py:86-100, :203-205):
//   h  = x0 + PixelShuffle(2)(u1)                    32 channels, bfloat16
//   o0 = ReLU(conv3x3(h, w0) + b0)                   32 -> 32, bfloat16
//   e  = conv3x3(o0, w1) + b1                        32 -> 1, float32
//   out = centre frame - e  (cropped, clipped)       float32 planes
// Rows stream through shared memory top to bottom: per row step the x0
// row and the u1 half row are loaded by TMA (one step ahead) and summed
// into an h row, and one batch of MMAs computes an o0 row and the output
// row two rows above it (implicit GEMMs, M = 128 pixels, K = 9 taps x 32
// channels = 18 MMAs of K 16 each, float32 accumulators in TMEM), reading
// rings of three h rows and four o0 rows in place through tap-shifted
// descriptors, as k_conv_thin_rd does; the centre pixels are loaded while
// the batch runs.  A staged row holds 130
// pixels as four 8-channel planes (pixel p of plane j at j * 2080 + 16 p:
// the K-major core-matrix layout, K-adjacent chunks one plane apart).  o0
// is computed for the strip's 126 output columns plus one on each side
// (128 = one MMA tile); o0 values outside the frame are zero (the zero
// padding of the second convolution).  Waits are bounded as in the thin
// convolution.
constexpr int kTailSeg = 126;                    // output columns per strip
constexpr int kTailPx = 130;                     // staged h pixels per row
constexpr int kTailPlane = kTailPx * 16;         // one 8-channel plane of a row
constexpr int kTailRow = 4 * kTailPlane;         // 32 channels
constexpr int kTailKC = 36;                      // 16-byte K chunks of a 3 x 3 x 32 filter
constexpr int kTailSBO = kTailKC * kCore;        // 8-row groups of a weight operand
constexpr int kTailTmem = 128;  // o0 accumulators at columns 0-31, 32-63; e at 64-79, 96-111
constexpr unsigned kTailLoad = kTailPx * 64 + 65 * 128;  // bytes of one row's two TMA boxes

struct alignas(1024) TailSmem {
    uint8_t sx[kTailPx * 64];              // x0 row: 130 px x 32 ch, 64-byte swizzle
    alignas(1024) uint8_t su[65 * 128];    // u1 half row: 65 px x 64 ch, 128-byte swizzle
    alignas(16) uint8_t h[4][kTailRow];
    alignas(16) uint8_t o[4][kTailRow];
    alignas(16) uint8_t w0[4 * kTailSBO];  // 32 filters
    // the output filter per row dy as 16 x 32 operands: filter n = 3 dy + dx
    // holds tap (dy, dx), the others zero, so the three rows' MMAs
    // accumulate D[m, 3 dy + dx] = sum_c o0(dy)[m, c] w1(dy, dx)[c]
    alignas(16) uint8_t w1[3][2 * 4 * kCore];
    float esum[3][kTailPx + 2];  // per dx: sum_dy D[m, 3 dy + dx]
    alignas(16) float b0[32];
    float b1;
    uint64_t lbar, abar[2], bbar[2];
    uint32_t tmem;
};
constexpr int kSmemTail = (int)sizeof(TailSmem) + 1024;
static_assert(kSmemTail <= 112 * 1024, "k_den_tail: two blocks per SM");


__device__ __forceinline__ void tma_load4(void *dst, const CUtensorMap *m, int c0, int c1, int c2,
                                          int c3, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
        "{%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(m)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
        "r"(smem_u32(bar))
        : "memory");
}

struct TailGeo {
    int64_t count, Hp, Wp, Ho, Wo, Hs, Ws, first;
    int nseg, nchunk, R;
};

struct TailUnit {
    int f, xs, ya, yb;
};

__device__ __forceinline__ TailUnit tail_unit(const TailGeo &g, int64_t u) {
    TailUnit t;
    const int64_t per_f = (int64_t)g.nseg * g.nchunk;
    t.f = (int)(u / per_f);
    const int rem = (int)(u - (int64_t)t.f * per_f);
    const int c = rem / g.nseg, sg = rem - c * g.nseg;
    t.xs = sg * kTailSeg;
    t.ya = c * g.R;
    t.yb = (int)((int64_t)(t.ya + g.R) < g.Ho ? (t.ya + g.R) : g.Ho);
    return t;
}

// thread 0: the TMA boxes of h row `hrow` of strip `t` (rows and columns
// outside the tensors read as zeros)
__device__ __forceinline__ void tail_issue(TailSmem &s, const CUtensorMap *mx,
                                           const CUtensorMap *mu, const TailUnit &t, int hrow) {
    mbar_expect_tx(&s.lbar, kTailLoad);
    tma_load4(s.sx, mx, 0, t.xs - 2, hrow, t.f, &s.lbar);
    tma_load4(s.su, mu, 64 * (hrow & 1), (t.xs - 2) >> 1, hrow >> 1, t.f, &s.lbar);
}

__device__ __forceinline__ uint4 add8_bf16(uint4 x, uint4 y) {
    uint4 r;
    const uint32_t *px = reinterpret_cast<const uint32_t *>(&x);
    const uint32_t *py = reinterpret_cast<const uint32_t *>(&y);
    uint32_t *pr = reinterpret_cast<uint32_t *>(&r);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const __nv_bfloat162 a = *reinterpret_cast<const __nv_bfloat162 *>(px + q);
        const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162 *>(py + q);
        const __nv_bfloat162 c = __floats2bfloat162_rn(__low2float(a) + __low2float(b),
                                                       __high2float(a) + __high2float(b));
        pr[q] = *reinterpret_cast<const uint32_t *>(&c);
    }
    return r;
}

// One row of the 3 x 3, 32 -> 32 convolution: 18 MMAs over the ring rows
// r0, r1, r2 (dy = 0, 1, 2), accumulator at TMEM address `tmem`.
__device__ __forceinline__ void tail_mma(uint32_t tmem, const uint8_t *r0, const uint8_t *r1,
                                         const uint8_t *r2, const uint8_t *w) {
    const uint8_t *rows[3] = {r0, r1, r2};
    const uint32_t wb = smem_u32(w);
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
        const uint32_t ra = smem_u32(rows[dy]);
#pragma unroll
        for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int tap = 3 * dy + dx;
                const uint64_t a = smem_desc_lbo(ra + (uint32_t)(2 * q * kTailPlane + dx * 16),
                                                 (uint32_t)kTailPlane, 128u);
                const uint64_t b = smem_desc_lbo(wb + (uint32_t)((tap * 4 + 2 * q) * kCore),
                                                 (uint32_t)kCore, (uint32_t)kTailSBO);
                tc_mma(tmem, a, b, instr_desc<32>(), (tap | q) ? 1u : 0u);
            }
    }
}

constexpr int kTailThr = kThr + 32;  // 4 worker warps (TMEM lanes 0-127) + the issuing warp

// The output convolution with its taps folded into N: per row dy two MMAs
// (K = 32 channels) of the unshifted o0 row against the row's three taps;
// the column shifts are applied in the epilogue.
__device__ __forceinline__ void tail_mma_fold(uint32_t tmem, const uint8_t *r0, const uint8_t *r1,
                                              const uint8_t *r2, const uint8_t (*w)[2 * 4 * kCore]) {
    const uint8_t *rows[3] = {r0, r1, r2};
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const uint64_t a = smem_desc_lbo(smem_u32(rows[dy]) + (uint32_t)(2 * q * kTailPlane),
                                             (uint32_t)kTailPlane, 128u);
            const uint64_t b = smem_desc_lbo(smem_u32(w[dy]) + (uint32_t)(2 * q * kCore),
                                             (uint32_t)kCore, (uint32_t)(4 * kCore));
            tc_mma(tmem, a, b, instr_desc<16>(), (dy | q) ? 1u : 0u);
        }
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(kTailThr, 2)
    k_den_tail(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap mu,
               const uint4 *__restrict__ w0, const float *__restrict__ b0,
               const uint4 *__restrict__ w1, const float *__restrict__ b1,
               const float *__restrict__ src, float *__restrict__ out, TailGeo g, int clip) {
    extern __shared__ uint8_t smem_raw[];
    TailSmem &s = *reinterpret_cast<TailSmem *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5;
    const bool worker = warp < 4, issuer = tid == kThr;  // issuer: lane 0 of warp 4
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    // filters as K-major core matrices: filter n, K chunk kc (tap * 4 + j)
    for (int i = tid; i < 32 * kTailKC; i += kTailThr) {
        const int n = i / kTailKC, kc = i % kTailKC;
        *reinterpret_cast<uint4 *>(s.w0 + (n >> 3) * kTailSBO + kc * kCore + (n & 7) * 16) = w0[i];
    }
    for (int i = tid; i < 3 * 16 * 4; i += kTailThr) {
        const int dy = i / 64, n = (i / 4) % 16, kc = i % 4;
        *reinterpret_cast<uint4 *>(s.w1[dy] + (n >> 3) * 4 * kCore + kc * kCore + (n & 7) * 16) =
            (n < 9 && n / 3 == dy) ? w1[n * 4 + kc] : zero;
    }
    for (int i = tid; i < 3 * 4; i += kTailThr) s.esum[i / 4][kTailPx - 2 + i % 4] = 0.f;
    for (int i = tid; i < 32; i += kTailThr) s.b0[i] = b0[i];
    if (tid == 0) s.b1 = b1 ? b1[0] : 0.f;
    // o0 ring pixels 128, 129 are read only by the strip's two unused MMA rows
    for (int i = tid; i < 4 * 4 * 2; i += kTailThr)
        *reinterpret_cast<uint4 *>(s.o[i / 8] + ((i / 2) % 4) * kTailPlane + (128 + i % 2) * 16) =
            zero;
    const int64_t nunits = g.count * g.nseg * g.nchunk, G = gridDim.x;
    if (tid == 0) {
        mbar_init(&s.lbar, 1);
        for (int i = 0; i < 2; ++i) {
            mbar_init(s.abar + i, 1);
            mbar_init(s.bbar + i, 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if ((int64_t)blockIdx.x < nunits) {
            const TailUnit t0 = tail_unit(g, blockIdx.x);
            tail_issue(s, &mx, &mu, t0, t0.ya - 2);
        }
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s.tmem)),
                     "r"(kTailTmem)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s.tmem;
    const uint32_t lane = (uint32_t)(warp * 32) << 16;
    // phase bits of the load barrier and of the two o0 / e barriers, and the
    // loads / commits not yet waited for (flipped and cleared only once a
    // step's barrier shows every wait succeeded, so that a block giving up
    // drains exactly what is still in flight)
    unsigned lphase = 0, aph = 0, bph = 0, apend = 0, bpend = 0;
    bool lpend = (int64_t)blockIdx.x < nunits;  // the prologue's load
    bool failed = false;
    for (int64_t u = blockIdx.x; u < nunits && !failed; u += G) {
        const TailUnit t = tail_unit(g, u);
        // Step k (KH = yb - ya + 3):
        //   A  (0 <= k <= KH)      h row ya - 2 + k from the staged rows
        //   B  (2 <= k <= KH)      MMAs of o0 row ya - 3 + k into o0 buffer k & 1
        //   C  (3 <= k <= KH + 1)  epilogue of o0 row ya - 4 + k (buffer (k - 1) & 1)
        //      (6 <= k <= KH + 2)  epilogue of output row ya + k - 6 (buffer (k - 1) & 1)
        //   D  (5 <= k <= KH + 1)  MMAs of output row ya + k - 5 into e buffer k & 1
        // so each batch of MMAs runs while the block forms the next h row and
        // the epilogue of the previous batch.
        const int KH = (t.yb - t.ya) + 3;
        for (int k = 0; k <= KH + 2; ++k) {
            const int x = t.xs + tid, y = t.ya + k - 6;
            const bool store = k >= 6 && tid < kTailSeg && x < g.Wo;
            float cen = 0.f;
            if (store) {  // the centre pixel, loaded while the step runs
                const int64_t gi = g.first + t.f;
                const int64_t yi = y < g.Hs ? y : 2 * (g.Hs - 1) - y;
                const int64_t xi = x < g.Ws ? x : 2 * (g.Ws - 1) - x;
                cen = __ldg(src + (gi * g.Hs + (yi < 0 ? 0 : yi)) * g.Ws + (xi < 0 ? 0 : xi));
            }
            // A (workers; the issuer is meanwhile issuing the previous step's D)
            bool ok = true;
            if (k <= KH) {
                if (worker) {
                    ok = mbar_wait(&s.lbar, lphase);
                    uint8_t *hr = s.h[k & 3];
                    for (int p = tid; p < kTailPx; p += kThr) {
                        const int q = p >> 1, b = p & 1;
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const uint4 xv = *reinterpret_cast<const uint4 *>(
                                s.sx + p * 64 + ((j ^ ((p >> 1) & 3)) << 4));
                            const uint4 uv = *reinterpret_cast<const uint4 *>(
                                s.su + q * 128 + (((4 * b + j) ^ (q & 7)) << 4));
                            *reinterpret_cast<uint4 *>(hr + j * kTailPlane + p * 16) =
                                add8_bf16(xv, uv);
                        }
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                }
            }
            tc_fence_before();
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            tc_fence_after();
            if (k <= KH) {
                lphase ^= 1u;
                // the next row's boxes, into the stage just consumed
                lpend = k + 1 <= KH || u + G < nunits;
            }
            if (k >= 2 && k <= KH) apend |= 1u << (k & 1);
            if (issuer && k <= KH) {  // the next row's boxes; B
                if (k + 1 <= KH) {
                    tail_issue(s, &mx, &mu, t, t.ya - 1 + k);
                } else if (u + G < nunits) {
                    const TailUnit tn = tail_unit(g, u + G);
                    tail_issue(s, &mx, &mu, tn, tn.ya - 2);
                }
                if (k >= 2) {
                    tail_mma(tmem + 32u * (k & 1), s.h[(k - 2) & 3], s.h[(k - 1) & 3],
                             s.h[k & 3], s.w0);
                    tc_commit(s.abar + (k & 1));
                }
            }
            // C (workers)
            if (k >= 3 && k <= KH + 1) {
                const int bi = (k - 1) & 1;
                if (worker) {
                    ok = mbar_wait(s.abar + bi, (aph >> bi) & 1u);
                    tc_fence_after();
                    uint32_t rr[32];
                    tc_ld32(tmem + lane + 32u * bi, rr);
                    const int orow = t.ya + k - 4, xo = t.xs - 1 + tid;  // this thread's o0 column
                    const bool inside = orow >= 0 && orow < g.Hp && xo >= 0 && xo < g.Wp;
                    uint8_t *orw = s.o[(k - 1) & 3];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float4 *b4 = reinterpret_cast<const float4 *>(s.b0 + j * 8);
                        const float4 ba = b4[0], bb = b4[1];
                        const float bv[8] = {ba.x, ba.y, ba.z, ba.w, bb.x, bb.y, bb.z, bb.w};
                        uint32_t w4[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int c = j * 8 + 2 * e;
                            float v0 = fmaxf(__uint_as_float(rr[c]) + bv[2 * e], 0.f);
                            float v1 = fmaxf(__uint_as_float(rr[c + 1]) + bv[2 * e + 1], 0.f);
                            if (!inside) v0 = v1 = 0.f;
                            const __nv_bfloat162 hb = __floats2bfloat162_rn(v0, v1);
                            w4[e] = *reinterpret_cast<const uint32_t *>(&hb);
                        }
                        *reinterpret_cast<uint4 *>(orw + j * kTailPlane + tid * 16) =
                            make_uint4(w4[0], w4[1], w4[2], w4[3]);
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                }
            }
            if (k >= 6) {
                const int bi = (k - 1) & 1;
                if (worker) {
                    ok = mbar_wait(s.bbar + bi, (bph >> bi) & 1u) && ok;
                    tc_fence_after();
                    uint32_t d[16];
                    tc_ld16(tmem + lane + 64u + 32u * bi, d);
#pragma unroll
                    for (int dx = 0; dx < 3; ++dx)
                        s.esum[dx][tid] = __uint_as_float(d[dx]) + __uint_as_float(d[3 + dx]) +
                                          __uint_as_float(d[6 + dx]);
                    asm volatile("bar.sync 1, 128;" ::: "memory");  // the four worker warps
                    const float ev = s.esum[0][tid] + s.esum[1][tid + 1] + s.esum[2][tid + 2];
                    if (store) {
                        float v = cen - (ev + s.b1);
                        if (clip) v = fminf(fmaxf(v, 0.f), 1.f);
                        out[((int64_t)t.f * g.Ho + y) * g.Wo + x] = v;
                    }
                }
            }
            tc_fence_before();
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            tc_fence_after();
            if (k >= 3 && k <= KH + 1) {  // C's o0 batch waited for
                aph ^= 1u << ((k - 1) & 1);
                apend &= ~(1u << ((k - 1) & 1));
            }
            if (k >= 6) {  // and the e batch
                bph ^= 1u << ((k - 1) & 1);
                bpend &= ~(1u << ((k - 1) & 1));
            }
            if (k >= 5 && k <= KH + 1) {  // D: output row ya + k - 5 from o0 rows ya + k - 6 ..
                if (issuer) {
                    tail_mma_fold(tmem + 64u + 32u * (k & 1), s.o[(k - 3) & 3], s.o[(k - 2) & 3],
                                  s.o[(k - 1) & 3], s.w1);
                    tc_commit(s.bbar + (k & 1));
                }
                bpend |= 1u << (k & 1);
            }
        }
    }
    if (failed && tid == 0) {
        atomicOr(&g_cnn_status, 1u);
        // let the copies and MMAs in flight land before the block ends
        if (lpend) mbar_wait(&s.lbar, lphase);
        for (int i = 0; i < 2; ++i) {
            if ((apend >> i) & 1u) mbar_wait(s.abar + i, (aph >> i) & 1u);
            if ((bpend >> i) & 1u) mbar_wait(s.bbar + i, (bph >> i) & 1u);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTailTmem)
                     : "memory");
}

// Row-segment tiles with bulk-copied input rows (k_conv_thin_rows): 1.84 ms
// for 8 x 2048 x 2048 -> 96 channels against 1.99 ms for the per-pixel
// gather (SCI_THIN_ROWS=0); the gather with a second A buffer and the next
// tile's copies in flight (2 blocks per SM) measured 2.37 ms.
// SCI_THIN_ROWS: 2 (the default) the staged rows read in place by the
// MMAs, 1 the im2col rows built from the staged rows, 0 the per-pixel
// gather.
template <int N>
int launch_thin_n(const void *in, const void *wts, const float *bias, void *out, int64_t F,
                  int64_t H, int64_t W, int relu, cudaStream_t st) {
    static const int form = [] {
        const char *e = getenv("SCI_THIN_ROWS");
        return e ? atoi(e) : 2;
    }();
    if (form >= 2) return launch_rd<N>(in, wts, bias, out, F, H, W, relu, st);
    if (form == 1) return launch_rows<N>(in, wts, bias, out, F, H, W, relu, st);
    return launch_thin<N>(in, wts, bias, out, F, H, W, relu, st);
}

// Tensor map over a bfloat16 tensor of `rank` dims (innermost first; byte
// strides of dims 1..rank-1), the box `box`, 64- or 128-byte swizzle.
static bool encode_map(CUtensorMap *m, const void *base, int rank, const cuuint64_t *dims,
                       const cuuint64_t *strides, const cuuint32_t *box, int swizzle_bytes) {
    const EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint32_t es[5] = {1u, 1u, 1u, 1u, 1u};
    const CUtensorMapSwizzle sw =
        swizzle_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void *>(base),
               dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

// Rows per strip of k_den_tail: the fewest whole waves of strips times the
// row steps each strip takes (its rows plus 6).  SCI_TAIL_ROWS overrides.
static int tail_rows(int64_t count, int nseg, int64_t Ho, int slots) {
    if (const char *e = getenv("SCI_TAIL_ROWS")) {
        const int v = atoi(e);
        if (v >= 8) return v;
    }
    int best = 64;
    int64_t best_cost = INT64_MAX;
    for (int R = 32; R <= 256; R += 8) {
        const int64_t units = count * nseg * ((Ho + R - 1) / R);
        const int64_t waves = (units + slots - 1) / slots;
        const int64_t cost = waves * (int64_t)(R + 6);
        if (cost < best_cost) best_cost = cost, best = R;
    }
    return best;
}

int launch_den_tail(const void *x0, const void *u1, const void *w0, const float *b0,
                    const void *w1, const float *b1, const float *src, int64_t Hs, int64_t Ws,
                    int64_t first, int64_t count, int64_t Hp, int64_t Wp, int64_t Ho, int64_t Wo,
                    int clip, float *out, cudaStream_t st) {
    CUtensorMap mx, mu;
    {
        const cuuint64_t dims[4] = {32, (cuuint64_t)Wp, (cuuint64_t)Hp, (cuuint64_t)count};
        const cuuint64_t str[3] = {64, (cuuint64_t)Wp * 64, (cuuint64_t)(Hp * Wp * 64)};
        const cuuint32_t box[4] = {32, (cuuint32_t)kTailPx, 1, 1};
        if (!encode_map(&mx, x0, 4, dims, str, box, 64)) {
            set_error("sci_cnn_den_tail: tensor map of x0 refused");
            return SCI_ERR_CUDA;
        }
    }
    {
        const int64_t h2 = Hp / 2, w2 = Wp / 2;
        const cuuint64_t dims[4] = {128, (cuuint64_t)w2, (cuuint64_t)h2, (cuuint64_t)count};
        const cuuint64_t str[3] = {256, (cuuint64_t)w2 * 256, (cuuint64_t)(h2 * w2 * 256)};
        const cuuint32_t box[4] = {64, 65, 1, 1};
        if (!encode_map(&mu, u1, 4, dims, str, box, 128)) {
            set_error("sci_cnn_den_tail: tensor map of u1 refused");
            return SCI_ERR_CUDA;
        }
    }
    TailGeo g;
    g.count = count, g.Hp = Hp, g.Wp = Wp, g.Ho = Ho, g.Wo = Wo, g.Hs = Hs, g.Ws = Ws;
    g.first = first;
    g.nseg = (int)((Wo + kTailSeg - 1) / kTailSeg);
    const int slots = kSMs * 2;
    g.R = tail_rows(count, g.nseg, Ho, slots);
    g.nchunk = (int)((Ho + g.R - 1) / g.R);
    const int64_t units = count * g.nseg * g.nchunk;
    const int grid = (int)(units < slots ? units : slots);
    SCI_CUDA(cudaFuncSetAttribute(k_den_tail, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kSmemTail));
    k_den_tail<<<grid, kTailThr, kSmemTail, st>>>(mx, mu, reinterpret_cast<const uint4 *>(w0), b0,
                                              reinterpret_cast<const uint4 *>(w1), b1, src, out,
                                              g, clip);
    SCI_LAUNCHED("k_den_tail");
    return SCI_OK;
}

}  // namespace

namespace cnn {
unsigned cnn_device_status(int clear) {
    unsigned v = 0;
    cudaMemcpyFromSymbol(&v, g_cnn_status, sizeof(v));
    if (clear) {
        const unsigned z = 0;
        cudaMemcpyToSymbol(g_cnn_status, &z, sizeof(z));
    }
    return v;
}
}  // namespace cnn
}  // namespace sci

using namespace sci;

extern "C" int sci_cnn_conv_thin(const void *in, const void *weights, const float *bias,
                                 void *out, int64_t nframes, int64_t H, int64_t W, int N,
                                 int relu, void *stream) {
    SCI_CHECK_ARG(in && weights && bias && out, "sci_cnn_conv_thin: null pointer");
    SCI_CHECK_ARG(nframes >= 1 && H >= 1 && W >= 1, "sci_cnn_conv_thin: invalid sizes");
    SCI_CHECK_ARG(nframes * H * W <= (int64_t(1) << 40), "sci_cnn_conv_thin: too many pixels");
    SCI_CHECK_ARG(aligned16(in) && aligned16(weights) && aligned16(out),
                  "sci_cnn_conv_thin: in, weights and out must be 16-byte aligned");
    const cudaStream_t st = as_stream(stream);
    switch (N) {
        case 64: return launch_thin_n<64>(in, weights, bias, out, nframes, H, W, relu, st);
        case 96: return launch_thin_n<96>(in, weights, bias, out, nframes, H, W, relu, st);
        default:
            set_error("sci_cnn_conv_thin: N = %d (64 or 96)", N);
            return SCI_ERR_UNSUPPORTED;
    }
}

extern "C" int sci_cnn_den_tail(const void *x0, const void *u1, const void *w0, const float *b0,
                                const void *w1, const float *b1, const float *src,
                                int64_t nframes, int64_t Hs, int64_t Ws, int64_t first,
                                int64_t count, int64_t Hp, int64_t Wp, int64_t Ho, int64_t Wo,
                                int clip, float *out, void *stream) {
    SCI_CHECK_ARG(x0 && u1 && w0 && b0 && w1 && src && out, "sci_cnn_den_tail: null pointer");
    SCI_CHECK_ARG(count >= 1 && first >= 0 && first + count <= nframes,
                  "sci_cnn_den_tail: frames [first, first + count) outside the source");
    SCI_CHECK_ARG(Hp >= 4 && Wp >= 4 && Hp % 2 == 0 && Wp % 2 == 0,
                  "sci_cnn_den_tail: Hp, Wp must be even and >= 4");
    SCI_CHECK_ARG(Hs >= 1 && Ws >= 1 && Hs <= Hp && Ws <= Wp && Hp - Hs < Hs && Wp - Ws < Ws,
                  "sci_cnn_den_tail: the padding must be less than the source size");
    SCI_CHECK_ARG(Ho >= 1 && Wo >= 1 && Ho <= Hp && Wo <= Wp,
                  "sci_cnn_den_tail: the crop must lie inside Hp x Wp");
    SCI_CHECK_ARG(count * Hp <= INT32_MAX && Wp <= INT32_MAX / 2,
                  "sci_cnn_den_tail: too large for the tensor coordinates");
    SCI_CHECK_ARG(aligned16(x0) && aligned16(u1) && aligned16(w0) && aligned16(w1),
                  "sci_cnn_den_tail: x0, u1, w0, w1 must be 16-byte aligned");
    return sci::launch_den_tail(x0, u1, w0, b0, w1, b1, src, Hs, Ws, first, count, Hp, Wp, Ho,
                                Wo, clip, out, as_stream(stream));
}
