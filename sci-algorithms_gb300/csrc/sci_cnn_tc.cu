// Thin-input 3 x 3 convolution on the 5th-generation tensor cores
// (tcgen05.mma, accumulator in tensor memory): the first layer of
// FastDVDnet's denoising block (6 input channels -> 90 features, padded to
// 8 -> 96; packages/fastdvdnet/models.py:29-43) and of FFDNet (5 -> 64,
// packages/ffdnet/models.py:37-42), where cuDNN falls back to slow kernels
// because each filter tap has only 8 input channels.
//
// Implicit GEMM per tile of kM = 128 consecutive output pixels (flattened
// frame, row, column order; TMEM lane m = pixel m of the tile):
//   D[m, n] = sum_k A[m, k] * B[n, k],  k = tap * 8 + c  (tap = 3 dy + dx),
// A = the tile's im2col rows (9 taps x 8 bf16 channels = 9 x 16 bytes, plus
// one zero chunk: K = 80 = 5 MMAs of K = 16), gathered from the NHWC8 input
// by cp.async (zero outside the frame); B = the N x 80 weights, staged once
// per block.  Both operands are K-major without swizzle: an 8-row x 16-byte
// core matrix is 128 contiguous bytes, K-adjacent core matrices are 128 B
// apart (LBO), 8-row groups kSBO = 10 x 128 B apart (SBO).  The epilogue
// reads D with tcgen05.ld (warp w owns lanes 32w..32w+31, i.e. thread t owns
// pixel t), adds the bias, applies ReLU, stages the tile's N bf16 channels
// per pixel in shared memory and writes them with one bulk copy (the
// tile's pixels are contiguous in the NHWC output), which drains while the
// block gathers its next tile.
//
// Persistent blocks of 128 threads; 64 KiB of shared memory per block caps
// residency at 3 blocks per SM (3 x 128 of the SM's 512 TMEM columns).
// The wait for each tile's MMAs is bounded: on timeout the block sets bit 0
// of the CNN status word, waits once more (bounded) for the MMAs in
// flight, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <cstdlib>

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
// shared memory requested per block: 64 KiB with one A buffer (3 blocks per
// SM), 100 KiB with two (2 blocks per SM)
template <int NBUF>
__host__ __device__ constexpr int smem_bytes() { return NBUF == 1 ? 64 * 1024 : 100 * 1024; }

template <int N, int NBUF>
struct alignas(1024) TcSmem {
    uint8_t a[NBUF][kATile];
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

// NBUF = 2: the gather of the block's next tile is issued before the
// current tile's MMAs and epilogue, so its latency overlaps them.
template <int N, int NBUF>
__global__ void __launch_bounds__(kThr, NBUF == 1 ? 3 : 2)
    k_conv_thin_tc(const uint4 *__restrict__ in, const uint4 *__restrict__ wts,
                   const float *__restrict__ bias, uint4 *__restrict__ out, int64_t F,
                   int64_t H, int64_t W, int relu) {
    static_assert(N % 32 == 0 && N >= 32 && N <= 256, "N: multiple of 32 up to 256");
    static_assert(sizeof(TcSmem<N, NBUF>) + 1024 <= smem_bytes<NBUF>(),
                  "shared memory layout too large");
    extern __shared__ uint8_t smem_raw[];
    TcSmem<N, NBUF> &s = *reinterpret_cast<TcSmem<N, NBUF> *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5;

    // weights into the core-matrix layout; the zero K chunk of A
    for (int i = tid; i < N * kKC; i += kThr) {
        const int n = i / kKC, kc = i % kKC;
        *reinterpret_cast<uint4 *>(s.b + (n >> 3) * kSBO + kc * kCore + (n & 7) * 16) = wts[i];
    }
    for (int i = tid; i < N; i += kThr) s.bias[i] = bias[i];
    const int row_off = (tid >> 3) * kSBO + (tid & 7) * 16;
#pragma unroll
    for (int b = 0; b < NBUF; ++b)
        *reinterpret_cast<uint4 *>(s.a[b] + row_off + 9 * kCore) = make_uint4(0u, 0u, 0u, 0u);
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
    if (NBUF == 2) {
        gather_row(in, s.a[0] + row_off, blockIdx.x * kM + tid, P, H, W);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    int buf = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, buf ^= (NBUF - 1)) {
        const int64_t p = tile * kM + tid;
        if (NBUF == 2) {
            const int64_t nxt = tile + gridDim.x;
            if (nxt < ntiles) gather_row(in, s.a[buf ^ 1] + row_off, nxt * kM + tid, P, H, W);
            asm volatile("cp.async.commit_group;" ::: "memory");
            asm volatile("cp.async.wait_group 1;" ::: "memory");  // this tile's copies
        } else {
            gather_row(in, s.a[0] + row_off, p, P, H, W);
            asm volatile("cp.async.wait_all;" ::: "memory");
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();  // the previous tile's tcgen05.ld before the barrier
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const uint32_t a_addr = smem_u32(s.a[buf]);
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

template <int N, int NBUF>
int launch_thin(const void *in, const void *wts, const float *bias, void *out, int64_t F,
                int64_t H, int64_t W, int relu, cudaStream_t st) {
    const int64_t ntiles = (F * H * W + kM - 1) / kM;
    const int64_t cap = int64_t(kSMs) * (NBUF == 1 ? 3 : 2);
    const int grid = int(ntiles < cap ? ntiles : cap);
    SCI_CUDA(cudaFuncSetAttribute(k_conv_thin_tc<N, NBUF>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem_bytes<NBUF>()));
    k_conv_thin_tc<N, NBUF><<<grid, kThr, smem_bytes<NBUF>(), st>>>(
        reinterpret_cast<const uint4 *>(in), reinterpret_cast<const uint4 *>(wts), bias,
        reinterpret_cast<uint4 *>(out), F, H, W, relu);
    SCI_LAUNCHED("k_conv_thin_tc");
    return SCI_OK;
}

template <int N>
int launch_thin_n(const void *in, const void *wts, const float *bias, void *out, int64_t F,
                  int64_t H, int64_t W, int relu, cudaStream_t st) {
    // one A buffer and 3 blocks per SM: 1.99 ms for 8 x 2048 x 2048 -> 96
    // channels; two buffers (next gather overlapping) and 2 blocks per SM:
    // 2.37 ms (SCI_THIN_NBUF=2)
    static const int nbuf = [] {
        const char *e = getenv("SCI_THIN_NBUF");
        return (e && e[0] == '2') ? 2 : 1;
    }();
    if (nbuf == 1) return launch_thin<N, 1>(in, wts, bias, out, F, H, W, relu, st);
    return launch_thin<N, 2>(in, wts, bias, out, F, H, W, relu, st);
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
