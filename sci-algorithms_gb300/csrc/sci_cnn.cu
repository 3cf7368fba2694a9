// Glue kernels of the CNN denoisers (FFDNet, FastDVDnet) on planar frame
// stacks: they build the networks' input tensors from the reconstruction's
// B x H x W float32 frames and turn the networks' outputs back into frames,
// so that every frame of a stack goes through one batched network call.
//
//   FFDNet input  (packages/ffdnet/functions.py:17-58): channel 0 = the
//     noise level, channels 1 + 2i + j = the pixels at offset (i, j) of each
//     2 x 2 cell (odd sizes: the last row / column repeated).
//   FFDNet output (functions.py:60-93 and test_ffdnet_ipol.py:174):
//     frame - depth_to_space(estimated noise).
//   FastDVDnet window (packages/fastdvdnet/fastdvdnet.py:117-131,
//     models.py:195-206): for centre frames g in [first, first + count),
//     channels
//     [src[g-1], s, src[g], s, src[g+1], s] (frame indices modulo the frame
//     count), reflect-padded at the bottom / right to Hp x Wp.
//   FastDVDnet output (models.py:205): centre frame - network output,
//     cropped to Ho x Wo.
//
// Layouts: SCI_CNN_NCHW_F32 (planar float32), SCI_CNN_NHWC8_BF16 (one
// 16-byte vector of 8 bfloat16 channels per pixel, unused channels 0) and
// SCI_CNN_NHWC8_F32 (8 float32 channels per pixel) for the channels-last
// tensor-core convolutions.  The noise level is read from device memory
// so that a captured CUDA graph replays with a new level.
#include <cuda_bf16.h>

#include "sci_common.cuh"

namespace sci {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int64_t reflect_hi(int64_t i, int64_t n) {
    // torch 'reflect' padding past the end: n + k -> n - 2 - k
    i = i < n ? i : 2 * (n - 1) - i;
    return i < 0 ? 0 : i;
}

__device__ __forceinline__ uint4 pack8(float a0, float a1, float a2, float a3, float a4,
                                       float a5, float a6, float a7) {
    __nv_bfloat162 p0 = __floats2bfloat162_rn(a0, a1);
    __nv_bfloat162 p1 = __floats2bfloat162_rn(a2, a3);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(a4, a5);
    __nv_bfloat162 p3 = __floats2bfloat162_rn(a6, a7);
    uint4 r;
    r.x = *reinterpret_cast<unsigned *>(&p0);
    r.y = *reinterpret_cast<unsigned *>(&p1);
    r.z = *reinterpret_cast<unsigned *>(&p2);
    r.w = *reinterpret_cast<unsigned *>(&p3);
    return r;
}

// 8 channels of one NHWC8 pixel: 8 bfloat16 (16 bytes) or 8 float32 (32 bytes)
template <int LAYOUT>
__device__ __forceinline__ void store8(void *out, int64_t t, float a0, float a1, float a2,
                                       float a3, float a4, float a5, float a6, float a7) {
    if (LAYOUT == SCI_CNN_NHWC8_BF16) {
        reinterpret_cast<uint4 *>(out)[t] = pack8(a0, a1, a2, a3, a4, a5, a6, a7);
    } else {
        float4 *o = reinterpret_cast<float4 *>(out) + 2 * t;
        o[0] = make_float4(a0, a1, a2, a3);
        o[1] = make_float4(a4, a5, a6, a7);
    }
}

// channel c of pixel p of an NHWC tensor with nch channels (bf16 or f32)
template <int LAYOUT>
__device__ __forceinline__ float load_ch(const void *r, int64_t p, int nch, int c) {
    if (LAYOUT == SCI_CNN_NHWC8_BF16)
        return __bfloat162float(reinterpret_cast<const __nv_bfloat16 *>(r)[p * nch + c]);
    return __ldg(reinterpret_cast<const float *>(r) + p * nch + c);
}

// ------------------------------------------------------------ FFDNet pack
template <int LAYOUT>
__global__ void k_ffdnet_pack(const float *__restrict__ x, int64_t F, int64_t H, int64_t W,
                              const float *__restrict__ sigma, void *__restrict__ out) {
    const int64_t H2 = (H + 1) / 2, W2 = (W + 1) / 2, n = F * H2 * W2;
    const float s = __ldg(sigma);
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t c = t % W2, r = (t / W2) % H2, f = t / (W2 * H2);
        const float *xf = x + f * H * W;
        const int64_t r0 = 2 * r, r1 = min(2 * r + 1, H - 1);
        const int64_t c0 = 2 * c, c1 = min(2 * c + 1, W - 1);
        const float d0 = __ldg(xf + r0 * W + c0), d1 = __ldg(xf + r0 * W + c1);
        const float d2 = __ldg(xf + r1 * W + c0), d3 = __ldg(xf + r1 * W + c1);
        if (LAYOUT != SCI_CNN_NCHW_F32) {
            store8<LAYOUT>(out, t, s, d0, d1, d2, d3, 0.f, 0.f, 0.f);
        } else {
            float *o = reinterpret_cast<float *>(out) + f * 5 * H2 * W2 + r * W2 + c;
            const int64_t pl = H2 * W2;
            o[0] = s;
            o[pl] = d0;
            o[2 * pl] = d1;
            o[3 * pl] = d2;
            o[4 * pl] = d3;
        }
    }
}

// -------------------------------------------------- FFDNet unpack + subtract
template <int LAYOUT>
__global__ void k_ffdnet_unpack_sub(const float *__restrict__ x, const void *__restrict__ noise,
                                    int64_t F, int64_t H, int64_t W, int nch, int clip,
                                    float *__restrict__ out) {
    const int64_t H2 = (H + 1) / 2, W2 = (W + 1) / 2, n = F * H2 * W2;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t c = t % W2, r = (t / W2) % H2, f = t / (W2 * H2);
        float e[4];
        if (LAYOUT == SCI_CNN_NHWC8_F32) {
            const float4 v = __ldg(reinterpret_cast<const float4 *>(
                reinterpret_cast<const float *>(noise) + t * nch));
            e[0] = v.x;
            e[1] = v.y;
            e[2] = v.z;
            e[3] = v.w;
        } else if (LAYOUT == SCI_CNN_NHWC8_BF16) {
            const __nv_bfloat16 *q = reinterpret_cast<const __nv_bfloat16 *>(noise) + t * nch;
            const uint2 v = *reinterpret_cast<const uint2 *>(q);
            const __nv_bfloat162 a = *reinterpret_cast<const __nv_bfloat162 *>(&v.x);
            const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162 *>(&v.y);
            e[0] = __low2float(a);
            e[1] = __high2float(a);
            e[2] = __low2float(b);
            e[3] = __high2float(b);
        } else {
            const float *q = reinterpret_cast<const float *>(noise) + f * 4 * H2 * W2 + r * W2 + c;
#pragma unroll
            for (int k = 0; k < 4; ++k) e[k] = __ldg(q + k * H2 * W2);
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int64_t y = 2 * r + i;
            if (y >= H) break;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int64_t xx = 2 * c + j;
                if (xx >= W) break;
                const int64_t idx = (f * H + y) * W + xx;
                float v = __ldg(x + idx) - e[2 * i + j];
                if (clip) v = fminf(fmaxf(v, 0.f), 1.f);
                out[idx] = v;
            }
        }
    }
}

// ------------------------------------------------------ FastDVDnet window
template <int LAYOUT>
__global__ void k_window(const float *__restrict__ src, int64_t F, int64_t Hs, int64_t Ws,
                         int64_t Hp, int64_t Wp, int64_t first, int64_t count,
                         const float *__restrict__ sigma, void *__restrict__ out) {
    const int64_t n = count * Hp * Wp;
    const float s = __ldg(sigma);
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t j = t % Wp, i = (t / Wp) % Hp, gl = t / (Wp * Hp), g = first + gl;
        const int64_t off = reflect_hi(i, Hs) * Ws + reflect_hi(j, Ws);
        const int64_t gm = (g + F - 1) % F, gp = (g + 1) % F;
        const float a = __ldg(src + gm * Hs * Ws + off);
        const float b = __ldg(src + g * Hs * Ws + off);
        const float c = __ldg(src + gp * Hs * Ws + off);
        if (LAYOUT != SCI_CNN_NCHW_F32) {
            store8<LAYOUT>(out, t, a, s, b, s, c, s, 0.f, 0.f);
        } else {
            const int64_t pl = Hp * Wp;
            float *o = reinterpret_cast<float *>(out) + gl * 6 * pl + i * Wp + j;
            o[0] = a;
            o[pl] = s;
            o[2 * pl] = b;
            o[3 * pl] = s;
            o[4 * pl] = c;
            o[5 * pl] = s;
        }
    }
}

// ---------------------------------------------- FastDVDnet centre - output
template <int LAYOUT>
__global__ void k_center_sub(const float *__restrict__ src, int64_t Hs, int64_t Ws,
                             int64_t first, int64_t count, const void *__restrict__ r, int nch,
                             int64_t Hp, int64_t Wp, int64_t Ho, int64_t Wo, int clip,
                             float *__restrict__ out) {
    const int64_t n = count * Ho * Wo;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t j = t % Wo, i = (t / Wo) % Ho, gl = t / (Wo * Ho), g = first + gl;
        const float cen = __ldg(src + g * Hs * Ws + reflect_hi(i, Hs) * Ws + reflect_hi(j, Ws));
        const int64_t p = (gl * Hp + i) * Wp + j;
        const float e = (LAYOUT == SCI_CNN_NCHW_F32) ? __ldg(reinterpret_cast<const float *>(r) + p)
                                                     : load_ch<LAYOUT>(r, p, nch, 0);
        float v = cen - e;
        if (clip) v = fminf(fmaxf(v, 0.f), 1.f);
        out[t] = v;
    }
}

// ------------------------------------- FastDVDnet upsampling + skip add
// u: N x h x w x 4C bfloat16 whose channel k*C + c holds sub-pixel k = 2a + b
// of output channel c (the upsampling convolution's outputs permuted so
// that each sub-pixel is one contiguous vector); a, out: N x 2h x 2w x C.
// out[n, 2i+a, 2j+b, c] = a[n, 2i+a, 2j+b, c] + u[n, i, j, (2a+b)*C + c],
// summed in float32 and rounded to bfloat16.
__device__ __forceinline__ uint4 add8(uint4 x, uint4 y) {
    uint4 r;
    const unsigned *px = reinterpret_cast<const unsigned *>(&x);
    const unsigned *py = reinterpret_cast<const unsigned *>(&y);
    unsigned *pr = reinterpret_cast<unsigned *>(&r);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const __nv_bfloat162 a = *reinterpret_cast<const __nv_bfloat162 *>(px + q);
        const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162 *>(py + q);
        const __nv_bfloat162 c = __floats2bfloat162_rn(__low2float(a) + __low2float(b),
                                                       __high2float(a) + __high2float(b));
        pr[q] = *reinterpret_cast<const unsigned *>(&c);
    }
    return r;
}

__global__ void k_shuffle_add(const uint4 *__restrict__ a, const uint4 *__restrict__ u,
                              uint4 *__restrict__ out, int64_t N, int64_t h, int64_t w,
                              int64_t V) {
    const int64_t n = N * h * w * 4 * V;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t v = t % V, k = (t / V) % 4, pix = t / (4 * V);
        const int64_t j = pix % w, i = (pix / w) % h, b = pix / (w * h);
        const int64_t o = ((b * 2 * h + 2 * i + (k >> 1)) * 2 * w + 2 * j + (k & 1)) * V + v;
        const uint4 uv = __ldg(u + t);
        out[o] = a ? add8(__ldg(a + o), uv) : uv;
    }
}

// the same on float32 NHWC (4 channels per 16-byte vector, V = C / 4)
__global__ void k_shuffle_add_f32(const float4 *__restrict__ a, const float4 *__restrict__ u,
                                  float4 *__restrict__ out, int64_t N, int64_t h, int64_t w,
                                  int64_t V) {
    const int64_t n = N * h * w * 4 * V;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t v = t % V, k = (t / V) % 4, pix = t / (4 * V);
        const int64_t j = pix % w, i = (pix / w) % h, b = pix / (w * h);
        const int64_t o = ((b * 2 * h + 2 * i + (k >> 1)) * 2 * w + 2 * j + (k & 1)) * V + v;
        const float4 uv = __ldg(u + t);
        if (a) {
            const float4 av = __ldg(a + o);
            out[o] = make_float4(av.x + uv.x, av.y + uv.y, av.z + uv.z, av.w + uv.w);
        } else {
            out[o] = uv;
        }
    }
}

int grid_for(int64_t n) {
    int64_t b = (n + kThreads - 1) / kThreads;
    const int64_t cap = int64_t(kSMs) * 16;
    return int(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace
}  // namespace sci

using namespace sci;

extern "C" {

int sci_cnn_ffdnet_pack(const float *x, int64_t nframes, int64_t H, int64_t W,
                        const float *sigma, void *out, int layout, void *stream) {
    SCI_CHECK_ARG(x && sigma && out, "sci_cnn_ffdnet_pack: null pointer");
    SCI_CHECK_ARG(nframes >= 1 && H >= 1 && W >= 1, "sci_cnn_ffdnet_pack: invalid sizes");
    SCI_CHECK_ARG(layout >= SCI_CNN_NCHW_F32 && layout <= SCI_CNN_NHWC8_F32,
                  "sci_cnn_ffdnet_pack: unknown layout %d", layout);
    SCI_CHECK_ARG(layout == SCI_CNN_NCHW_F32 || aligned16(out),
                  "sci_cnn_ffdnet_pack: NHWC8 output must be 16-byte aligned");
    const int64_t n = nframes * ((H + 1) / 2) * ((W + 1) / 2);
    const cudaStream_t st = as_stream(stream);
    if (layout == SCI_CNN_NHWC8_BF16)
        k_ffdnet_pack<SCI_CNN_NHWC8_BF16><<<grid_for(n), kThreads, 0, st>>>(x, nframes, H, W,
                                                                           sigma, out);
    else if (layout == SCI_CNN_NHWC8_F32)
        k_ffdnet_pack<SCI_CNN_NHWC8_F32><<<grid_for(n), kThreads, 0, st>>>(x, nframes, H, W,
                                                                          sigma, out);
    else
        k_ffdnet_pack<SCI_CNN_NCHW_F32><<<grid_for(n), kThreads, 0, st>>>(x, nframes, H, W,
                                                                         sigma, out);
    SCI_LAUNCHED("k_ffdnet_pack");
    return SCI_OK;
}

int sci_cnn_ffdnet_unpack_sub(const float *x, const void *noise, int64_t nframes, int64_t H,
                              int64_t W, int layout, int channels, int clip, float *out,
                              void *stream) {
    SCI_CHECK_ARG(x && noise && out, "sci_cnn_ffdnet_unpack_sub: null pointer");
    SCI_CHECK_ARG(nframes >= 1 && H >= 1 && W >= 1, "sci_cnn_ffdnet_unpack_sub: invalid sizes");
    SCI_CHECK_ARG(layout >= SCI_CNN_NCHW_F32 && layout <= SCI_CNN_NHWC8_F32,
                  "sci_cnn_ffdnet_unpack_sub: unknown layout %d", layout);
    SCI_CHECK_ARG(layout == SCI_CNN_NCHW_F32 ||
                      ((channels == 4 || channels == 8) &&
                       (reinterpret_cast<uintptr_t>(noise) & 15u) == 0),
                  "sci_cnn_ffdnet_unpack_sub: NHWC noise needs 4 or 8 channels, 16-byte aligned");
    const int64_t n = nframes * ((H + 1) / 2) * ((W + 1) / 2);
    const cudaStream_t st = as_stream(stream);
    if (layout == SCI_CNN_NHWC8_BF16)
        k_ffdnet_unpack_sub<SCI_CNN_NHWC8_BF16><<<grid_for(n), kThreads, 0, st>>>(
            x, noise, nframes, H, W, channels, clip, out);
    else if (layout == SCI_CNN_NHWC8_F32)
        k_ffdnet_unpack_sub<SCI_CNN_NHWC8_F32><<<grid_for(n), kThreads, 0, st>>>(
            x, noise, nframes, H, W, channels, clip, out);
    else
        k_ffdnet_unpack_sub<SCI_CNN_NCHW_F32><<<grid_for(n), kThreads, 0, st>>>(
            x, noise, nframes, H, W, 4, clip, out);
    SCI_LAUNCHED("k_ffdnet_unpack_sub");
    return SCI_OK;
}

int sci_cnn_window(const float *src, int64_t nframes, int64_t Hs, int64_t Ws, int64_t Hp,
                   int64_t Wp, int64_t first, int64_t count, const float *sigma, void *out,
                   int layout, void *stream) {
    SCI_CHECK_ARG(src && sigma && out, "sci_cnn_window: null pointer");
    SCI_CHECK_ARG(nframes >= 1 && Hs >= 1 && Ws >= 1 && Hp >= Hs && Wp >= Ws,
                  "sci_cnn_window: invalid sizes");
    SCI_CHECK_ARG(first >= 0 && count >= 1 && first + count <= nframes,
                  "sci_cnn_window: centre frames [%lld, %lld) outside %lld frames",
                  (long long)first, (long long)(first + count), (long long)nframes);
    SCI_CHECK_ARG((Hp == Hs || Hp - Hs < Hs) && (Wp == Ws || Wp - Ws < Ws),
                  "sci_cnn_window: reflect padding must be shorter than the frame");
    SCI_CHECK_ARG(layout >= SCI_CNN_NCHW_F32 && layout <= SCI_CNN_NHWC8_F32,
                  "sci_cnn_window: unknown layout %d", layout);
    SCI_CHECK_ARG(layout == SCI_CNN_NCHW_F32 || aligned16(out),
                  "sci_cnn_window: NHWC8 output must be 16-byte aligned");
    const int64_t n = count * Hp * Wp;
    const cudaStream_t st = as_stream(stream);
    if (layout == SCI_CNN_NHWC8_BF16)
        k_window<SCI_CNN_NHWC8_BF16><<<grid_for(n), kThreads, 0, st>>>(
            src, nframes, Hs, Ws, Hp, Wp, first, count, sigma, out);
    else if (layout == SCI_CNN_NHWC8_F32)
        k_window<SCI_CNN_NHWC8_F32><<<grid_for(n), kThreads, 0, st>>>(
            src, nframes, Hs, Ws, Hp, Wp, first, count, sigma, out);
    else
        k_window<SCI_CNN_NCHW_F32><<<grid_for(n), kThreads, 0, st>>>(
            src, nframes, Hs, Ws, Hp, Wp, first, count, sigma, out);
    SCI_LAUNCHED("k_window");
    return SCI_OK;
}

int sci_cnn_center_sub(const float *src, int64_t nframes, int64_t Hs, int64_t Ws,
                       int64_t first, int64_t count, const void *r, int layout, int channels,
                       int64_t Hp, int64_t Wp, int64_t Ho, int64_t Wo, int clip, float *out,
                       void *stream) {
    SCI_CHECK_ARG(src && r && out, "sci_cnn_center_sub: null pointer");
    SCI_CHECK_ARG(nframes >= 1 && Hs >= 1 && Ws >= 1 && Ho >= 1 && Wo >= 1 && Ho <= Hp &&
                      Wo <= Wp && Hp >= Hs && Wp >= Ws,
                  "sci_cnn_center_sub: invalid sizes");
    SCI_CHECK_ARG(first >= 0 && count >= 1 && first + count <= nframes,
                  "sci_cnn_center_sub: centre frames outside the stack");
    SCI_CHECK_ARG((Hp == Hs || Hp - Hs < Hs) && (Wp == Ws || Wp - Ws < Ws),
                  "sci_cnn_center_sub: reflect padding must be shorter than the frame");
    SCI_CHECK_ARG(layout >= SCI_CNN_NCHW_F32 && layout <= SCI_CNN_NHWC8_F32,
                  "sci_cnn_center_sub: unknown layout %d", layout);
    SCI_CHECK_ARG(layout == SCI_CNN_NCHW_F32 || channels >= 1,
                  "sci_cnn_center_sub: an NHWC output needs its channel count");
    const int64_t n = count * Ho * Wo;
    const cudaStream_t st = as_stream(stream);
    if (layout == SCI_CNN_NHWC8_BF16)
        k_center_sub<SCI_CNN_NHWC8_BF16><<<grid_for(n), kThreads, 0, st>>>(
            src, Hs, Ws, first, count, r, channels, Hp, Wp, Ho, Wo, clip, out);
    else if (layout == SCI_CNN_NHWC8_F32)
        k_center_sub<SCI_CNN_NHWC8_F32><<<grid_for(n), kThreads, 0, st>>>(
            src, Hs, Ws, first, count, r, channels, Hp, Wp, Ho, Wo, clip, out);
    else
        k_center_sub<SCI_CNN_NCHW_F32><<<grid_for(n), kThreads, 0, st>>>(
            src, Hs, Ws, first, count, r, 1, Hp, Wp, Ho, Wo, clip, out);
    SCI_LAUNCHED("k_center_sub");
    return SCI_OK;
}

int sci_cnn_shuffle_add(const void *a, const void *u, void *out, int64_t N, int64_t h,
                        int64_t w, int64_t C, void *stream) {
    SCI_CHECK_ARG(u && out, "sci_cnn_shuffle_add: null pointer");
    SCI_CHECK_ARG(N >= 1 && h >= 1 && w >= 1 && C >= 8 && C % 8 == 0,
                  "sci_cnn_shuffle_add: invalid sizes (C must be a multiple of 8)");
    SCI_CHECK_ARG(aligned16(u) && aligned16(out) && (!a || aligned16(a)),
                  "sci_cnn_shuffle_add: buffers must be 16-byte aligned");
    SCI_CHECK_ARG(out != u, "sci_cnn_shuffle_add: out must not alias u");
    const int64_t n = N * h * w * 4 * (C / 8);
    k_shuffle_add<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(
        reinterpret_cast<const uint4 *>(a), reinterpret_cast<const uint4 *>(u),
        reinterpret_cast<uint4 *>(out), N, h, w, C / 8);
    SCI_LAUNCHED("k_shuffle_add");
    return SCI_OK;
}

int sci_cnn_shuffle_add_f32(const float *a, const float *u, float *out, int64_t N, int64_t h,
                            int64_t w, int64_t C, void *stream) {
    SCI_CHECK_ARG(u && out, "sci_cnn_shuffle_add_f32: null pointer");
    SCI_CHECK_ARG(N >= 1 && h >= 1 && w >= 1 && C >= 4 && C % 4 == 0,
                  "sci_cnn_shuffle_add_f32: invalid sizes (C must be a multiple of 4)");
    SCI_CHECK_ARG(aligned16(u) && aligned16(out) && (!a || aligned16(a)),
                  "sci_cnn_shuffle_add_f32: buffers must be 16-byte aligned");
    SCI_CHECK_ARG(out != u, "sci_cnn_shuffle_add_f32: out must not alias u");
    const int64_t n = N * h * w * 4 * (C / 4);
    k_shuffle_add_f32<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(
        reinterpret_cast<const float4 *>(a), reinterpret_cast<const float4 *>(u),
        reinterpret_cast<float4 *>(out), N, h, w, C / 4);
    SCI_LAUNCHED("k_shuffle_add_f32");
    return SCI_OK;
}

}  // extern "C"
