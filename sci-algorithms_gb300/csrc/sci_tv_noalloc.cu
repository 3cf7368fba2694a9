// Chambolle TV for callers that cannot allocate device memory.
//
// sci_tv_chambolle needs a small device workspace (per-frame float64 energy
// sums for the stop test, and per-frame flags) that the caller allocates.
// Some callers cannot do that: a host framework that owns every device byte
// through its own pool and forbids cudaMalloc outside it, a plug-in that is
// handed only its input and output buffers, or a latency-critical loop where
// cudaMalloc/cudaFree would synchronise the device.  This entry point serves
// them: its scratch lives in a fixed array in this library's device image,
// so a call allocates nothing.
//
// Limits and behaviour:
//  * the scratch array is 64 KiB; a call fits when n_iter_max <= 5 (one
//    pipeline pass, so the dual field stays on chip) and the per-frame
//    energy slots fit: nframes * n_iter_max * 16 bytes (+ 8 bytes a frame
//    for the stop flags and decisions, with alignment) <= 64 KiB, i.e.
//    nframes <= 742 at n_iter_max = 5.  Larger requests
//    are rejected with SCI_ERR_INVALID_ARG and a message;
//  * every GPU that loads the library keeps the 64 KiB until the process
//    exits;
//  * all calls share the one array: the energy sums are cleared on the
//    stream at the start of every call, but calls whose work overlaps on
//    the GPU (other streams, or other host threads) race on the array and
//    must be ordered by the caller;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current) and caches it; make
//    that first call before any stream capture on the device.  Later calls
//    read the cached address without taking a lock.  The cache does not
//    survive a reset of the device's primary context (cudaDeviceReset, or a
//    host framework that resets the device): the library's device image is
//    unloaded with the context, so do not call this entry point again in a
//    process that has reset the device.
#include <atomic>
#include <mutex>

#include "sci_common.cuh"

namespace sci {

int tv_launch(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
              int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
              void *workspace, size_t ws_bytes, cudaStream_t s, int force_R);
size_t tv_workspace_bytes(int64_t nf, int64_t H, int64_t W, int K);

namespace {

constexpr size_t kScratchBytes = 64 * 1024;
constexpr int kMaxDevices = 64;

// The scratch itself.  Host code must not use this name as an address: on
// the host it is only a stand-in symbol; the device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_tv_scratch[kScratchBytes];

std::mutex g_mu;  // serialises the first lookup on a device
std::atomic<void *> g_addr[kMaxDevices] = {};

// Device address of the scratch on the current device (looked up once; a
// cached address is read without the lock).
int scratch_address(void **out) {
    int dev = 0;
    SCI_CUDA(cudaGetDevice(&dev));
    SCI_CHECK_ARG(dev >= 0 && dev < kMaxDevices, "no-alloc TV: device ordinal %d out of range",
                  dev);
    void *p = g_addr[dev].load(std::memory_order_acquire);
    if (!p) {
        std::lock_guard<std::mutex> lk(g_mu);
        p = g_addr[dev].load(std::memory_order_relaxed);
        if (!p) {
            const cudaError_t e = cudaGetSymbolAddress(&p, g_tv_scratch);
            if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_tv_scratch)");
            g_addr[dev].store(p, std::memory_order_release);
        }
    }
    *out = p;
    return SCI_OK;
}

}  // namespace
}  // namespace sci

extern "C" int sci_tv_chambolle_noalloc(const float *f, float *u, float *resid, int64_t nframes,
                                        int64_t H, int64_t W, float weight, float eps,
                                        int n_iter_max, int *steps, void *stream) {
    using namespace sci;
    SCI_CHECK_ARG(f && u && nframes >= 1 && H >= 1 && W >= 1 && n_iter_max >= 1,
                  "sci_tv_chambolle_noalloc: bad arguments");
    SCI_CHECK_ARG(n_iter_max <= 5,
                  "sci_tv_chambolle_noalloc: n_iter_max = %d exceeds the limit of 5 of the "
                  "allocation-free variant (use sci_tv_chambolle with a workspace)",
                  n_iter_max);
    const size_t need = tv_workspace_bytes(nframes, H, W, n_iter_max);
    SCI_CHECK_ARG(need <= kScratchBytes,
                  "sci_tv_chambolle_noalloc: %lld frames x %d steps need %zu bytes of scratch, "
                  "more than its fixed %zu bytes (use sci_tv_chambolle with a workspace)",
                  (long long)nframes, n_iter_max, need, kScratchBytes);
    void *scratch = nullptr;
    if (int e = scratch_address(&scratch)) return e;
    return tv_launch(f, u, resid, nframes, H, W, H * W, weight, eps, n_iter_max, steps, nullptr,
                     scratch, kScratchBytes, as_stream(stream), 0);
}
