// Cached CUDA graphs of whole enqueued sequences: a GAP / ADMM solve, a
// batched solve, an unrolled forward or reverse pass, a spectral solve.
// Each is keyed by every argument that shapes the launches (pointers,
// sizes, schedules) and by the SCI_* environment switches; the first call captures the sequence on a private
// stream and instantiates it, later calls replay it with one launch.  One
// process-wide cache (most recently used first, bounded) behind a mutex.
#pragma once
#include <string>

#include "sci_common.cuh"

namespace sci {

// The SCI_* environment switches (sorted "name=value" pairs): they select
// kernels and launch shapes at capture time, so they are part of every key.
std::string env_switches();

// Launches the graph cached under key on s (under the cache's lock, so that
// no other thread evicts it meanwhile); *found says whether there was one.
int graph_replay(const std::string &key, cudaStream_t s, bool *found);
// Launches g on s and caches it under key (the cache owns it from then on;
// the least recently used entries beyond the bound are destroyed).
int graph_store_and_launch(const std::string &key, cudaGraphExec_t g, cudaStream_t s);

// Appends the bytes of each value to a key.
template <typename... T>
void key_append(std::string &k, const T &...v) {
    (k.append(reinterpret_cast<const char *>(&v), sizeof(T)), ...);
}

// Replays the graph cached under (what, key) on stream s, or captures
// enqueue(stream) into a new graph first.  `what` names the sequence in
// error messages and keeps the keys of different callers apart.
template <typename F>
int run_graph(const char *what, const std::string &key, cudaStream_t s, F enqueue) {
    const std::string k = std::string(what) + '\0' + env_switches() + '\0' + key;
    bool found = false;
    const int r = graph_replay(k, s, &found);
    if (found || r) return r;
    cudaStream_t cs;
    SCI_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    const cudaError_t cb = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = SCI_OK;
    if (cb == cudaSuccess) rc = enqueue(cs);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = (cb == cudaSuccess) ? cudaStreamEndCapture(cs, &graph) : cb;
    cudaStreamDestroy(cs);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (ce != cudaSuccess) return cuda_status(ce, what);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ci = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ci != cudaSuccess) return cuda_status(ci, "cudaGraphInstantiate");
    return graph_store_and_launch(k, exec, s);
}

}  // namespace sci
