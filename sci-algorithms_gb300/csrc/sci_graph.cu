// The process-wide cache of instantiated CUDA graphs (sci_graph.cuh).
#include <algorithm>
#include <cstring>
#include <list>
#include <mutex>
#include <utility>
#include <vector>

#include "sci_graph.cuh"

extern char **environ;

namespace sci {
namespace {

constexpr size_t kMaxGraphs = 32;

struct GraphCache {
    std::mutex mu;
    std::list<std::pair<std::string, cudaGraphExec_t>> entries;  // most recent first
};

GraphCache &cache() {
    static GraphCache c;
    return c;
}

}  // namespace

std::string env_switches() {
    std::vector<std::string> v;
    for (char **e = environ; e && *e; ++e)
        if (std::strncmp(*e, "SCI_", 4) == 0) v.emplace_back(*e);
    std::sort(v.begin(), v.end());
    std::string k;
    for (const std::string &s : v) {
        k += s;
        k += '\n';
    }
    return k;
}

int graph_replay(const std::string &key, cudaStream_t s, bool *found) {
    GraphCache &c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    *found = false;
    for (auto it = c.entries.begin(); it != c.entries.end(); ++it)
        if (it->first == key) {
            c.entries.splice(c.entries.begin(), c.entries, it);
            *found = true;
            SCI_CUDA(cudaGraphLaunch(c.entries.front().second, s));
            return SCI_OK;
        }
    return SCI_OK;
}

int graph_store_and_launch(const std::string &key, cudaGraphExec_t g, cudaStream_t s) {
    GraphCache &c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    c.entries.emplace_front(key, g);
    while (c.entries.size() > kMaxGraphs) {
        cudaGraphExecDestroy(c.entries.back().second);
        c.entries.pop_back();
    }
    SCI_CUDA(cudaGraphLaunch(g, s));
    return SCI_OK;
}

}  // namespace sci
