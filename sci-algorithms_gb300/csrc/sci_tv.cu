// Host driver of the Chambolle TV (all passes of one call) and its C ABI.
// The kernels are in sci_tv.cuh (instantiated in sci_tv_k4.cu,
// sci_tv_k123.cu and sci_tv_fix.cu).
#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <queue>
#include <tuple>
#include <vector>

#include "sci_tv.cuh"

namespace sci {
namespace tv {

__global__ void k_init_done(int *done, int *steps, int K, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        done[i] = -1;
        if (steps) steps[i] = K;
    }
}

__global__ void k_copy_frames(const float *f, float *u, float *resid, int64_t n, int *steps,
                              int nf) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        u[i] = f[i];
        if (resid) resid[i] = 0.f;
        if (steps && i < nf) steps[i] = 1;
    }
}

static inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

struct Workspace {
    double *energy;  // [nf][K][2]
    int *done;       // [nf]
    float *pa, *pb;  // [nf][2][H][W] each (multi-pass only)
    int *stopj;      // [nf]: the stop decision of the current pass
    unsigned *ticket;  // right after the energies, so that one memset clears both
};

static size_t ws_layout(int64_t nf, int64_t H, int64_t W, int K, Workspace *w, char *base) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~size_t(255);
        return o;
    };
    const size_t ne = sizeof(double) * (size_t)(nf * K * 2);
    const size_t oe = take(ne + sizeof(double));
    const size_t od = take(sizeof(int) * (size_t)nf);
    const size_t oj = take(sizeof(int) * (size_t)nf);
    size_t opa = 0, opb = 0;
    if (K - 1 > SMAX) {
        opa = take(sizeof(float) * (size_t)(nf * 2 * H * W));
        opb = take(sizeof(float) * (size_t)(nf * 2 * H * W));
    }
    if (w) {
        w->energy = reinterpret_cast<double *>(base + oe);
        w->ticket = reinterpret_cast<unsigned *>(base + oe + ne);
        w->done = reinterpret_cast<int *>(base + od);
        w->stopj = reinterpret_cast<int *>(base + oj);
        w->pa = (K - 1 > SMAX) ? reinterpret_cast<float *>(base + opa) : nullptr;
        w->pb = (K - 1 > SMAX) ? reinterpret_cast<float *>(base + opb) : nullptr;
    }
    return off;
}

// Chooses rows per chunk so that the grid fills the GPU about twice.
// Chooses rows per chunk so that the grid fills the GPU about twice, down
// to 16 rows (a chunk of R rows costs R + 2S pipeline steps).  Measured on
// the spectral workload (28 frames of 256 x 256): 16 rows 4.06 ms per solve,
// 32 rows 4.25 ms, 8 rows 5.24 ms (2 columns per lane).
static int choose_R(int64_t nf, int nbands, int H) {
    if (const char *e = getenv("SCI_TV_R")) {
        const int v = atoi(e);
        if (v >= 8) return v;
    }
    const int64_t want = (int64_t)kSMs * 16 * 2;  // warps
    int R = 256;
    while (R > 16 && nf * nbands * ((H + R - 1) / R) < want) R >>= 1;
    return R;
}

// Finish time of a grid whose blocks (WPB consecutive work items each, in
// launch order) are taken by `slots` resident block slots, each slot taking
// the next block as soon as it is free; a block costs its longest item.
static double grid_makespan(const std::vector<int> &item_cost, int slots) {
    std::priority_queue<double, std::vector<double>, std::greater<double>> free_at;
    for (int i = 0; i < slots; ++i) free_at.push(0.0);
    double end = 0.0;
    for (size_t b = 0; b < item_cost.size(); b += WPB) {
        int c = 0;
        for (size_t i = b; i < std::min(item_cost.size(), b + WPB); ++i)
            c = std::max(c, item_cost[i]);
        const double t = free_at.top() + c;
        free_at.pop();
        free_at.push(t);
        end = std::max(end, t);
    }
    return end;
}

// Rows per chunk for the register-lean pass: a work item of R rows costs
// about R + S + 4 pipeline steps, and the chunk count whose grid finishes
// first in the slot model of grid_makespan is taken (a last wave that is
// half empty costs a whole wave there).  Results are cached per shape.
// Measured: this choice 2311 iter/s on the 2048 x 2048 x 24 GAP-TV solve
// against 2294 for the wave-count formula it replaced; tall chunks followed
// by short ones for the grid's tail (1 % shorter in the model) measured no
// faster (a partly empty last wave costs less than the model says: the
// SMs that run fewer blocks run them faster).
static int choose_R_slim(int64_t nf, int nbands, int H, int S, int slots) {
    if (const char *e = getenv("SCI_TV_R")) {
        const int v = atoi(e);
        if (v >= 8) return v;
    }
    static std::mutex mu;
    static std::map<std::tuple<int64_t, int, int, int, int>, int> cache;
    const auto key = std::make_tuple(nf, nbands, H, S, slots);
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    const int64_t cols = nf * (int64_t)nbands;  // items per chunk row
    std::vector<int> cost;
    int best_R = H;
    double best_t = -1.0;
    const int max_chunks = std::max(1, H / 16);
    for (int nc = 1; nc <= max_chunks; ++nc) {
        const int R = (H + nc - 1) / nc;
        cost.clear();
        for (int r0 = 0; r0 < H; r0 += R)
            cost.insert(cost.end(), (size_t)cols, std::min(R, H - r0) + S + 4);
        const double t = grid_makespan(cost, slots);
        if (best_t < 0.0 || t < best_t - 1e-9) {
            best_t = t;
            best_R = R;
        }
    }
    std::lock_guard<std::mutex> lock(mu);
    cache[key] = best_R;
    return best_R;
}

}  // namespace tv

// Register-lean TV pass (sci_tv_slim.cuh) for single-pass scikit-image runs
// on aligned frames; SCI_TV_SLIM=0 selects the generic pipeline instead.
// SCI_SLIM_MINB picks its register budget for n_iter_max = 5 (resident
// blocks per SM: 3 or 4 with 4 columns per lane, 5, 6 or 7 with 2).
static bool slim_enabled() {
    const char *e = getenv("SCI_TV_SLIM");
    return !e || atoi(e) != 0;
}
static int slim_minb(int cpl) {
    const char *e = getenv("SCI_SLIM_MINB");
    const int v = e ? atoi(e) : 0;
    if (cpl == 4) return v == 3 ? 3 : 4;
    return (v == 5 || v == 7) ? v : 6;
}

// Columns per lane: 4 halves the halo overhead of a band (8 of 128 columns
// instead of 8 of 64) but doubles the registers of the pipeline state; 2
// keeps ~1.3x more warps resident.  Measured at 2048 x 2048 x 24, 4 is
// faster (0.44 vs 0.52 ms).  SCI_TV_CPL overrides the choice.
// Work-item order (SCI_TV_ORDER: 0 bands of a frame adjacent, 1 frames of
// a tile adjacent).  Frame-fastest is faster for both variants at
// 2048 x 2048 x 24 (385 vs 395 us plain; the on-load projection shares the
// tile's map rows across frames in L1/L2).
static int frame_fast_order(bool) {
    if (const char *e = getenv("SCI_TV_ORDER")) return atoi(e) ? 1 : 0;
    return 1;
}

// Pipeline lag (1: chained stages, 2: independent stages); SCI_TV_LAG
// overrides the choice.
static int choose_lag() {
    if (const char *e = getenv("SCI_TV_LAG")) {
        const int v = atoi(e);
        if (v == 1 || v == 2) return v;
    }
    return 1;
}

static int choose_cpl(int64_t W) {
    if (const char *e = getenv("SCI_TV_CPL")) {
        const int v = atoi(e);
        if (v == 2 || v == 4) return v;
    }
    // narrow frames: a 128-column band wastes up to half its columns on a
    // 256-wide frame, and 64-column bands give twice the warps (spectral
    // workload, 256 x 256 x 28: 4.06 vs 4.36 ms per solve)
    return W <= 512 ? 2 : 4;
}

// Host driver: all passes of one TV call.  Used by the C ABI and the solvers.
// flags & 1: run all n_iter_max steps without the stop test (the unrolled,
// differentiable form).  proj (nullable): apply the GAP projection
// f = x + lam (c phi_b) while loading the input x (see tv_proj_supported).
// Update rule of a pipeline run: RULE_SKIMAGE takes tau = 1/4 and
// tau / weight; the MATLAB rules their own constants and run without the
// stop test (see sci_tv.cuh).
struct RuleArgs {
    int rule = tv::RULE_SKIMAGE;
    float tau = 0.f, tw = 0.f, c1 = 0.f, c2 = 0.f;
    float *tape_p = nullptr, *tape_u = nullptr;  // single-pass tape (sci_tv_tape.cu)
    // with the on-load projection: also store t = u + (u - f) (the lean
    // pass only, PROJ 3; the fused ADMM iteration's next t = theta + b)
    float *tout = nullptr;
};

static int tv_launch_core(const float *f, float *u, float *resid, int64_t nf, int64_t H,
                          int64_t W, int64_t fs, float weight, float eps, int K, int *steps,
                          double *energy_out, void *workspace, size_t ws_bytes, cudaStream_t s,
                          int force_R, int flags, const uint32_t *proj_bits, const float *proj_c,
                          float proj_lam, const RuleArgs &ra) {
    const bool tape = ra.tape_p != nullptr;
    const bool no_stop = (flags & 1) != 0 || ra.rule != tv::RULE_SKIMAGE || tape;
    const bool proj = proj_bits != nullptr;
    using namespace tv;
    SCI_CHECK_ARG(!tape || (ra.tape_u && K >= 2 && K - 1 <= SMAX && !proj && !resid &&
                            ra.rule == RULE_SKIMAGE),
                  "tv: a tape needs one pass (2 <= K <= 5), no projection, no resid");
    SCI_CHECK_ARG(f && u && nf >= 1 && H >= 1 && W >= 1, "tv: bad arguments");
    SCI_CHECK_ARG(K >= 1, "tv: n_iter_max must be >= 1");
    SCI_CHECK_ARG(weight > 0.f, "tv: weight must be > 0 (got %g)", (double)weight);
    SCI_CHECK_ARG(!proj || ra.rule == RULE_SKIMAGE, "tv: on-load projection needs the default rule");
    SCI_CHECK_ARG(f != u, "tv: input and output must not alias");
    SCI_CHECK_ARG(H <= (1 << 30) && W <= (1 << 30) && nf <= (1 << 30), "tv: sizes too large");
    const size_t need = ws_layout(nf, H, W, K, nullptr, nullptr);
    SCI_CHECK_ARG(workspace && ws_bytes >= need, "tv: workspace of %zu bytes needed, got %zu",
                  need, ws_bytes);
    if (proj) {
        SCI_CHECK_ARG(proj_c && nf <= 32 && K >= 2 && K <= SMAX + 1 && !resid && !no_stop,
                      "tv: on-load projection needs K in [2, 5], nf <= 32, no resid");
    }
    if (K == 1) {
        k_copy_frames<<<(unsigned)std::min<int64_t>((nf * fs + 255) / 256, kSMs * 16), 256, 0, s>>>(
            f, u, resid, nf * fs, steps, (int)nf);
        SCI_LAUNCHED("k_copy_frames");
        return SCI_OK;
    }
    Workspace w;
    ws_layout(nf, H, W, K, &w, static_cast<char *>(workspace));
    double *energy = energy_out ? energy_out : w.energy;
    const size_t ne = sizeof(double) * (size_t)(nf * K * 2);
    // flags & 4: the caller's preceding kernel cleared the energy sums and
    // the ticket (tv_clear_region), so that this launch follows it directly
    // (a memset node between two kernels of the solver graphs cost about
    // 6 us per iteration); runs without a stop test read neither
    SCI_CHECK_ARG(!(flags & 4) || energy == w.energy,
                  "tv: pre-cleared sums need the workspace's own energy buffer");
    if ((flags & 4) || (no_stop && !energy_out)) {
    } else if (energy == w.energy) {
        SCI_CUDA(cudaMemsetAsync(energy, 0, ne + sizeof(unsigned), s));  // and the ticket
    } else {
        SCI_CUDA(cudaMemsetAsync(energy, 0, ne, s));
        SCI_CUDA(cudaMemsetAsync(w.ticket, 0, sizeof(unsigned), s));
    }
    const int U = K - 1;  // dual updates
    // done flags are read only by later passes; steps are written by the
    // stop-test launch of the last window (K >= 3) or here
    if (U > SMAX || ((K < 3 || no_stop) && steps)) {
        k_init_done<<<(unsigned)((nf + 255) / 256), 256, 0, s>>>(w.done, steps, K, (int)nf);
        SCI_LAUNCHED("k_init_done");
    }

    // the generic pipeline's on-load projection and MATLAB rules are built
    // for 4 columns; the lean pass takes 2 or 4
    const int lag = (proj || tape || ra.rule != RULE_SKIMAGE) ? 1 : choose_lag();
    const bool slim_ok = slim_enabled() && ra.rule == RULE_SKIMAGE && !tape && !resid &&
                         U <= SMAX && lag == 1;
    auto aligned_for = [&](int c) {
        return (W % c == 0) && (fs % c == 0) && W >= c &&
               ((reinterpret_cast<uintptr_t>(f) | reinterpret_cast<uintptr_t>(u) |
                 reinterpret_cast<uintptr_t>(resid) | reinterpret_cast<uintptr_t>(proj_bits) |
                 reinterpret_cast<uintptr_t>(proj_c)) % (4 * c) == 0);
    };
    // flags bits 8-11: columns per lane forced by the caller (2 or 4)
    const int fcpl = (flags >> 8) & 0xf;
    const int cpl_pick = (fcpl == 2 || fcpl == 4) ? fcpl : choose_cpl(W);
    const bool slim = slim_ok && aligned_for(cpl_pick) &&
                      (!ra.tout || (reinterpret_cast<uintptr_t>(ra.tout) % (4 * cpl_pick)) == 0);
    SCI_CHECK_ARG(!ra.tout || (proj && slim), "tv: the t output needs the lean pass with the "
                                              "on-load projection (aligned frames)");
    const int pmode = proj ? (ra.tout ? 3 : 1) : 0;  // the lean pass's PROJ
    const int cpl = slim ? cpl_pick : ((proj || ra.rule != RULE_SKIMAGE) ? 4 : cpl_pick);
    const bool vec = (W % cpl == 0) && (fs % cpl == 0) &&
                     ((reinterpret_cast<uintptr_t>(f) | reinterpret_cast<uintptr_t>(u) |
                       reinterpret_cast<uintptr_t>(resid)) % (4 * cpl) == 0);
    const int minb = slim_minb(cpl);
    const float *pin = nullptr;
    float *pbuf[2] = {w.pa, w.pb};
    int pi = 0;
    for (int a = 0; a < U; a += SMAX) {
        const int SG = std::min(SMAX, U - a);
        const bool PIN = a > 0, FINAL = (a + SG == U);
        Pass P{};
        P.f = f;
        P.u = u;
        P.resid = resid;
        P.p_in = pin;
        P.p_out = FINAL ? nullptr : pbuf[pi];
        P.energy = energy;
        P.done = w.done;
        P.steps = steps;
        P.fs = fs;
        P.nf = (int)nf;
        P.H = (int)H;
        P.W = (int)W;
        P.K = K;
        P.a = a;
        if (ra.rule == RULE_SKIMAGE) {
            P.tau = 0.25f;
            P.tw = 0.25f / weight;
        } else {
            P.tau = ra.tau;
            P.tw = ra.tw;
            P.c1 = ra.c1;
            P.c2 = ra.c2;
        }
        P.weight = weight;
        P.eps = eps;
        P.cpl = cpl;
        P.hl = round_up(SG + (PIN ? 1 : 0), cpl);
        P.hr = round_up(SG, cpl);
        P.own = 32 * cpl - P.hl - P.hr;
        P.ht = SG + (PIN ? 1 : 0);
        P.lag = lag;
        P.proj = proj ? 1 : 0;
        P.tout = ra.tout;
        P.bits = proj_bits;
        P.cmap = proj_c;
        P.lam = proj_lam;
        P.frame_fast = frame_fast_order(proj);
        P.nbands = band_count((int)W, 32 * cpl, P.hl, P.hr);
        if (force_R > 0) P.R = force_R;
        else if (slim)
            P.R = choose_R_slim(nf, P.nbands, (int)H, SG,
                                kSMs * slim_resident_blocks(cpl, SG, minb, pmode));
        else P.R = choose_R(nf, P.nbands, (int)H);
        P.nchunks = (int)((H + P.R - 1) / P.R);
        P.S = SG;
        P.vec = vec ? 1 : 0;
        P.tape_p = ra.tape_p;
        P.tape_u = ra.tape_u;
        // the stop test can change the result only when a step k in
        // [1, K-2] lies in this pass's window; then the main launch's last
        // block decides it per frame
        const bool stop_test = !no_stop && std::max(1, a) <= std::min(a + SG - 1, K - 2);
        P.stopj = stop_test ? w.stopj : nullptr;
        P.ticket = stop_test ? w.ticket : nullptr;
        const int per_frame_blocks = (P.nbands * P.nchunks + WPB - 1) / WPB;
        P.gpf = std::max(1, std::min(per_frame_blocks, 16));
        if (slim) {
            launch_slim(P, SG, minb, pmode, s);
        } else if (tape) {
            launch_tape(P, SG, s);
        } else if (ra.rule == RULE_CHAM_ITV) {
            launch_rule1(P, SG, PIN, FINAL, s);
        } else if (ra.rule == RULE_CHAM_ATV) {
            launch_rule2(P, SG, PIN, FINAL, s);
        } else if (ra.rule == RULE_CLIP) {
            launch_rule3(P, SG, PIN, FINAL, s);
        } else if (proj) {
            launch_main_proj(P, SG, s);
        } else if (SG == SMAX) {
            if (lag == 2) launch_main4_lag2(P, PIN, FINAL, s);
            else if (cpl == 2) launch_main4_c2(P, PIN, FINAL, s);
            else launch_main4_c4(P, PIN, FINAL, s);
        } else {
            launch_main123(P, SG, PIN, s);
        }
        SCI_LAUNCHED("k_tv_main");
        if (stop_test) {
            if (slim) launch_slim_fix(P, pmode, s);
            else if (proj) launch_fixup_proj(P, s);
            else launch_fixup(P, PIN, s);
            SCI_LAUNCHED("k_tv_fixup");
        }
        pin = P.p_out;
        pi ^= 1;
    }
    return SCI_OK;
}

int tv_launch_impl(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
                   int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
                   void *workspace, size_t ws_bytes, cudaStream_t s, int force_R, int flags,
                   const uint32_t *proj_bits, const float *proj_c, float proj_lam) {
    return tv_launch_core(f, u, resid, nf, H, W, fs, weight, eps, K, steps, energy_out,
                          workspace, ws_bytes, s, force_R, flags, proj_bits, proj_c, proj_lam,
                          RuleArgs{});
}

// tv_launch_impl with the on-load projection that also stores t = u + (u -
// f) into tout (the lean pass; see RuleArgs::tout).
int tv_launch_tout(const float *f, float *u, int64_t nf, int64_t H, int64_t W, int64_t fs,
                   float weight, float eps, int K, int *steps, void *workspace, size_t ws_bytes,
                   cudaStream_t s, int flags, const uint32_t *proj_bits, const float *proj_c,
                   float proj_lam, float *tout) {
    RuleArgs ra;
    ra.tout = tout;
    return tv_launch_core(f, u, nullptr, nf, H, W, fs, weight, eps, K, steps, nullptr,
                          workspace, ws_bytes, s, 0, flags, proj_bits, proj_c, proj_lam, ra);
}

// A MATLAB-rule run of `updates` dual updates (rule, tau, tw, c1, c2 as in
// sci_tv.cuh); the workspace is tv_workspace_bytes(nf, H, W, updates + 1).
// TV of nf frames (K Chambolle steps, 2 <= K <= 5, no stop test) that also
// writes its tape: p_1..p_{K-1} to tape_p [K-1][nf][2][H][W] and
// u_1..u_{K-2} to tape_u [K-2][nf][H][W].
int tv_launch_tape(const float *f, float *u, int64_t nf, int64_t H, int64_t W, float weight,
                   int K, float *tape_p, float *tape_u, void *workspace, size_t ws_bytes,
                   cudaStream_t s) {
    SCI_CHECK_ARG(tape_p && tape_u, "tv: null tape");
    RuleArgs ra;
    ra.tape_p = tape_p;
    ra.tape_u = tape_u;
    return tv_launch_core(f, u, nullptr, nf, H, W, H * W, weight, 0.f, K, nullptr, nullptr,
                          workspace, ws_bytes, s, 0, 1, nullptr, nullptr, 0.f, ra);
}

int tv_launch_rule(int rule, const float *f, float *u, float *resid, int64_t nf, int64_t H,
                   int64_t W, int updates, float tau, float tw, float c1, float c2, int *steps,
                   void *workspace, size_t ws_bytes, cudaStream_t s) {
    SCI_CHECK_ARG(rule >= tv::RULE_CHAM_ITV && rule <= tv::RULE_CLIP && updates >= 0,
                  "tv: bad rule arguments");
    RuleArgs ra;
    ra.rule = rule;
    ra.tau = tau;
    ra.tw = tw;
    ra.c1 = c1;
    ra.c2 = c2;
    return tv_launch_core(f, u, resid, nf, H, W, H * W, 1.0f, 0.f, updates + 1, steps, nullptr,
                          workspace, ws_bytes, s, 0, 1, nullptr, nullptr, 0.f, ra);
}

int tv_launch_flags(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
                    int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
                    void *workspace, size_t ws_bytes, cudaStream_t s, int force_R, int flags) {
    return tv_launch_impl(f, u, resid, nf, H, W, fs, weight, eps, K, steps, energy_out,
                          workspace, ws_bytes, s, force_R, flags, nullptr, nullptr, 0.f);
}

int tv_launch(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
              int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
              void *workspace, size_t ws_bytes, cudaStream_t s, int force_R) {
    return tv_launch_flags(f, u, resid, nf, H, W, fs, weight, eps, K, steps, energy_out,
                           workspace, ws_bytes, s, force_R, 0);
}

// The on-load projection path covers one measurement of <= 32 frames with a
// packed mask, 2..5 Chambolle steps (one pass) and 16-byte aligned rows.
// On by default (SCI_FUSED_PROJ=0 turns it off): with the lean TV pass,
// whose input rows come through shared-memory rings, the projection costs
// the pass little, and the iteration at 2048 x 2048 x 24 goes from 2123 to
// 2180-2187 iter/s (residual pass 73 us instead of the 141 us projection).
// With the generic pipeline it was slower (552 + 73 us against 385 + 179).
bool tv_proj_supported(int64_t nf, int64_t W, int K) {
    const char *e = getenv("SCI_FUSED_PROJ");
    return !(e && atoi(e) == 0) && slim_enabled() && nf <= 32 && K >= 2 &&
           K <= tv::SMAX + 1 && W % 4 == 0 && !getenv("SCI_TV_LAG");
}

size_t tv_workspace_bytes(int64_t nf, int64_t H, int64_t W, int K) {
    return tv::ws_layout(nf, H, W, K, nullptr, nullptr);
}

// The stop-test sums and ticket of a TV workspace, as 8-byte words to clear
// (see flags & 4 of tv_launch_core).
double *tv_clear_region(int64_t nf, int64_t H, int64_t W, int K, void *workspace, int *words) {
    tv::Workspace w;
    tv::ws_layout(nf, H, W, K, &w, static_cast<char *>(workspace));
    *words = (int)(nf * K * 2) + 1;
    return w.energy;
}

}  // namespace sci

extern "C" {

int sci_tv_workspace_bytes(int64_t nframes, int64_t H, int64_t W, int n_iter_max,
                           size_t *bytes) {
    SCI_CHECK_ARG(bytes && nframes >= 1 && H >= 1 && W >= 1 && n_iter_max >= 1,
                  "sci_tv_workspace_bytes: bad argument");
    *bytes = sci::tv_workspace_bytes(nframes, H, W, n_iter_max);
    return SCI_OK;
}

int sci_tv_chambolle(const float *f, float *u, float *resid, int64_t nframes, int64_t H,
                     int64_t W, float weight, float eps, int n_iter_max, int *steps,
                     double *energy, void *workspace, size_t workspace_bytes, void *stream) {
    return sci::tv_launch(f, u, resid, nframes, H, W, H * W, weight, eps, n_iter_max, steps,
                          energy, workspace, workspace_bytes, sci::as_stream(stream), 0);
}

}  // extern "C"
