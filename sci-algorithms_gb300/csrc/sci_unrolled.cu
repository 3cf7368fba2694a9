// Differentiable unrolled GAP-TV: forward with outer-iterate checkpoints and
// a hand-written reverse pass.
//
// Model (a batch of N scenes sharing one learnable mask):
//   Phi = sigmoid(logits) (B x H x W), Phi_sum = sum_b Phi_b,
//   y_n = A(x_true_n), x^0 = At(y / Phi_sum),
//   for k < K (GAP with acceleration, pnp_sci_algo.py:641-643):
//     yb = A(x^k); y1 += y - yb; q = (y1 - yb) / Phi_sum;
//     v^k = x^k + lambda_k At(q);   x^{k+1} = TV(v^k)   (fixed T Chambolle
//     steps, no stop test: the stop rule is not differentiable)
//   loss = mean (x^K - x_true)^2.
// The forward keeps x^k and y1^k and the reverse pass recomputes v^k and
// each TV call from v^k step by step; with SCI_UNROLLED_TAPE=1 the forward
// also keeps, when they fit (up to 48 GiB), v^k and the tape (u_k, p_{k+1})
// its TV pipeline writes as it runs, and the reverse pass reads them.  The reverse
// pass runs the adjoint of every TV step:
//   p_{k+1} = (p_k - tau g_k) r_k,  r_k = 1 / (1 + (tau/w) n_k),  n_k = |g_k|,
//   gbar_k = -tau r_k pbar_{k+1} - (tau/w) r_k (g_k / n_k) <pbar_{k+1}, p_{k+1}>
//            (0 for the second term where n_k = 0: the safe-norm convention),
//   ubar_k = -div gbar_k,  fbar += ubar_k,  pbar_k = r_k pbar_{k+1} + grad ubar_k.
// then the adjoint of the projection (including d/dPhi through A, At and
// Phi_sum, and d/dlambda_k), and finally of the measurement and x^0.
#include <cstdlib>
#include <string>

#include "sci_common.cuh"
#include "sci_graph.cuh"

namespace sci {

int tv_launch_flags(const float *f, float *u, float *resid, int64_t nf, int64_t H, int64_t W,
                    int64_t fs, float weight, float eps, int K, int *steps, double *energy_out,
                    void *workspace, size_t ws_bytes, cudaStream_t s, int force_R, int flags);
int tv_launch_tape(const float *f, float *u, int64_t nf, int64_t H, int64_t W, float weight,
                   int K, float *tape_p, float *tape_u, void *workspace, size_t ws_bytes,
                   cudaStream_t s);
size_t tv_workspace_bytes(int64_t nf, int64_t H, int64_t W, int K);

namespace unr {

constexpr int kNoStop = 1;  // tv_launch_flags: run all steps, no stop test

inline dim3 grid1(int64_t n, int t) {
    int64_t b = (n + t - 1) / t;
    if (b > (int64_t)kSMs * 16) b = (int64_t)kSMs * 16;
    return dim3((unsigned)(b < 1 ? 1 : b));
}

#define GRID_LOOP(i, n)                                                          \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n);    \
         i += (int64_t)gridDim.x * blockDim.x)

// One thread per pixel of a frame stack on a (W/32, H/8, frames) grid of
// 32 x 8 blocks (grid3): column c, row r, frame f, in-frame index p,
// stack index i.  No index divisions.
#define PIXEL_3D(H, W)                                                          \
    const int c = blockIdx.x * blockDim.x + threadIdx.x;                        \
    const int r = blockIdx.y * blockDim.y + threadIdx.y;                        \
    if (r >= (H) || c >= (W)) return;                                           \
    const int64_t f = blockIdx.z;                                               \
    const int64_t p = (int64_t)r * (W) + c, i = f * hw + p;                     \
    (void)i

inline dim3 grid3(int64_t nf, int64_t H, int64_t W) {
    return dim3((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8), (unsigned)nf);
}
const dim3 kBlk3(32, 8);

// ------------------------------------------------------------- forward
__global__ void k_mask(const float *__restrict__ logits, float *__restrict__ phi,
                       float *__restrict__ ps, int B, int64_t hw) {
    GRID_LOOP(p, hw) {
        float s = 0.f;
        for (int b = 0; b < B; ++b) {
            const float m = 1.f / (1.f + expf(-logits[b * hw + p]));
            phi[b * hw + p] = m;
            s += m;
        }
        ps[p] = s;
    }
}

// y_n = A(x_true_n); x^0_n = At(y_n / Phi_sum)
__global__ void k_meas_x0(const float *__restrict__ xt, const float *__restrict__ phi,
                          const float *__restrict__ ps, float *__restrict__ y,
                          float *__restrict__ x0, int N, int B, int64_t hw) {
    GRID_LOOP(i, (int64_t)N * hw) {
        const int n = (int)(i / hw);
        const int64_t p = i - (int64_t)n * hw;
        const float *xn = xt + (int64_t)n * B * hw;
        float s = 0.f;
        for (int b = 0; b < B; ++b) s = fmaf(xn[b * hw + p], phi[b * hw + p], s);
        y[i] = s;
        const float s0 = s / ps[p];
        float *x0n = x0 + (int64_t)n * B * hw;
        for (int b = 0; b < B; ++b) x0n[b * hw + p] = phi[b * hw + p] * s0;
    }
}

// yb = A(x); y1 = y1_prev + (y - yb); v = x + lambda (phi (y1 - yb)/Phi_sum)
__global__ void k_proj_fwd(const float *__restrict__ x, const float *__restrict__ phi,
                           const float *__restrict__ ps, const float *__restrict__ y,
                           const float *__restrict__ y1_prev, float *__restrict__ y1,
                           float *__restrict__ v, const float *__restrict__ lambdas, int k,
                           int N, int B, int64_t hw) {
    const float lam = lambdas[k];
    GRID_LOOP(i, (int64_t)N * hw) {
        const int n = (int)(i / hw);
        const int64_t p = i - (int64_t)n * hw;
        const float *xn = x + (int64_t)n * B * hw;
        float yb = 0.f;
        for (int b = 0; b < B; ++b) yb = fmaf(xn[b * hw + p], phi[b * hw + p], yb);
        const float t = (y1_prev ? y1_prev[i] : 0.f) + (y[i] - yb);
        y1[i] = t;
        const float q = (t - yb) / ps[p];
        float *vn = v + (int64_t)n * B * hw;
        for (int b = 0; b < B; ++b) vn[b * hw + p] = fmaf(lam, q * phi[b * hw + p], xn[b * hw + p]);
    }
}

__global__ void k_mse(const float *__restrict__ a, const float *__restrict__ b,
                      float *__restrict__ grad, float gscale, int64_t n, double *out) {
    double acc = 0.0;
    GRID_LOOP(i, n) {
        const float d = a[i] - b[i];
        acc += (double)d * d;
        if (grad) grad[i] = gscale * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && out) atomicAdd(out, acc);
}

// ------------------------------------------------------- TV tape (recompute)
// One recomputed tape step on a 32 x 8 tile: p_{j+1} from u_j (and p_j;
// none for j = 0) on the tile and a one-pixel halo above / left of it, then
// u_{j+1} = f - div p_{j+1} on the tile (unless LASTP: the final p is not
// followed by a u).  Writes p_{j+1} and u_{j+1} to the tape.
template <bool P0, bool LASTP>
__global__ void __launch_bounds__(32 * 8) k_tape_step(
    const float *__restrict__ u, const float *__restrict__ pin, const float *__restrict__ f,
    float *__restrict__ pout, float *__restrict__ uout, int H, int W, float tau, float tw) {
    __shared__ float pr_s[9][33], pc_s[9][33];
    const int64_t hw = (int64_t)H * W;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
    const int64_t fo = (int64_t)blockIdx.z * hw;
    const float *uf = u + fo;
    const float *pir = pin + 2 * fo, *pic = pir + hw;
    float *por = pout + 2 * fo, *poc = por + hw;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    // p_{j+1} on [y0-1, y0+8) x [x0-1, x0+32); 0 outside the frame
    // two fixed rounds (297 cells, 256 threads), unrolled so that the loads
    // of both rounds are in flight together
#pragma unroll
    for (int rnd = 0; rnd < 2; ++rnd) {
        const int cidx = tid + rnd * 256;
        if (cidx >= 9 * 33) break;
        const int ly = cidx / 33, lx = cidx - ly * 33;
        const int i = y0 - 1 + ly, j = x0 - 1 + lx;
        float a = 0.f, b = 0.f;
        if (i >= 0 && i < H && j >= 0 && j < W) {
            const int64_t o = (int64_t)i * W + j;
            const float uc = uf[o];
            const float gr = (i + 1 < H) ? uf[o + W] - uc : 0.f;
            const float gc = (j + 1 < W) ? uf[o + 1] - uc : 0.f;
            const float ri = rcp_approx(fmaf(tw, sqrt_approx(fmaf(gr, gr, gc * gc)), 1.f));
            const float qr = P0 ? 0.f : pir[o], qc = P0 ? 0.f : pic[o];
            a = fmaf(-tau, gr, qr) * ri;
            b = fmaf(-tau, gc, qc) * ri;
            if (ly > 0 && lx > 0) {  // the tile itself goes to the tape
                por[o] = a;
                poc[o] = b;
            }
        }
        pr_s[ly][lx] = a;
        pc_s[ly][lx] = b;
    }
    if (LASTP) return;
    __syncthreads();
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int i = y0 + ty, j = x0 + tx;
    if (i >= H || j >= W) return;
    const int64_t o = (int64_t)i * W + j;
    const float d = ((pr_s[ty + 1][tx + 1] + pc_s[ty + 1][tx + 1]) - pr_s[ty][tx + 1]) -
                    pc_s[ty + 1][tx];
    uout[fo + o] = f[fo + o] - d;
}

// ---------------------------------------------------------- TV adjoint
// Per dual update k (last to first): with g_k = grad u_k, n_k = |g_k|,
// r_k = 1 / (1 + tw n_k) and p_{k+1} = r_k (p_k - tau g_k):
//   gbar_k = -tau r_k pbar_{k+1} - (tw r_k / n_k) <pbar_{k+1}, p_{k+1}> g_k
//   ubar_k = -div gbar_k;  fbar += ubar_k;  pbar_k = r_k pbar_{k+1} + grad ubar_k
// One adjoint step on a 32 x 8 tile of one frame: gbar on the
// tile and a one-pixel halo in shared memory, ubar = -div gbar on the tile
// and its right / bottom halo, then fbar += ubar and (not LAST) pbar_k =
// r_k pbar_{k+1} + grad ubar.  FIRST: pbar_{k+1} = grad xbar and fbar
// starts at xbar (u_T = f - div p_T with ubar_T = xbar).  gbar never
// leaves the chip: 9 planes of HBM traffic per step (16 when gbar was
// written out and read back by a second kernel).
constexpr int TBX = 32, TBY = 8;

template <bool FIRST, bool LAST>
__global__ void __launch_bounds__(TBX * TBY) k_tvb_step(
    const float *__restrict__ u, const float *__restrict__ pnext, const float *__restrict__ pb,
    const float *__restrict__ xbar, float *__restrict__ pb_out, float *__restrict__ fb,
    int H, int W, float tau, float tw) {
    __shared__ float gr_s[TBY + 2][TBX + 2], gc_s[TBY + 2][TBX + 2], ri_s[TBY + 2][TBX + 2];
    __shared__ float ub_s[TBY + 1][TBX + 1];
    const int64_t hw = (int64_t)H * W;
    const int x0 = blockIdx.x * TBX, y0 = blockIdx.y * TBY;
    const int64_t fo = (int64_t)blockIdx.z * hw;
    const float *uf = u + fo, *xb = xbar + fo;
    const float *pnr = pnext + 2 * fo, *pnc = pnr + hw;
    const float *pbr = pb + 2 * fo, *pbc = pbr + hw;
    const int tid = threadIdx.y * TBX + threadIdx.x;
    // 1. gbar (and r = 1 / (1 + tw |grad u|)) on [y0-1, y0+TBY] x [x0-1, x0+TBX]
    // two fixed rounds (340 cells, 256 threads), unrolled so that the loads
    // of both rounds are in flight together
#pragma unroll
    for (int rnd = 0; rnd < 2; ++rnd) {
        const int cidx = tid + rnd * TBX * TBY;
        if (cidx >= (TBY + 2) * (TBX + 2)) break;
        const int ly = cidx / (TBX + 2), lx = cidx - ly * (TBX + 2);
        const int i = y0 - 1 + ly, j = x0 - 1 + lx;
        float g1 = 0.f, g2 = 0.f, ri = 0.f;
        if (i >= 0 && i < H && j >= 0 && j < W) {
            const int64_t o = (int64_t)i * W + j;
            const bool hr = i + 1 < H, hc = j + 1 < W;
            const float uc = uf[o];
            const float gr = hr ? uf[o + W] - uc : 0.f;
            const float gc = hc ? uf[o + 1] - uc : 0.f;
            const float nrm = sqrt_approx(fmaf(gr, gr, gc * gc));
            ri = rcp_approx(fmaf(tw, nrm, 1.f));
            float br, bc;
            if (FIRST) {
                const float xc = xb[o];
                br = hr ? xb[o + W] - xc : 0.f;
                bc = hc ? xb[o + 1] - xc : 0.f;
            } else {
                br = pbr[o];
                bc = pbc[o];
            }
            const float dot = br * pnr[o] + bc * pnc[o];
            const float coef = nrm > 0.f ? -tw * ri * dot / nrm : 0.f;
            g1 = hr ? fmaf(-tau * ri, br, coef * gr) : 0.f;
            g2 = hc ? fmaf(-tau * ri, bc, coef * gc) : 0.f;
        }
        gr_s[ly][lx] = g1;
        gc_s[ly][lx] = g2;
        ri_s[ly][lx] = ri;
    }
    __syncthreads();
    // 2. ubar = -div gbar on [y0, y0+TBY] x [x0, x0+TBX] (gbar is 0 outside
    //    the frame, which gives div's zero boundary terms)
    for (int cidx = tid; cidx < (TBY + 1) * (TBX + 1); cidx += TBX * TBY) {
        const int ly = cidx / (TBX + 1), lx = cidx - ly * (TBX + 1);
        ub_s[ly][lx] = -(((gr_s[ly + 1][lx + 1] + gc_s[ly + 1][lx + 1]) - gr_s[ly][lx + 1]) -
                         gc_s[ly + 1][lx]);
    }
    __syncthreads();
    // 3. fbar and pbar_k on the tile
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int i = y0 + ty, j = x0 + tx;
    if (i >= H || j >= W) return;
    const int64_t o = (int64_t)i * W + j;
    const float ub = ub_s[ty][tx];
    fb[fo + o] = (FIRST ? xb[o] : fb[fo + o]) + ub;
    if (!LAST) {
        const bool hr = i + 1 < H, hc = j + 1 < W;
        float br, bc;
        if (FIRST) {
            const float xc = xb[o];
            br = hr ? xb[o + W] - xc : 0.f;
            bc = hc ? xb[o + 1] - xc : 0.f;
        } else {
            br = pbr[o];
            bc = pbc[o];
        }
        const float ri = ri_s[ty + 1][tx + 1];
        const float ubr = hr ? ub_s[ty + 1][tx] - ub : 0.f;
        const float ubc = hc ? ub_s[ty][tx + 1] - ub : 0.f;
        float *por = pb_out + 2 * fo, *poc = por + hw;
        por[o] = fmaf(ri, br, ubr);
        poc[o] = fmaf(ri, bc, ubc);
    }
}

// --------------------------------------------------- projection adjoint
// One thread per pixel, looping over the N items; accumulates dPhi, dPhi_sum
// and d lambda_k, carries dy1 and dy, and writes xbar^k.
__global__ void k_proj_bwd(const float *__restrict__ vb, const float *__restrict__ x,
                           const float *__restrict__ phi, const float *__restrict__ ps,
                           const float *__restrict__ y1, const float *__restrict__ lambdas, int k,
                           float *__restrict__ y1c, float *__restrict__ ybar,
                           float *__restrict__ phib, float *__restrict__ psb,
                           double *__restrict__ lamb, float *__restrict__ xb, int N, int B,
                           int64_t hw) {
    const float lam = lambdas[k];
    double lacc = 0.0;
    GRID_LOOP(p, hw) {
        const float s = ps[p];
        float psacc = 0.f;
        for (int n = 0; n < N; ++n) {
            const float *xn = x + (int64_t)n * B * hw;
            const float *vn = vb + (int64_t)n * B * hw;
            float yb = 0.f, pv = 0.f;
            for (int b = 0; b < B; ++b) {
                const float m = phi[b * hw + p];
                yb = fmaf(xn[b * hw + p], m, yb);
                pv = fmaf(vn[b * hw + p], m, pv);
            }
            const int64_t i = (int64_t)n * hw + p;
            const float q = (y1[i] - yb) / s;
            lacc += (double)pv * q;
            const float qb = lam * pv;
            const float y1t = y1c[i] + qb / s;
            psacc -= qb * q / s;
            const float ybb = -qb / s - y1t;
            ybar[i] += y1t;
            y1c[i] = y1t;
            float *xbn = xb + (int64_t)n * B * hw;
            for (int b = 0; b < B; ++b) {
                const float m = phi[b * hw + p];
                const float v = vn[b * hw + p];
                xbn[b * hw + p] = fmaf(m, ybb, v);
                phib[b * hw + p] += fmaf(q * lam, v, xn[b * hw + p] * ybb);
            }
        }
        psb[p] += psacc;
    }
    for (int o = 16; o > 0; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(lamb + k, lacc);
}

// The same adjoint with the items spread over IL lanes (threadIdx.y) of a
// 32-pixel block: lane l takes items l, l+IL, ... (at most IMAX, their
// per-item scalars in registers); the sums over items (dPhi_b, dPhi_sum)
// are reduced over the lanes in shared memory in a fixed order, so the
// result does not depend on scheduling.
constexpr int IL = 8, IMAX = 8;  // item lanes; items per lane (N <= 64)

__global__ void __launch_bounds__(32 * IL) k_proj_bwd_par(
    const float *__restrict__ vb, const float *__restrict__ x, const float *__restrict__ phi,
    const float *__restrict__ ps, const float *__restrict__ y1, const float *__restrict__ lambdas,
    int k, float *__restrict__ y1c, float *__restrict__ ybar, float *__restrict__ phib,
    float *__restrict__ psb, double *__restrict__ lamb, float *__restrict__ xb, int N, int B,
    int64_t hw) {
    __shared__ float red[IL][32];
    __shared__ double lred[IL];
    extern __shared__ float red_b[];  // [B][IL][32]
    const int64_t p = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool in = p < hw;
    const float lam = lambdas[k];
    const float s = in ? ps[p] : 1.f;
    float ql[IMAX], yl[IMAX];  // q * lambda and dL/dyb per item of this lane
    float psacc = 0.f;
    double lacc = 0.0;
#pragma unroll
    for (int t = 0; t < IMAX; ++t) {
        const int n = threadIdx.y + t * IL;
        ql[t] = yl[t] = 0.f;
        if (!in || n >= N) continue;
        const float *xn = x + (int64_t)n * B * hw;
        const float *vn = vb + (int64_t)n * B * hw;
        float yb = 0.f, pv = 0.f;
        for (int b = 0; b < B; ++b) {
            const float m = phi[b * hw + p];
            yb = fmaf(xn[b * hw + p], m, yb);
            pv = fmaf(vn[b * hw + p], m, pv);
        }
        const int64_t i = (int64_t)n * hw + p;
        const float q = (y1[i] - yb) / s;
        lacc += (double)pv * q;
        const float qb = lam * pv;
        const float y1t = y1c[i] + qb / s;
        psacc -= qb * q / s;
        const float ybb = -qb / s - y1t;
        ybar[i] += y1t;
        y1c[i] = y1t;
        ql[t] = q * lam;
        yl[t] = ybb;
    }
    // per frame: x bar of every item, and this lane's part of dPhi_b
    // (red_b[b][lane][pixel], summed over the lanes after one barrier)
    for (int b = 0; b < B; ++b) {
        float part = 0.f;
        const float m = in ? phi[b * hw + p] : 0.f;
#pragma unroll
        for (int t = 0; t < IMAX; ++t) {
            const int n = threadIdx.y + t * IL;
            if (!in || n >= N) continue;
            const int64_t o = (int64_t)n * B * hw + b * hw + p;
            const float v = vb[o];
            xb[o] = fmaf(m, yl[t], v);
            part += fmaf(ql[t], v, x[o] * yl[t]);
        }
        red_b[(b * IL + threadIdx.y) * 32 + threadIdx.x] = part;
    }
    red[threadIdx.y][threadIdx.x] = psacc;
    __syncthreads();
    if (in) {
        for (int b = threadIdx.y; b < B; b += IL) {
            float tot = 0.f;
#pragma unroll
            for (int l = 0; l < IL; ++l) tot += red_b[(b * IL + l) * 32 + threadIdx.x];
            phib[b * hw + p] += tot;
        }
        if (threadIdx.y == 0) {
            float tot = 0.f;
#pragma unroll
            for (int l = 0; l < IL; ++l) tot += red[l][threadIdx.x];
            psb[p] += tot;
        }
    }
    for (int o = 16; o > 0; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
    if (threadIdx.x == 0) lred[threadIdx.y] = lacc;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        double tot = 0.0;
        for (int l = 0; l < IL; ++l) tot += lred[l];
        atomicAdd(lamb + k, tot);
    }
}

// Adjoint of x^0 = At(y / Phi_sum), y = A(x_true), Phi_sum = sum Phi_b and
// Phi = sigmoid(logits): writes dlogits.
__global__ void k_init_bwd(const float *__restrict__ x0b, const float *__restrict__ xt,
                           const float *__restrict__ phi, const float *__restrict__ ps,
                           const float *__restrict__ y, const float *__restrict__ ybar,
                           float *__restrict__ phib, const float *__restrict__ psb,
                           float *__restrict__ glog, float gscale, int N, int B, int64_t hw) {
    GRID_LOOP(p, hw) {
        const float s = ps[p];
        float psacc = psb[p];
        for (int n = 0; n < N; ++n) {
            const int64_t i = (int64_t)n * hw + p;
            const float *xbn = x0b + (int64_t)n * B * hw;
            const float *xtn = xt + (int64_t)n * B * hw;
            const float s0 = y[i] / s;
            float s0b = 0.f;
            for (int b = 0; b < B; ++b) s0b = fmaf(phi[b * hw + p], xbn[b * hw + p], s0b);
            const float yt = ybar[i] + s0b / s;
            psacc -= s0b * s0 / s;
            for (int b = 0; b < B; ++b)
                phib[b * hw + p] += fmaf(s0, xbn[b * hw + p], xtn[b * hw + p] * yt);
        }
        for (int b = 0; b < B; ++b) {
            const float m = phi[b * hw + p];
            glog[b * hw + p] = gscale * (phib[b * hw + p] + psacc) * m * (1.f - m);
        }
    }
}

struct Ws {
    float *phi, *ps, *y, *X, *Y1, *V;          // forward
    float *tu, *tp;                            // tape: u_1..u_{T-1}, p_1..p_{T-1}
    // stored tapes (when they fit): per outer iteration k, v^k and the
    // forward TV's tape, so that the reverse pass recomputes neither
    bool stored;
    float *Vall, *tpall, *tuall;               // [K][nbhw], [K][U][2 nbhw], [K][U-1][nbhw]
    float *pb0, *pb1, *fb, *xb, *y1c, *ybar, *phib, *psb;  // reverse
    double *loss;
    void *tv;
    size_t tv_bytes;
};

// Whether the forward keeps v^k and the TV tape of every outer iteration
// (3 (T-1) planes per iteration) for the reverse pass.  By default it keeps
// only the outer iterates and the reverse pass recomputes each inner TV
// loop (the checkpoint-only form); SCI_UNROLLED_TAPE=1 stores the tapes
// instead when they fit in 48 GiB.
bool stored_tape(int64_t N, int64_t B, int64_t H, int64_t W, int K, int T) {
    const char *e = getenv("SCI_UNROLLED_TAPE");
    if (!(e && e[0] == '1')) return false;
    const double bytes = 4.0 * (double)(N * B * H * W) * 3.0 * (T - 1) * K;
    return bytes <= 48.0 * (1ull << 30);
}

size_t layout(int64_t N, int64_t B, int64_t H, int64_t W, int K, int T, Ws *w, char *base) {
    const size_t hw = (size_t)(H * W), nbhw = (size_t)(N * B) * hw, nhw = (size_t)N * hw;
    const int U = T - 1;
    const bool st = stored_tape(N, B, H, W, K, T);
    size_t off = 0;
    auto take = [&](size_t floats) {
        size_t o = off;
        off += (floats * 4 + 255) & ~size_t(255);
        return o;
    };
    const size_t o_phi = take(B * hw), o_ps = take(hw), o_y = take(nhw);
    const size_t o_X = take((K + 1) * nbhw), o_Y1 = take((size_t)K * nhw), o_V = take(nbhw);
    const size_t o_tu = take((size_t)(U > 1 ? U - 1 : 1) * nbhw), o_tp = take((size_t)U * 2 * nbhw);
    const size_t o_pb0 = take(2 * nbhw), o_pb1 = take(2 * nbhw);
    const size_t o_fb = take(nbhw), o_xb = take(nbhw), o_y1c = take(nhw), o_ybar = take(nhw);
    const size_t o_phib = take(B * hw), o_psb = take(hw), o_loss = take(4);
    size_t o_Vall = 0, o_tpall = 0, o_tuall = 0;
    if (st) {
        o_Vall = take((size_t)K * nbhw);
        o_tpall = take((size_t)K * U * 2 * nbhw);
        o_tuall = take((size_t)K * (U > 1 ? U - 1 : 1) * nbhw);
    }
    const size_t tvb = tv_workspace_bytes(N * B, H, W, T);
    const size_t o_tv = off;
    off += (tvb + 255) & ~size_t(255);
    if (w) {
        auto F = [&](size_t o) { return reinterpret_cast<float *>(base + o); };
        w->phi = F(o_phi); w->ps = F(o_ps); w->y = F(o_y); w->X = F(o_X); w->Y1 = F(o_Y1);
        w->V = F(o_V); w->tu = F(o_tu); w->tp = F(o_tp); w->pb0 = F(o_pb0); w->pb1 = F(o_pb1);
        w->fb = F(o_fb); w->xb = F(o_xb); w->y1c = F(o_y1c);
        w->ybar = F(o_ybar); w->phib = F(o_phib); w->psb = F(o_psb);
        w->loss = reinterpret_cast<double *>(base + o_loss);
        w->stored = st;
        w->Vall = st ? F(o_Vall) : nullptr;
        w->tpall = st ? F(o_tpall) : nullptr;
        w->tuall = st ? F(o_tuall) : nullptr;
        w->tv = base + o_tv;
        w->tv_bytes = tvb;
    }
    return off;
}

int check(int64_t N, int64_t B, int64_t H, int64_t W, int K, int T, float weight) {
    SCI_CHECK_ARG(N >= 1 && B >= 1 && H >= 1 && W >= 1 && K >= 1, "unrolled: invalid sizes");
    SCI_CHECK_ARG(N * B <= 65535 && H <= (1 << 19), "unrolled: N * B <= 65535 frames");
    SCI_CHECK_ARG(T >= 2 && T <= 5, "unrolled: tv_iters must be in [2, 5] (got %d)", T);
    SCI_CHECK_ARG(weight > 0.f, "unrolled: tv_weight must be > 0");
    return SCI_OK;
}

// forward: fills the checkpoints; loss (device double) = mean sq. error
int forward(const float *logits, const float *lambdas, const float *xt, int64_t N, int64_t B,
            int64_t H, int64_t W, int K, int T, float weight, Ws &w, cudaStream_t s) {
    const int64_t hw = H * W, nbhw = N * B * hw;
    const dim3 g = grid1(N * hw, 256);
    k_mask<<<grid1(hw, 256), 256, 0, s>>>(logits, w.phi, w.ps, (int)B, hw);
    k_meas_x0<<<g, 256, 0, s>>>(xt, w.phi, w.ps, w.y, w.X, (int)N, (int)B, hw);
    SCI_LAUNCHED("k_meas_x0");
    const int U = T - 1;
    for (int k = 0; k < K; ++k) {
        float *V = w.stored ? w.Vall + k * nbhw : w.V;
        k_proj_fwd<<<g, 256, 0, s>>>(w.X + k * nbhw, w.phi, w.ps, w.y,
                                     k ? w.Y1 + (k - 1) * N * hw : nullptr, w.Y1 + k * N * hw,
                                     V, lambdas, k, (int)N, (int)B, hw);
        SCI_LAUNCHED("k_proj_fwd");
        int e = w.stored
                    ? tv_launch_tape(V, w.X + (k + 1) * nbhw, N * B, H, W, weight, T,
                                     w.tpall + (int64_t)k * U * 2 * nbhw,
                                     w.tuall + (int64_t)k * (U > 1 ? U - 1 : 1) * nbhw, w.tv,
                                     w.tv_bytes, s)
                    : tv_launch_flags(V, w.X + (k + 1) * nbhw, nullptr, N * B, H, W, hw, weight,
                                      0.f, T, nullptr, nullptr, w.tv, w.tv_bytes, s, 0, kNoStop);
        if (e) return e;
    }
    SCI_CUDA(cudaMemsetAsync(w.loss, 0, sizeof(double), s));
    k_mse<<<grid1(nbhw, 256), 256, 0, s>>>(w.X + K * nbhw, xt, nullptr, 0.f, nbhw, w.loss);
    SCI_LAUNCHED("k_mse");
    return SCI_OK;
}

// Whole forward / reverse passes run as cached CUDA graphs (sci_graph.cuh),
// keyed by every argument: the reverse pass is ~20 launches per outer
// iteration.
template <typename... T>
std::string make_key(const T &...v) {
    std::string k;
    (k.append(reinterpret_cast<const char *>(&v), sizeof(T)), ...);
    return k;
}

}  // namespace unr
}  // namespace sci

using namespace sci;
using namespace sci::unr;

extern "C" {

int sci_unrolled_workspace_bytes(int64_t N, int64_t B, int64_t H, int64_t W, int K, int tv_iters,
                                 size_t *bytes) {
    SCI_CHECK_ARG(bytes, "null bytes");
    if (int e = check(N, B, H, W, K, tv_iters, 1.f)) return e;
    *bytes = layout(N, B, H, W, K, tv_iters, nullptr, nullptr);
    return SCI_OK;
}

int sci_unrolled_fwd(const float *logits, const float *lambdas, const float *x_true, int64_t N,
                     int64_t B, int64_t H, int64_t W, int K, int tv_iters, float tv_weight,
                     double *loss, float *x_out, void *workspace, size_t workspace_bytes,
                     void *stream) {
    if (int e = check(N, B, H, W, K, tv_iters, tv_weight)) return e;
    SCI_CHECK_ARG(logits && lambdas && x_true, "sci_unrolled_fwd: null pointer");
    const size_t need = layout(N, B, H, W, K, tv_iters, nullptr, nullptr);
    SCI_CHECK_ARG(workspace && workspace_bytes >= need,
                  "sci_unrolled_fwd: workspace of %zu bytes needed, got %zu", need,
                  workspace_bytes);
    Ws w;
    layout(N, B, H, W, K, tv_iters, &w, static_cast<char *>(workspace));
    const int64_t nbhw = N * B * H * W;
    auto body = [&](cudaStream_t s) -> int {
        if (int e = forward(logits, lambdas, x_true, N, B, H, W, K, tv_iters, tv_weight, w, s))
            return e;
        if (loss)
            SCI_CUDA(cudaMemcpyAsync(loss, w.loss, sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (x_out)
            SCI_CUDA(cudaMemcpyAsync(x_out, w.X + (int64_t)K * nbhw, 4 * nbhw,
                                     cudaMemcpyDeviceToDevice, s));
        return SCI_OK;
    };
    const std::string key = make_key(1, logits, lambdas, x_true, N, B, H, W, K, tv_iters,
                                     tv_weight, loss, x_out, workspace, (int)w.stored);
    return run_graph("unrolled graph capture", key, as_stream(stream), body);
}

int sci_unrolled_bwd(const float *logits, const float *lambdas, const float *x_true, int64_t N,
                     int64_t B, int64_t H, int64_t W, int K, int tv_iters, float tv_weight,
                     float grad_loss, float *grad_logits, double *grad_lambdas,
                     void *workspace, size_t workspace_bytes, void *stream) {
    if (int e = check(N, B, H, W, K, tv_iters, tv_weight)) return e;
    SCI_CHECK_ARG(logits && lambdas && x_true && grad_logits && grad_lambdas,
                  "sci_unrolled_bwd: null pointer");
    const size_t need = layout(N, B, H, W, K, tv_iters, nullptr, nullptr);
    SCI_CHECK_ARG(workspace && workspace_bytes >= need,
                  "sci_unrolled_bwd: workspace of %zu bytes needed, got %zu", need,
                  workspace_bytes);
    Ws w;
    layout(N, B, H, W, K, tv_iters, &w, static_cast<char *>(workspace));
    const std::string key = make_key(2, logits, lambdas, x_true, N, B, H, W, K, tv_iters,
                                     tv_weight, grad_loss, grad_logits, grad_lambdas, workspace,
                                     (int)w.stored);
    return run_graph("unrolled graph capture", key, as_stream(stream), [&](cudaStream_t s) -> int {
    // The checkpoints of the preceding sci_unrolled_fwd call on this
    // workspace (same arguments) are used as they are.
    const int64_t hw = H * W, nbhw = N * B * hw, nhw = N * hw, nf = N * B;
    const int T = tv_iters, U = T - 1;
    const float tau = 0.25f, tw = 0.25f / tv_weight;
    const dim3 g = grid1(nbhw, 256), gp = grid1(hw, 128), g3 = grid3(nf, H, W);
    // dL/dx^K = grad_loss * 2 (x^K - x_true) / numel
    k_mse<<<g, 256, 0, s>>>(w.X + (int64_t)K * nbhw, x_true, w.xb,
                            2.f * grad_loss / (float)nbhw, nbhw, nullptr);
    SCI_LAUNCHED("k_mse");
    SCI_CUDA(cudaMemsetAsync(w.y1c, 0, 4 * nhw, s));
    SCI_CUDA(cudaMemsetAsync(w.ybar, 0, 4 * nhw, s));
    SCI_CUDA(cudaMemsetAsync(w.phib, 0, 4 * B * hw, s));
    SCI_CUDA(cudaMemsetAsync(w.psb, 0, 4 * hw, s));
    SCI_CUDA(cudaMemsetAsync(grad_lambdas, 0, sizeof(double) * K, s));
    for (int k = K - 1; k >= 0; --k) {
        // v^k and the TV tape: kept by the forward, or recomputed
        const float *V = w.stored ? w.Vall + k * nbhw : w.V;
        const float *tp = w.stored ? w.tpall + (int64_t)k * U * 2 * nbhw : w.tp;
        const float *tu = w.stored ? w.tuall + (int64_t)k * (U > 1 ? U - 1 : 1) * nbhw : w.tu;
        if (!w.stored) {
            k_proj_fwd<<<grid1(nhw, 256), 256, 0, s>>>(
                w.X + k * nbhw, w.phi, w.ps, w.y, k ? w.Y1 + (k - 1) * nhw : nullptr,
                w.Y1 + k * nhw, w.V, lambdas, k, (int)N, (int)B, hw);
            const float *u_prev = w.V;  // u_0 = f = v^k
            for (int j = 0; j < U; ++j) {
                float *pj = w.tp + (int64_t)j * 2 * nbhw;  // p_{j+1}
                const float *pprev = j ? w.tp + (int64_t)(j - 1) * 2 * nbhw : nullptr;
                float *uj = w.tu + (int64_t)j * nbhw;      // u_{j+1}
                const bool p0 = j == 0, lastp = j + 1 == U;
                if (p0 && lastp)
                    k_tape_step<true, true><<<g3, kBlk3, 0, s>>>(u_prev, pprev, w.V, pj, uj, (int)H,
                                                                 (int)W, tau, tw);
                else if (p0)
                    k_tape_step<true, false><<<g3, kBlk3, 0, s>>>(u_prev, pprev, w.V, pj, uj, (int)H,
                                                                  (int)W, tau, tw);
                else if (lastp)
                    k_tape_step<false, true><<<g3, kBlk3, 0, s>>>(u_prev, pprev, w.V, pj, uj, (int)H,
                                                                  (int)W, tau, tw);
                else
                    k_tape_step<false, false><<<g3, kBlk3, 0, s>>>(u_prev, pprev, w.V, pj, uj,
                                                                   (int)H, (int)W, tau, tw);
                u_prev = uj;
            }
            SCI_LAUNCHED("tv tape");
        }
        // TV adjoint: fbar = d/dv^k, one fused step per dual update
        float *pb_in = w.pb0, *pb_out = w.pb1;
        for (int j = U - 1; j >= 0; --j) {
            const float *uj = j == 0 ? V : tu + (int64_t)(j - 1) * nbhw;  // u_j
            const float *pn = tp + (int64_t)j * 2 * nbhw;                 // p_{j+1}
            const bool first = j == U - 1, last = j == 0;
            if (first && last)
                k_tvb_step<true, true><<<g3, kBlk3, 0, s>>>(uj, pn, pb_in, w.xb, pb_out, w.fb,
                                                            (int)H, (int)W, tau, tw);
            else if (first)
                k_tvb_step<true, false><<<g3, kBlk3, 0, s>>>(uj, pn, pb_in, w.xb, pb_out, w.fb,
                                                             (int)H, (int)W, tau, tw);
            else if (last)
                k_tvb_step<false, true><<<g3, kBlk3, 0, s>>>(uj, pn, pb_in, w.xb, pb_out, w.fb,
                                                             (int)H, (int)W, tau, tw);
            else
                k_tvb_step<false, false><<<g3, kBlk3, 0, s>>>(uj, pn, pb_in, w.xb, pb_out, w.fb,
                                                              (int)H, (int)W, tau, tw);
            float *t = pb_in;
            pb_in = pb_out;
            pb_out = t;
        }
        SCI_LAUNCHED("tv adjoint");
        // projection adjoint: xbar^k
        if (N <= IL * IMAX && B <= 40)
            k_proj_bwd_par<<<(unsigned)((hw + 31) / 32), dim3(32, IL),
                             sizeof(float) * (size_t)B * IL * 32, s>>>(
                w.fb, w.X + k * nbhw, w.phi, w.ps, w.Y1 + k * nhw, lambdas, k, w.y1c, w.ybar,
                w.phib, w.psb, grad_lambdas, w.xb, (int)N, (int)B, hw);
        else
            k_proj_bwd<<<gp, 128, 0, s>>>(w.fb, w.X + k * nbhw, w.phi, w.ps, w.Y1 + k * nhw,
                                           lambdas, k, w.y1c, w.ybar, w.phib, w.psb,
                                           grad_lambdas, w.xb, (int)N, (int)B, hw);
        SCI_LAUNCHED("k_proj_bwd");
    }
    k_init_bwd<<<gp, 128, 0, s>>>(w.xb, x_true, w.phi, w.ps, w.y, w.ybar, w.phib, w.psb,
                                  grad_logits, 1.f, (int)N, (int)B, hw);
    SCI_LAUNCHED("k_init_bwd");
    return SCI_OK;
    });
}

}  // extern "C"
