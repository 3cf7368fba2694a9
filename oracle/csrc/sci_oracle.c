/*
 * CPU oracle in C: float64 restatement of the GAP-TV / ADMM-TV path.
 *
 * TEST INFRASTRUCTURE ONLY.  The product never links, loads or calls this
 * library; tests/ and the CPU-baseline leg of bench.py load it through
 * ctypes, as the checker for sizes the numpy oracle (oracle/reference_port.py)
 * cannot finish in seconds.  It is pinned against that numpy oracle on
 * small inputs (tests/test_oracle.py, relative error <= 1e-12), and the
 * numpy oracle is pinned bit for bit against the reference's own code.
 *
 * Layout: planar, frame-major (B x H x W, W fastest), float64.
 *
 * Follows:
 *   A_   PnP_SCI/python/utils.py:10-15      y = sum_b phi_b x_b
 *   At_  PnP_SCI/python/utils.py:17-26      x_b = phi_b y
 *   GAP  PnP_SCI/python/pnp_sci_algo.py:636-650 (accelerated: 641-643)
 *   ADMM PnP_SCI/python/pnp_sci_algo.py:805-836
 *   TV   scikit-image 0.16 denoise_tv_chambolle (Chambolle 2004), called
 *        per frame at pnp_sci_algo.py:650 and :812; see
 *        oracle/tv_chambolle.py for the statement of the recurrence.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* y[h,w] = sum_b x[b,h,w] * phi[b,h,w] */
void orc_A(const double *x, const double *phi, double *y, i64 B, i64 H, i64 W) {
    const i64 hw = H * W;
#pragma omp parallel for schedule(static)
    for (i64 i = 0; i < hw; ++i) {
        double s = 0.0;
        for (i64 b = 0; b < B; ++b) s += x[b * hw + i] * phi[b * hw + i];
        y[i] = s;
    }
}

/* x[b,h,w] = y[h,w] * phi[b,h,w] */
void orc_At(const double *y, const double *phi, double *x, i64 B, i64 H, i64 W) {
    const i64 hw = H * W;
#pragma omp parallel for schedule(static)
    for (i64 i = 0; i < B * hw; ++i) x[i] = y[i % hw] * phi[i];
}

/*
 * Chambolle TV of `nframes` independent H x W frames.
 * steps_out[f] (nullable): executed steps of frame f.
 * energies_out (nullable): nframes x n_iter_max energies E_k (unset -> NAN).
 */
void orc_tv_chambolle(const double *f, double *u, i64 nframes, i64 H, i64 W,
                      double weight, double eps, int n_iter_max,
                      int *steps_out, double *energies_out) {
    const i64 hw = H * W;
    const double tau = 0.25;
    double *pr = (double *)calloc((size_t)(nframes * hw), sizeof(double));
    double *pc = (double *)calloc((size_t)(nframes * hw), sizeof(double));
    double *rowd = (double *)calloc((size_t)(nframes * H), sizeof(double));
    double *rown = (double *)calloc((size_t)(nframes * H), sizeof(double));
    int *active = (int *)malloc(sizeof(int) * (size_t)nframes);
    double *e_init = (double *)malloc(sizeof(double) * (size_t)nframes);
    double *e_prev = (double *)malloc(sizeof(double) * (size_t)nframes);
    for (i64 fr = 0; fr < nframes; ++fr) {
        active[fr] = 1;
        if (steps_out) steps_out[fr] = 0;
    }
    if (energies_out)
        for (i64 i = 0; i < nframes * n_iter_max; ++i) energies_out[i] = NAN;
    memcpy(u, f, sizeof(double) * (size_t)(nframes * hw));

    for (int k = 0; k < n_iter_max; ++k) {
        /* pass 1: u = f - div p (k > 0) and sum of (div p)^2 per row */
#pragma omp parallel for collapse(2) schedule(static)
        for (i64 fr = 0; fr < nframes; ++fr) {
            for (i64 i = 0; i < H; ++i) {
                if (!active[fr]) continue;
                const i64 o = fr * hw + i * W;
                double sd = 0.0;
                if (k > 0) {
                    for (i64 j = 0; j < W; ++j) {
                        double dv = pr[o + j] + pc[o + j];
                        if (i > 0) dv -= pr[o + j - W];
                        if (j > 0) dv -= pc[o + j - 1];
                        u[o + j] = f[o + j] - dv;
                        sd += dv * dv;
                    }
                }
                rowd[fr * H + i] = sd;
            }
        }
        /* pass 2: gradient of u, norm, p update (k < n_iter_max-1 only
           matters for the output but the energy needs the norm) */
#pragma omp parallel for collapse(2) schedule(static)
        for (i64 fr = 0; fr < nframes; ++fr) {
            for (i64 i = 0; i < H; ++i) {
                if (!active[fr]) continue;
                const i64 o = fr * hw + i * W;
                double sn = 0.0;
                for (i64 j = 0; j < W; ++j) {
                    const double uc = u[o + j];
                    const double gr = (i + 1 < H) ? u[o + j + W] - uc : 0.0;
                    const double gc = (j + 1 < W) ? u[o + j + 1] - uc : 0.0;
                    const double nrm = sqrt(gr * gr + gc * gc);
                    sn += nrm;
                    const double den = 1.0 + nrm * (tau / weight);
                    pr[o + j] = (pr[o + j] - tau * gr) / den;
                    pc[o + j] = (pc[o + j] - tau * gc) / den;
                }
                rown[fr * H + i] = sn;
            }
        }
        for (i64 fr = 0; fr < nframes; ++fr) {
            if (!active[fr]) continue;
            double sd = 0.0, sn = 0.0;
            for (i64 i = 0; i < H; ++i) {
                sd += rowd[fr * H + i];
                sn += rown[fr * H + i];
            }
            const double e = (sd + weight * sn) / (double)hw;
            if (energies_out) energies_out[fr * n_iter_max + k] = e;
            if (steps_out) steps_out[fr] = k + 1;
            if (k == 0) {
                e_init[fr] = e;
                e_prev[fr] = e;
            } else if (fabs(e_prev[fr] - e) < eps * e_init[fr]) {
                active[fr] = 0;
            } else {
                e_prev[fr] = e;
            }
        }
    }
    free(pr); free(pc); free(rowd); free(rown);
    free(active); free(e_init); free(e_prev);
}

/*
 * GAP-TV (accelerate != 0: GAP_acc) over `iters` iterations.
 * lambdas / weights: per-iteration arrays (length iters).
 * x: in = x0, out = result.  psnr_all (nullable, length iters) with orig.
 */
void orc_gap_tv(const double *y, const double *phi, const double *phisum,
                double *x, i64 B, i64 H, i64 W, int iters,
                const double *lambdas, const double *weights,
                int tv_iter_max, double eps, int accelerate,
                const double *orig, double *psnr_all) {
    const i64 hw = H * W, n = B * hw;
    double *yb = (double *)malloc(sizeof(double) * (size_t)hw);
    double *y1 = (double *)calloc((size_t)hw, sizeof(double));
    double *xp = (double *)malloc(sizeof(double) * (size_t)n);
    for (int it = 0; it < iters; ++it) {
        const double lam = lambdas[it];
        orc_A(x, phi, yb, B, H, W);
#pragma omp parallel for schedule(static)
        for (i64 i = 0; i < hw; ++i) {
            double r;
            if (accelerate) {
                y1[i] = y1[i] + (y[i] - yb[i]);
                r = (y1[i] - yb[i]) / phisum[i];
            } else {
                r = (y[i] - yb[i]) / phisum[i];
            }
            for (i64 b = 0; b < B; ++b)
                xp[b * hw + i] = x[b * hw + i] + lam * (r * phi[b * hw + i]);
        }
        orc_tv_chambolle(xp, x, B, H, W, weights[it], eps, tv_iter_max, NULL, NULL);
        if (orig && psnr_all) {
            double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
            for (i64 i = 0; i < n; ++i) {
                const double d = orig[i] - x[i];
                s += d * d;
            }
            const double mse = s / (double)n;
            psnr_all[it] = (mse == 0.0) ? 100.0 : 20.0 * log10(1.0 / sqrt(mse));
        }
    }
    free(yb); free(y1); free(xp);
}

/*
 * ADMM-TV over `iters` iterations: yb = A(theta+b);
 * x = theta + b + lambda At((y - yb)/(phisum + gamma)); theta = TV(x - b);
 * b = b - (x - theta).  x: in = x0 (theta_0 = x0, b_0 = 0), out = the last x.
 */
void orc_admm_tv(const double *y, const double *phi, const double *phisum,
                 double *x, i64 B, i64 H, i64 W, int iters,
                 const double *lambdas, const double *weights, double gamma,
                 int tv_iter_max, double eps,
                 const double *orig, double *psnr_all) {
    const i64 hw = H * W, n = B * hw;
    double *yb = (double *)malloc(sizeof(double) * (size_t)hw);
    double *theta = (double *)malloc(sizeof(double) * (size_t)n);
    double *bb = (double *)calloc((size_t)n, sizeof(double));
    double *tb = (double *)malloc(sizeof(double) * (size_t)n);
    double *xmb = (double *)malloc(sizeof(double) * (size_t)n);
    memcpy(theta, x, sizeof(double) * (size_t)n);
    for (int it = 0; it < iters; ++it) {
        const double lam = lambdas[it];
#pragma omp parallel for schedule(static)
        for (i64 i = 0; i < n; ++i) tb[i] = theta[i] + bb[i];
        orc_A(tb, phi, yb, B, H, W);
#pragma omp parallel for schedule(static)
        for (i64 i = 0; i < hw; ++i) {
            const double r = (y[i] - yb[i]) / (phisum[i] + gamma);
            for (i64 b = 0; b < B; ++b) {
                const i64 j = b * hw + i;
                x[j] = tb[j] + lam * (r * phi[j]);
                xmb[j] = x[j] - bb[j];
            }
        }
        orc_tv_chambolle(xmb, theta, B, H, W, weights[it], eps, tv_iter_max, NULL, NULL);
#pragma omp parallel for schedule(static)
        for (i64 i = 0; i < n; ++i) bb[i] = bb[i] - (x[i] - theta[i]);
        if (orig && psnr_all) {
            double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
            for (i64 i = 0; i < n; ++i) {
                const double d = orig[i] - x[i];
                s += d * d;
            }
            const double mse = s / (double)n;
            psnr_all[it] = (mse == 0.0) ? 100.0 : 20.0 * log10(1.0 / sqrt(mse));
        }
    }
    free(yb); free(theta); free(bb); free(tb); free(xmb);
}
