/*
 * ORACLE — CPU restatement of USTB's delay-and-sum hot loop.
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker / CPU baseline.  The product
 * library (ustb_gb300/) never links, loads or calls this file.
 *
 * Two entry points:
 *
 *  oracle_das_f32  — single-precision restatement of the reference's das_c
 *                    inner loop (+mex/source/das_c.cpp:355-409), operation for
 *                    operation: delay = tx + rx (:372), denay = (delay - t0)*Fs
 *                    (:375), n0 = trunc, b = denay - floor (:376-379), validity
 *                    0 < n0 < L-1 (:381), weight = exp(i*wd*delay)*apo (:385-387),
 *                    4-term real/imag dot products in the same order (:389-399),
 *                    wd = 2*(float)PI*fd only when |fd| > 1e-6 (:240-244),
 *                    output strides per sum mode (:324-353).  Built with
 *                    -ffp-contract=off so every operation rounds as on x86
 *                    without FMA; with the reference compiled the same way the
 *                    two agree bit for bit (pinned in tests/test_oracle.py).
 *
 *  oracle_das_f64  — the same formula in double precision (the "FP64 oracle"
 *                    the reduced-precision GPU path is checked against).  Takes
 *                    double tables and data.  edge_rule 0 = das_c's validity
 *                    rule; 1 = the tools.matlab_beamformer / interp1 rule
 *                    (+tools/matlab_beamformer.m:30: t in [t_0, t_{L-1}]).
 *
 * Layouts are MATLAB column-major (first index fastest):
 *   ch  [L, N, W, F] interleaved complex; tables [P, W] / [P, N];
 *   out [P, N|1, W|1, F] interleaved complex, accumulated into (caller zeroes).
 * Pixels are split over `threads` pthreads; each pixel's sum is sequential, so
 * the result does not depend on the thread count.
 */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_EPS 1e-6
#define ORACLE_PI 3.14159265359

typedef struct {
    int64_t L, N, W, F, P;
    int64_t rx_f, w_f, f_f; /* output strides (complex elements) */
    int dim;
    int edge_rule;
    /* f32 */
    const float* ch32; const float *atx32, *arx32, *dtx32, *drx32; float* out32;
    float fs32, t032, wd32;
    /* f64 */
    const double* ch64; const double *atx64, *arx64, *dtx64, *drx64; double* out64;
    double fs64, t064, wd64;
    int64_t p_begin, p_end;
} job_t;

static void strides(int dim, int64_t P, int64_t N, int64_t W, int64_t* rx_f, int64_t* w_f, int64_t* f_f) {
    switch (dim) {
        case 0: *rx_f = P; *w_f = P * N; *f_f = P * N * W; break; /* none */
        case 1: *rx_f = 0; *w_f = P;     *f_f = P * W;     break; /* receive */
        case 2: *rx_f = P; *w_f = 0;     *f_f = P * N;     break; /* transmit */
        default: *rx_f = 0; *w_f = 0;    *f_f = P;         break; /* both */
    }
}

static void* run_f32(void* arg) {
    const job_t* j = (const job_t*)arg;
    const int64_t L = j->L, N = j->N, W = j->W, F = j->F, P = j->P;
    const int64_t LN = L * N, LNW = LN * W;
    for (int64_t p = j->p_begin; p < j->p_end; ++p) {
        for (int64_t w = 0; w < W; ++w) {
            const float tx_delay = j->dtx32[P * w + p];
            const float tx_apo = j->atx32[P * w + p];
            if (tx_apo == 0.0f) continue;
            for (int64_t n = 0; n < N; ++n) {
                const float rx_delay = j->drx32[P * n + p];
                const float rx_apo = j->arx32[P * n + p];
                if (rx_apo == 0.0f) continue;
                const float delay = tx_delay + rx_delay;
                const float apo = tx_apo * rx_apo;
                const float denay = (delay - j->t032) * j->fs32;
                const float n0f = floorf(denay);
                const int n0 = (int)denay;
                const float b = denay - n0f;
                const float a = 1.0f - b;
                if (!(n0 > 0 && n0 < (L - 1))) continue;
                const float phase = j->wd32 * delay;
                const float complex e = cexpf(I * phase);
                const float wr = crealf(e) * apo;
                const float wi = cimagf(e) * apo;
                const float cr[4] = {a * wr, -a * wi, b * wr, -b * wi};
                const float ci[4] = {a * wi, a * wr, b * wi, b * wr};
                const float* x = j->ch32 + 2 * (L * n + LN * w + n0);
                float* o = j->out32 + 2 * (j->rx_f * n + j->w_f * w + p);
                for (int64_t f = 0; f < F; ++f) {
                    float re = 0.0f, im = 0.0f;
                    for (int v = 0; v < 4; ++v) {
                        re += cr[v] * x[v];
                        im += ci[v] * x[v];
                    }
                    o[0] += re;
                    o[1] += im;
                    x += 2 * LNW;
                    o += 2 * j->f_f;
                }
            }
        }
    }
    return NULL;
}

static void* run_f64(void* arg) {
    const job_t* j = (const job_t*)arg;
    const int64_t L = j->L, N = j->N, W = j->W, F = j->F, P = j->P;
    const int64_t LN = L * N, LNW = LN * W;
    for (int64_t p = j->p_begin; p < j->p_end; ++p) {
        for (int64_t w = 0; w < W; ++w) {
            const double tx_delay = j->dtx64[P * w + p];
            const double tx_apo = j->atx64[P * w + p];
            if (tx_apo == 0.0) continue;
            for (int64_t n = 0; n < N; ++n) {
                const double rx_delay = j->drx64[P * n + p];
                const double rx_apo = j->arx64[P * n + p];
                if (rx_apo == 0.0) continue;
                const double delay = tx_delay + rx_delay;
                const double apo = tx_apo * rx_apo;
                const double denay = (delay - j->t064) * j->fs64;
                const double fl = floor(denay);
                double b = denay - fl;
                int64_t n0;
                if (j->edge_rule == 0) {
                    if (!(denay < 9.0e18 && denay > -9.0e18)) continue;
                    n0 = (int64_t)denay;
                    if (!(n0 > 0 && n0 < L - 1)) continue;
                } else {
                    /* interp1(t, x, tau, 'linear', 0): t_0 <= tau <= t_{L-1} */
                    if (!(denay >= 0.0 && denay <= (double)(L - 1))) continue;
                    n0 = (int64_t)fl;
                    if (n0 == L - 1) { n0 = L - 2; b = 1.0; }
                }
                const double a = 1.0 - b;
                const double complex e = cexp(I * (j->wd64 * delay)) * apo;
                const double* x = j->ch64 + 2 * (L * n + LN * w + n0);
                double* o = j->out64 + 2 * (j->rx_f * n + j->w_f * w + p);
                for (int64_t f = 0; f < F; ++f) {
                    const double complex v = (a * x[0] + b * x[2]) + I * (a * x[1] + b * x[3]);
                    const double complex r = e * v;
                    o[0] += creal(r);
                    o[1] += cimag(r);
                    x += 2 * LNW;
                    o += 2 * j->f_f;
                }
            }
        }
    }
    return NULL;
}

static int run_threads(job_t* base, int threads, void* (*fn)(void*)) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    if (base->P < threads) threads = base->P > 0 ? (int)base->P : 1;
    job_t jobs[256];
    pthread_t tid[256];
    /* interleave small blocks so deep and shallow pixels spread evenly */
    const int64_t P = base->P;
    const int64_t per = (P + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        jobs[t] = *base;
        jobs[t].p_begin = t * per < P ? t * per : P;
        jobs[t].p_end = (t + 1) * per < P ? (t + 1) * per : P;
    }
    for (int t = 1; t < threads; ++t)
        if (pthread_create(&tid[t], NULL, fn, &jobs[t]) != 0) return -1;
    fn(&jobs[0]);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
    return 0;
}

/* Returns 0 on success, 1 on an argument error (das_c's checks that matter
 * numerically: sum mode range, fd with real data is the caller's business). */
int oracle_das_f32(const float* ch, int64_t L, int64_t N, int64_t W, int64_t F, float fs, float t0,
                   const float* apo_tx, const float* apo_rx, const float* delay_tx,
                   const float* delay_rx, int64_t P, float fd, int32_t dim, float* out,
                   int threads) {
    if (dim < 0 || dim > 3) return 1;
    job_t j;
    memset(&j, 0, sizeof j);
    j.L = L; j.N = N; j.W = W; j.F = F; j.P = P; j.dim = dim;
    strides(dim, P, N, W, &j.rx_f, &j.w_f, &j.f_f);
    j.ch32 = ch; j.atx32 = apo_tx; j.arx32 = apo_rx; j.dtx32 = delay_tx; j.drx32 = delay_rx;
    j.out32 = out;
    j.fs32 = fs; j.t032 = t0;
    j.wd32 = 0.0f;
    if (fabsf(fd) > ORACLE_EPS) j.wd32 = 2 * (float)ORACLE_PI * fd;
    return run_threads(&j, threads, run_f32) == 0 ? 0 : 2;
}

int oracle_das_f64(const double* ch, int64_t L, int64_t N, int64_t W, int64_t F, double fs,
                   double t0, const double* apo_tx, const double* apo_rx, const double* delay_tx,
                   const double* delay_rx, int64_t P, double fd, int32_t dim, int32_t edge_rule,
                   double* out, int threads) {
    if (dim < 0 || dim > 3) return 1;
    job_t j;
    memset(&j, 0, sizeof j);
    j.L = L; j.N = N; j.W = W; j.F = F; j.P = P; j.dim = dim; j.edge_rule = edge_rule;
    strides(dim, P, N, W, &j.rx_f, &j.w_f, &j.f_f);
    j.ch64 = ch; j.atx64 = apo_tx; j.arx64 = apo_rx; j.dtx64 = delay_tx; j.drx64 = delay_rx;
    j.out64 = out;
    j.fs64 = fs; j.t064 = t0;
    j.wd64 = (fabs(fd) > ORACLE_EPS) ? 2.0 * M_PI * fd : 0.0;
    return run_threads(&j, threads, run_f64) == 0 ? 0 : 2;
}
