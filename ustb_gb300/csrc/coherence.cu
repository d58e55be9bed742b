// Adaptive weights on the kept channel (or wave) cube of a dimension.transmit (or
// dimension.receive) result, one thread per pixel and frame, reading the cube
// [F][K][P] (pixel fastest: coalesced across threads):
//
// Phase coherence factor (+postprocess/phase_coherence_factor.m:64-129), over the
// K values s_k of a pixel with weights w_k (the apodization, or ones):
//   phi = angle(s), psi = phi - pi (phi > 0) or phi + pi,
//   std(x) = sqrt(sum w (x - mean_w x)^2 / sum w)     (tools/weigthed_std.m)
//   FCA = max(0, 1 - gamma / sigma0 * min(std phi, std psi))   (NaN -> 0)
//   FCC = 1 - sqrt(var_w(cos phi) + var_w(sin phi)),  image = FCC * sum s
// computed in one pass with weighted incremental updates (the reference's
// mean-then-variance to rounding), four threads per pixel over a quarter of the K
// values each, merged pairwise.
//
// Generalized coherence factor (+postprocess/generalized_coherence_factor.m:66-97):
//   GCF = sum_{k in LF} |DFT_K(s)[k]|^2 / sum_k |DFT_K(s)[k]|^2   (NaN -> 0),
//   LF = MATLAB indices [1:M0+1, K-M0+1:K] (repeats counted twice, as indexing does)
//   when M0 > 1, else [1];  image = GCF * sum s.  The total is K * sum |s|^2
//   (Parseval); the low-frequency bins (at most 15: M0 <= 7) are DFTs over a twiddle
//   table in shared memory, summed in registers by four threads per pixel.  K <= 1024
//   keeps that table and the partial sums within the default 48 KB.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace {

constexpr int kThreads = 256;
constexpr float kPi = 3.14159265358979f;

constexpr int kParts = 4;                    // threads per pixel, each over a quarter of K
constexpr int kPix = kThreads / kParts;      // pixels per CTA (64: two warps of pixels per part)

// weighted running mean and sum of squared deviations (West's incremental update,
// the algorithm of tools/weighted_incremental_variance.m): var = S / W; partial runs
// merge exactly (Chan et al.'s pairwise update)
struct WRun {
    float mean = 0.f, S = 0.f;
    __device__ __forceinline__ void add(float x, float w, float w_over_W) {
        const float d = x - mean;
        mean = fmaf(w_over_W, d, mean);
        S = fmaf(w * d, x - mean, S);
    }
    __device__ __forceinline__ void merge(float Wa, float Wb, float mb, float Sb) {
        const float Wt = Wa + Wb;
        if (Wb == 0.f) return;
        if (Wa == 0.f) { mean = mb; S = Sb; return; }
        const float d = mb - mean;
        mean = fmaf(d, Wb / Wt, mean);
        S = S + Sb + d * d * (Wa * Wb / Wt);
    }
};

// CTA layout: thread = (part g, pixel slot i), g = tid / kPix, i = tid % kPix, so a
// warp reads 32 consecutive pixels of one k (coalesced); part g takes k = g, g+4, ...
__global__ void __launch_bounds__(kThreads) pcf_kernel(const float2* __restrict__ cube, const float* __restrict__ wts,
                                                       int64_t P, int64_t K, int64_t F, float gamma_over_sigma,
                                                       float* fca, float* fcc, float2* image) {
    __shared__ float red[kParts][11][kPix];
    const int g = threadIdx.x / kPix, i = threadIdx.x % kPix;
    const int64_t total = P * F;
    for (int64_t t0 = (int64_t)blockIdx.x * kPix; t0 < total; t0 += (int64_t)gridDim.x * kPix) {
        const int64_t t = t0 + i;
        const bool ok = t < total;
        const int64_t f = ok ? t / P : 0, p = ok ? t - f * P : 0;
        const float2* s = cube + f * K * P + p;
        float W = 0.f;
        WRun rphi, rpsi, rc, rs;
        float2 sum = make_float2(0.f, 0.f);
        if (ok) {
            for (int64_t k = g; k < K; k += kParts) {
                const float2 v = __ldg(s + k * P);
                const float w = wts ? __ldg(wts + k * P + p) : 1.f;
                sum.x += v.x;
                sum.y += v.y;
                if (w == 0.f) continue;  // zero weight: no change to any weighted statistic
                W += w;
                const float q = w / W;
                const float phi = atan2f(v.y, v.x);
                const float psi = phi <= 0.f ? phi + kPi : phi - kPi;
                float sn, cs;
                sincosf(phi, &sn, &cs);
                rphi.add(phi, w, q);
                rpsi.add(psi, w, q);
                rc.add(cs, w, q);
                rs.add(sn, w, q);
            }
        }
        const float v11[11] = {W, rphi.mean, rphi.S, rpsi.mean, rpsi.S, rc.mean, rc.S, rs.mean, rs.S, sum.x, sum.y};
#pragma unroll
        for (int j = 0; j < 11; ++j) red[g][j][i] = v11[j];
        __syncthreads();
        if (g == 0 && ok) {
            for (int h = 1; h < kParts; ++h) {
                const float Wb = red[h][0][i];
                rphi.merge(W, Wb, red[h][1][i], red[h][2][i]);
                rpsi.merge(W, Wb, red[h][3][i], red[h][4][i]);
                rc.merge(W, Wb, red[h][5][i], red[h][6][i]);
                rs.merge(W, Wb, red[h][7][i], red[h][8][i]);
                W += Wb;
                sum.x += red[h][9][i];
                sum.y += red[h][10][i];
            }
            const float inv = 1.f / W;  // W = 0: NaN statistics, as the reference's 0/0
            const float sf = fminf(sqrtf(rphi.S * inv), sqrtf(rpsi.S * inv));
            float a = 1.f - gamma_over_sigma * sf;
            if (a < 0.f) a = 0.f;
            if (a != a) a = 0.f;
            const float c = 1.f - sqrtf((rc.S + rs.S) * inv);
            const int64_t o = f * P + p;
            if (fca) fca[o] = a;
            if (fcc) fcc[o] = c;
            if (image) image[o] = make_float2(c * sum.x, c * sum.y);
        }
        __syncthreads();
    }
}

struct Bins {
    int n;
    int b[64];
};

template <int NB>  // number of low-frequency bins, 1 or 2 M0 + 1
__global__ void __launch_bounds__(kThreads) gcf_kernel(const float2* __restrict__ cube, int64_t P, int64_t K,
                                                       int64_t F, const Bins bins, float* gcf, float2* image) {
    extern __shared__ float2 tw[];  // tw[m] = exp(-i 2 pi m / K)
    __shared__ float2 red[kParts][NB + 1][kPix];
    __shared__ float rede[kParts][kPix];
    for (int m = threadIdx.x; m < K; m += blockDim.x) {
        float sn, cs;
        sincospif(-2.f * (float)m / (float)K, &sn, &cs);
        tw[m] = make_float2(cs, sn);
    }
    __syncthreads();
    const int g = threadIdx.x / kPix, i = threadIdx.x % kPix;
    const int64_t total = P * F;
    for (int64_t t0 = (int64_t)blockIdx.x * kPix; t0 < total; t0 += (int64_t)gridDim.x * kPix) {
        const int64_t t = t0 + i;
        const bool ok = t < total;
        const int64_t f = ok ? t / P : 0, p = ok ? t - f * P : 0;
        const float2* s = cube + f * K * P + p;
        float e = 0.f;
        float2 sum = make_float2(0.f, 0.f);
        float2 X[NB];
        int mb[NB], step[NB];
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            X[b] = make_float2(0.f, 0.f);
            const int bin = bins.b[b];
            mb[b] = (int)(((int64_t)bin * g) % K);             // twiddle index of k = g
            step[b] = (int)(((int64_t)bin * kParts) % K);      // advance per k += kParts
        }
        if (ok) {
            for (int64_t k = g; k < K; k += kParts) {
                const float2 v = __ldg(s + k * P);
                e += v.x * v.x + v.y * v.y;
                sum.x += v.x;
                sum.y += v.y;
#pragma unroll
                for (int b = 0; b < NB; ++b) {
                    const float2 w = tw[mb[b]];
                    X[b].x += v.x * w.x - v.y * w.y;
                    X[b].y += v.x * w.y + v.y * w.x;
                    mb[b] += step[b];
                    if (mb[b] >= K) mb[b] -= (int)K;
                }
            }
        }
#pragma unroll
        for (int b = 0; b < NB; ++b) red[g][b][i] = X[b];
        red[g][NB][i] = sum;
        rede[g][i] = e;
        __syncthreads();
        if (g == 0 && ok) {
            float lf = 0.f;
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                float2 x = X[b];
                for (int h = 1; h < kParts; ++h) {
                    x.x += red[h][b][i].x;
                    x.y += red[h][b][i].y;
                }
                lf += x.x * x.x + x.y * x.y;
            }
            for (int h = 1; h < kParts; ++h) {
                e += rede[h][i];
                sum.x += red[h][NB][i].x;
                sum.y += red[h][NB][i].y;
            }
            float gv = lf / ((float)K * e);
            if (gv != gv) gv = 0.f;
            const int64_t o = f * P + p;
            if (gcf) gcf[o] = gv;
            if (image) image[o] = make_float2(gv * sum.x, gv * sum.y);
        }
        __syncthreads();
    }
}

unsigned grid_for(int64_t total) {  // CTAs of kPix pixels
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + kPix - 1) / kPix, (int64_t)std::max(sms, 1) * 32));
}

// Coherence factor over the channels, the waves or both of a kept cube [P, N, W, F]
// (pixel fastest), +postprocess/coherence_factor.m:100-135:
//   CF = |sum s|^2 / sum |s|^2 * (1 / M)  (NaN -> 0),  image = CF * sum s,
// M = the count of active units per pixel given by the caller, or the number summed
// (the reference's Python CoherenceFactor, python/src/ustb/postprocess/coherence_factor.py:29-47).
// One thread per (pixel, remaining index); a warp reads 32 consecutive pixels.
__global__ void __launch_bounds__(kThreads) cf_kernel(const float2* __restrict__ cube, const float* __restrict__ M,
                                                      int64_t P, int64_t K, int64_t S, int64_t J0, int64_t B0,
                                                      int64_t B1, int64_t pblocks, float* __restrict__ cf,
                                                      float2* __restrict__ img) {
    const int64_t j = blockIdx.x / pblocks;
    const int64_t p = (blockIdx.x - j * pblocks) * kThreads + threadIdx.x;
    if (p >= P) return;
    const int64_t j1 = j / J0, j0 = j - j1 * J0;
    const float2* x = cube + j0 * B0 + j1 * B1 + p;
    float2 sum = make_float2(0.f, 0.f);
    float e = 0.f;
    for (int64_t k = 0; k < K; ++k) {
        const float2 v = __ldg(x + k * S);
        sum.x += v.x;
        sum.y += v.y;
        e = fmaf(v.x, v.x, fmaf(v.y, v.y, e));
    }
    const float m = M ? __ldg(M + p) : (float)K;
    float c = (sum.x * sum.x + sum.y * sum.y) / e * (1.f / m);
    if (c != c) c = 0.f;  // NaN -> 0 (coherence_factor.m:132)
    if (cf) cf[p + P * j] = c;
    if (img) img[p + P * j] = make_float2(c * sum.x, c * sum.y);
}

}  // namespace

extern "C" int ustb_phase_coherence(const void* cube, int64_t P, int64_t K, int64_t F, const float* weights,
                                    float gamma, float sigma0, float* fca, float* fcc, void* image, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(P >= 0 && K >= 0 && F >= 0, USTB_E_SHAPE, "negative size");
    USTB_REQUIRE(K >= 2, USTB_E_SHAPE, "Not enough channels to compute factor (K = %lld)", (long long)K);
    USTB_REQUIRE(sigma0 > 0.f, USTB_E_ARG, "sigma_0 must be > 0");
    if (P == 0 || F == 0) return USTB_OK;
    USTB_REQUIRE(cube && (fca || fcc || image), USTB_E_ARG, "NULL pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    pcf_kernel<<<grid_for(P * F), kThreads, 0, s>>>(static_cast<const float2*>(cube), weights, P, K, F,
                                                     gamma / sigma0, fca, fcc, static_cast<float2*>(image));
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}

extern "C" int ustb_generalized_coherence(const void* cube, int64_t P, int64_t K, int64_t F, int32_t M0, float* gcf,
                                          void* image, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(P >= 0 && K >= 0 && F >= 0, USTB_E_SHAPE, "negative size");
    USTB_REQUIRE(K >= 2, USTB_E_SHAPE, "Not enough channels to compute factor (K = %lld)", (long long)K);
    USTB_REQUIRE(K <= 1024, USTB_E_SHAPE, "at most 1024 values per pixel");
    USTB_REQUIRE(M0 >= 0 && M0 <= 7, USTB_E_ARG, "M0 must be in [0, 7]");
    USTB_REQUIRE(M0 <= 1 || K > M0, USTB_E_SHAPE, "M0 = %d needs more than %d values per pixel (K = %lld)", (int)M0,
                 (int)M0, (long long)K);
    if (P == 0 || F == 0) return USTB_OK;
    USTB_REQUIRE(cube && (gcf || image), USTB_E_ARG, "NULL pointer");
    // the reference's 1-based indices [1:M0+1, K-M0+1:K] (M0 > 1), else [1], as 0-based bins
    Bins bins;
    bins.n = 0;
    if (M0 > 1) {
        for (int i = 0; i <= M0; ++i) bins.b[bins.n++] = i;
        for (int64_t i = K - M0; i < K; ++i) bins.b[bins.n++] = (int)i;
    } else {
        bins.b[bins.n++] = 0;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned grid = grid_for(P * F);
    const size_t smem = sizeof(float2) * (size_t)K;
    const float2* c = static_cast<const float2*>(cube);
    float2* im = static_cast<float2*>(image);
    switch (bins.n) {
        case 1: gcf_kernel<1><<<grid, kThreads, smem, s>>>(c, P, K, F, bins, gcf, im); break;
        case 5: gcf_kernel<5><<<grid, kThreads, smem, s>>>(c, P, K, F, bins, gcf, im); break;
        case 7: gcf_kernel<7><<<grid, kThreads, smem, s>>>(c, P, K, F, bins, gcf, im); break;
        case 9: gcf_kernel<9><<<grid, kThreads, smem, s>>>(c, P, K, F, bins, gcf, im); break;
        case 11: gcf_kernel<11><<<grid, kThreads, smem, s>>>(c, P, K, F, bins, gcf, im); break;
        case 13: gcf_kernel<13><<<grid, kThreads, smem, s>>>(c, P, K, F, bins, gcf, im); break;
        default: gcf_kernel<15><<<grid, kThreads, smem, s>>>(c, P, K, F, bins, gcf, im); break;
    }
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}

extern "C" int ustb_coherence_factor(const void* cube, int64_t P, int64_t N, int64_t W, int64_t F, int32_t dimension,
                                     const float* active_count, float* cf, void* image, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(dimension == USTB_DIM_RECEIVE || dimension == USTB_DIM_TRANSMIT || dimension == USTB_DIM_BOTH,
                 USTB_E_ARG, "dimension must be receive (1), transmit (2) or both (3), got %d", (int)dimension);
    USTB_REQUIRE(P >= 0 && N >= 0 && W >= 0 && F >= 0, USTB_E_SHAPE, "negative size");
    int64_t K, S, J0, B0, B1;
    if (dimension == USTB_DIM_RECEIVE) {  // over channels; remaining (wave, frame)
        K = N; S = P; J0 = W * F; B0 = P * N; B1 = 0;
    } else if (dimension == USTB_DIM_TRANSMIT) {  // over waves; remaining (channel, frame)
        K = W; S = P * N; J0 = N; B0 = P; B1 = P * N * W;
    } else {  // over both; remaining frames
        K = N * W; S = P; J0 = F; B0 = P * N * W; B1 = 0;
    }
    const int64_t J = (dimension == USTB_DIM_RECEIVE) ? W * F : (dimension == USTB_DIM_TRANSMIT ? N * F : F);
    if (P == 0 || J == 0) return USTB_OK;
    USTB_REQUIRE(cube && (cf || image), USTB_E_ARG, "NULL pointer");
    const int64_t pblocks = (P + kThreads - 1) / kThreads;
    USTB_REQUIRE(pblocks * J <= INT32_MAX, USTB_E_SHAPE, "too many pixels x remaining slices");
    cf_kernel<<<(unsigned)(pblocks * J), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float2*>(cube), active_count, P, K, S, J0, B0, B1, pblocks, cf,
        static_cast<float2*>(image));
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}
