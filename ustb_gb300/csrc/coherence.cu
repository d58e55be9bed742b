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
// computed in two passes over the K values, as the reference's mean-then-variance.
//
// Generalized coherence factor (+postprocess/generalized_coherence_factor.m:66-97):
//   GCF = sum_{k in LF} |DFT_K(s)[k]|^2 / sum_k |DFT_K(s)[k]|^2   (NaN -> 0),
//   LF = MATLAB indices [1:M0+1, K-M0+1:K] (repeats counted twice, as indexing does)
//   when M0 > 1, else [1];  image = GCF * sum s.  The total is K * sum |s|^2
//   (Parseval); the low-frequency bins are DFTs over a twiddle table in shared memory.
//   K <= 4096 keeps that table within the default 48 KB.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace {

constexpr int kThreads = 256;
constexpr float kPi = 3.14159265358979f;

__global__ void __launch_bounds__(kThreads) pcf_kernel(const float2* __restrict__ cube, const float* __restrict__ wts,
                                                       int64_t P, int64_t K, int64_t F, float gamma_over_sigma,
                                                       float* fca, float* fcc, float2* image) {
    const int64_t total = P * F;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = t / P, p = t - f * P;
        const float2* s = cube + f * K * P + p;
        float sw = 0.f, sphi = 0.f, spsi = 0.f, sc = 0.f, ss = 0.f;
        float2 sum = make_float2(0.f, 0.f);
        for (int64_t k = 0; k < K; ++k) {
            const float2 v = __ldg(s + k * P);
            const float w = wts ? __ldg(wts + k * P + p) : 1.f;
            const float phi = atan2f(v.y, v.x);
            const float psi = phi <= 0.f ? phi + kPi : phi - kPi;
            float sn, cs;
            sincosf(phi, &sn, &cs);
            sw += w;
            sphi += w * phi;
            spsi += w * psi;
            sc += w * cs;
            ss += w * sn;
            sum.x += v.x;
            sum.y += v.y;
        }
        const float inv = 1.f / sw;
        const float mphi = sphi * inv, mpsi = spsi * inv, mc = sc * inv, ms = ss * inv;
        float vphi = 0.f, vpsi = 0.f, vcs = 0.f;
        for (int64_t k = 0; k < K; ++k) {
            const float2 v = __ldg(s + k * P);
            const float w = wts ? __ldg(wts + k * P + p) : 1.f;
            const float phi = atan2f(v.y, v.x);
            const float psi = phi <= 0.f ? phi + kPi : phi - kPi;
            float sn, cs;
            sincosf(phi, &sn, &cs);
            vphi += w * (phi - mphi) * (phi - mphi);
            vpsi += w * (psi - mpsi) * (psi - mpsi);
            vcs += w * ((cs - mc) * (cs - mc) + (sn - ms) * (sn - ms));
        }
        const float sf = fminf(sqrtf(vphi * inv), sqrtf(vpsi * inv));
        float a = 1.f - gamma_over_sigma * sf;
        if (a < 0.f) a = 0.f;
        if (a != a) a = 0.f;
        const float c = 1.f - sqrtf(vcs * inv);
        const int64_t o = f * P + p;
        if (fca) fca[o] = a;
        if (fcc) fcc[o] = c;
        if (image) image[o] = make_float2(c * sum.x, c * sum.y);
    }
}

struct Bins {
    int n;
    int b[64];
};

__global__ void __launch_bounds__(kThreads) gcf_kernel(const float2* __restrict__ cube, int64_t P, int64_t K,
                                                       int64_t F, const Bins bins, float* gcf, float2* image) {
    extern __shared__ float2 tw[];  // tw[m] = exp(-i 2 pi m / K)
    for (int m = threadIdx.x; m < K; m += blockDim.x) {
        float sn, cs;
        sincospif(-2.f * (float)m / (float)K, &sn, &cs);
        tw[m] = make_float2(cs, sn);
    }
    __syncthreads();
    const int64_t total = P * F;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = t / P, p = t - f * P;
        const float2* s = cube + f * K * P + p;
        float e = 0.f;
        float2 sum = make_float2(0.f, 0.f);
        for (int64_t k = 0; k < K; ++k) {
            const float2 v = __ldg(s + k * P);
            e += v.x * v.x + v.y * v.y;
            sum.x += v.x;
            sum.y += v.y;
        }
        float lf = 0.f;
        for (int b = 0; b < bins.n; ++b) {
            const int bin = bins.b[b];
            float2 X = make_float2(0.f, 0.f);
            int m = 0;  // bin * k mod K
            for (int64_t k = 0; k < K; ++k) {
                const float2 v = __ldg(s + k * P);
                const float2 w = tw[m];
                X.x += v.x * w.x - v.y * w.y;
                X.y += v.x * w.y + v.y * w.x;
                m += bin;
                if (m >= K) m -= (int)K;
            }
            lf += X.x * X.x + X.y * X.y;
        }
        float g = lf / ((float)K * e);
        if (g != g) g = 0.f;
        const int64_t o = f * P + p;
        if (gcf) gcf[o] = g;
        if (image) image[o] = make_float2(g * sum.x, g * sum.y);
    }
}

unsigned grid_for(int64_t total) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + kThreads - 1) / kThreads, (int64_t)std::max(sms, 1) * 16));
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
    USTB_REQUIRE(K <= 4096, USTB_E_SHAPE, "at most 4096 values per pixel");
    USTB_REQUIRE(M0 >= 0 && M0 <= 31, USTB_E_ARG, "M0 must be in [0, 31]");
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
    gcf_kernel<<<grid_for(P * F), kThreads, sizeof(float2) * (size_t)K, s>>>(static_cast<const float2*>(cube), P, K, F,
                                                                            bins, gcf, static_cast<float2*>(image));
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}
