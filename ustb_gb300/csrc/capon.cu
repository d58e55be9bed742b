// Capon minimum-variance beamforming on a kept channel cube
// (+postprocess/capon_minimum_variance.m:117-177), one warp per pixel.
//
// For pixel (iz, ix) of a scan grid with depth fastest, over the M values x[c] of
// its channels (or waves) and the rows r of its depth window [iz-K, iz+K] (clipped):
//   active channels c: |apod[c]| > criterion; first a, last b, count Ma.
//   All |x| <= eps -> 0; Ma < 2 -> sum_c x[c].
//   L = clamp(floor(L_elements / M * Ma), 1, Ma - 1); subarray starts l = a .. b-L+1.
//   R = sum_r sum_l X_r[l:l+L]^H X_r[l:l+L] / ((2K+1)(Ma - L + 1))  (rows of A' * A),
//   optionally R = (R + J conj(R) J) / 2 (forward-backward),
//   w = (R + I regCoef/L trace R)^-1 1 / (1^T (...)^-1 1),
//   z = Ma / (Ma - L + 1) * sum_l conj(w)^T conj(x_iz[l:l+L])   (w' * x', as written).
//
// R is accumulated in shared memory along its diagonals: lane d owns diagonal d and
// walks it with a sliding window, G(i+1, i+1+d) = G(i, i+d) + conj(x[l1+i+1]) x[l1+i+1+d]
// - conj(x[l0+i]) x[l0+i+d], so a row costs (#l + 2L) products per lane instead of
// #l * L.  The system is solved by a Cholesky factorisation R = U^H U in shared
// memory, lanes over columns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace {

constexpr int kLMax = 32;        // subarray length <= one lane per diagonal
constexpr int kWarps = 4;        // pixels per CTA
constexpr int kMMax = 256;       // channels per pixel

struct CaponArgs {
    int64_t nz, nx, F, M;
    int K;                 // depth half-window in samples
    float l_frac;          // L_elements / M
    float crit;            // active-element criterion
    float reg;             // regularisation coefficient
    int fb;                // forward-backward averaging
};

__device__ __forceinline__ float2 cmul_conj(float2 a, float2 b) {  // conj(a) * b
    return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

__global__ void __launch_bounds__(32 * kWarps) capon_kernel(const float2* __restrict__ cube,
                                                            const float* __restrict__ apod, float2* __restrict__ out,
                                                            const CaponArgs a) {
    __shared__ float2 sR[kWarps][kLMax][kLMax + 1];
    __shared__ float2 srow[kWarps][kMMax];
    __shared__ float2 sv[kWarps][kLMax];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 (*R)[kLMax + 1] = sR[wi];
    float2* row = srow[wi];
    float2* v = sv[wi];
    const int64_t P = a.nz * a.nx;
    const int64_t total = P * a.F;
    const int M = (int)a.M;
    for (int64_t t = (int64_t)blockIdx.x * kWarps + wi; t < total; t += (int64_t)gridDim.x * kWarps) {
        const int64_t f = t / P, p = t - f * P;
        const int64_t ix = p / a.nz, iz = p - ix * a.nz;
        const float2* base = cube + f * a.M * P;  // [M][P]
        // active channels, all-zero test and the plain sum of the pixel's own row
        int first = M, last = -1, cnt = 0;
        bool any = false;
        float2 sum = make_float2(0.f, 0.f);
        for (int c = lane; c < M; c += 32) {
            const float2 x = __ldg(base + (int64_t)c * P + p);
            any |= hypotf(x.x, x.y) > 2.220446049250313e-16f;
            sum.x += x.x;
            sum.y += x.y;
            if (fabsf(__ldg(apod + (int64_t)c * P + p)) > a.crit) {
                first = min(first, c);
                last = max(last, c);
                ++cnt;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
            last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            sum.x += __shfl_xor_sync(0xffffffffu, sum.x, o);
            sum.y += __shfl_xor_sync(0xffffffffu, sum.y, o);
        }
        any = __any_sync(0xffffffffu, any);
        if (!any) {
            if (lane == 0) out[t] = make_float2(0.f, 0.f);
            continue;
        }
        if (cnt < 2) {
            if (lane == 0) out[t] = sum;
            continue;
        }
        int L = (int)floorf(a.l_frac * (float)cnt);
        L = max(1, min(L, cnt - 1));
        if (last - L + 1 < first) {  // no subarray fits: plain sum
            if (lane == 0) out[t] = sum;
            continue;
        }
        const int l0 = first, l1 = last - L + 1;  // subarray starts
        // R = sum over rows of the depth window
        for (int i = lane; i < L * (kLMax + 1); i += 32) (&R[0][0])[i] = make_float2(0.f, 0.f);
        const int64_t r0 = max((int64_t)0, iz - a.K), r1 = min(a.nz - 1, iz + a.K);
        for (int64_t r = r0; r <= r1; ++r) {
            __syncwarp();
            for (int c = lane; c < M; c += 32) row[c] = __ldg(base + (int64_t)c * P + ix * a.nz + r);
            __syncwarp();
            const int d = lane;
            if (d < L) {
                float2 g = make_float2(0.f, 0.f);  // G(0, d)
                for (int l = l0; l <= l1; ++l) {
                    const float2 q = cmul_conj(row[l], row[l + d]);
                    g.x += q.x;
                    g.y += q.y;
                }
                for (int i = 0; i + d < L; ++i) {
                    R[i][i + d].x += g.x;
                    R[i][i + d].y += g.y;
                    if (i + 1 + d < L) {  // slide to G(i+1, i+1+d)
                        const float2 add = cmul_conj(row[l1 + i + 1], row[l1 + i + 1 + d]);
                        const float2 sub = cmul_conj(row[l0 + i], row[l0 + i + d]);
                        g.x += add.x - sub.x;
                        g.y += add.y - sub.y;
                    }
                }
            }
        }
        __syncwarp();
        // normalise, mirror to the lower triangle, forward-backward, diagonal loading
        const float norm = 1.f / ((float)(2 * a.K + 1) * (float)(cnt - L + 1));
        for (int idx = lane; idx < L * L; idx += 32) {
            const int i = idx / L, j = idx - (idx / L) * L;
            if (j >= i) {
                R[i][j].x *= norm;
                R[i][j].y *= norm;
            }
        }
        __syncwarp();
        for (int idx = lane; idx < L * L; idx += 32) {
            const int i = idx / L, j = idx - (idx / L) * L;
            if (j < i) R[i][j] = make_float2(R[j][i].x, -R[j][i].y);
        }
        __syncwarp();
        if (a.fb) {
            // (J conj(R) J)[i][j] = conj(R[L-1-i][L-1-j]); average the upper triangle
            float2 nv[kLMax];
            int n = 0;
            for (int idx = lane; idx < L * L; idx += 32, ++n) {
                const int i = idx / L, j = idx - (idx / L) * L;
                const float2 q = R[L - 1 - i][L - 1 - j];
                nv[n] = make_float2(0.5f * (R[i][j].x + q.x), 0.5f * (R[i][j].y - q.y));
            }
            __syncwarp();
            n = 0;
            for (int idx = lane; idx < L * L; idx += 32, ++n) {
                const int i = idx / L, j = idx - (idx / L) * L;
                R[i][j] = nv[n];
            }
            __syncwarp();
        }
        float tr = lane < L ? R[lane][lane].x : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
        if (lane < L) R[lane][lane].x += a.reg / (float)L * tr;
        __syncwarp();
        // Cholesky R = U^H U (U upper, over R's upper triangle)
        for (int k = 0; k < L; ++k) {
            float dkk = R[k][k].x;
            for (int m = 0; m < k; ++m) dkk -= R[m][k].x * R[m][k].x + R[m][k].y * R[m][k].y;
            const float ukk = sqrtf(fmaxf(dkk, 1e-30f));
            const int j = lane;
            float2 ukj = make_float2(0.f, 0.f);
            if (j > k && j < L) {
                float2 s = R[k][j];
                for (int m = 0; m < k; ++m) {
                    const float2 q = cmul_conj(R[m][k], R[m][j]);
                    s.x -= q.x;
                    s.y -= q.y;
                }
                ukj = make_float2(s.x / ukk, s.y / ukk);
            }
            __syncwarp();
            if (j > k && j < L) R[k][j] = ukj;
            if (lane == 0) R[k][k] = make_float2(ukk, 0.f);
            __syncwarp();
        }
        // U^H y = 1 (forward), U x = y (backward); v holds y then x
        if (lane == 0) {
            for (int i = 0; i < L; ++i) {
                float2 s = make_float2(1.f, 0.f);
                for (int m = 0; m < i; ++m) {  // (U^H)[i][m] = conj(U[m][i])
                    const float2 q = cmul_conj(R[m][i], v[m]);
                    s.x -= q.x;
                    s.y -= q.y;
                }
                v[i] = make_float2(s.x / R[i][i].x, s.y / R[i][i].x);
            }
            for (int i = L - 1; i >= 0; --i) {
                float2 s = v[i];
                for (int m = i + 1; m < L; ++m) {
                    const float2 u = R[i][m], x = v[m];
                    s.x -= u.x * x.x - u.y * x.y;
                    s.y -= u.x * x.y + u.y * x.x;
                }
                v[i] = make_float2(s.x / R[i][i].x, s.y / R[i][i].x);
            }
        }
        __syncwarp();
        // w = x / (1^T x); z = sum_l sum_i conj(w_i) conj(x_iz[l + i]) * Ma / (Ma - L + 1)
        float2 den = lane < L ? v[lane] : make_float2(0.f, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            den.x += __shfl_xor_sync(0xffffffffu, den.x, o);
            den.y += __shfl_xor_sync(0xffffffffu, den.y, o);
        }
        // the pixel's own row
        for (int c = lane; c < M; c += 32) row[c] = __ldg(base + (int64_t)c * P + p);
        __syncwarp();
        float2 z = make_float2(0.f, 0.f);
        if (lane < L) {
            const float dd = den.x * den.x + den.y * den.y;
            const float2 xi = v[lane];
            const float2 w = make_float2((xi.x * den.x + xi.y * den.y) / dd, (xi.y * den.x - xi.x * den.y) / dd);
            for (int l = l0; l <= l1; ++l) {
                const float2 x = row[l + lane];
                // conj(w) * conj(x) = conj(w * x)
                z.x += w.x * x.x - w.y * x.y;
                z.y -= w.x * x.y + w.y * x.x;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            z.x += __shfl_xor_sync(0xffffffffu, z.x, o);
            z.y += __shfl_xor_sync(0xffffffffu, z.y, o);
        }
        if (lane == 0) {
            const float sc = (float)cnt / (float)(cnt - L + 1);
            out[t] = make_float2(z.x * sc, z.y * sc);
        }
        __syncwarp();
    }
}

}  // namespace

extern "C" int ustb_capon(const void* cube, const float* apodization, int64_t nz, int64_t nx, int64_t M, int64_t F,
                          float L_elements, int32_t K_samples, float regularisation, float criterion,
                          int32_t forward_backward, void* out, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(nz >= 0 && nx >= 0 && M >= 0 && F >= 0, USTB_E_SHAPE, "negative size");
    USTB_REQUIRE(M >= 2 && M <= kMMax, USTB_E_SHAPE, "Capon needs 2..%d channels per pixel, got %lld", kMMax,
                 (long long)M);
    USTB_REQUIRE(L_elements >= 1.f, USTB_E_ARG, "L_elements must be >= 1");
    USTB_REQUIRE(K_samples >= 0 && K_samples < 4096, USTB_E_ARG, "K_samples must be in [0, 4096)");
    USTB_REQUIRE(regularisation >= 0.f, USTB_E_ARG, "regularisation must be >= 0");
    if (nz == 0 || nx == 0 || F == 0) return USTB_OK;
    USTB_REQUIRE(cube && apodization && out, USTB_E_ARG, "NULL pointer");
    CaponArgs a;
    a.nz = nz; a.nx = nx; a.F = F; a.M = M;
    a.K = K_samples;
    a.l_frac = L_elements / (float)M;
    a.crit = criterion;
    a.reg = regularisation;
    a.fb = forward_backward ? 1 : 0;
    // the subarray length the active count can produce must fit one warp
    USTB_REQUIRE((int)floorf(a.l_frac * (float)M) <= kLMax, USTB_E_ARG,
                 "L_elements = %g gives subarrays longer than %d", (double)L_elements, kLMax);
    int dev = 0, sms = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t total = nz * nx * F;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + kWarps - 1) / kWarps,
                                                                          (int64_t)sms * 64));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    capon_kernel<<<grid, 32 * kWarps, 0, s>>>(static_cast<const float2*>(cube), apodization,
                                              static_cast<float2*>(out), a);
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}
