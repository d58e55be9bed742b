// RF -> IQ demodulation fused with the conversion into the fast path's storage type:
// down-mix, low-pass FIR and decimation in one pass over the RF samples
// (+preprocess/fast_demodulation.m:121-167 and :286-293 for the filter):
//
//   mix[j] = scale * x[j] * exp(-i 2 pi fc t_j),   t_j = t0 + j / fs
//   y[m]   = sum_k b[k] * mix[m*D - k]              (causal FIR, zero before j = 0)
//
// for m = 0 .. ceil(L/D) - 1 (MATLAB's data(1:D:end,...)).  The caller shifts the
// output's initial time by the filter delay (ntaps - 1) / 2 / fs.
//
// One CTA computes kout (<= 1024) consecutive outputs of one trace: it stages the
// taps and the mixed samples the outputs need (kout*D + ntaps - 1 of them, at most
// about 8192) in shared memory, the samples in polyphase order (phase-major) so that the
// 32 outputs of a warp read 32 consecutive samples for each tap; each thread forms 4
// outputs with independent accumulators.  The mixer phase
// is formed in cycles as c0 + j*step with step split into two floats and the
// product's rounding error recovered by an FMA, so the phase stays exact to
// ~1e-7 cycles over any trace length.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "common.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kOPT = 4;                  // outputs per thread
constexpr int kStage = 8192;             // staged samples per CTA at most (64 KB), when kout allows

template <typename S>
__device__ __forceinline__ float rf_sample(const S* p, int64_t i);
template <>
__device__ __forceinline__ float rf_sample<float>(const float* p, int64_t i) { return __ldg(p + i); }
template <>
__device__ __forceinline__ float rf_sample<int16_t>(const int16_t* p, int64_t i) { return (float)__ldg(p + i); }
template <>
__device__ __forceinline__ float rf_sample<__half>(const __half* p, int64_t i) { return __half2float(__ldg(p + i)); }

// 4 consecutive samples starting at an index whose address is 4-sample aligned
template <typename S>
__device__ __forceinline__ float4 rf_vec4(const S* p, int64_t i);
template <>
__device__ __forceinline__ float4 rf_vec4<float>(const float* p, int64_t i) {
    return __ldg(reinterpret_cast<const float4*>(p + i));
}
template <>
__device__ __forceinline__ float4 rf_vec4<int16_t>(const int16_t* p, int64_t i) {
    const uint2 u = __ldg(reinterpret_cast<const uint2*>(p + i));
    return make_float4((float)(int16_t)(u.x & 0xFFFF), (float)(int16_t)(u.x >> 16), (float)(int16_t)(u.y & 0xFFFF),
                       (float)(int16_t)(u.y >> 16));
}
template <>
__device__ __forceinline__ float4 rf_vec4<__half>(const __half* p, int64_t i) {
    const uint2 u = __ldg(reinterpret_cast<const uint2*>(p + i));
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
}

template <typename D>
__device__ __forceinline__ void store_iq(D* out, int64_t i, float2 v);
template <>
__device__ __forceinline__ void store_iq<float>(float* out, int64_t i, float2 v) {
    reinterpret_cast<float2*>(out)[i] = v;
}
template <>
__device__ __forceinline__ void store_iq<__half>(__half* out, int64_t i, float2 v) {
    reinterpret_cast<__half2*>(out)[i] = __floats2half2_rn(v.x, v.y);
}
template <>
__device__ __forceinline__ void store_iq<__nv_bfloat16>(__nv_bfloat16* out, int64_t i, float2 v) {
    reinterpret_cast<__nv_bfloat162*>(out)[i] = __floats2bfloat162_rn(v.x, v.y);
}

struct DemodArgs {
    int64_t L, Ld, n_traces;
    int D, ntaps, kout;  // kout: outputs per CTA (<= kThreads * kOPT)
    float c0;              // fractional part of fc * t0 (cycles)
    float step_hi, step_lo;  // fc / fs split into two floats
    float scale;
};

template <typename S, typename D>
__global__ void __launch_bounds__(kThreads) demod_kernel(const S* __restrict__ rf, D* __restrict__ iq,
                                                         const float* __restrict__ taps, const DemodArgs a) {
    // shared: taps[ntaps], then the mixed samples [kout * D + ntaps - 1]
    extern __shared__ float2 smem2[];
    float* tap = reinterpret_cast<float*>(smem2);
    float2* mix = smem2 + (a.ntaps + 1) / 2;
    const int64_t chunks = (a.Ld + a.kout - 1) / a.kout;
    const int64_t trace = blockIdx.x / chunks;
    const int64_t m0 = (blockIdx.x - trace * chunks) * a.kout;
    if (trace >= a.n_traces) return;
    for (int k = threadIdx.x; k < a.ntaps; k += kThreads) tap[k] = __ldg(taps + k);
    const S* x = rf + trace * a.L;
    // staged window [j0, j0 + nstage), stored from jb <= j0 where the address of
    // sample jb is 4-sample aligned, so that threads load 4 samples per instruction
    const int64_t j0 = m0 * a.D - (a.ntaps - 1);  // first needed sample (may be negative)
    const int off = (int)((((trace * a.L + j0) % 4) + 4) % 4);
    const int64_t jb = j0 - off;
    const int nstage = a.kout * a.D + a.ntaps - 1 + off;
    // the staged samples are stored polyphase: sample s at mix[(s % D) * Q + s / D], so
    // that for one tap the 32 outputs of a warp read 32 consecutive float2
    const int Q = (nstage + a.D - 1) / a.D;
    for (int s0 = 4 * threadIdx.x; s0 < nstage; s0 += 4 * kThreads) {
        const int64_t jv = jb + s0;
        float r[4];
        if (jv >= 0 && jv + 3 < a.L) {
            const float4 v = rf_vec4<S>(x, jv);
            r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
        } else {
#pragma unroll
            for (int u = 0; u < 4; ++u) r[u] = (jv + u >= 0 && jv + u < a.L) ? rf_sample<S>(x, jv + u) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int s = s0 + u;
            if (s >= nstage) break;
            const int64_t j = jv + u;
            float2 v = make_float2(0.f, 0.f);
            if (j >= 0 && j < a.L) {
                const float jf = (float)j;  // exact: L < 2^24
                const float p = jf * a.step_hi;
                const float e = fmaf(jf, a.step_hi, -p);  // rounding error of the product
                const float cyc = (a.c0 + (p - rintf(p))) + fmaf(jf, a.step_lo, e);
                float sn, cs;
                __sincosf(-6.283185307179586f * (cyc - rintf(cyc)), &sn, &cs);
                const float rr = a.scale * r[u];
                v = make_float2(rr * cs, rr * sn);
            }
            mix[(s % a.D) * Q + s / a.D] = v;  // polyphase: phase-major
        }
    }
    __syncthreads();
    // outputs o = threadIdx.x + kThreads * q, kOPT per thread: independent accumulators
    float2 acc[kOPT];
#pragma unroll
    for (int q = 0; q < kOPT; ++q) acc[q] = make_float2(0.f, 0.f);
    const int last = a.ntaps - 1 + off;
    // tap k reads staged sample o*D + last - k: phase (last - k) % D, offset (last - k) / D,
    // stepped down incrementally instead of divided per tap
    auto fir = [&](auto full) {
        int ph = last % a.D, qo = last / a.D;
        for (int k = 0; k < a.ntaps; ++k) {
            const float b = tap[k];
            const float2* row = mix + ph * Q + qo;
#pragma unroll
            for (int q = 0; q < kOPT; ++q) {
                const int o = threadIdx.x + kThreads * q;
                if (decltype(full)::value || o < a.kout) {
                    const float2 v = row[o];
                    acc[q].x = fmaf(b, v.x, acc[q].x);
                    acc[q].y = fmaf(b, v.y, acc[q].y);
                }
            }
            if (ph == 0) {
                ph = a.D - 1;
                --qo;
            } else {
                --ph;
            }
        }
    };
    if (a.kout == kThreads * kOPT) fir(std::true_type{});
    else fir(std::false_type{});
#pragma unroll
    for (int q = 0; q < kOPT; ++q) {
        const int o = threadIdx.x + kThreads * q;
        const int64_t m = m0 + o;
        if (o < a.kout && m < a.Ld) store_iq<D>(iq, trace * a.Ld + m, acc[q]);
    }
}

template <typename S>
int launch_demod(const S* rf, void* iq, int32_t dst_type, const float* taps, const DemodArgs& a, cudaStream_t s) {
    const int64_t chunks = (a.Ld + a.kout - 1) / a.kout;
    const int64_t blocks = chunks * a.n_traces;
    USTB_REQUIRE(blocks <= INT32_MAX, USTB_E_SHAPE, "too many traces x output chunks");
    const size_t smem = sizeof(float2) * ((size_t)(a.ntaps + 1) / 2 + (size_t)(a.kout * a.D + a.ntaps - 1 + 3) + a.D);
    int dev = 0, optin = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    USTB_REQUIRE(smem <= (size_t)optin, USTB_E_SHAPE, "decimation %d with %d taps needs %zu bytes of shared memory",
                 a.D, a.ntaps, smem);
    switch (dst_type) {
        case USTB_STORE_F32:
            USTB_CUDA(cudaFuncSetAttribute(demod_kernel<S, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            demod_kernel<S, float><<<(unsigned)blocks, kThreads, smem, s>>>(rf, (float*)iq, taps, a);
            break;
        case USTB_STORE_F16:
            USTB_CUDA(cudaFuncSetAttribute(demod_kernel<S, __half>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            demod_kernel<S, __half><<<(unsigned)blocks, kThreads, smem, s>>>(rf, (__half*)iq, taps, a);
            break;
        default:
            USTB_CUDA(cudaFuncSetAttribute(demod_kernel<S, __nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            demod_kernel<S, __nv_bfloat16><<<(unsigned)blocks, kThreads, smem, s>>>(rf, (__nv_bfloat16*)iq, taps, a);
            break;
    }
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}

// ---------------------------------------------------------------------------
// Zero-phase variant, python/src/ustb/preprocess/fast_demodulation.py:71-134: the
// mixed trace is filtered forward and backward with the FIR (scipy filtfilt with its
// defaults: odd extension by P = 3 * ntaps samples at both ends, steady-state initial
// conditions in both directions) and then sampled every D-th sample from the first,
// with t0 unchanged:
//
//   E[m] = odd extension of mix, m in [0, L + 2P):
//          2 mix[0] - mix[P - m]            m < P
//          mix[m - P]                       P <= m < P + L
//          2 mix[L-1] - mix[2L + P - 2 - m] m >= P + L
//   f[n] = sum_k b[k] E[max(n - k, 0)]              (forward, steady state before E[0])
//   g[n] = sum_k b[k] f[min(n + k, L + 2P - 1)]     (backward, steady state after the end)
//   y[i] = g[i*D + P]
//
// The outputs only need f at n >= P, where n - k >= 2P/3 + 1 > 0, so the forward
// clamp never applies there.  One CTA forms kout consecutive outputs of one trace: it
// stages the E window they need, computes f over it into a second shared array,
// then each thread forms outputs from f.
struct FiltfiltArgs {
    int64_t L, Ld, n_traces;
    int D, ntaps, P, kout;
    float c0, step_hi, step_lo, scale;
};

template <typename S>
__device__ __forceinline__ float2 mixed_sample(const S* x, int64_t j, const FiltfiltArgs& a) {
    const float jf = (float)j;  // exact: L < 2^24
    const float p = jf * a.step_hi;
    const float e = fmaf(jf, a.step_hi, -p);
    const float cyc = (a.c0 + (p - rintf(p))) + fmaf(jf, a.step_lo, e);
    float sn, cs;
    __sincosf(-6.283185307179586f * (cyc - rintf(cyc)), &sn, &cs);
    const float r = a.scale * rf_sample<S>(x, j);
    return make_float2(r * cs, r * sn);
}

template <typename S>
__device__ __forceinline__ float2 extended_sample(const S* x, int64_t m, const FiltfiltArgs& a) {
    if (m < a.P) {
        const float2 e0 = mixed_sample<S>(x, 0, a), v = mixed_sample<S>(x, a.P - m, a);
        return make_float2(2.f * e0.x - v.x, 2.f * e0.y - v.y);
    }
    if (m < a.P + a.L) return mixed_sample<S>(x, m - a.P, a);
    const float2 e1 = mixed_sample<S>(x, a.L - 1, a), v = mixed_sample<S>(x, 2 * a.L + a.P - 2 - m, a);
    return make_float2(2.f * e1.x - v.x, 2.f * e1.y - v.y);
}

template <typename S, typename D>
__global__ void __launch_bounds__(kThreads) filtfilt_kernel(const S* __restrict__ rf, D* __restrict__ iq,
                                                            const float* __restrict__ taps, const FiltfiltArgs a) {
    extern __shared__ float2 smem2[];
    const int M = a.ntaps;
    float* tap = reinterpret_cast<float*>(smem2);
    const int64_t chunks = (a.Ld + a.kout - 1) / a.kout;
    const int64_t trace = blockIdx.x / chunks;
    const int64_t m0 = (blockIdx.x - trace * chunks) * a.kout;
    if (trace >= a.n_traces) return;
    const int nout = (int)(a.Ld - m0 < a.kout ? a.Ld - m0 : a.kout);
    const int64_t Ne = a.L + 2 * a.P;
    const int64_t flo = m0 * a.D + a.P;                                      // first f needed
    const int64_t fend = (m0 + nout - 1) * a.D + a.P + M - 1;
    const int64_t fhi = fend < Ne - 1 ? fend : Ne - 1;  // last f needed
    const int nF = (int)(fhi - flo + 1), nE = nF + M - 1;
    const int64_t elo = flo - (M - 1);
    float2* Es = smem2 + (M + 1) / 2;
    float2* Fs = Es + nE;
    for (int k = threadIdx.x; k < M; k += kThreads) tap[k] = __ldg(taps + k);
    const S* x = rf + trace * a.L;
    for (int e = threadIdx.x; e < nE; e += kThreads) Es[e] = extended_sample<S>(x, elo + e, a);
    __syncthreads();
    for (int q = threadIdx.x; q < nF; q += kThreads) {
        float2 acc = make_float2(0.f, 0.f);
        const float2* row = Es + q + (M - 1);
        for (int k = 0; k < M; ++k) {
            const float b = tap[k];
            const float2 v = row[-k];
            acc.x = fmaf(b, v.x, acc.x);
            acc.y = fmaf(b, v.y, acc.y);
        }
        Fs[q] = acc;
    }
    __syncthreads();
    for (int o = threadIdx.x; o < nout; o += kThreads) {
        const int64_t n = (m0 + o) * a.D + a.P;
        float2 acc = make_float2(0.f, 0.f);
        for (int k = 0; k < M; ++k) {
            const float b = tap[k];
            const float2 v = Fs[(n + k < Ne - 1 ? n + k : Ne - 1) - flo];
            acc.x = fmaf(b, v.x, acc.x);
            acc.y = fmaf(b, v.y, acc.y);
        }
        store_iq<D>(iq, trace * a.Ld + m0 + o, acc);
    }
}

template <typename S>
int launch_filtfilt(const S* rf, void* iq, int32_t dst_type, const float* taps, const FiltfiltArgs& a, cudaStream_t s) {
    const int64_t chunks = (a.Ld + a.kout - 1) / a.kout;
    const int64_t blocks = chunks * a.n_traces;
    USTB_REQUIRE(blocks <= INT32_MAX, USTB_E_SHAPE, "too many traces x output chunks");
    const size_t nF = (size_t)(a.kout - 1) * a.D + a.ntaps;
    const size_t smem = sizeof(float2) * ((size_t)(a.ntaps + 1) / 2 + 2 * nF + a.ntaps);
    int dev = 0, optin = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    USTB_REQUIRE(smem <= (size_t)optin, USTB_E_SHAPE, "decimation %d with %d taps needs %zu bytes of shared memory",
                 a.D, a.ntaps, smem);
    switch (dst_type) {
        case USTB_STORE_F32:
            USTB_CUDA(cudaFuncSetAttribute(filtfilt_kernel<S, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            filtfilt_kernel<S, float><<<(unsigned)blocks, kThreads, smem, s>>>(rf, (float*)iq, taps, a);
            break;
        case USTB_STORE_F16:
            USTB_CUDA(cudaFuncSetAttribute(filtfilt_kernel<S, __half>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            filtfilt_kernel<S, __half><<<(unsigned)blocks, kThreads, smem, s>>>(rf, (__half*)iq, taps, a);
            break;
        default:
            USTB_CUDA(cudaFuncSetAttribute(filtfilt_kernel<S, __nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            filtfilt_kernel<S, __nv_bfloat16><<<(unsigned)blocks, kThreads, smem, s>>>(rf, (__nv_bfloat16*)iq, taps, a);
            break;
    }
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}

}  // namespace

extern "C" int ustb_demodulate(const void* rf, int32_t src_type, void* iq, int32_t dst_type, int64_t L,
                               int64_t n_traces, double fs, double t0, double fc, int32_t decimation,
                               const float* taps, int32_t ntaps, float scale, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(src_type >= 0 && src_type <= 2, USTB_E_DTYPE, "unknown source type %d", (int)src_type);
    USTB_REQUIRE(dst_type >= 0 && dst_type <= 2, USTB_E_DTYPE, "unknown storage type %d", (int)dst_type);
    USTB_REQUIRE(L >= 0 && n_traces >= 0, USTB_E_SHAPE, "negative size");
    USTB_REQUIRE(L < (1 << 24), USTB_E_SHAPE, "at most 2^24 samples per trace");
    USTB_REQUIRE(decimation >= 1 && decimation <= 64, USTB_E_ARG, "decimation must be in [1, 64], got %d",
                 (int)decimation);
    USTB_REQUIRE(ntaps >= 1 && ntaps <= 4096, USTB_E_ARG, "ntaps must be in [1, 4096], got %d", (int)ntaps);
    USTB_REQUIRE(fs > 0.0, USTB_E_ARG, "sampling frequency must be > 0");
    if (L == 0 || n_traces == 0) return USTB_OK;
    USTB_REQUIRE(rf && iq && taps, USTB_E_ARG, "NULL pointer");
    DemodArgs a;
    a.L = L;
    a.Ld = (L + decimation - 1) / decimation;
    a.n_traces = n_traces;
    a.D = decimation;
    a.ntaps = ntaps;
    a.kout = (int)std::max<int64_t>(32, std::min<int64_t>(kThreads * kOPT, (kStage - ntaps) / decimation));
    const double c0 = fc * t0;
    a.c0 = (float)(c0 - std::floor(c0));
    const double step = fc / fs;
    a.step_hi = (float)step;
    a.step_lo = (float)(step - (double)a.step_hi);
    a.scale = scale;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (src_type) {
        case USTB_SRC_F32: return launch_demod<float>((const float*)rf, iq, dst_type, taps, a, s);
        case USTB_SRC_I16: return launch_demod<int16_t>((const int16_t*)rf, iq, dst_type, taps, a, s);
        default: return launch_demod<__half>((const __half*)rf, iq, dst_type, taps, a, s);
    }
}

extern "C" int ustb_demodulate_filtfilt(const void* rf, int32_t src_type, void* iq, int32_t dst_type, int64_t L,
                                        int64_t n_traces, double fs, double t0, double fc, int32_t decimation,
                                        const float* taps, int32_t ntaps, float scale, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(src_type >= 0 && src_type <= 2, USTB_E_DTYPE, "unknown source type %d", (int)src_type);
    USTB_REQUIRE(dst_type >= 0 && dst_type <= 2, USTB_E_DTYPE, "unknown storage type %d", (int)dst_type);
    USTB_REQUIRE(L >= 0 && n_traces >= 0, USTB_E_SHAPE, "negative size");
    USTB_REQUIRE(L < (1 << 24), USTB_E_SHAPE, "at most 2^24 samples per trace");
    USTB_REQUIRE(decimation >= 1 && decimation <= 64, USTB_E_ARG, "decimation must be in [1, 64], got %d",
                 (int)decimation);
    USTB_REQUIRE(ntaps >= 1 && ntaps <= 1024, USTB_E_ARG, "ntaps must be in [1, 1024], got %d", (int)ntaps);
    USTB_REQUIRE(fs > 0.0, USTB_E_ARG, "sampling frequency must be > 0");
    if (n_traces == 0) return USTB_OK;
    // scipy filtfilt: the trace must be longer than the padding
    USTB_REQUIRE(L > 3 * (int64_t)ntaps, USTB_E_SHAPE,
                 "the trace (%lld samples) must be longer than the padding 3 * ntaps = %d", (long long)L,
                 3 * (int)ntaps);
    USTB_REQUIRE(rf && iq && taps, USTB_E_ARG, "NULL pointer");
    FiltfiltArgs a;
    a.L = L;
    a.Ld = (L + decimation - 1) / decimation;
    a.n_traces = n_traces;
    a.D = decimation;
    a.ntaps = ntaps;
    a.P = 3 * ntaps;
    a.kout = (int)std::max<int64_t>(32, std::min<int64_t>(kThreads * kOPT, (kStage / 2 - ntaps) / decimation + 1));
    const double c0 = fc * t0;
    a.c0 = (float)(c0 - std::floor(c0));
    const double step = fc / fs;
    a.step_hi = (float)step;
    a.step_lo = (float)(step - (double)a.step_hi);
    a.scale = scale;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (src_type) {
        case USTB_SRC_F32: return launch_filtfilt<float>((const float*)rf, iq, dst_type, taps, a, s);
        case USTB_SRC_I16: return launch_filtfilt<int16_t>((const int16_t*)rf, iq, dst_type, taps, a, s);
        default: return launch_filtfilt<__half>((const __half*)rf, iq, dst_type, taps, a, s);
    }
}
