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
// about 8192) in shared memory, the samples in polyphase order (phase-major): output o
// reads, for tap k, position o + (last - k)/D of row (last - k) % D, so the taps of one
// row step one position at a time.  Each thread forms 4 consecutive outputs and, per
// block of 4 taps of a row, loads the 7 samples they span once (a shared load per
// 4.6 FMA instead of per 2); a float2 of padding after every 16 keeps the half-warps'
// loads on distinct banks.  The mixer phase
// is formed in cycles as c0 + j*step with step split into two floats and the
// product's rounding error recovered by an FMA, so the phase stays exact to
// ~1e-7 cycles over any trace length.
//
// The zero-phase variant (ustb_demodulate_filtfilt, the reference's Python port,
// python/src/ustb/preprocess/fast_demodulation.py:47-76) is the same pass with the
// taps replaced by the autocorrelation of b (2 ntaps - 1 of them, formed per CTA),
// the sequence shifted by ntaps - 1 samples so the filter is centred, and the
// trace odd-extended about its end samples (scipy filtfilt's padding) instead of
// zero-extended.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "common.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kOPT = 4;                  // consecutive outputs per thread
constexpr int kTB = 4;                   // taps per register block (one float4 of a tap row)
static_assert(kTB == 4, "a tap block is read as one float4");

// staged row position q with one float2 of padding after every 16, so that the 16
// lanes of a half-warp, whose first outputs are 4 apart, read 16 different bank pairs
__device__ __forceinline__ int row_pad(int q) { return q + (q >> 4); }
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
    int mb, shift;         // zero-phase: taps of the reference filter, and mb - 1
    int Qa, Qp;            // staged samples per polyphase row, and the padded row stride
    int T4, Cap;           // taps rounded up to 4; taps per polyphase row (a multiple of 4)
    float c0;              // fractional part of fc * t0 (cycles)
    float step_hi, step_lo;  // fc / fs split into two floats
    float scale;
};

// scale * x * exp(-i 2 pi fc (t0 + j/fs)) for raw sample value x at index j
__device__ __forceinline__ float2 mix_value(float x, int64_t j, const DemodArgs& a) {
    const float jf = (float)j;  // exact: |j| < 2^24
    const float p = jf * a.step_hi;
    const float e = fmaf(jf, a.step_hi, -p);  // rounding error of the product
    const float cyc = (a.c0 + (p - rintf(p))) + fmaf(jf, a.step_lo, e);
    float sn, cs;
    __sincosf(-6.283185307179586f * (cyc - rintf(cyc)), &sn, &cs);
    const float rr = a.scale * x;
    return make_float2(rr * cs, rr * sn);
}

// mixed sample j of the sequence the FIR runs over: the trace with zeros outside it,
// or (zero-phase) its odd extension about both end samples, zero beyond one reflection
template <typename S, bool ZP>
__device__ __forceinline__ float2 edge_value(const S* x, int64_t j, const DemodArgs& a) {
    if (j >= 0 && j < a.L) return mix_value(rf_sample<S>(x, j), j, a);
    if (!ZP) return make_float2(0.f, 0.f);
    int64_t e, r;  // end sample and reflected sample
    if (j < 0) {
        e = 0;
        r = -j;
    } else {
        e = a.L - 1;
        r = 2 * a.L - 2 - j;
    }
    if (r < 0 || r >= a.L) return make_float2(0.f, 0.f);
    const float2 ve = mix_value(rf_sample<S>(x, e), e, a), vr = mix_value(rf_sample<S>(x, r), r, a);
    return make_float2(2.f * ve.x - vr.x, 2.f * ve.y - vr.y);
}

template <typename S, typename D, bool ZP>
__global__ void __launch_bounds__(kThreads) demod_kernel(const S* __restrict__ rf, D* __restrict__ iq,
                                                         const float* __restrict__ taps, const DemodArgs a) {
    // shared: taps[ntaps], then the mixed samples [kout * D + ntaps - 1]
    extern __shared__ float2 smem2[];
    float* tap = reinterpret_cast<float*>(smem2);  // zero-phase: the taps formed per CTA
    float* trow = tap + a.T4;                       // taps by polyphase row, zero-padded
    float2* mix = reinterpret_cast<float2*>(trow + a.D * a.Cap);
    const int64_t chunks = (a.Ld + a.kout - 1) / a.kout;
    const int64_t trace = blockIdx.x / chunks;
    const int64_t m0 = (blockIdx.x - trace * chunks) * a.kout;
    if (trace >= a.n_traces) return;
    if constexpr (ZP) {
        // the single FIR equal to filtfilt at the kept samples: the autocorrelation
        // h[t] = sum_j b[j] b[j - t], |t| < mb, staged from b in the sample area
        float* bt = reinterpret_cast<float*>(mix);
        for (int k = threadIdx.x; k < a.mb; k += kThreads) bt[k] = __ldg(taps + k);
        __syncthreads();
        // two neighbouring threads per tap, each summing half of the products
        for (int i0 = 0; i0 < 2 * a.ntaps; i0 += kThreads) {  // bounds uniform across the CTA
            const int i = i0 + threadIdx.x, k = i >> 1;
            float h = 0.f;
            if (k < a.ntaps) {
                const int t = k - (a.mb - 1);
                const int lo = max(0, t), hi = min(a.mb, a.mb + t), mid = (lo + hi) >> 1;
                for (int j = (i & 1) ? mid : lo; j < ((i & 1) ? hi : mid); ++j) h = fmaf(bt[j], bt[j - t], h);
            }
            h += __shfl_xor_sync(0xffffffffu, h, 1);
            if (k < a.ntaps && !(i & 1)) tap[k] = h;
        }
        __syncthreads();
    }
    const S* x = rf + trace * a.L;
    // staged window [j0, j0 + nstage) of the filtered sequence, whose sample j is
    // trace sample j + shift, stored from jb <= j0 where the address of trace sample
    // jb + shift is 4-sample aligned, so that threads load 4 samples per instruction
    const int64_t j0 = m0 * a.D - (a.ntaps - 1);  // first needed sample (may be negative)
    const int off = (int)((((trace * a.L + j0 + a.shift) % 4) + 4) % 4);
    const int64_t jb = j0 - off;
    const int nstage = a.kout * a.D + a.ntaps - 1 + off;
    // the staged samples are stored polyphase: sample s at mix[(s % D) * Qp + row_pad(s / D)];
    // the rows' tails, read by the last outputs' padded tap blocks, are zeros
    const int Qp = a.Qp;
    // tap k belongs to row (last - k) % D at m = (last - k) / D: trow[ph][m]
    const int last = a.ntaps - 1 + off;
    for (int i = threadIdx.x; i < a.D * a.Cap; i += kThreads) {
        const int ph = i / a.Cap, m = i - ph * a.Cap;
        const int k = last - ph - m * a.D;
        float b = 0.f;
        if (k >= 0 && k < a.ntaps) b = ZP ? tap[k] : __ldg(taps + k);
        trow[i] = b;
    }
    for (int t = nstage + threadIdx.x; t < a.Qa * a.D; t += kThreads)
        mix[(t % a.D) * Qp + row_pad(t / a.D)] = make_float2(0.f, 0.f);
    for (int s0 = 4 * threadIdx.x; s0 < nstage; s0 += 4 * kThreads) {
        const int64_t jv = jb + s0 + a.shift;  // trace index of staged sample s0
        float2 v[4];
        if (jv >= 0 && jv + 3 < a.L) {
            const float4 q = rf_vec4<S>(x, jv);
            v[0] = mix_value(q.x, jv, a);
            v[1] = mix_value(q.y, jv + 1, a);
            v[2] = mix_value(q.z, jv + 2, a);
            v[3] = mix_value(q.w, jv + 3, a);
        } else {
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = edge_value<S, ZP>(x, jv + u, a);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int s = s0 + u;
            if (s >= nstage) break;
            mix[(s % a.D) * Qp + row_pad(s / a.D)] = v[u];  // polyphase: phase-major
        }
    }
    __syncthreads();
    // kOPT consecutive outputs per thread.  Output o at tap k reads staged sample
    // o*D + last - k, i.e. row (last - k) % D at o + (last - k) / D: the taps of one
    // row, k = last - ph - m*D, step the read position by one.  For each block of kTB
    // taps of a row the thread loads the kOPT + kTB - 1 samples they span once.
    float2 acc[kOPT];
#pragma unroll
    for (int q = 0; q < kOPT; ++q) acc[q] = make_float2(0.f, 0.f);
    const int o0 = threadIdx.x * kOPT;
    if (o0 < a.kout) {
        for (int ph = 0; ph < a.D && ph <= last; ++ph) {
            const int mhi = (last - ph) / a.D;  // taps k = last - ph - m D >= 0 (zero where k >= ntaps)
            const float2* row = mix + ph * Qp;
            const float* tr = trow + ph * a.Cap;
            for (int m0 = 0; m0 <= mhi; m0 += kTB) {
                const float4 b4 = *reinterpret_cast<const float4*>(tr + m0);
                const float bb[kTB] = {b4.x, b4.y, b4.z, b4.w};
                float2 v[kOPT + kTB - 1];
#pragma unroll
                for (int j = 0; j < kOPT + kTB - 1; ++j) v[j] = row[row_pad(o0 + m0 + j)];
#pragma unroll
                for (int mm = 0; mm < kTB; ++mm) {
#pragma unroll
                    for (int q = 0; q < kOPT; ++q) {
                        acc[q].x = fmaf(bb[mm], v[q + mm].x, acc[q].x);
                        acc[q].y = fmaf(bb[mm], v[q + mm].y, acc[q].y);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < kOPT; ++q) {
        const int o = o0 + q;
        const int64_t m = m0 + o;
        if (o < a.kout && m < a.Ld) store_iq<D>(iq, trace * a.Ld + m, acc[q]);
    }
}

// staged row length and padded stride: the rows hold the chunk's samples and the
// farthest position a thread's last tap block reads, o + m + j < kout + (ntaps + 2)/D + kOPT + kTB
void set_rows(DemodArgs& a) {
    a.Qa = a.kout + (a.ntaps + 2) / a.D + kOPT + kTB;
    a.Qp = (a.Qa - 1) + ((a.Qa - 1) >> 4) + 1;
    a.T4 = (a.ntaps + 3) / 4 * 4;
    a.Cap = ((a.ntaps + 2) / a.D + 1 + 3) / 4 * 4;  // m <= (ntaps - 1 + 3) / D
}

// outputs per CTA: the trace's Ld outputs split into the fewest chunks of at most kmax,
// all of the same size (a last, short chunk would leave most of its CTA idle)
int balanced_chunk(int64_t Ld, int64_t kmax) {
    const int64_t chunks = (Ld + kmax - 1) / kmax;
    return (int)((Ld + chunks - 1) / chunks);
}

template <typename S, bool ZP>
int launch_demod(const S* rf, void* iq, int32_t dst_type, const float* taps, const DemodArgs& a, cudaStream_t s) {
    const int64_t chunks = (a.Ld + a.kout - 1) / a.kout;
    const int64_t blocks = chunks * a.n_traces;
    USTB_REQUIRE(blocks <= INT32_MAX, USTB_E_SHAPE, "too many traces x output chunks");
    const size_t smem = sizeof(float) * ((size_t)a.T4 + (size_t)a.D * (size_t)a.Cap) +
                        sizeof(float2) * (size_t)a.D * (size_t)a.Qp;
    int dev = 0, optin = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    USTB_REQUIRE(smem <= (size_t)optin, USTB_E_SHAPE, "decimation %d with %d taps needs %zu bytes of shared memory",
                 a.D, a.ntaps, smem);
    switch (dst_type) {
        case USTB_STORE_F32:
            USTB_CUDA(cudaFuncSetAttribute(demod_kernel<S, float, ZP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            demod_kernel<S, float, ZP><<<(unsigned)blocks, kThreads, smem, s>>>(rf, (float*)iq, taps, a);
            break;
        case USTB_STORE_F16:
            USTB_CUDA(cudaFuncSetAttribute(demod_kernel<S, __half, ZP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            demod_kernel<S, __half, ZP><<<(unsigned)blocks, kThreads, smem, s>>>(rf, (__half*)iq, taps, a);
            break;
        default:
            USTB_CUDA(cudaFuncSetAttribute(demod_kernel<S, __nv_bfloat16, ZP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            demod_kernel<S, __nv_bfloat16, ZP><<<(unsigned)blocks, kThreads, smem, s>>>(rf, (__nv_bfloat16*)iq, taps, a);
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
    a.kout = balanced_chunk(a.Ld, std::max<int64_t>(32, std::min<int64_t>(kThreads * kOPT, (kStage - ntaps) / decimation)));
    set_rows(a);
    const double c0 = fc * t0;
    a.c0 = (float)(c0 - std::floor(c0));
    const double step = fc / fs;
    a.step_hi = (float)step;
    a.step_lo = (float)(step - (double)a.step_hi);
    a.scale = scale;
    a.mb = ntaps;
    a.shift = 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (src_type) {
        case USTB_SRC_F32: return launch_demod<float, false>((const float*)rf, iq, dst_type, taps, a, s);
        case USTB_SRC_I16: return launch_demod<int16_t, false>((const int16_t*)rf, iq, dst_type, taps, a, s);
        default: return launch_demod<__half, false>((const __half*)rf, iq, dst_type, taps, a, s);
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
    // At every kept sample, filtfilt equals one FIR with the 2 ntaps - 1 taps of b's
    // autocorrelation applied to the odd-extended mixed trace: the kept outputs only
    // use forward values at least 2 ntaps + 1 samples into the extension and backward
    // sums that end at least 2 ntaps samples before its end, so neither pass's
    // steady-state start is reached.
    DemodArgs a;
    a.L = L;
    a.Ld = (L + decimation - 1) / decimation;
    a.n_traces = n_traces;
    a.D = decimation;
    a.ntaps = 2 * ntaps - 1;
    a.mb = ntaps;
    a.shift = ntaps - 1;
    a.kout = balanced_chunk(a.Ld, std::max<int64_t>(32, std::min<int64_t>(kThreads * kOPT, (kStage - a.ntaps) / decimation)));
    set_rows(a);
    const double c0 = fc * t0;
    a.c0 = (float)(c0 - std::floor(c0));
    const double step = fc / fs;
    a.step_hi = (float)step;
    a.step_lo = (float)(step - (double)a.step_hi);
    a.scale = scale;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (src_type) {
        case USTB_SRC_F32: return launch_demod<float, true>((const float*)rf, iq, dst_type, taps, a, s);
        case USTB_SRC_I16: return launch_demod<int16_t, true>((const int16_t*)rf, iq, dst_type, taps, a, s);
        default: return launch_demod<__half, true>((const __half*)rf, iq, dst_type, taps, a, s);
    }
}
