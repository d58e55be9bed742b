// Depth-direction FIR filtering of beamformed images, the band-pass step of
// the simplified delay-multiply-and-sum post-process
// (+postprocess/simplified_delay_multiply_and_sum.m:170-176):
//   filtered = filter(b, 1, [y; zeros(d)]);  out = filtered(d+1:end)
// i.e. out[z] = sum_k b[k] * y[z + d - k] with y = 0 outside [0, Nz).
#include <algorithm>

#include "common.cuh"

namespace {

constexpr int kMaxTaps = 1024;
constexpr int kR = 8;  // consecutive outputs per thread

// shared index of staged sample s: one word of padding after every 32, so that the
// 32 lanes of a warp, whose windows start 8 samples apart, hit 32 different banks
__device__ __forceinline__ int pad(int s) { return s + (s >> 5); }

// One CTA filters a run of nthreads * kR consecutive depths of one column.  It
// stages the taps (zero-padded to a multiple of kR) and the input samples the run
// needs (zeros outside [0, nz)); each thread then forms kR consecutive outputs,
// loading for every block of kR taps the 2 kR - 1 samples they span once and reusing
// them from registers.
__global__ void fir_depth_kernel(const float* __restrict__ in, float* __restrict__ out,
                                 const float* __restrict__ taps, int ntaps, int delay, int64_t nz,
                                 int64_t runs) {
    extern __shared__ float sh[];
    const int K = (ntaps + kR - 1) / kR * kR;  // padded tap count
    float* tp = sh;
    float* sm = sh + K;
    const int nrun = blockDim.x * kR;
    const int64_t col = blockIdx.x / runs;
    const int64_t z0 = (blockIdx.x - col * runs) * nrun;
    const float* x = in + col * nz;
    for (int k = threadIdx.x; k < K; k += blockDim.x) tp[k] = k < ntaps ? taps[k] : 0.f;
    // output z reads x[z + delay - k]; staged sample s is x[j0 + s], with kR - 1
    // extra samples in front for the padded taps
    const int64_t j0 = z0 + delay - (K - 1);
    const int ns = nrun + K - 1;
    for (int s = threadIdx.x; s < ns; s += blockDim.x) {
        const int64_t j = j0 + s;
        sm[pad(s)] = (j >= 0 && j < nz) ? __ldg(x + j) : 0.f;
    }
    __syncthreads();
    float acc[kR];
#pragma unroll
    for (int r = 0; r < kR; ++r) acc[r] = 0.f;
    const int base = threadIdx.x * kR + K - 1;  // output r at tap k reads staged sample base + r - k
    for (int k0 = 0; k0 < K; k0 += kR) {
        float v[2 * kR - 1];
#pragma unroll
        for (int j = 0; j < 2 * kR - 1; ++j) v[j] = sm[pad(base - k0 - (kR - 1) + j)];
#pragma unroll
        for (int kk = 0; kk < kR; ++kk) {
            const float b = tp[k0 + kk];
#pragma unroll
            for (int r = 0; r < kR; ++r) acc[r] = fmaf(b, v[r - kk + kR - 1], acc[r]);
        }
    }
#pragma unroll
    for (int r = 0; r < kR; ++r) {
        const int64_t z = z0 + threadIdx.x * kR + r;
        if (z < nz) out[col * nz + z] = acc[r];
    }
}

}  // namespace

extern "C" int ustb_fir_depth(const float* in, float* out, int64_t nz, int64_t ncols, const float* taps,
                              int32_t ntaps, int32_t delay, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(nz >= 0 && ncols >= 0, USTB_E_SHAPE, "negative size");
    USTB_REQUIRE(ntaps >= 1 && ntaps <= kMaxTaps, USTB_E_ARG, "ntaps must be in [1, %d]", kMaxTaps);
    USTB_REQUIRE(delay >= 0, USTB_E_ARG, "delay must be >= 0");
    if (nz == 0 || ncols == 0) return USTB_OK;
    USTB_REQUIRE(in && out && taps && in != out, USTB_E_ARG, "NULL or aliased pointer");
    // threads per CTA: enough for the column (a multiple of 32), at most 256
    const int64_t nthreads = std::min<int64_t>(256, ((nz + kR - 1) / kR + 31) / 32 * 32);
    const int64_t runs = (nz + nthreads * kR - 1) / (nthreads * kR);
    const int64_t blocks = runs * ncols;
    USTB_REQUIRE(blocks <= INT32_MAX, USTB_E_SHAPE, "too many columns");
    const int K = (ntaps + kR - 1) / kR * kR;
    const int ns = (int)nthreads * kR + K - 1;
    const size_t smem = sizeof(float) * ((size_t)K + (size_t)ns + (size_t)(ns >> 5) + 1);
    fir_depth_kernel<<<(unsigned)blocks, (unsigned)nthreads, smem, static_cast<cudaStream_t>(stream)>>>(
        in, out, taps, ntaps, delay, nz, runs);
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}
