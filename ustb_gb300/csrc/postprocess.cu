// Depth-direction FIR filtering of beamformed images, the band-pass step of
// the simplified delay-multiply-and-sum post-process
// (+postprocess/simplified_delay_multiply_and_sum.m:170-176):
//   filtered = filter(b, 1, [y; zeros(d)]);  out = filtered(d+1:end)
// i.e. out[z] = sum_k b[k] * y[z + d - k] with y = 0 outside [0, Nz).
#include "common.cuh"

namespace {

constexpr int kMaxTaps = 1024;

__global__ void fir_depth_kernel(const float* __restrict__ in, float* __restrict__ out,
                                 const float* __restrict__ taps, int ntaps, int delay, int64_t nz,
                                 int64_t ncols) {
    extern __shared__ float sh_taps[];
    for (int k = threadIdx.x; k < ntaps; k += blockDim.x) sh_taps[k] = taps[k];
    __syncthreads();
    const int64_t total = nz * ncols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t col = i / nz, z = i - col * nz;
        const float* x = in + col * nz;
        const int64_t hi = z + delay;  // newest input sample of this output
        float acc = 0.f;
        const int kmin = (int)max((int64_t)0, hi - (nz - 1));
        const int kmax = (int)min((int64_t)(ntaps - 1), hi);
        for (int k = kmin; k <= kmax; ++k) acc = fmaf(sh_taps[k], __ldg(x + hi - k), acc);
        out[i] = acc;
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
    int dev = 0, sms = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t total = nz * ncols;
    const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, (int64_t)sms * 8);
    fir_depth_kernel<<<grid, 256, ntaps * sizeof(float), static_cast<cudaStream_t>(stream)>>>(
        in, out, taps, ntaps, delay, nz, ncols);
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}
