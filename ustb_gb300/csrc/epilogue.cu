// Per-pixel phase epilogue of midprocess.das (+midprocess/das.m:306-309):
// bf(p, ...) *= exp(-i*2*w0*reference_distance(p)/c).  The factor is formed on
// the host in double (as MATLAB does) and applied here in single precision.
#include "common.cuh"

namespace {

__global__ void apply_phase_kernel(float2* __restrict__ data, const float2* __restrict__ ph,
                                   int64_t P, int64_t total) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float2 f = __ldg(ph + (i % P));
        const float2 v = data[i];
        data[i] = make_float2(v.x * f.x - v.y * f.y, v.x * f.y + v.y * f.x);
    }
}

}  // namespace

extern "C" int ustb_apply_pixel_phase(void* data, int64_t P, int64_t rest, const void* phase,
                                      void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(P >= 0 && rest >= 0, USTB_E_SHAPE, "negative size");
    const int64_t total = P * rest;
    if (total == 0) return USTB_OK;
    USTB_REQUIRE(data && phase, USTB_E_ARG, "NULL pointer");
    int dev = 0, sms = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t want = (total + 255) / 256;
    const unsigned grid = (unsigned)std::min<int64_t>(want, (int64_t)sms * 8);
    apply_phase_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<float2*>(data), static_cast<const float2*>(phase), P, total);
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}
