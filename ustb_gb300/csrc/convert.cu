// Channel-data conversion into the device storage type of the fast path
// (e.g. int16 I/Q scanner samples or complex64 into half), with a scale.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"

namespace {

template <typename S>
__device__ __forceinline__ float load_src(const S* p, int64_t i);
template <>
__device__ __forceinline__ float load_src<float>(const float* p, int64_t i) { return __ldg(p + i); }
template <>
__device__ __forceinline__ float load_src<int16_t>(const int16_t* p, int64_t i) { return (float)__ldg(p + i); }
template <>
__device__ __forceinline__ float load_src<__half>(const __half* p, int64_t i) { return __half2float(__ldg(p + i)); }

template <typename D>
__device__ __forceinline__ D to_dst(float v);
template <>
__device__ __forceinline__ float to_dst<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half to_dst<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 to_dst<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

template <typename S, typename D>
__global__ void convert_kernel(const S* __restrict__ src, D* __restrict__ dst, int64_t n, float scale) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = to_dst<D>(load_src<S>(src, i) * scale);
}

template <typename S>
int launch_dst(const S* src, void* dst, int32_t dst_type, int64_t n, float scale, cudaStream_t s) {
    int dev = 0, sms = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16);
    switch (dst_type) {
        case USTB_STORE_F32: convert_kernel<S, float><<<grid, 256, 0, s>>>(src, (float*)dst, n, scale); break;
        case USTB_STORE_F16: convert_kernel<S, __half><<<grid, 256, 0, s>>>(src, (__half*)dst, n, scale); break;
        default: convert_kernel<S, __nv_bfloat16><<<grid, 256, 0, s>>>(src, (__nv_bfloat16*)dst, n, scale); break;
    }
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}

}  // namespace

extern "C" int ustb_convert_channels(const void* src, int32_t src_type, void* dst, int32_t dst_type,
                                     int64_t count, float scale, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(count >= 0, USTB_E_SHAPE, "negative count");
    USTB_REQUIRE(src_type >= 0 && src_type <= 2, USTB_E_DTYPE, "unknown source type %d", (int)src_type);
    USTB_REQUIRE(dst_type >= 0 && dst_type <= 2, USTB_E_DTYPE, "unknown storage type %d", (int)dst_type);
    if (count == 0) return USTB_OK;
    USTB_REQUIRE(src && dst, USTB_E_ARG, "NULL pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (src_type) {
        case USTB_SRC_F32: return launch_dst((const float*)src, dst, dst_type, count, scale, s);
        case USTB_SRC_I16: return launch_dst((const int16_t*)src, dst, dst_type, count, scale, s);
        default: return launch_dst((const __half*)src, dst, dst_type, count, scale, s);
    }
}
