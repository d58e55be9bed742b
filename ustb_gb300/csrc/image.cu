// Image formation after the beamformer, headless: envelope, compression and scan
// conversion of a sector-scan image into a Cartesian device buffer.
//
//   compression (+uff/beamformed_data.m:300-316, get_image):
//     log   20 log10(|b| / max|b|)   (max over every pixel of every frame)
//     sqrt  sqrt(|b|)
//     abs   |b|
//   scan conversion (+tools/scan_convert.m): the compressed image on its
//   (depth, azimuth) grid is interpolated bilinearly in (azimuth, depth) at
//   theta = atan2(x, z), r = hypot(x, z) of every pixel of a uniform (x, z) grid;
//   pixels outside the sector get -inf (interp2's extrapolation value there).
//
// Both passes are HBM-bound and small: a max reduction (log only) and one thread
// per output pixel that reads its 4 neighbours.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace {

__device__ __forceinline__ float mag(const void* data, int cplx, int64_t i) {
    if (cplx) {
        const float2 v = __ldg(reinterpret_cast<const float2*>(data) + i);
        return hypotf(v.x, v.y);
    }
    return fabsf(__ldg(reinterpret_cast<const float*>(data) + i));
}

// max |b| over n values into *peak (non-negative floats order like their bits)
__global__ void peak_kernel(const void* data, int cplx, int64_t n, float* peak) {
    float m = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, mag(data, cplx, i));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int*>(peak), __float_as_int(m));
}

__device__ __forceinline__ float compress(float a, int mode, float inv_peak) {
    if (mode == 0) return 20.f * log10f(a * inv_peak);
    if (mode == 1) return sqrtf(a);
    return a;
}

// index i with axis[i] <= v <= axis[i + 1] of an increasing axis, or -1 outside
__device__ __forceinline__ int bracket(const float* axis, int n, float v) {
    if (!(v >= axis[0] && v <= axis[n - 1]) || n < 2) return -1;
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (axis[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

struct ConvArgs {
    int64_t nd, na, F, sx, sz;
    float x0, dx, z0, dz;
    int cplx, mode;
};

__global__ void scan_convert_kernel(const void* data, const float* depth, const float* azim, const float* peak,
                                    float* out, const ConvArgs a) {
    const int64_t total = a.F * a.sx * a.sz;
    const float inv_peak = (a.mode == 0) ? 1.f / __ldg(peak) : 1.f;
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < total; o += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = o / (a.sx * a.sz);
        const int64_t rem = o - f * a.sx * a.sz;
        const int64_t ix = rem / a.sz, iz = rem - ix * a.sz;  // z fastest, as MATLAB's [sizeZ, sizeX]
        const float x = a.x0 + a.dx * (float)ix, z = a.z0 + a.dz * (float)iz;
        const float th = atan2f(x, z), r = hypotf(x, z);
        const int i = bracket(depth, (int)a.nd, r), j = bracket(azim, (int)a.na, th);
        float v = -INFINITY;
        if (i >= 0 && j >= 0) {
            const float u = (r - depth[i]) / (depth[i + 1] - depth[i]);
            const float w = (th - azim[j]) / (azim[j + 1] - azim[j]);
            const int64_t b = f * a.nd * a.na;
            const float v00 = compress(mag(data, a.cplx, b + j * a.nd + i), a.mode, inv_peak);
            const float v10 = compress(mag(data, a.cplx, b + j * a.nd + i + 1), a.mode, inv_peak);
            const float v01 = compress(mag(data, a.cplx, b + (j + 1) * a.nd + i), a.mode, inv_peak);
            const float v11 = compress(mag(data, a.cplx, b + (j + 1) * a.nd + i + 1), a.mode, inv_peak);
            v = (1.f - u) * ((1.f - w) * v00 + w * v01) + u * ((1.f - w) * v10 + w * v11);
        }
        out[o] = v;
    }
}

}  // namespace

extern "C" int ustb_scan_convert(const void* data, int32_t is_complex, int32_t compression, int64_t n_depth,
                                 int64_t n_azimuth, int64_t n_frames, const float* depth_axis,
                                 const float* azimuth_axis, float* peak, float* out, int64_t size_x,
                                 int64_t size_z, float x0, float dx, float z0, float dz, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(compression >= 0 && compression <= 2, USTB_E_ARG, "compression must be 0 (log), 1 (sqrt) or 2 (abs)");
    USTB_REQUIRE(n_depth >= 2 && n_azimuth >= 2 && n_frames >= 0 && size_x >= 0 && size_z >= 0, USTB_E_SHAPE,
                 "need at least 2 depths and 2 azimuths");
    USTB_REQUIRE(n_depth < INT32_MAX && n_azimuth < INT32_MAX, USTB_E_SHAPE, "axes too long");
    const int64_t total = n_frames * size_x * size_z;
    if (total == 0) return USTB_OK;
    USTB_REQUIRE(data && depth_axis && azimuth_axis && out && (compression != 0 || peak), USTB_E_ARG, "NULL pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (compression == 0) {
        const int64_t n = n_depth * n_azimuth * n_frames;
        USTB_CUDA(cudaMemsetAsync(peak, 0, sizeof(float), s));
        const unsigned g = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)sms * 8);
        peak_kernel<<<g, 256, 0, s>>>(data, is_complex ? 1 : 0, n, peak);
        USTB_CUDA(cudaGetLastError());
    }
    ConvArgs a;
    a.nd = n_depth; a.na = n_azimuth; a.F = n_frames; a.sx = size_x; a.sz = size_z;
    a.x0 = x0; a.dx = dx; a.z0 = z0; a.dz = dz;
    a.cplx = is_complex ? 1 : 0;
    a.mode = compression;
    const unsigned g = (unsigned)std::min<int64_t>((total + 255) / 256, (int64_t)sms * 16);
    scan_convert_kernel<<<g, 256, 0, s>>>(data, depth_axis, azimuth_axis, peak, out, a);
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}
