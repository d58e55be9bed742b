// Shared plumbing for the ustb_gb300 C-ABI: status codes, the thread-local
// error message and argument/CUDA checking helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/ustb_gb300.h"

namespace ustb {

// Thread-local message behind ustb_last_error().
void set_error(const char* fmt, ...);
void clear_error();

// Record a CUDA failure (with the call site) and return USTB_E_CUDA, or
// USTB_E_OOM for allocation failures.
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

}  // namespace ustb

#define USTB_CUDA(call)                                                              \
    do {                                                                             \
        cudaError_t ustb_e_ = (call);                                                \
        if (ustb_e_ != cudaSuccess) return ustb::cuda_fail(ustb_e_, #call, __FILE__, __LINE__); \
    } while (0)

#define USTB_REQUIRE(cond, code, ...)            \
    do {                                         \
        if (!(cond)) {                           \
            ustb::set_error(__VA_ARGS__);        \
            return (code);                       \
        }                                        \
    } while (0)

// Output strides (in elements) of the four `dimension` modes, as laid out by
// das_c (+mex/source/das_c.cpp:324-353): out[p + rx_f*n + w_f*w + f_f*f].
struct OutStrides {
    int64_t rx_f, w_f, f_f;
};

static inline OutStrides out_strides(int dim, int64_t P, int64_t N, int64_t W) {
    switch (dim) {
        case USTB_DIM_NONE: return {P, P * N, P * N * W};
        case USTB_DIM_RECEIVE: return {0, P, P * W};
        case USTB_DIM_TRANSMIT: return {P, 0, P * N};
        default: return {0, 0, P};
    }
}

static inline int64_t out_elems(int dim, int64_t P, int64_t N, int64_t W, int64_t F) {
    switch (dim) {
        case USTB_DIM_NONE: return P * N * W * F;
        case USTB_DIM_RECEIVE: return P * W * F;
        case USTB_DIM_TRANSMIT: return P * N * F;
        default: return P * F;
    }
}
