/*
 * C-ABI driver around a MEX function with das_c's argument layout: the
 * reference's own das_c (+mex/source/das_c.cpp, compiled unmodified against
 * oracle/shim/), or — compiled with -DMEX_RUN_NAME=... by the tests — the
 * product's MEX gateway, so that the MATLAB boundary is exercised without MATLAB.
 * TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/libdas_c_ref.so, which the
 * tests use to pin the oracle port and to make golden fixtures, and (with
 * -DMEX_GPU_ID, around the reference's das_cuda) into oracle/_ref/libdas_cuda_ref.so,
 * which the reference arm of bench.py times.  The product library never links or
 * loads either.
 *
 * das_c_ref_run() wraps caller buffers in mxArrays with das.m's argument layout
 * (das.m:251-259): ch [L,N,W,F] complex single, fs, t0 (single scalars),
 * apo_tx [P,W], apo_rx [P,N], delay_tx [P,W], delay_rx [P,N] (single),
 * fd (single scalar), int32 dimension.  The output is copied into `out`
 * (interleaved complex single, [P, N|1, W|1, F]).  Returns 0, or 1 with the
 * MEX error id and message in errbuf.
 */
#include "mex.h"

#include <cstdint>
#include <cstdlib>
#include <cstring>

mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity cplx) {
    mxArray* a = new mxArray();
    a->dims.assign(dims, dims + ndim);
    a->cls = cls;
    a->complex_ = (cplx == mxCOMPLEX);
    size_t el = (cls == mxDOUBLE_CLASS) ? 8 : 4;
    if (a->complex_) el *= 2;
    a->data = std::calloc(mxGetNumberOfElements(a) ? mxGetNumberOfElements(a) : 1, el);
    a->owned = true;
    return a;
}

static void destroy(mxArray* a) {
    if (!a) return;
    if (a->owned) std::free(a->data);
    delete a;
}

static mxArray wrap(void* data, std::initializer_list<mwSize> dims, mxClassID cls, bool cplx) {
    mxArray a;
    a.dims.assign(dims.begin(), dims.end());
    a.cls = cls;
    a.complex_ = cplx;
    a.data = data;
    a.owned = false;
    return a;
}

#ifndef MEX_RUN_NAME
#define MEX_RUN_NAME das_c_ref_run
#endif

// With -DMEX_GPU_ID the MEX function takes das_cuda's tenth argument, int32 gpu_id
// (das.m:262-271), passed as `gpu` (the reference's +mex/source/das_cuda.cu).
#ifdef MEX_GPU_ID
#define USTB_GPU_PARAM , int32_t gpu
#define USTB_NRHS 10
#else
#define USTB_GPU_PARAM
#define USTB_NRHS 9
#endif

extern "C" int MEX_RUN_NAME(const float* ch, int64_t L, int64_t N, int64_t W, int64_t F,
                             float fs, float t0, const float* apo_tx, const float* apo_rx,
                             const float* delay_tx, const float* delay_rx, int64_t P, float fd,
                             int32_t dim, float* out, char* errbuf, int errlen USTB_GPU_PARAM) {
    mxArray m_ch = wrap((void*)ch, {(mwSize)L, (mwSize)N, (mwSize)W, (mwSize)F}, mxSINGLE_CLASS, true);
    mxArray m_fs = wrap(&fs, {1, 1}, mxSINGLE_CLASS, false);
    mxArray m_t0 = wrap(&t0, {1, 1}, mxSINGLE_CLASS, false);
    mxArray m_atx = wrap((void*)apo_tx, {(mwSize)P, (mwSize)W}, mxSINGLE_CLASS, false);
    mxArray m_arx = wrap((void*)apo_rx, {(mwSize)P, (mwSize)N}, mxSINGLE_CLASS, false);
    mxArray m_dtx = wrap((void*)delay_tx, {(mwSize)P, (mwSize)W}, mxSINGLE_CLASS, false);
    mxArray m_drx = wrap((void*)delay_rx, {(mwSize)P, (mwSize)N}, mxSINGLE_CLASS, false);
    mxArray m_fd = wrap(&fd, {1, 1}, mxSINGLE_CLASS, false);
    mxArray m_dim = wrap(&dim, {1, 1}, mxINT32_CLASS, false);
#ifdef MEX_GPU_ID
    mxArray m_gpu = wrap(&gpu, {1, 1}, mxINT32_CLASS, false);
    const mxArray* prhs[USTB_NRHS] = {&m_ch, &m_fs, &m_t0, &m_atx, &m_arx, &m_dtx, &m_drx, &m_fd, &m_dim, &m_gpu};
#else
    const mxArray* prhs[USTB_NRHS] = {&m_ch, &m_fs, &m_t0, &m_atx, &m_arx, &m_dtx, &m_drx, &m_fd, &m_dim};
#endif
    mxArray* plhs[1] = {nullptr};
    try {
        mexFunction(1, plhs, USTB_NRHS, prhs);
    } catch (const MexError& e) {
        if (errbuf && errlen > 0) std::snprintf(errbuf, errlen, "%s: %s", e.id.c_str(), e.what());
        destroy(plhs[0]);
        return 1;
    }
    std::memcpy(out, plhs[0]->data, mxGetNumberOfElements(plhs[0]) * 2 * sizeof(float));
    destroy(plhs[0]);
    return 0;
}
