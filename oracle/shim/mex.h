/*
 * Minimal stand-in for MATLAB's mex.h / matrix.h (interleaved-complex API,
 * -R2018a), sufficient to compile the reference's +mex/source/das_c.cpp
 * unmodified outside MATLAB.  TEST INFRASTRUCTURE ONLY: this header is part of
 * the oracle and is never linked into the product library.
 *
 * Error calls (mexErrMsgIdAndTxt / mexErrMsgTxt) throw a C++ exception that the
 * driver in oracle/ref_driver.cpp turns into a status code, mirroring how a MEX
 * error unwinds back into the MATLAB interpreter.
 */
#ifndef USTB_ORACLE_MEX_SHIM_H
#define USTB_ORACLE_MEX_SHIM_H

#include <cstddef>
#include <cstdarg>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

typedef size_t mwSize;
typedef size_t mwIndex;

typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7, mxINT32_CLASS = 12 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

typedef struct { float real, imag; } mxComplexSingle;

struct mxArray {
    std::vector<mwSize> dims;
    mxClassID cls = mxUNKNOWN_CLASS;
    bool complex_ = false;
    void* data = nullptr;   /* borrowed or owned, see owned */
    bool owned = false;
};

struct MexError : public std::runtime_error {
    std::string id;
    MexError(const std::string& i, const std::string& m) : std::runtime_error(m), id(i) {}
};

static inline std::string ustb_shim_vfmt(const char* fmt, va_list ap) {
    char buf[1024];
    vsnprintf(buf, sizeof buf, fmt, ap);
    return std::string(buf);
}

static inline mwSize mxGetNumberOfDimensions(const mxArray* a) { return a->dims.size(); }
static inline const mwSize* mxGetDimensions(const mxArray* a) { return a->dims.data(); }
static inline bool mxIsDouble(const mxArray* a) { return a->cls == mxDOUBLE_CLASS; }
static inline bool mxIsComplex(const mxArray* a) { return a->complex_; }
static inline void* mxGetData(const mxArray* a) { return a->data; }
static inline size_t mxGetNumberOfElements(const mxArray* a) {
    size_t n = 1;
    for (mwSize d : a->dims) n *= d;
    return n;
}
static inline bool mxIsScalar(const mxArray* a) { return mxGetNumberOfElements(a) == 1; }
static inline mxComplexSingle* mxGetComplexSingles(const mxArray* a) {
    /* MATLAB returns NULL for a real array; keep that behaviour. */
    if (a->cls != mxSINGLE_CLASS || !a->complex_) return nullptr;
    return (mxComplexSingle*)a->data;
}
static inline float* mxGetSingles(const mxArray* a) {
    if (a->cls != mxSINGLE_CLASS || a->complex_) return nullptr;
    return (float*)a->data;
}
static inline int* mxGetInt32s(const mxArray* a) {
    if (a->cls != mxINT32_CLASS) return nullptr;
    return (int*)a->data;
}
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity cplx);

[[noreturn]] static inline void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::string m = ustb_shim_vfmt(fmt, ap);
    va_end(ap);
    throw MexError(id, m);
}
[[noreturn]] static inline void mexErrMsgTxt(const char* msg) { throw MexError("", msg); }
static inline int mexPrintf(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    int r = vprintf(fmt, ap);
    va_end(ap);
    return r;
}
static inline int mexEvalString(const char*) { return 0; }

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);

#endif
