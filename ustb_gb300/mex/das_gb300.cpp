/*
 * MATLAB MEX gateway: das_gb300(ch_data, fs, t0, apoTx, apoRx, dTx, dRx, fd, int32 dim [, int32 gpu_id])
 *
 * Drop-in for mex.das_c / mex.das_cuda as called by +midprocess/das.m:251-271:
 * same right-hand sides (prhs[0..8]), optional prhs[9] = gpu_id (das_cuda's
 * extra argument, default 0), one output: complex single [P, N|1, W|1, F]
 * (real single for real RF input).  Argument checks follow das_c
 * (+mex/source/das_c.cpp:52-252) and raise the same "Toolbox:SRP_SRC:*" ids;
 * failures inside the library are raised as Toolbox:SRP_SRC:<status>.
 *
 * Build in MATLAB (R2018a interleaved-complex API), with the library built by
 * `python -m ustb_gb300.build`:
 *   mex -R2018a -I<repo>/include das_gb300.cpp -L<repo>/ustb_gb300 -lustb_gb300
 */
#include <mex.h>

#include <cmath>
#include <cstdint>

#include "ustb_gb300.h"

#define M_P prhs[0]
#define M_FS prhs[1]
#define M_T0 prhs[2]
#define M_APO_TX prhs[3]
#define M_APO_RX prhs[4]
#define M_DELAY_TX prhs[5]
#define M_DELAY_RX prhs[6]
#define M_FD prhs[7]
#define M_SUM prhs[8]
#define M_GPU prhs[9]

static const char* status_id(int rc) {
    switch (rc) {
        case USTB_E_ARG: return "Toolbox:SRP_SRC:Argument";
        case USTB_E_SHAPE: return "Toolbox:SRP_SRC:Dimensions";
        case USTB_E_DTYPE: return "Toolbox:SRP_SRC:Type";
        case USTB_E_OOM: return "Toolbox:SRP_SRC:Memory";
        default: return "Toolbox:SRP_SRC:GPU";
    }
}

static void table_dims(const mxArray* a, const char* what, mwSize& rows, mwSize& cols) {
    if (mxGetNumberOfDimensions(a) > 2)
        mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Dimensions", "Unknown %s format. Expected 2 dimensions", what);
    if (mxIsDouble(a) || mxIsComplex(a))
        mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Type", "The %s should be real single precision", what);
    const mwSize* d = mxGetDimensions(a);
    rows = d[0];
    cols = mxGetNumberOfDimensions(a) == 2 ? d[1] : 1;
}

static float scalar(const mxArray* a, const char* what) {
    if (mxGetNumberOfElements(a) != 1) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Argument", "The %s should be an escalar", what);
    if (mxIsDouble(a)) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Type", "The %s should be single precision", what);
    return *static_cast<const float*>(mxGetData(a));
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
    if (nrhs < 9) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:nrhs", "Too few input arguments");
    if (nrhs > 10) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:nrhs", "Too many input arguments");
    if (nlhs > 1) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:nlhs", "Too many output arguments");

    const int dim = *static_cast<const int*>(mxGetData(M_SUM));
    if (dim < 0 || dim > 3) mexErrMsgTxt("Unknown sum mode. Available: 0 -> NONE, 1->RX, 2->TX, 3->BOTH");
    const int gpu = nrhs == 10 ? *static_cast<const int*>(mxGetData(M_GPU)) : 0;

    const int ndim = (int)mxGetNumberOfDimensions(M_P);
    if (ndim < 2 || ndim > 4)
        mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Dimensions",
                          "Unknown channel data format. Expected from 2 to 4 dimensions: [time, channel, wave, frame]");
    if (mxIsDouble(M_P)) mexErrMsgTxt("The channel data should be single precision");
    const mwSize* pd = mxGetDimensions(M_P);
    const int64_t L = (int64_t)pd[0], N = (int64_t)pd[1];
    const int64_t W = ndim > 2 ? (int64_t)pd[2] : 1, F = ndim > 3 ? (int64_t)pd[3] : 1;
    const bool cplx = mxIsComplex(M_P);

    mwSize P, Wc, P2, Nc, P3, Wa, P4, Na;
    table_dims(M_DELAY_TX, "transmit delay", P, Wc);
    if ((int64_t)Wc != W) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Dimensions", "Number of waves in channel data & transmit delays do not match.");
    table_dims(M_DELAY_RX, "receive delay", P2, Nc);
    if (P2 != P) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Dimensions", "Number of pixels in transmit and receive delays do not match.");
    if ((int64_t)Nc != N) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Dimensions", "Number of channels in channel data & receive delays do not match.");
    table_dims(M_APO_TX, "transmit apodization", P3, Wa);
    if (P3 != P) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Dimensions", "Number of pixels in transmit apodization and transmit delays do not match.");
    if ((int64_t)Wa != W) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Dimensions", "Number of waves in channel data & transmit apodization do not match.");
    table_dims(M_APO_RX, "receive apodization", P4, Na);
    if (P4 != P) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Dimensions", "Number of pixels in receive apodization and receive delays do not match.");
    if ((int64_t)Na != N) mexErrMsgIdAndTxt("Toolbox:SRP_SRC:Dimensions", "Number of channels in channel data & receive apodization do not match.");

    const float fs = scalar(M_FS, "sampling frequency");
    const float t0 = scalar(M_T0, "initial time");
    const float fd = scalar(M_FD, "modulation frequency");
    if (std::fabs(fd) > 1e-6f && !cplx)
        mexErrMsgTxt("The modulation frequency > 0 but the input data is real. Check inputs.");

    mwSize out_size[4] = {P, (dim == USTB_DIM_NONE || dim == USTB_DIM_TRANSMIT) ? (mwSize)N : 1,
                          (dim == USTB_DIM_NONE || dim == USTB_DIM_RECEIVE) ? (mwSize)W : 1, (mwSize)F};
    plhs[0] = mxCreateNumericArray(4, out_size, mxSINGLE_CLASS, cplx ? mxCOMPLEX : mxREAL);
    void* out = mxGetData(plhs[0]);

    const int rc = ustb_das_table_f32_host(mxGetData(M_P), cplx ? 1 : 0, L, N, W, F, fs, t0,
                                           static_cast<const float*>(mxGetData(M_APO_TX)),
                                           static_cast<const float*>(mxGetData(M_APO_RX)),
                                           static_cast<const float*>(mxGetData(M_DELAY_TX)),
                                           static_cast<const float*>(mxGetData(M_DELAY_RX)), (int64_t)P, fd,
                                           dim, out, gpu);
    if (rc != USTB_OK) mexErrMsgIdAndTxt(status_id(rc), "%s", ustb_last_error());
}
