/*
 * ustb_gb300 — C-ABI of the GB300 (sm_103a) delay-and-sum beamformer that
 * drops in behind USTB's midprocess.das.
 *
 * Conventions
 *  - Every entry point returns an int status (USTB_OK = 0); on failure the
 *    calling thread's message is available from ustb_last_error().
 *  - Arrays use MATLAB's column-major layout (first index fastest), exactly as
 *    das.m hands them to the MEX call (+midprocess/das.m:251-259):
 *      channel data  [L samples, N channels, W waves, F frames]
 *      tx tables     [P pixels, W waves]      (delay in s, apodization)
 *      rx tables     [P pixels, N channels]
 *      output        [P, N|1, W|1, F]  (which dims are kept follows `dimension`)
 *    Complex data is interleaved (re, im) single precision, like
 *    mxGetComplexSingles.
 *  - "Device" entry points take device pointers and a cudaStream_t (passed as
 *    void*, NULL = legacy default stream); they are asynchronous with respect to
 *    the host and stream-ordered.  "_host" entry points take host pointers,
 *    copy in and out themselves and return after the result is in host memory.
 *  - The caller owns every buffer.  No entry point keeps a pointer after it
 *    returns (plans excepted, see ustb_plan_*).
 */
#ifndef USTB_GB300_H
#define USTB_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The MEX gateway maps them to "Toolbox:SRP_SRC:<kind>" error
 * ids, the prefix das_c uses (+mex/source/das_c.cpp:53-252). */
enum {
    USTB_OK = 0,
    USTB_E_ARG = 1,      /* bad scalar argument or enum value */
    USTB_E_SHAPE = 2,    /* inconsistent array sizes */
    USTB_E_DTYPE = 3,    /* unsupported element type / real-vs-complex mismatch */
    USTB_E_CUDA = 4,     /* a CUDA runtime call failed */
    USTB_E_OOM = 5,      /* device memory could not be obtained */
    USTB_E_TIMEOUT = 6,  /* a bounded device-side wait gave up */
    USTB_E_OVERFLOW = 7, /* a tile's sample window did not fit its stage slot */
    USTB_E_BUSY = 8      /* a plan/server slot is in use */
};

/* `dimension` enum, same int32 values as USTB's dimension.m:27-32. */
enum { USTB_DIM_NONE = 0, USTB_DIM_RECEIVE = 1, USTB_DIM_TRANSMIT = 2, USTB_DIM_BOTH = 3 };

/* Thread-local description of the last failure on this thread ("" if none). */
const char* ustb_last_error(void);

/* ABI version of this library (major*10000 + minor*100 + patch). */
int ustb_abi_version(void);

/*
 * Plain single-precision DAS on precomputed delay/apodization tables: the
 * das_c drop-in.
 *
 * Replaces: mex.das_c(ch_data, fs, t0, apoTx, apoRx, dTx, dRx, fd, int32(dim))
 *   called at +midprocess/das.m:251-259 and implemented by
 *   +mex/source/das_c.cpp:46-418 (the hot loop is :355-409).
 * Semantics follow das_c: units with a zero tx or rx apodization are skipped,
 * delay = dTx + dRx, s = (delay - t0)*fs, n0 = trunc(s), valid iff
 * 0 < n0 < L-1, linear interpolation between samples n0 and n0+1, phase
 * rotation exp(i*2*pi*fd*delay) when |fd| > 1e-6, apodization dTx*dRx weight,
 * summation per `dimension`.  Every output element is written (das_c's output is
 * zero-initialised), so `out` need not be cleared.
 *
 * ch_complex = 1: `ch` holds interleaved complex single samples and `out` is
 *   interleaved complex single.
 * ch_complex = 0: `ch` holds real single samples (RF), fd must be 0, and `out`
 *   is real single; it equals real(das_c(hilbert(rf))) as das.m computes for
 *   RF input (+midprocess/das.m:211-214).
 * Device pointers; stream-ordered on `stream`.
 */
int ustb_das_table_f32(const void* ch, int32_t ch_complex, int64_t L, int64_t N, int64_t W,
                       int64_t F, float fs, float t0, const float* apo_tx, const float* apo_rx,
                       const float* delay_tx, const float* delay_rx, int64_t P, float fd,
                       int32_t dimension, void* out, void* stream);

/*
 * Host-pointer form of ustb_das_table_f32 (the MEX gateway's call).
 * Replaces the same das.m:251-259 call, and das.m:262-271 (mex.das_cuda with
 * int32 gpu_id) when `device` is given.  Copies the inputs to `device`, runs
 * the kernel, copies the result into `out` and synchronises.
 */
int ustb_das_table_f32_host(const void* ch, int32_t ch_complex, int64_t L, int64_t N, int64_t W,
                            int64_t F, float fs, float t0, const float* apo_tx,
                            const float* apo_rx, const float* delay_tx, const float* delay_rx,
                            int64_t P, float fd, int32_t dimension, void* out, int32_t device);


/*
 * Per-pixel phase epilogue: data[p + P*j] *= phase[p] for j < rest
 * (interleaved complex single).  Replaces the MATLAB step
 * bf .* exp(-1j*2*w0*scan.reference_distance/c) at +midprocess/das.m:306-309;
 * the caller forms phase[p] from the reference distance in double.
 * Device pointers; stream-ordered.
 */
int ustb_apply_pixel_phase(void* data, int64_t P, int64_t rest, const void* phase, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* USTB_GB300_H */
