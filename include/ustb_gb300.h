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
int ustb_abi_version(void); /* 10300: ustb_serve_create_ex; 10200: ustb_das_geometry.stage_shape */

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
 * the kernel, copies the result into `out` and synchronises.  The calling
 * thread's current device is restored before the call returns.  Sizes whose
 * byte counts overflow 64 bits are rejected with USTB_E_SHAPE.
 */
int ustb_das_table_f32_host(const void* ch, int32_t ch_complex, int64_t L, int64_t N, int64_t W,
                            int64_t F, float fs, float t0, const float* apo_tx,
                            const float* apo_rx, const float* delay_tx, const float* delay_rx,
                            int64_t P, float fd, int32_t dimension, void* out, int32_t device);


/*
 * Allocation-free form of ustb_das_table_f32_host.  No counterpart in the
 * reference: das_cuda (+mex/source/das_cuda.cu:190-220) and
 * ustb_das_table_f32_host both obtain device memory per call.
 *
 * For callers that must not allocate device memory while they run.  Examples
 * are acquisition or serving loops with a hard latency budget (cudaMalloc can
 * block and synchronise the device), and host applications that keep a fixed
 * memory budget or let another allocator own the GPU (a MATLAB or PyTorch
 * process with a caching pool), where a fresh cudaMalloc may fail or evict.
 *
 * Same arguments and result as ustb_das_table_f32_host.  The device staging
 * buffers (channel data, the four tables and the output, each rounded up to
 * 256 bytes) come from one static device array of USTB_NOALLOC_SCRATCH_BYTES
 * that every GPU which loads this library holds until the process exits.
 * Requests that need more (including sizes whose byte counts overflow 64 bits)
 * are rejected with USTB_E_SHAPE before any copy.  The call makes no
 * cudaMalloc/cudaFree, uses the per-thread default stream and restores the
 * calling thread's current device before it returns.
 * Its first call on a device looks up the array's device address (set-up, once
 * per device); make that first call before any stream capture on that device.
 * All calls share the one array and nothing in it is cleared (every byte used is
 * rewritten by the call): calls that overlap on the GPU, e.g. from two host
 * threads on one device, race on it and must be serialised by the caller.
 */
#define USTB_NOALLOC_SCRATCH_BYTES (64u << 20)
int ustb_das_table_f32_host_noalloc(const void* ch, int32_t ch_complex, int64_t L, int64_t N,
                                    int64_t W, int64_t F, float fs, float t0, const float* apo_tx,
                                    const float* apo_rx, const float* delay_tx,
                                    const float* delay_rx, int64_t P, float fd, int32_t dimension,
                                    void* out, int32_t device);

/*
 * Per-pixel phase epilogue: data[p + P*j] *= phase[p] for j < rest
 * (interleaved complex single).  Replaces the MATLAB step
 * bf .* exp(-1j*2*w0*scan.reference_distance/c) at +midprocess/das.m:306-309;
 * the caller forms phase[p] from the reference distance in double.
 * Device pointers; stream-ordered.
 */
int ustb_apply_pixel_phase(void* data, int64_t P, int64_t rest, const void* phase, void* stream);

/* ------------------------------------------------------------------------ */
/* Fast path: reduced-precision channel storage, on-the-fly geometry         */
/* ------------------------------------------------------------------------ */

/* Channel-data storage on the device (arithmetic is always single precision). */
enum { USTB_STORE_F32 = 0, USTB_STORE_F16 = 1, USTB_STORE_BF16 = 2 };

/* Source types of ustb_convert_channels. */
enum { USTB_SRC_F32 = 0, USTB_SRC_I16 = 1, USTB_SRC_F16 = 2 };

/* Transmit-delay models of ustb_wave.kind (+midprocess/das.m:110-206). */
enum {
    USTB_WAVE_PLANE = 0,     /* tau = (dir . x)/c - delay                          das.m:193 */
    USTB_WAVE_SPHERICAL = 1, /* tau = (sigma*|x - src| + offset)/c - delay,
                                sigma = -1 where z < src_z                 das.m:120-132 */
    USTB_WAVE_ZERO = 2,      /* tau = -delay (photoacoustic)                    das.m:196-197 */
    USTB_WAVE_TABLE = 3      /* tau read from ustb_das_geometry.tx_delay_table [P,W] */
};

/* One transmit event.  48 bytes, 4-byte aligned members. */
typedef struct {
    int32_t kind;        /* USTB_WAVE_* */
    float dir[3];        /* plane: (sin az cos el, sin el, cos az cos el) */
    float src[3];        /* spherical: virtual source position, m */
    float offset;        /* spherical: -|distance| (diverging) or +distance (focused), m */
    float sound_speed;   /* wave.sound_speed, m/s */
    float delay;         /* wave.delay, s */
    float apodization;   /* constant transmit apodization (when tx_apo_table is NULL) */
    float reserved;
} ustb_wave;

/* Receive window ids (same values as +uff/window.m). */
enum {
    USTB_WIN_NONE = 0, USTB_WIN_BOXCAR = 1, USTB_WIN_HANNING = 2, USTB_WIN_HAMMING = 3,
    USTB_WIN_TUKEY25 = 4, USTB_WIN_TUKEY50 = 5, USTB_WIN_TUKEY75 = 6, USTB_WIN_TRIANGLE = 9
};

/* Pixels per tile of the fast path (one CTA). */
#define USTB_TILE_PIXELS 512

/*
 * Geometry of one beamforming request.  All pointers are device pointers.
 * Pixels are processed in tiles of USTB_TILE_PIXELS: tile_pixels[t][j] is the
 * pixel index handled by lane j of tile t (-1 = idle lane; lane 0 of every tile
 * must be live).  Compact tiles keep each channel/wave sample window short.
 */
typedef struct {
    int64_t n_elements;
    const float* element_xyz;    /* [N][3] m */
    int64_t n_pixels;
    const float* pixel_xyz;      /* [P][3] m */
    int64_t n_tiles;
    const int32_t* tile_pixels;  /* [n_tiles][USTB_TILE_PIXELS] */
    int64_t n_waves;
    const ustb_wave* waves;      /* [W] */
    const float* tx_delay_table; /* [P,W] s for USTB_WAVE_TABLE waves, else NULL */
    const float* tx_apo_table;   /* [P,W] or NULL (then ustb_wave.apodization) */
    const float* rx_apo_table;   /* [P,N] or NULL (then the receive window below) */
    const float* pixel_phase;    /* [P] interleaved complex factor applied to every output, or NULL */
    float fs, t0, fd, sound_speed, lens_delay;
    /* receive apodization, +uff/apodization.m:323-468 (flat probe, no tilt) */
    int32_t rx_window;           /* USTB_WIN_* */
    float rx_f_number[2];
    float rx_min_aperture[2];
    float rx_max_aperture[2];
    int32_t rx_use_origin;       /* 0: aperture centred under each pixel; 1: at rx_origin (sector scans) */
    float rx_origin[3];
    float cf_threshold;          /* coherence factor: elements with rx apodization > this count in M */
    int32_t ctas_per_tile;       /* dimension.both, one launch per request: 1 to 4 CTAs per tile (each
                                    adds its partial sum over an equal part of the tile's work; with 3
                                    or 4 the sums are added in completion order, so repeated runs may
                                    differ in the last bits); 0 = the library picks 2 when there are
                                    fewer than 4 tiles per SM */
    int32_t stage_shape;         /* (channel, wave) pairs per shared-memory stage and loop order:
                                    1 = waves outer, 2 channels x 16 waves (dimension.both / receive);
                                    2 = channels outer, 8 x 4; 3 = channels outer, 16 x 2
                                    (dimension.both / transmit / none); 0 = the library's choice */
} ustb_das_geometry;

/* Outputs of ustb_das_fast (device pointers; unused ones NULL). */
typedef struct {
    void* cube;       /* [P, N|1, W|1, F] per `dimension`: complex single (or real single for RF) */
    void* das;        /* epilogue: [P, F] complex, the channel sum (the dimension.both image) */
    float* cf;        /* epilogue: [P, F] coherence factor |sum s|^2 / (M * sum |s|^2) */
    void* cf_image;   /* epilogue: [P, F] complex, cf * sum s */
    float* sdmas;     /* epilogue: [P, F] ((sum sign(re s) sqrt|re s|)^2 - sum |re s|)/2 */
} ustb_das_outputs;

/* ustb_das_fast flag bits (written to *flags, device memory). */
#define USTB_FLAG_WINDOW_OVERFLOW 1u

/*
 * Delay-and-sum with channel data stored as single, half or bfloat16 and the
 * delays, apodization and phase formed on the fly in single precision (the
 * reference forms them as tables in MATLAB: +midprocess/das.m:91-209, then calls
 * das_c: +mex/source/das_c.cpp:355-409).  Same formula as das_c — validity
 * 0 < n0 < L-1, linear interpolation, exp(i 2 pi fd tau) rotation, tx x rx
 * apodization, summation per `dimension` — with the phase factored per
 * pixel-wave and pixel-channel.  Results are checked against a double-precision
 * oracle of that formula, not bit-for-bit against das_c.
 *
 * ch: [L,N,W,F] of the given storage; complex (interleaved) when is_complex,
 * else real RF (fd must be 0; outputs are then real).
 * epilogue = 1 (dimension.transmit, complex only) also produces the coherence
 * factor (+postprocess/coherence_factor.m:100-135, over channels) and the
 * per-pixel simplified-DMAS value (+postprocess/simplified_delay_multiply_and_sum.m:140-148)
 * without writing the channel cube (out->cube may be NULL).
 * flags: device uint32, cleared by the call; USTB_FLAG_WINDOW_OVERFLOW means a
 * tile was too large for its sample windows (re-plan with smaller tiles).
 * The call first rewrites the channel data as FP32 interpolation entries
 * {x_i, x_(i+1) - x_i} (16 bytes per complex sample, 8 per real one) in a
 * stream-ordered scratch array that the library allocates from its own memory
 * pool and frees before returning (USTB_E_OOM when it does not fit).
 */
int ustb_das_fast(const void* ch, int32_t storage, int32_t is_complex, int64_t L, int64_t N,
                  int64_t W, int64_t F, const ustb_das_geometry* geometry, int32_t dimension,
                  int32_t epilogue, const ustb_das_outputs* out, uint32_t* flags, void* stream);

/*
 * The two halves of ustb_das_fast, for callers that beamform the same channel data
 * more than once (several scans, apodizations or dimension modes on one
 * acquisition) or that own the working memory: ustb_build_entries writes the FP32
 * interpolation entries of ch (ustb_entries_bytes bytes, 16-byte aligned, device)
 * and ustb_das_fast_entries beamforms from them.  Together they give ustb_das_fast's
 * results.  No reference counterpart (das_c reads the samples directly).
 */
int64_t ustb_entries_bytes(int64_t L, int64_t N, int64_t W, int64_t F, int32_t is_complex);
int ustb_build_entries(const void* ch, int32_t storage, int32_t is_complex, int64_t L, int64_t N, int64_t W,
                       int64_t F, void* entries, void* stream);
int ustb_das_fast_entries(const void* entries, int32_t is_complex, int64_t L, int64_t N, int64_t W, int64_t F,
                          const ustb_das_geometry* geometry, int32_t dimension, int32_t epilogue,
                          const ustb_das_outputs* out, uint32_t* flags, void* stream);

/* One request of a persistent batched launch (host struct; pointers inside as
 * for ustb_das_fast). */
typedef struct {
    const void* ch;
    int32_t storage;
    int32_t is_complex;
    int64_t L, N, W, F;
    const ustb_das_geometry* geometry;
    int32_t dimension;
    int32_t epilogue;
    const ustb_das_outputs* out;
} ustb_das_request;

/*
 * Batched, persistent form of ustb_das_fast: every request is cut into
 * (frame, tile) work items and one CTA per SM pulls items from a queue until all
 * are done, so requests of different scans, probes, frame counts and sizes share
 * one launch and balance across the GPU (one launch per kernel variant, i.e. per
 * dimension / real-complex / epilogue combination present).  Each request's
 * entry array (see ustb_das_fast) lives in library scratch until the launches are done.  The
 * reference runs requests one at a time (+midprocess/das.m:77-317,
 * +mex/source/das_cuda.cu:253-283 pipelines only frames).
 * scratch: device memory of at least 8*(n+1) bytes; word 0 receives the
 * USTB_FLAG_* bits of all requests (low 32 bits), words 1.. are queue counters.
 * Stream-ordered; results are as ustb_das_fast gives them for each request.
 */
int ustb_das_fast_batch(const ustb_das_request* reqs, int32_t n, uint64_t* scratch, void* stream);

/*
 * Device bytes that ustb_das_fast_batch_ws needs as workspace for this batch:
 * the FP32 interpolation entries of every request, each on a 256-byte boundary.
 * No reference counterpart (the reference keeps no device working set).
 */
int64_t ustb_das_fast_workspace_bytes(const ustb_das_request* reqs, int32_t n);

/*
 * ustb_das_fast_batch with the entry arrays carved from a caller-owned device
 * workspace (256-byte aligned, at least ustb_das_fast_workspace_bytes bytes)
 * instead of the library's memory pool, so the call performs no stream-ordered
 * allocation: for callers that account device memory themselves (a serving
 * budget) or that record the launch into a CUDA graph.  Same results as
 * ustb_das_fast_batch; USTB_E_SHAPE when the workspace is too small.
 */
int ustb_das_fast_batch_ws(const ustb_das_request* reqs, int32_t n, uint64_t* scratch, void* workspace,
                           int64_t workspace_bytes, void* stream);

/*
 * ustb_das_fast_batch / _ws with a bound on the persistent launch's CTAs:
 * max_ctas > 0 runs at most that many CTAs (one per SM), leaving the other SMs to
 * launches on other streams, e.g. small requests served while a large one runs;
 * 0 = one CTA per SM.  workspace may be NULL (library pool, as
 * ustb_das_fast_batch).  No reference counterpart (the reference serves nothing).
 */
int ustb_das_fast_batch_ex(const ustb_das_request* reqs, int32_t n, uint64_t* scratch, void* workspace,
                           int64_t workspace_bytes, int32_t max_ctas, void* stream);

/* ------------------------------------------------------------------------ */
/* Resident plans and the continuous-batching server                         */
/* ------------------------------------------------------------------------ */

/*
 * A plan keeps one acquisition's geometry on the device -- element and pixel
 * positions, transmit events, optional tables and the tile map -- with the
 * request shape, so every later frame of that acquisition needs only its
 * channel data.  The reference rebuilds its delay and apodization tables on
 * every go() (+midprocess/das.m:91-209) and copies them with each das_cuda call
 * (+mex/source/das_cuda.cu:171-216).  A plan is immutable once created: any
 * number of threads may execute it, or submit it to servers, at the same time.
 */
typedef struct ustb_plan_s* ustb_plan;

typedef struct {
    ustb_das_geometry geometry; /* pointer members are HOST arrays here; ustb_plan_create copies
                                   them to the device.  tile_pixels may be NULL: the library then
                                   tiles the pixels itself (over pixel_grid when it is given) */
    int64_t pixel_grid[3];      /* the pixels' grid, first axis fastest, product n_pixels (e.g.
                                   {N_z, N_x, N_y} of a linear scan, {N_depth, N_azimuth, 1} of a
                                   sector scan); {0, 0, 0}: no grid */
    int64_t L, F;               /* samples per trace, frames per request */
    int32_t storage;            /* USTB_STORE_* of the channel data */
    int32_t is_complex;
    int32_t dimension;          /* USTB_DIM_* */
    int32_t epilogue;           /* as for ustb_das_fast */
} ustb_plan_desc;

/* Copy the geometry to the device and plan its tiles.  Synchronous. */
int ustb_plan_create(const ustb_plan_desc* desc, ustb_plan* plan);
/* The tile map ustb_plan_create would use for this descriptor, planned on the host
 * without a GPU: up to `capacity` tiles of USTB_TILE_PIXELS lanes are written to the
 * host array `tiles` (may be NULL); returns the number of tiles, or -status. */
int64_t ustb_plan_tiles_host(const ustb_plan_desc* desc, int32_t* tiles, int64_t capacity);
/* Free a plan's device memory.  No call that uses the plan may still be in flight. */
int ustb_plan_destroy(ustb_plan plan);
/* Number of tiles of a plan (negative status on a NULL plan). */
int64_t ustb_plan_tiles(ustb_plan plan);
/* ustb_das_fast on the plan's geometry: ch [L,N,W,F] of the plan's storage (device). */
int ustb_plan_execute(ustb_plan plan, const void* ch, const ustb_das_outputs* out, uint32_t* flags,
                      void* stream);

/*
 * Continuous-batching server.  ustb_serve_submit queues one request (a plan, its
 * device channel data and outputs; both must stay valid until the request is
 * done) and returns at once with a ticket.  A request with more than `large_units`
 * pixel x channel x wave x frame units (0: 2e9) is large.  A scheduler thread takes
 * small requests in arrival order into batches whose interpolation entries fit
 * `workspace_budget` bytes (at most `max_batch` requests, at most 40; a request
 * whose entries alone exceed the budget runs alone) and launches each batch as
 * ustb_das_fast_batch_ex, alternating between two streams of its own with a
 * workspace each.  Large requests launch one per batch on a third stream (at most
 * two queued there), so small batches never wait behind a large launch on a stream;
 * ustb_serve_create_ex's `reserve_sms` > 0 also caps a large launch at SMs -
 * reserve_sms persistent CTAs, keeping that many SMs for small batches while it
 * runs (0: a large launch may use every SM, which favours throughput).  One
 * completion thread per class (small, large) waits for its batches and marks their
 * tickets done.  The reference serves no requests: das.m beamforms one call at a
 * time.
 */
typedef struct ustb_server_s* ustb_server;

int ustb_serve_create(int64_t workspace_budget, int32_t max_batch, int64_t large_units, ustb_server* server);
/* ustb_serve_create with SMs kept free of large launches (ABI 10300). */
int ustb_serve_create_ex(int64_t workspace_budget, int32_t max_batch, int64_t large_units, int32_t reserve_sms,
                         ustb_server* server);
int ustb_serve_submit(ustb_server server, ustb_plan plan, const void* ch, const ustb_das_outputs* out,
                      uint64_t* ticket);
/* Wait until the ticket's request is done (timeout_ms < 0: no limit); USTB_E_TIMEOUT
 * if it is not done in time (the ticket stays valid), else the request's status,
 * with its USTB_FLAG_* bits in *flags (may be NULL).  A finished ticket is released. */
int ustb_serve_wait(ustb_server server, uint64_t ticket, int32_t timeout_ms, uint32_t* flags);
/* Finish every queued request, stop the threads and free the server. */
int ustb_serve_destroy(ustb_server server);

/*
 * Convert channel data to a device storage type: count scalars from `src`
 * (USTB_SRC_*) times `scale` into `dst` (USTB_STORE_*), e.g. int16 I/Q scanner
 * samples or complex64 into half.  Device pointers; stream-ordered.
 */
int ustb_convert_channels(const void* src, int32_t src_type, void* dst, int32_t dst_type,
                          int64_t count, float scale, void* stream);

/*
 * RF -> IQ demodulation fused with the conversion into a storage type, for the
 * channel data the fast path consumes (+preprocess/fast_demodulation.m:121-167):
 * iq[t][m] = sum_k taps[k] * scale * rf[t][m*D - k] * exp(-i 2 pi fc (t0 + (m*D - k)/fs))
 * for m < ceil(L/D), rf[t][j] = 0 for j < 0; one down-mix, FIR and decimation pass.
 * rf: n_traces x L samples (USTB_SRC_*); iq: n_traces x ceil(L/D) complex samples
 * of the storage type (USTB_STORE_*), interleaved.  taps: device float[ntaps]
 * (the reference designs them with kaiserord + fir1 'noscale', :286-293).  The
 * caller sets the output's initial time to t0 - (ntaps - 1) / 2 / fs and its
 * sampling frequency to fs / D, as the reference does (:170-175).
 */
int ustb_demodulate(const void* rf, int32_t src_type, void* iq, int32_t dst_type, int64_t L,
                    int64_t n_traces, double fs, double t0, double fc, int32_t decimation,
                    const float* taps, int32_t ntaps, float scale, void* stream);

/*
 * Zero-phase RF -> IQ demodulation of the reference's Python port
 * (python/src/ustb/preprocess/fast_demodulation.py:71-134): mix with
 * exp(-i 2 pi fc (t0 + j/fs)), filter forward and backward with the taps as scipy's
 * filtfilt(b, 1, x) does (odd extension by 3 * ntaps samples at each end,
 * steady-state initial conditions in both passes), then keep every D-th sample from
 * the first; the initial time stays t0.  Arguments and layouts as ustb_demodulate;
 * L must exceed 3 * ntaps (filtfilt's padding), else USTB_E_SHAPE.
 */
int ustb_demodulate_filtfilt(const void* rf, int32_t src_type, void* iq, int32_t dst_type, int64_t L,
                             int64_t n_traces, double fs, double t0, double fc, int32_t decimation,
                             const float* taps, int32_t ntaps, float scale, void* stream);

/*
 * Headless image formation of a sector-scan result: envelope and compression
 * (+uff/beamformed_data.m:300-316 get_image: 0 = log, 20 log10(|b| / max|b|) with the
 * maximum over all frames; 1 = sqrt(|b|); 2 = |b|), then scan conversion onto a
 * uniform Cartesian grid by bilinear interpolation in (azimuth, depth) with -inf
 * outside the sector (+tools/scan_convert.m).  data: [n_depth, n_azimuth, n_frames]
 * (depth fastest) complex or real single; depth/azimuth axes: increasing device
 * float arrays; out: [n_frames][size_x][size_z] floats (z fastest), pixel (ix, iz) at
 * x = x0 + ix*dx, z = z0 + iz*dz.  peak: device float that receives max|b| (log only).
 */
int ustb_scan_convert(const void* data, int32_t is_complex, int32_t compression, int64_t n_depth,
                      int64_t n_azimuth, int64_t n_frames, const float* depth_axis,
                      const float* azimuth_axis, float* peak, float* out, int64_t size_x,
                      int64_t size_z, float x0, float dx, float z0, float dz, void* stream);

/*
 * Coherence factor of a kept cube (+postprocess/coherence_factor.m:100-135): over the
 * channels (dimension USTB_DIM_RECEIVE), the waves (USTB_DIM_TRANSMIT) or both
 * (USTB_DIM_BOTH) of cube [P, N, W, F] (complex single, pixel fastest):
 * cf = |sum s|^2 / sum |s|^2 / M (NaN -> 0) and image = cf * sum s, both [P, J] with J
 * the remaining dimensions in order (W*F, N*F or F).  active_count: [P] counts M (the
 * reference's M = elements with apodization > active_element_criterium), or NULL for
 * M = the number of terms summed (the Python port's rule).  cf or image may be NULL.
 */
int ustb_coherence_factor(const void* cube, int64_t P, int64_t N, int64_t W, int64_t F, int32_t dimension,
                          const float* active_count, float* cf, void* image, void* stream);

/*
 * Phase coherence factor on a kept cube (+postprocess/phase_coherence_factor.m:64-129):
 * cube [F][K][P] complex single (pixel fastest: the channels of a dimension.transmit
 * result, or the waves of a dimension.receive one), weights [K][P] (the apodization
 * of the summed dimension, as MATLAB's [P, K]) or NULL for ones.  Outputs [F][P]
 * (any may be NULL): fca = max(0, 1 - gamma/sigma0 * min(std phase, std shifted
 * phase)), fcc = 1 - sqrt(var cos + var sin) (weighted, tools/weigthed_std.m),
 * image = fcc * sum.  The optional centre-frequency re-phasing of the reference is
 * not applied.
 */
int ustb_phase_coherence(const void* cube, int64_t P, int64_t K, int64_t F, const float* weights,
                         float gamma, float sigma0, float* fca, float* fcc, void* image, void* stream);

/*
 * Generalized coherence factor on a kept cube
 * (+postprocess/generalized_coherence_factor.m:66-97): gcf = energy of the DFT bins
 * [0..M0] and [K-M0..K-1] (only bin 0 when M0 <= 1) over the total energy along the
 * K values of each pixel; image = gcf * sum.  Layout as ustb_phase_coherence.
 */
int ustb_generalized_coherence(const void* cube, int64_t P, int64_t K, int64_t F, int32_t M0, float* gcf,
                               void* image, void* stream);

/*
 * Capon minimum-variance beamforming on a kept cube (+postprocess/capon_minimum_variance.m:117-177),
 * per pixel of an nz x nx grid (depth fastest), over the M channels (or waves) of
 * cube [F][M][nz*nx] complex single: spatial smoothing over subarrays of
 * L = clamp(floor(L_elements/M * active), 1, active - 1) elements spanning the active
 * aperture (|apodization [M][nz*nx]| > criterion), temporal averaging over
 * 2*K_samples + 1 depth samples, diagonal loading regularisation/L * trace R,
 * optional forward-backward averaging; out [F][nz*nx] complex single.  L <= 32.
 */
int ustb_capon(const void* cube, const float* apodization, int64_t nz, int64_t nx, int64_t M, int64_t F,
               float L_elements, int32_t K_samples, float regularisation, float criterion,
               int32_t forward_backward, void* out, void* stream);

/*
 * FIR filter along depth with delay compensation, for the band-pass step of the
 * simplified-DMAS post-process (+postprocess/simplified_delay_multiply_and_sum.m:170-176):
 * out[c][z] = sum_k taps[k] * in[c][z + delay - k], zero outside [0, nz).
 * in/out: ncols columns of nz real samples each (depth fastest).  Device pointers.
 */
int ustb_fir_depth(const float* in, float* out, int64_t nz, int64_t ncols, const float* taps,
                   int32_t ntaps, int32_t delay, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* USTB_GB300_H */
