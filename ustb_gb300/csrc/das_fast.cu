// Fast delay-and-sum: reduced-precision channel storage, geometry formed on the
// fly, factored phase, sample windows staged in shared memory.
//
// Same formula as the reference's das_c (+mex/source/das_c.cpp:355-409), with
// the tables das.m builds in MATLAB (+midprocess/das.m:91-209) computed per
// pixel-channel and pixel-wave in registers:
//
//   y = sum_w sum_n  A_w(p) * B_n(p) * lerp(x_{n,w}, s_tx(p,w) + s_rx(p,n))
//   A_w = apo_tx * exp(i 2 pi fd tau_tx),  B_n = apo_rx * exp(i 2 pi fd tau_rx)
//
// One CTA beamforms a tile of 512 pixels (one per thread) for one frame.  The
// (channel, wave) pairs are processed in stages of CG x KW = 32 slots; for each
// pair the tile needs a short window of samples starting at i0 = base_n + base_w,
// where base_n / base_w are integer lower bounds of the tile's receive / transmit
// delays (in samples) derived from the tile's bounding box.
//
// A pre-pass (build_entries_kernel) rewrites the channel data, whatever its
// storage type, as FP32 interpolation entries {x_i, x_{i+1} - x_i} with das_c's
// validity rule (0 < i < L-1) folded in as zero entries.  A stage's windows are
// then plain runs of 16-byte (complex) or 8-byte (real) entries that the CTA
// copies with cp.async into one of two shared-memory buffers while it computes
// the stage before; no per-sample work is left in the staging.  A unit costs:
//   s = s_tx_loc + s_rx_loc; j = floor(s); b = s - j; e = slot[j];
//   v = e.x + b*e.d;  acc += weight * v.
// Delays relative to the tile bases stay below 80 samples, so j and b keep
// full sub-sample precision in FP32.
//
// Loop orders: waves outer / channels inner for dimension.both and .receive
// (rx weight per unit, tx weight once per wave chunk); channels outer / waves
// inner for .transmit and .none (tx weight per unit).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "phasor.cuh"

namespace {

constexpr int kTile = USTB_TILE_PIXELS;
constexpr int kSlot = 160;                      // entries per (channel, wave) window
constexpr int kRing = 2;                        // stage buffers: stage s + kRing - 1 is copied during stage s
constexpr float kHalf = (float)(kSlot / 2 - 1);  // max relative delay of each component
constexpr float kMagic = 8388608.0f;            // 2^23: floor via round-toward-zero add
constexpr int kMagicBits = 0x4B000000;
constexpr int kBothShape = 1;                   // dimension.both: channels outer, 8 x 4 stages

struct Params {
    const void* entries;  // [F][W][N][Lp] interpolation entries (float4 complex, float2 real)
    int64_t L, Lp, N, W, F, P;
    const float* el;
    const float* px;
    const int32_t* tiles;
    int64_t n_tiles;
    const ustb_wave* waves;
    const float* tx_delay_tab;
    const float* tx_apo_tab;
    const float* rx_apo_tab;
    const float2* pix_phase;
    float fs, t0, fd, inv_c, lens;
    int rx_window;
    float win_r1, win_a, win_e, win_b, win_c, win_d;  // see window_coeffs()
    float fnx, fny, minx, miny, maxx, maxy;
    int rx_origin;
    float ox, oy, oz;
    float cf_thr;
    void* cube;
    float2* o_das;
    float* o_cf;
    float2* o_cfimg;
    float* o_sdmas;
    int64_t rx_f, w_f, f_f;
    uint32_t* flags;
    int split;  // grid kernel, dimension.both: CTAs per tile (parts of the stage list, 1-4); 0 = auto
    int shape;  // stage shape (Shape<> index)
    int fpi;    // persistent kernel: frames per work item (one tile, consecutive frames)
};

// ---------------------------------------------------------------------------
// apodization windows, +uff/apodization.m:172-223 (0 beyond ratio 1/2)
//
// Every window has the form
//   w(r) = 1                                  for r <= r1
//        = a + e*r + b*cos(c*(r - d))          for r1 < r <= 1/2
//        = 0                                   beyond
// with per-window constants (window_coeffs), so the kernel evaluates it without
// branching on the window type:
//   boxcar    r1 = 1/2
//   hanning   r1 = -1, a = b = 1/2, c = 2*pi, d = 0
//   hamming   r1 = -1, a = 0.53836, b = 0.46164, c = 2*pi, d = 0
//   tukey(R)  r1 = (1-R)/2, a = b = 1/2, c = 2*pi/R, d = R/2 + 1/2
//   triangle  r1 = -1, a = 1, e = -2
// (Tukey's strict r < 1/2 edge gives the same value, 0, at r = 1/2.)
// ---------------------------------------------------------------------------
struct WinCoeffs {
    float r1, a, e, b, c, d;
};

static WinCoeffs window_coeffs(int win) {
    const float twopi = 6.283185307179586f;
    switch (win) {
        case USTB_WIN_BOXCAR: return {0.5f, 0.f, 0.f, 0.f, 0.f, 0.f};
        case USTB_WIN_HANNING: return {-1.f, 0.5f, 0.f, 0.5f, twopi, 0.f};
        case USTB_WIN_HAMMING: return {-1.f, 0.53836f, 0.f, 0.46164f, twopi, 0.f};
        case USTB_WIN_TUKEY25: return {0.375f, 0.5f, 0.f, 0.5f, twopi / 0.25f, 0.625f};
        case USTB_WIN_TUKEY50: return {0.25f, 0.5f, 0.f, 0.5f, twopi / 0.5f, 0.75f};
        case USTB_WIN_TUKEY75: return {0.125f, 0.5f, 0.f, 0.5f, twopi / 0.75f, 0.875f};
        case USTB_WIN_TRIANGLE: return {-1.f, 1.f, -2.f, 0.f, 0.f, 0.f};
        default: return {3.4e38f, 0.f, 0.f, 0.f, 0.f, 0.f};  // none: 1 everywhere
    }
}

__device__ __forceinline__ float window(const Params& A, float r) {
    const float taper = fmaf(A.win_e, r, A.win_a) + A.win_b * __cosf(A.win_c * (r - A.win_d));
    const float w = r <= 0.5f ? taper : 0.f;
    return r <= A.win_r1 ? 1.f : w;  // NaN ratios (0/0) give 0
}

__device__ __forceinline__ float msign(float v) { return (float)((v > 0.f) - (v < 0.f)); }

// min/max aperture clamps of apodization.m:452-462 (MATLAB sign(0) = 0)
__device__ __forceinline__ float clamp_ap(float z, float fnum, float minap, float maxap) {
    const float a = fminf(fmaxf(fabsf(z), minap * fnum), maxap * fnum);
    return copysignf(a, z) * (z != 0.f ? 1.f : 0.f);
}

__device__ __forceinline__ float rx_apodization(const Params& A, float ex, float ey, float ez, float px,
                                                float py, float pz) {
    if (A.rx_window == USTB_WIN_NONE) return 1.f;
    float xd, yd, zd;
    if (A.rx_origin) {
        xd = ex - A.ox;
        yd = ey - A.oy;
        const float qx = px - A.ox, qy = py - A.oy, qz = pz - A.oz;
        zd = sqrtf(qx * qx + qy * qy + qz * qz);
    } else {
        xd = px - ex;
        yd = py - ey;
        zd = pz - ez;
    }
    const float zx = clamp_ap(zd, A.fnx, A.minx, A.maxx);
    const float rt = fabsf(A.fnx * __fdividef(xd, zx));
    const float wx = window(A, rt);
    if (yd == 0.f) return wx;  // elevation ratio 0: every window is 1 there
    const float zy = clamp_ap(zd, A.fny, A.miny, A.maxy);
    const float rp = fabsf(A.fny * __fdividef(yd, zy));
    return wx * window(A, rp);
}

// exp(i 2 pi fd tau) from the phase in cycles
__device__ __forceinline__ float2 phasor_cycles(float cyc) {
    const float k = rintf(cyc);
    const float fr = cyc - k;  // exact for |cyc| < 2^22
    float s, c;
    __sincosf(6.283185307179586f * fr, &s, &c);
    return make_float2(c, s);
}

struct Box {
    float lo[3], hi[3];
};

__device__ __forceinline__ void dist_range(const Box& b, float x, float y, float z, float& dmin, float& dmax) {
    const float q[3] = {x, y, z};
    float n2 = 0.f, f2 = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float dl = b.lo[i] - q[i], dh = q[i] - b.hi[i];
        const float dn = fmaxf(0.f, fmaxf(dl, dh));
        const float df = fmaxf(fabsf(q[i] - b.lo[i]), fabsf(q[i] - b.hi[i]));
        n2 += dn * dn;
        f2 += df * df;
    }
    dmin = sqrtf(n2);
    dmax = sqrtf(f2);
}

// lower / upper bound of a wave's transmit delay (s) over the tile box
__device__ __forceinline__ void tx_tau_range(const ustb_wave& wv, const Box& b, float& lo, float& hi) {
    switch (wv.kind) {
        case USTB_WAVE_PLANE: {
            float mn = 0.f, mx = 0.f;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float u = wv.dir[i] * b.lo[i], v = wv.dir[i] * b.hi[i];
                mn += fminf(u, v);
                mx += fmaxf(u, v);
            }
            lo = mn / wv.sound_speed - wv.delay;
            hi = mx / wv.sound_speed - wv.delay;
            return;
        }
        case USTB_WAVE_SPHERICAL: {
            float dmin, dmax;
            dist_range(b, wv.src[0], wv.src[1], wv.src[2], dmin, dmax);
            float vlo, vhi;
            if (b.lo[2] >= wv.src[2]) { vlo = dmin; vhi = dmax; }
            else if (b.hi[2] < wv.src[2]) { vlo = -dmax; vhi = -dmin; }
            else { vlo = -dmax; vhi = dmax; }
            lo = (vlo + wv.offset) / wv.sound_speed - wv.delay;
            hi = (vhi + wv.offset) / wv.sound_speed - wv.delay;
            return;
        }
        default:
            lo = hi = -wv.delay;
            return;
    }
}

// block-wide min/max of one float (all threads call; result broadcast)
__device__ __forceinline__ float2 block_minmax(float vmin, float vmax, float2* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
        vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[warp] = make_float2(vmin, vmax);
    __syncthreads();
    float2 r = red[0];
#pragma unroll
    for (int i = 1; i < kTile / 32; ++i) {
        r.x = fminf(r.x, red[i].x);
        r.y = fmaxf(r.y, red[i].y);
    }
    return r;
}

template <bool CPLX>
struct EntryT { using type = float4; };
template <>
struct EntryT<false> { using type = float2; };

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// one stored sample (global memory) as float2
template <int ST, bool CPLX>
__device__ __forceinline__ float2 load_sample(const void* ch, int64_t i) {
    if constexpr (CPLX) {
        if constexpr (ST == USTB_STORE_F32) return __ldg(reinterpret_cast<const float2*>(ch) + i);
        else if constexpr (ST == USTB_STORE_F16) return __half22float2(reinterpret_cast<const __half2*>(ch)[i]);
        else return __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(ch)[i]);
    } else {
        if constexpr (ST == USTB_STORE_F32) return make_float2(__ldg(reinterpret_cast<const float*>(ch) + i), 0.f);
        else if constexpr (ST == USTB_STORE_F16) return make_float2(__half2float(reinterpret_cast<const __half*>(ch)[i]), 0.f);
        else return make_float2(__bfloat162float(reinterpret_cast<const __nv_bfloat16*>(ch)[i]), 0.f);
    }
}

// Interpolation entries of every trace: E[t][i] = {x_i, x_{i+1} - x_i} for
// 0 < i < L-1 (das_c.cpp:381-383's validity rule), zero elsewhere.  HBM-bound:
// one pass over the channel data.
template <int ST, bool CPLX>
__global__ void __launch_bounds__(256) build_entries_kernel(const void* __restrict__ ch,
                                                            void* __restrict__ entries, int64_t L, int64_t Lp,
                                                            int64_t n_traces) {
    // CTAs stride over traces, threads over the samples of a trace (no 64-bit divisions)
    for (int64_t t = blockIdx.x; t < n_traces; t += gridDim.x) {
        const int64_t in0 = t * L, out0 = t * Lp;
        for (int i = threadIdx.x; i < (int)Lp; i += blockDim.x) {
            float2 x0 = make_float2(0.f, 0.f), d = make_float2(0.f, 0.f);
            if (i >= 1 && i < (int)L - 1) {
                x0 = load_sample<ST, CPLX>(ch, in0 + i);
                const float2 x1 = load_sample<ST, CPLX>(ch, in0 + i + 1);
                d = make_float2(x1.x - x0.x, x1.y - x0.y);
            }
            if constexpr (CPLX) reinterpret_cast<float4*>(entries)[out0 + i] = make_float4(x0.x, x0.y, d.x, d.y);
            else reinterpret_cast<float2*>(entries)[out0 + i] = make_float2(x0.x, d.x);
        }
    }
}

// ---- asynchronous global -> shared copies (cp.async, 16 or 8 bytes per thread) -----
template <int BYTES>
__device__ __forceinline__ void cp_async(uint32_t dst, const void* src) {
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
// all but the newest N commit groups of this thread have landed
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Conservative test that channel `n`'s receive window is zero over the whole tile
// box: every window is 0 for ratio > 1/2 (apodization.m:172-186), and the ratio
// F#*|x_dist|/|z| is bounded below by the box.
__device__ __forceinline__ bool rx_active(const Params& A, const Box& b, float ex, float ey, float ez) {
    if (A.rx_apo_tab || A.rx_window == USTB_WIN_NONE) return true;
    float xd, yd, zmax;
    if (A.rx_origin) {
        xd = fabsf(ex - A.ox);
        yd = fabsf(ey - A.oy);
        float dmin, dmax;
        dist_range(b, A.ox, A.oy, A.oz, dmin, dmax);
        zmax = dmax;
    } else {
        xd = fmaxf(0.f, fmaxf(b.lo[0] - ex, ex - b.hi[0]));
        yd = fmaxf(0.f, fmaxf(b.lo[1] - ey, ey - b.hi[1]));
        zmax = fmaxf(fabsf(b.lo[2] - ez), fabsf(b.hi[2] - ez));
    }
    const float zx = fminf(fmaxf(zmax, A.minx * A.fnx), A.maxx * A.fnx);
    const float zy = fminf(fmaxf(zmax, A.miny * A.fny), A.maxy * A.fny);
    if (!(zx > 0.f) || !(zy > 0.f)) return true;
    const float lim = 0.5f * (1.f + 1e-4f);
    return !(A.fnx * xd / zx > lim || A.fny * yd / zy > lim);
}

template <bool CPLX>
struct CtasPerSm {
    static constexpr int value = 1;  // 512 threads x 128 registers fill the register file
};

// Stage shapes: a stage is CG channels x KW waves = 32 (channel, wave) slots.
//   shape 0: waves outer (2 channels x 16 waves); per-wave accumulators, the
//            receive geometry of a channel is formed once per 16-wave chunk
//   shape 1: channels outer (8 channels x 4 waves); per-channel accumulators,
//            the receive geometry is formed once per (pixel, channel) and the
//            transmit geometry once per stage
//   shape 2: channels outer (16 channels x 2 waves)
// dimension.receive needs waves outer, dimension.transmit/none channels outer;
// dimension.both runs with any of the three.
template <int SHAPE>
struct Shape;
template <>
struct Shape<0> {
    static constexpr bool WAVES_OUTER = true;
    static constexpr int CG = 2, KW = 16;
};
template <>
struct Shape<1> {
    static constexpr bool WAVES_OUTER = false;
    static constexpr int CG = 8, KW = 4;
};
template <>
struct Shape<2> {
    static constexpr bool WAVES_OUTER = false;
    static constexpr int CG = 16, KW = 2;
};
constexpr int kStageSlots = 32;

// Shared memory of one CTA: kRing stage buffers of kStageSlots slots x kSlot entries,
// then the per-tile tables (their size depends on N, W and the stage shape).
template <bool CPLX>
constexpr size_t slot_buffer_bytes() {
    return (size_t)kRing * kStageSlots * kSlot * (CPLX ? 16 : 8);
}

// Byte offsets of the per-tile tables (16-byte records first).
struct TileTables {
    size_t el4, txc, txp, bl, base_n, len_n, rxph, base_w, len_w, stages, olist, act_n, act_w, act_g, act_c, total;
};

// Per-channel tables hold NG * CG records and per-wave tables NC * KW records: the
// channels / waves past N / W are padding with zero weight, so a stage never needs
// bounds checks.
__host__ __device__ __forceinline__ TileTables tile_tables(int64_t N, int64_t W, int64_t NG, int64_t NC, int CG,
                                                           int KW) {
    TileTables t;
    const size_t NP = (size_t)(NG * CG), WP = (size_t)(NC * KW);
    (void)N;
    (void)W;
    size_t o = 0;
    t.el4 = o;    o += 16 * NP;        // float4 per channel: x, y, z, window base
    t.txc = o;    o += 16 * WP;        // float4 per wave: delay coefficients
    t.txp = o;    o += 16 * WP;        // float4 per wave: phase offset, apodization, fs/c, kind
    t.bl = o;     o += 8 * (NP + WP);  // int2 {window base, length}: channels, then waves
    t.base_n = o; o += 4 * NP;
    t.len_n = o;  o += 4 * NP;
    t.rxph = o;   o += 4 * NP;         // phase (cycles) of each channel's window base
    t.base_w = o; o += 4 * WP;
    t.len_w = o;  o += 4 * WP;
    t.stages = o; o += 4 * (size_t)(NG * NC);  // (outer << 16) | inner, loop order
    t.olist = o;  o += 4 * (size_t)(NG + NC);  // active outer indices, then active inner indices
    t.act_n = o;  o += NP;
    t.act_w = o;  o += WP;
    t.act_g = o;  o += (size_t)NG;                       // channel groups
    t.act_c = o;  o += (size_t)NC;                       // wave chunks
    t.total = (o + 15) & ~size_t(15);
    return t;
}

// Once per CTA, before its first tile: zero the stage buffers, so that units with
// zero weight, which may read past a window's end, never read uninitialised words.
template <bool CPLX>
__device__ __forceinline__ void zero_slots() {
    extern __shared__ __align__(16) unsigned char smem[];
    float4* z = reinterpret_cast<float4*>(smem);
    for (int i = threadIdx.x; i < (int)(slot_buffer_bytes<CPLX>() / 16); i += blockDim.x)
        z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
}

__device__ __forceinline__ float frac_cycles(double v) { return (float)(v - floor(v)); }

// Beamform one tile of one frame (the whole CTA participates).
//
// Delays are kept relative to integer window bases of the tile: for pixel p,
//   s_tx(p, w) = (tau_tx - t0) fs - base_w,   s_rx(p, n) = tau_rx fs - base_n,
// both in [0, kHalf], and the unit's sample position in slot (n, w) is
// s_tx + s_rx.  The phase factors exp(i 2 pi fd tau) are formed from these
// relative delays and a per-tile offset of each base (computed in double):
//   fd tau_tx = (fd/fs) s_tx + frac(fd (base_w/fs + t0)),  fd tau_rx = (fd/fs) s_rx + frac(fd base_n / fs).
// A plane or photoacoustic wave's s_tx is affine in the pixel position and a
// spherical wave's is sigma |p - src| fs/c + const; the per-tile coefficients
// sit in shared memory (txc, txp).
//
// FRAMES (persistent kernel): frames f_first .. f_first + nfr - 1 of the tile in turn,
// after one build of the tile's tables and stage list (the geometry is the same for
// every frame of a request).
template <int MODE, bool CPLX, bool EPI, int SHAPE, bool FRAMES = false>
__device__ __forceinline__ void das_tile(const Params& A, int tile, int64_t f_first, int half = -1, int nfr = 1) {
    constexpr bool ORDER_A = Shape<SHAPE>::WAVES_OUTER;
    constexpr int CG = Shape<SHAPE>::CG;
    constexpr int KW = Shape<SHAPE>::KW;
    constexpr int NS = CG * KW;
    static_assert(NS == kStageSlots, "stage buffers hold kStageSlots slots");
    static_assert(MODE != USTB_DIM_RECEIVE || ORDER_A, "dimension.receive keeps waves outer");
    static_assert((MODE != USTB_DIM_TRANSMIT && MODE != USTB_DIM_NONE) || !ORDER_A,
                  "dimension.transmit / none keep channels outer");
    using Entry = typename EntryT<CPLX>::type;
    constexpr int ES = (int)sizeof(Entry);

    const int64_t N = A.N, W = A.W, P = A.P;
    extern __shared__ __align__(16) unsigned char smem[];
    Entry* slots = reinterpret_cast<Entry*>(smem);
    const int NG = (int)((N + CG - 1) / CG), NC = (int)((W + KW - 1) / KW);
    const TileTables tt = tile_tables(N, W, NG, NC, CG, KW);
    unsigned char* tb = smem + slot_buffer_bytes<CPLX>();
    float4* el4 = reinterpret_cast<float4*>(tb + tt.el4);
    float4* txc = reinterpret_cast<float4*>(tb + tt.txc);
    float4* txp = reinterpret_cast<float4*>(tb + tt.txp);
    int2* bl_n = reinterpret_cast<int2*>(tb + tt.bl);
    int2* bl_w = bl_n + NG * CG;
    float* base_n = reinterpret_cast<float*>(tb + tt.base_n);
    int* len_n = reinterpret_cast<int*>(tb + tt.len_n);
    float* rxph = reinterpret_cast<float*>(tb + tt.rxph);
    float* base_w = reinterpret_cast<float*>(tb + tt.base_w);
    int* len_w = reinterpret_cast<int*>(tb + tt.len_w);
    int* stage_list = reinterpret_cast<int*>(tb + tt.stages);
    unsigned char* act_n = tb + tt.act_n;
    unsigned char* act_w = tb + tt.act_w;
    unsigned char* act_g = tb + tt.act_g;
    unsigned char* act_c = tb + tt.act_c;
    __shared__ float2 s_red[kTile / 32];
    __shared__ int s_nstages;
    __shared__ int s_tx_general;  // a spherical or tabulated wave, or tabulated tx apodization
    __shared__ int s_tx_sph;      // every active wave spherical, and no tx tables

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int32_t* tl = A.tiles + (int64_t)tile * kTile;
    // tile entries outside [0, P) are idle lanes; lane 0 names the tile's anchor pixel
    const int32_t p_own = __ldg(tl + tid);
    const bool live = p_own >= 0 && (int64_t)p_own < A.P;
    const int32_t p_anchor = __ldg(tl);
    const int64_t p = live ? p_own : ((p_anchor >= 0 && (int64_t)p_anchor < A.P) ? p_anchor : 0);
    const float px = __ldg(A.px + 3 * p), py = __ldg(A.px + 3 * p + 1), pz = __ldg(A.px + 3 * p + 2);

    Box box;
    {
        const float big = 3.4e38f;
        float2 r = block_minmax(live ? px : big, live ? px : -big, s_red);
        box.lo[0] = r.x; box.hi[0] = r.y;
        r = block_minmax(live ? py : big, live ? py : -big, s_red);
        box.lo[1] = r.x; box.hi[1] = r.y;
        r = block_minmax(live ? pz : big, live ? pz : -big, s_red);
        box.lo[2] = r.x; box.hi[2] = r.y;
    }

    // ---- per-tile window bases, lengths, activity and delay/phase coefficients ----
    const double fd_fs = (double)A.fd / (double)A.fs;
    if (tid == 0) {
        s_tx_general = A.tx_apo_tab != nullptr || A.tx_delay_tab != nullptr;
        s_tx_sph = !s_tx_general;
    }
    for (int n = (int)N + tid; n < NG * CG; n += kTile) {  // padding channels: never active
        el4[n] = make_float4(0.f, 0.f, 0.f, 0.f);
        base_n[n] = 0.f;
        len_n[n] = 0;
        rxph[n] = 0.f;
        act_n[n] = 0;
    }
    for (int w = (int)W + tid; w < NC * KW; w += kTile) {  // padding waves: zero weight
        txc[w] = make_float4(0.f, 0.f, 0.f, 0.f);
        txp[w] = make_float4(0.f, 0.f, 0.f, (float)USTB_WAVE_ZERO);
        base_w[w] = 0.f;
        len_w[w] = 0;
        act_w[w] = 0;
    }
    __syncthreads();  // s_tx_general is set before the wave loop may raise it
    for (int64_t n = tid; n < N; n += kTile) {
        const float ex = __ldg(A.el + 3 * n), ey = __ldg(A.el + 3 * n + 1), ez = __ldg(A.el + 3 * n + 2);
        float dmin, dmax;
        dist_range(box, ex, ey, ez, dmin, dmax);
        const float lo = (dmin * A.inv_c + A.lens) * A.fs, hi = (dmax * A.inv_c + A.lens) * A.fs;
        const float base = floorf(lo) - 1.f;
        const bool ok = (hi - base <= kHalf - 2.f) && fabsf(base) < 1.0e9f;
        const bool act = rx_active(A, box, ex, ey, ez);
        if (!ok && act) atomicOr(A.flags, USTB_FLAG_WINDOW_OVERFLOW);
        base_n[n] = fminf(fmaxf(base, -1.0e9f), 1.0e9f);
        el4[n] = make_float4(ex, ey, ez, base_n[n]);
        len_n[n] = (int)fminf(fmaxf(ceilf(hi - base), 0.f), kHalf);
        act_n[n] = act ? 1 : 0;
        rxph[n] = frac_cycles(fd_fs * (double)base_n[n]);
    }
    for (int64_t w = tid; w < W; w += kTile) {
        const ustb_wave wv = A.waves[w];
        if (wv.kind == USTB_WAVE_TABLE) continue;  // bases from the table below
        float lo, hi;
        tx_tau_range(wv, box, lo, hi);
        lo = (lo - A.t0) * A.fs;
        hi = (hi - A.t0) * A.fs;
        const float base = floorf(lo) - 1.f;
        const bool ok = (hi - base <= kHalf - 2.f) && fabsf(base) < 1.0e9f;
        const bool act = A.tx_apo_tab != nullptr || wv.apodization != 0.f;
        if (!ok && act) atomicOr(A.flags, USTB_FLAG_WINDOW_OVERFLOW);
        if (wv.kind == USTB_WAVE_SPHERICAL && act) s_tx_general = 1;
        if (wv.kind != USTB_WAVE_SPHERICAL && act) s_tx_sph = 0;
        const float bw = fminf(fmaxf(base, -1.0e9f), 1.0e9f);
        base_w[w] = bw;
        len_w[w] = (int)fminf(fmaxf(ceilf(hi - base), 0.f), kHalf);
        act_w[w] = act ? 1 : 0;
        // s_tx(p) = (tau(p) - t0) fs - base_w; constant part in double
        const double fs_c = (double)A.fs / (double)wv.sound_speed;
        const double c0 = -((double)wv.delay + (double)A.t0) * (double)A.fs - (double)bw;
        if (wv.kind == USTB_WAVE_PLANE)
            txc[w] = make_float4((float)(wv.dir[0] * fs_c), (float)(wv.dir[1] * fs_c), (float)(wv.dir[2] * fs_c),
                                 (float)c0);
        else if (wv.kind == USTB_WAVE_SPHERICAL)
            txc[w] = make_float4(wv.src[0], wv.src[1], wv.src[2], (float)(c0 + (double)wv.offset * fs_c));
        else
            txc[w] = make_float4(0.f, 0.f, 0.f, (float)c0);
        txp[w] = make_float4(frac_cycles(fd_fs * ((double)bw + (double)A.t0 * (double)A.fs)), wv.apodization,
                             (float)fs_c, (float)wv.kind);
    }
    if (A.tx_delay_tab) {  // tabulated transmit delays: the tile's actual range
        for (int64_t w = 0; w < W; ++w) {
            const ustb_wave wv = A.waves[w];
            if (wv.kind != USTB_WAVE_TABLE) continue;
            const float s = (__ldg(A.tx_delay_tab + w * P + p) - A.t0) * A.fs;
            const float2 r = block_minmax(live ? s : 3.4e38f, live ? s : -3.4e38f, s_red);
            if (tid == 0) {
                const float base = floorf(r.x) - 1.f;
                const bool ok = (r.y - base <= kHalf - 2.f) && fabsf(base) < 1.0e9f;
                if (!ok) atomicOr(A.flags, USTB_FLAG_WINDOW_OVERFLOW);
                const float bw = fminf(fmaxf(base, -1.0e9f), 1.0e9f);
                base_w[w] = bw;
                len_w[w] = (int)fminf(fmaxf(ceilf(r.y - base), 0.f), kHalf);
                act_w[w] = 1;
                txc[w] = make_float4(0.f, 0.f, 0.f, 0.f);
                txp[w] = make_float4(frac_cycles(fd_fs * ((double)bw + (double)A.t0 * (double)A.fs)),
                                     wv.apodization, 0.f, (float)USTB_WAVE_TABLE);
            }
        }
    } else {
        for (int64_t w = tid; w < W; w += kTile) {  // table waves without a table: tau = -delay
            const ustb_wave wv = A.waves[w];
            if (wv.kind != USTB_WAVE_TABLE) continue;
            const float lo = (-wv.delay - A.t0) * A.fs;
            const float base = floorf(lo) - 1.f;
            const bool act = A.tx_apo_tab != nullptr || wv.apodization != 0.f;
            const float bw = fminf(fmaxf(base, -1.0e9f), 1.0e9f);
            base_w[w] = bw;
            len_w[w] = (int)fminf(fmaxf(ceilf(lo - base), 0.f), kHalf);
            act_w[w] = act ? 1 : 0;
            const double c0 = -((double)wv.delay + (double)A.t0) * (double)A.fs - (double)bw;
            txc[w] = make_float4(0.f, 0.f, 0.f, (float)c0);
            txp[w] = make_float4(frac_cycles(fd_fs * ((double)bw + (double)A.t0 * (double)A.fs)), wv.apodization,
                                 0.f, (float)USTB_WAVE_ZERO);
        }
    }
    __syncthreads();
    for (int i = tid; i < NG * CG + NC * KW; i += kTile) {
        int2 v = make_int2(0, -(1 << 20));
        if (i < NG * CG) {
            if (i < N && act_n[i]) v = make_int2((int)base_n[i], len_n[i]);
        } else {
            const int w = i - NG * CG;
            if (w < W && act_w[w]) v = make_int2((int)base_w[w], len_w[w]);
        }
        bl_n[i] = v;
    }
    for (int g = tid; g < NG; g += kTile) {
        bool a = false;
        for (int c = 0; c < CG; ++c) a |= (g * CG + c < N) && act_n[g * CG + c];
        act_g[g] = a;
    }
    for (int k = tid; k < NC; k += kTile) {
        bool a = false;
        for (int j = 0; j < KW; ++j) a |= (k * KW + j < W) && act_w[k * KW + j];
        act_c[k] = a;
    }
    __syncthreads();
    // stage list: every (active outer, active inner) pair in loop order.  Warp 0
    // compacts the active outer and inner indices (ballots), then all threads fill in
    // the pairs.
    __shared__ int s_nout, s_nin;
    {
        const int NO = ORDER_A ? NC : NG, NI = ORDER_A ? NG : NC;
        const unsigned char* ao = ORDER_A ? act_c : act_g;
        const unsigned char* ai = ORDER_A ? act_g : act_c;
        int* olist = reinterpret_cast<int*>(tb + tt.olist);
        int* ilist = olist + NO;
        if (warp == 0) {
            int cnt = 0;
            for (int b = 0; b < NO; b += 32) {
                const bool a = b + lane < NO && ao[b + lane];
                const unsigned m = __ballot_sync(0xffffffffu, a);
                if (a) olist[cnt + __popc(m & ((1u << lane) - 1u))] = b + lane;
                cnt += __popc(m);
            }
            int cin = 0;
            for (int b = 0; b < NI; b += 32) {
                const bool a = b + lane < NI && ai[b + lane];
                const unsigned m = __ballot_sync(0xffffffffu, a);
                if (a) ilist[cin + __popc(m & ((1u << lane) - 1u))] = b + lane;
                cin += __popc(m);
            }
            if (lane == 0) {
                s_nout = cnt;
                s_nin = cin;
                s_nstages = cnt * cin;
            }
        }
        __syncthreads();
        const int no = s_nout, ni = s_nin;
        for (int t = tid; t < no * ni; t += kTile) {
            const int r = t / ni, q = t - r * ni;
            stage_list[t] = (olist[r] << 16) | ilist[q];
        }
    }
    __syncthreads();
    const int nstages = s_nstages;

    auto frame = [&](const int64_t f) {
    const float2 ph = A.pix_phase ? __ldg(A.pix_phase + p) : make_float2(1.f, 0.f);
    const float fdfs = (float)fd_fs;
    const int64_t frame_tr = f * W * N;  // first trace of this frame
    const int Lc = (int)A.L;             // entries per trace
    const uint32_t slots_s = (uint32_t)__cvta_generic_to_shared(slots);
    unsigned bufoff = 0;                 // byte offset of the current stage's buffer
    auto stage_o = [&](int si) { return stage_list[si] >> 16; };
    auto stage_i = [&](int si) { return stage_list[si] & 0xFFFF; };
    auto stage_w0 = [&](int si) { return (ORDER_A ? stage_o(si) : stage_i(si)) * KW; };
    auto stage_n0 = [&](int si) { return (ORDER_A ? stage_i(si) : stage_o(si)) * CG; };

    // Stage si's windows into buffer `buf`.  Half-warp h of warp v stages slot
    // v + 16 h: its 16 lanes copy the window [i0, i0 + len) entry by entry with
    // cp.async, and store zeros for the entries outside the trace (bounds are
    // checked only for windows that cross an end of the trace).  i0 and len come
    // from the packed per-tile {base, length} of the slot's channel and wave; an
    // inactive channel or wave has a negative length.  Slots without work are left
    // as they are: their units carry zero weight and read finite stale entries.
    constexpr int NWARPS = kTile / 32;
    const Entry* ent_f = reinterpret_cast<const Entry*>(A.entries) + frame_tr * A.Lp;
    const int Nn = (int)N;
    auto issue = [&](int si, int buf) {
        static_assert(NS == 2 * NWARPS, "two slots per warp");
        const int w0 = stage_w0(si), n0 = stage_n0(si);
        const int sl = warp + NWARPS * (lane >> 4);  // half-warp h of warp v: slot v + NWARPS h
        const int c = sl / KW, k = sl - (sl / KW) * KW;
        const int n = n0 + c, w = w0 + k;
        const int2 a = bl_n[n], b = bl_w[w];
        const int len = min(kSlot, a.y + b.y + 3);
        const int i0 = a.x + b.x;
        const Entry* src = ent_f + (int64_t)(w * Nn + n) * A.Lp;
        const uint32_t dst = slots_s + (uint32_t)((buf * NS + sl) * kSlot * ES);
        const int hl = lane & 15;
        if (i0 >= 0 && i0 + len <= Lc) {
            const Entry* sp = src + i0 + hl;
            const uint32_t dp = dst + (uint32_t)(hl * ES);
            for (int j = 0; j < len - hl; j += 16) cp_async<ES>(dp + (uint32_t)(j * ES), sp + j);
        } else {
            for (int j = hl; j < len; j += 16) {
                const int i = i0 + j;
                if ((unsigned)i < (unsigned)Lc) {
                    cp_async<ES>(dst + (uint32_t)(j * ES), src + i);
                } else {
                    if constexpr (CPLX)
                        asm volatile("st.shared.v4.f32 [%0], {%1, %1, %1, %1};\n" ::"r"(dst + (uint32_t)(j * ES)), "f"(0.f) : "memory");
                    else
                        asm volatile("st.shared.v2.f32 [%0], {%1, %1};\n" ::"r"(dst + (uint32_t)(j * ES)), "f"(0.f) : "memory");
                }
            }
        }
        cp_async_commit();
    };

    // per-thread geometry
    float srx[CG];
    float2 B[CG];
    float rxapo[CG];
    float stx[KW];
    float2 Aw[KW];
    constexpr int NACC = ORDER_A ? KW : CG;
    float accr[NACC], acci[NACC];
    float2 Y = make_float2(0.f, 0.f);
    float2 eS = make_float2(0.f, 0.f);
    float eI = 0.f, eM = 0.f, eR = 0.f, eQ = 0.f;

    // Closed-form window (no table): the same arithmetic as rx_apodization without
    // per-channel branches, centred under the pixel or, for sector scans, at the
    // aperture origin (lateral offsets from the origin per channel, the pixel's distance
    // to it per pixel); padding channels are inactive, so their weight is 0.
    const bool rx_plain = !A.rx_apo_tab && A.rx_window != USTB_WIN_NONE;
    float zo = 0.f;
    if (A.rx_origin) {
        const float qx = px - A.ox, qy = py - A.oy, qz = pz - A.oz;
        zo = sqrtf(qx * qx + qy * qy + qz * qz);
    }
    auto setup_rx_plain = [&](int n0, auto org) {
#pragma unroll
        for (int c = 0; c < CG; ++c) {
            const int n = n0 + c;
            const float4 e4 = el4[n];
            const float dx = px - e4.x, dy = py - e4.y, dz = pz - e4.z;
            const float r2 = fmaxf(dx * dx + dy * dy + dz * dz, 1e-30f);
            const float r = r2 * rsqrtf(r2);
            const float s = (r * A.inv_c + A.lens) * A.fs - e4.w;
            constexpr bool ORG = decltype(org)::value;
            const float xd = ORG ? e4.x - A.ox : -dx;
            const float yd = ORG ? e4.y - A.oy : -dy;
            const float zd = ORG ? zo : dz;
            const float zx = clamp_ap(zd, A.fnx, A.minx, A.maxx);
            const float wx = window(A, fabsf(A.fnx * __fdividef(xd, zx)));
            const float zy = clamp_ap(zd, A.fny, A.miny, A.maxy);
            const float wy = yd == 0.f ? 1.f : window(A, fabsf(A.fny * __fdividef(yd, zy)));
            const float apo = (live && n < N && act_n[n]) ? (yd == 0.f ? wx : wx * wy) : 0.f;
            float2 bb;
            if (CPLX) {
                const float2 e = phasor_cycles(fmaf(s, fdfs, rxph[n]));
                bb = make_float2(apo * e.x, apo * e.y);
            } else {
                bb = make_float2(apo, 0.f);
            }
            srx[c] = fminf(fmaxf(s, 0.f), kHalf);  // NaN -> 0: stays inside the slot
            B[c] = bb;
            rxapo[c] = apo;
        }
    };
    auto setup_rx = [&](int n0) {
        // the origin form only outside dimension.both (the sector scans' transmit mode):
        // in the dimension.both kernels a second unrolled copy made 75-wave plane-wave
        // compounding 2 % slower
        if (rx_plain && !A.rx_origin) {
            setup_rx_plain(n0, std::false_type{});
            return;
        }
        if constexpr (MODE != USTB_DIM_BOTH) {
            if (rx_plain) {
                setup_rx_plain(n0, std::true_type{});
                return;
            }
        }
#pragma unroll
        for (int c = 0; c < CG; ++c) {
            const int n = n0 + c;
            float s = 0.f, apo = 0.f;
            float2 bb = make_float2(0.f, 0.f);
            if (n < N && act_n[n]) {
                const float4 e4 = el4[n];
                const float ex = e4.x, ey = e4.y, ez = e4.z;
                const float dx = px - ex, dy = py - ey, dz = pz - ez;
                const float r2 = fmaxf(dx * dx + dy * dy + dz * dz, 1e-30f);
                const float r = r2 * rsqrtf(r2);
                s = (r * A.inv_c + A.lens) * A.fs - e4.w;
                apo = A.rx_apo_tab ? __ldg(A.rx_apo_tab + (int64_t)n * P + p) : rx_apodization(A, ex, ey, ez, px, py, pz);
                if (!live) apo = 0.f;
                if (CPLX) {
                    const float2 e = phasor_cycles(fmaf(s, fdfs, rxph[n]));
                    bb = make_float2(apo * e.x, apo * e.y);
                } else {
                    bb = make_float2(apo, 0.f);
                }
            }
            srx[c] = fminf(fmaxf(s, 0.f), kHalf);  // NaN -> 0: stays inside the slot
            B[c] = bb;
            rxapo[c] = apo;
        }
    };
    // Plane and photoacoustic waves (every tile without spherical or tabulated waves
    // and without a tx apodization table): s_tx is affine in the pixel position and
    // the weight is the wave's constant apodization times the phasor; padding and
    // inactive waves carry apodization 0.  No branches.
    const bool tx_affine = !s_tx_general;
    // Diverging and focused waves (every active wave spherical, no tables): the same
    // arithmetic as the general setup below without its per-wave branches; padding and
    // inactive waves carry apodization 0, and a table wave without a table has fs/c = 0
    // there, so its s_tx is the constant term as in the general setup.
    const bool tx_sph = s_tx_sph != 0;
    auto setup_tx_affine = [&](int w0) {
#pragma unroll
        for (int k = 0; k < KW; ++k) {
            const float4 cw = txc[w0 + k];
            const float2 q = *reinterpret_cast<const float2*>(&txp[w0 + k]);
            const float s = fmaf(cw.x, px, fmaf(cw.y, py, fmaf(cw.z, pz, cw.w)));
            stx[k] = fminf(fmaxf(s, 0.f), kHalf);
            if (CPLX) {
                const float2 e = phasor_cycles(fmaf(s, fdfs, q.x));
                Aw[k] = make_float2(q.y * e.x, q.y * e.y);
            } else {
                Aw[k] = make_float2(q.y, 0.f);
            }
        }
    };
    auto setup_tx = [&](int w0) {
        if (tx_affine) {
            setup_tx_affine(w0);
            return;
        }
        if (tx_sph) {
#pragma unroll
            for (int k = 0; k < KW; ++k) {
                const float4 cw = txc[w0 + k];
                const float4 q = txp[w0 + k];
                const float dx = px - cw.x, dy = py - cw.y, dz = pz - cw.z;
                const float d = sqrtf(dx * dx + dy * dy + dz * dz);
                const float sv = fmaf(pz < cw.z ? -d : d, q.z, cw.w);
                stx[k] = fminf(fmaxf(sv, 0.f), kHalf);
                if (CPLX) {
                    const float2 e = phasor_cycles(fmaf(sv, fdfs, q.x));
                    Aw[k] = make_float2(q.y * e.x, q.y * e.y);
                } else {
                    Aw[k] = make_float2(q.y, 0.f);
                }
            }
            return;
        }
#pragma unroll
        for (int k = 0; k < KW; ++k) {
            const int w = w0 + k;
            float s = 0.f;
            float2 a = make_float2(0.f, 0.f);
            if (w < W && act_w[w]) {
                const float4 cw = txc[w];
                const float4 q = txp[w];
                const int kind = (int)q.w;
                if (kind == USTB_WAVE_SPHERICAL) {
                    const float dx = px - cw.x, dy = py - cw.y, dz = pz - cw.z;
                    const float d = sqrtf(dx * dx + dy * dy + dz * dz);
                    s = fmaf(pz < cw.z ? -d : d, q.z, cw.w);
                } else if (kind == USTB_WAVE_TABLE) {
                    s = (__ldg(A.tx_delay_tab + w * P + p) - A.t0) * A.fs - base_w[w];
                } else {  // plane; photoacoustic (zero coefficients)
                    s = fmaf(cw.x, px, fmaf(cw.y, py, fmaf(cw.z, pz, cw.w)));
                }
                float apo = A.tx_apo_tab ? __ldg(A.tx_apo_tab + (int64_t)w * P + p) : q.y;
                if (!live) apo = 0.f;
                if (CPLX) {
                    const float2 e = phasor_cycles(fmaf(s, fdfs, q.x));
                    a = make_float2(apo * e.x, apo * e.y);
                } else {
                    a = make_float2(apo, 0.f);
                }
            }
            stx[k] = fminf(fmaxf(s, 0.f), kHalf);
            Aw[k] = a;
        }
    };

    // shared address of entry 0 of slot 0, minus the bias of the 2^23 floor trick
    const unsigned slot0 = (unsigned)__cvta_generic_to_shared(slots) - (unsigned)kMagicBits * (unsigned)sizeof(Entry);
    auto interp = [&](int c, int k, float s) -> float2 {
        const float t = __fadd_rz(s, kMagic);
        const float b = s - (t - kMagic);
        const unsigned addr = (unsigned)__float_as_int(t) * (unsigned)sizeof(Entry) + (slot0 + bufoff) +
                              (unsigned)((c * KW + k) * kSlot * (int)sizeof(Entry));
        if constexpr (CPLX) {
            float4 e;
            asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];\n"
                         : "=f"(e.x), "=f"(e.y), "=f"(e.z), "=f"(e.w) : "r"(addr));
            return make_float2(fmaf(b, e.z, e.x), fmaf(b, e.w, e.y));
        } else {
            float2 e;
            asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];\n" : "=f"(e.x), "=f"(e.y) : "r"(addr));
            return make_float2(fmaf(b, e.y, e.x), 0.f);
        }
    };

    auto store_cube = [&](int64_t o, float2 y) {
        if (!live || !A.cube) return;
        if constexpr (CPLX) reinterpret_cast<float2*>(A.cube)[o] = y;
        else reinterpret_cast<float*>(A.cube)[o] = y.x;
    };

    // Double-buffered pipeline over the tile's active stages: stage si + 1's windows
    // are copied while stage si is computed.  One barrier per stage: it makes stage
    // si's entries visible to every warp and frees the other buffer (read by stage
    // si - 1) for stage si + 1's copies.
    // half = k >= 0: this CTA takes part k of A.split equal parts of the stage list and
    // adds its partial sum to the (zeroed) output; -1: the whole list, plain stores
    const int parts = half < 0 ? 1 : A.split;
    const int s_lo = half < 0 ? 0 : (int)((int64_t)nstages * half / parts);
    const int s_hi = half < 0 ? nstages : (int)((int64_t)nstages * (half + 1) / parts);
    // A ring of kRing stage buffers: the copies of the first kRing - 1 stages are
    // issued up front, then stage si waits for its own copies (older commit groups),
    // one barrier publishes them and frees stage si - 1's buffer, which takes stage
    // si + kRing - 1's copies.  Stages past the end commit empty groups, so that every
    // thread's count of outstanding groups stays kRing - 1.
#pragma unroll
    for (int d = 0; d < kRing - 1; ++d) {
        if (s_lo + d < s_hi) issue(s_lo + d, d);
        else cp_async_commit();
    }
    auto begin_stage = [&](int si) {
        cp_async_wait_group<kRing - 2>();
        __syncthreads();
        const int nx = si + kRing - 1;
        if (nx < s_hi) issue(nx, (nx - s_lo) % kRing);
        else cp_async_commit();
        bufoff = (unsigned)(((si - s_lo) % kRing) * NS * kSlot * ES);
    };
    const float2 zero2 = make_float2(0.f, 0.f);
    // dimension.both: the pixel's sum, plain store or (split tiles) one of the partial sums
    auto store_both = [&]() {
        const float2 y = CPLX ? cmul(Y, ph) : Y;
        if (half < 0) {
            store_cube(p + A.f_f * f, y);
        } else if (live && A.cube) {  // partial sums: two give fl(a + b) in either order; three or
                                      // four are added in completion order (last-bit differences)
            if constexpr (CPLX) {
                atomicAdd(&reinterpret_cast<float2*>(A.cube)[p + A.f_f * f].x, y.x);
                atomicAdd(&reinterpret_cast<float2*>(A.cube)[p + A.f_f * f].y, y.y);
            } else {
                atomicAdd(&reinterpret_cast<float*>(A.cube)[p + A.f_f * f], y.x);
            }
        }
    };

    if constexpr (ORDER_A) {
        int cur = -1;  // current wave chunk
        auto zero_chunks = [&](int from, int to) {  // receive mode: skipped chunks are zero
            if constexpr (MODE == USTB_DIM_RECEIVE)
                for (int w = from * KW; w < min(to * KW, (int)W); ++w) store_cube(p + A.w_f * w + A.f_f * f, zero2);
        };
        auto finish_chunk = [&]() {
            const int w0 = cur * KW;
            const int kw = min(KW, (int)W - w0);
#pragma unroll
            for (int k = 0; k < KW; ++k) {
                if (k >= kw) continue;
                float2 y;
                if constexpr (CPLX) y = cmul(Aw[k], make_float2(accr[k], acci[k]));
                else y = make_float2(Aw[k].x * accr[k], 0.f);
                if (MODE == USTB_DIM_BOTH) {
                    Y.x += y.x;
                    Y.y += y.y;
                } else {
                    store_cube(p + A.w_f * (w0 + k) + A.f_f * f, CPLX ? cmul(y, ph) : y);
                }
            }
        };
        for (int si = s_lo; si < s_hi; ++si) {
            const int oc = stage_o(si);
            if (oc != cur) {
                if (cur >= 0) finish_chunk();
                zero_chunks(cur + 1, oc);
                cur = oc;
                setup_tx(oc * KW);
#pragma unroll
                for (int k = 0; k < KW; ++k) accr[k] = acci[k] = 0.f;
            }
            const int n0 = stage_n0(si);
            setup_rx(n0);
            begin_stage(si);
            const int kw = min(KW, (int)W - cur * KW);
            auto units = [&](auto full) {
#pragma unroll
                for (int c = 0; c < CG; ++c) {
                    const float2 b = B[c];
                    // a channel whose receive weight is zero for the whole warp adds
                    // nothing (das_c skips zero-apodization units too)
                    if (!__any_sync(0xffffffffu, b.x != 0.f || b.y != 0.f)) continue;
#pragma unroll
                    for (int k = 0; k < KW; ++k) {
                        if (!decltype(full)::value && k >= kw) continue;  // last, partial wave chunk
                        const float2 v = interp(c, k, stx[k] + srx[c]);
                        if constexpr (CPLX) {
                            accr[k] = fmaf(b.x, v.x, fmaf(-b.y, v.y, accr[k]));
                            acci[k] = fmaf(b.x, v.y, fmaf(b.y, v.x, acci[k]));
                        } else {
                            accr[k] = fmaf(b.x, v.x, accr[k]);
                        }
                    }
                }
            };
            if (kw == KW) units(std::true_type{});
            else units(std::false_type{});
        }
        if (cur >= 0) finish_chunk();
        zero_chunks(cur + 1, NC);
        if (MODE == USTB_DIM_BOTH) store_both();
    } else {
        if (MODE == USTB_DIM_NONE) {  // units outside the active stages are zero
            for (int n = 0; n < N; ++n)
                for (int w = 0; w < W; ++w) store_cube(p + A.rx_f * n + A.w_f * w + A.f_f * f, zero2);
        }
        int cur = -1;  // current channel group
        auto zero_groups = [&](int from, int to) {
            if constexpr (MODE == USTB_DIM_TRANSMIT)
                for (int n = from * CG; n < min(to * CG, (int)N); ++n) store_cube(p + A.rx_f * n + A.f_f * f, zero2);
        };
        auto finish_group = [&]() {
            if constexpr (MODE == USTB_DIM_NONE) return;
            const int n0 = cur * CG;
            const int cg = min(CG, (int)N - n0);
#pragma unroll
            for (int c = 0; c < CG; ++c) {
                if (c >= cg) continue;
                float2 y;
                if constexpr (CPLX) y = cmul(B[c], make_float2(accr[c], acci[c]));
                else y = make_float2(B[c].x * accr[c], 0.f);
                if constexpr (MODE == USTB_DIM_BOTH) {
                    Y.x += y.x;
                    Y.y += y.y;
                } else {
                    if constexpr (CPLX) y = cmul(y, ph);
                    store_cube(p + A.rx_f * (n0 + c) + A.f_f * f, y);
                    if constexpr (EPI) {
                        eS.x += y.x;
                        eS.y += y.y;
                        eI += y.x * y.x + y.y * y.y;
                        eM += rxapo[c] > A.cf_thr ? 1.f : 0.f;
                        const float re = y.x;
                        eR += msign(re) * sqrtf(fabsf(re));
                        eQ += fabsf(re);
                    }
                }
            }
        };
        unsigned gmask = 0;  // channels of the current group with a nonzero weight in this warp
        constexpr unsigned kAll = (1u << CG) - 1u;
        auto units = [&](int n0, int w0, auto all) {
#pragma unroll
            for (int c = 0; c < CG; ++c) {
                if (!decltype(all)::value && !((gmask >> c) & 1u)) continue;
#pragma unroll
                for (int k = 0; k < KW; ++k) {
                    const float2 v = interp(c, k, stx[k] + srx[c]);
                    if (MODE == USTB_DIM_NONE) {
                        if (n0 + c < N && w0 + k < W && act_n[n0 + c] && act_w[w0 + k]) {
                            const float2 y = CPLX ? cmul(cmul(cmul(Aw[k], B[c]), v), ph)
                                                  : make_float2(Aw[k].x * B[c].x * v.x, 0.f);
                            store_cube(p + A.rx_f * (n0 + c) + A.w_f * (w0 + k) + A.f_f * f, y);
                        }
                    } else if constexpr (CPLX) {
                        accr[c] = fmaf(Aw[k].x, v.x, fmaf(-Aw[k].y, v.y, accr[c]));
                        acci[c] = fmaf(Aw[k].x, v.y, fmaf(Aw[k].y, v.x, acci[c]));
                    } else {
                        accr[c] = fmaf(Aw[k].x, v.x, accr[c]);
                    }
                }
            }
        };
        for (int si = s_lo; si < s_hi; ++si) {
            const int code = stage_list[si];
            const int og = code >> 16, w0 = (code & 0xFFFF) * KW, n0 = og * CG;
            if (og != cur) {
                if (cur >= 0) finish_group();
                zero_groups(cur + 1, og);
                cur = og;
                setup_rx(n0);
                gmask = 0;
#pragma unroll
                for (int c = 0; c < CG; ++c)
                    if (MODE == USTB_DIM_NONE || __any_sync(0xffffffffu, B[c].x != 0.f || B[c].y != 0.f)) gmask |= 1u << c;
#pragma unroll
                for (int c = 0; c < CG; ++c) accr[c] = acci[c] = 0.f;
            }
            setup_tx(w0);
            begin_stage(si);
            if (gmask == kAll) units(n0, w0, std::true_type{});
            else units(n0, w0, std::false_type{});
        }
        if (cur >= 0) finish_group();
        zero_groups(cur + 1, NG);
        if constexpr (MODE == USTB_DIM_BOTH) store_both();
        if constexpr (EPI) {
            if (live) {
                const int64_t o = p + P * f;
                float cf = (eS.x * eS.x + eS.y * eS.y) / eI * (1.f / eM);
                if (cf != cf) cf = 0.f;  // NaN -> 0 (coherence_factor.m:132)
                if (A.o_das) A.o_das[o] = eS;
                if (A.o_cf) A.o_cf[o] = cf;
                if (A.o_cfimg) A.o_cfimg[o] = make_float2(cf * eS.x, cf * eS.y);
                if (A.o_sdmas) A.o_sdmas[o] = 0.5f * (eR * eR - eQ);
            }
        }
    }
    cp_async_wait_all();  // only empty groups remain
    __syncthreads();      // the buffers are reused by the next frame, the tables by the next tile
    };
    if constexpr (FRAMES) {
        for (int64_t f = f_first; f < f_first + nfr; ++f) frame(f);
    } else {
        frame(f_first);
    }
}

// One launch per request: grid = (tiles x CTAs per tile, frames).
template <int MODE, bool CPLX, bool EPI, int SHAPE>
__global__ void __launch_bounds__(kTile, (CtasPerSm<CPLX>::value)) das_fast_kernel(const Params A) {
    zero_slots<CPLX>();
    if (MODE == USTB_DIM_BOTH && A.split >= 2)
        das_tile<MODE, CPLX, EPI, SHAPE>(A, (int)(blockIdx.x / A.split), (int64_t)blockIdx.y,
                                         (int)(blockIdx.x % A.split));
    else
        das_tile<MODE, CPLX, EPI, SHAPE>(A, (int)blockIdx.x, (int64_t)blockIdx.y);
}

// Persistent form: one CTA per SM pulls (request, tile, frames) work items from a
// queue counter until the batch is done, so requests of different scans, channel
// counts and frame counts share one launch and balance across SMs.  An item is one
// tile over up to 8 consecutive frames of a request (fewer while that leaves each CTA
// under 8 items), so the tile's tables are built once for those frames.
constexpr int kMaxBatch = 40;
struct BatchParams {
    Params req[kMaxBatch];
    int64_t first_item[kMaxBatch + 1];  // prefix sums of tiles * frames
    int n;
    unsigned long long* counter;        // queue head (device scratch, zeroed per launch)
};

template <int MODE, bool CPLX, bool EPI, int SHAPE>
__global__ void __launch_bounds__(kTile, 1) das_fast_persistent(const __grid_constant__ BatchParams B) {
    __shared__ long long s_item;
    zero_slots<CPLX>();
    const int64_t total = B.first_item[B.n];
    for (;;) {
        if (threadIdx.x == 0) s_item = (long long)atomicAdd(B.counter, 1ull);
        __syncthreads();
        const int64_t item = s_item;
        __syncthreads();
        if (item >= total) break;
        int r = 0;
        while (r + 1 < B.n && B.first_item[r + 1] <= item) ++r;
        const Params& A = B.req[r];
        const int64_t local = item - B.first_item[r];
        const int64_t f0 = (local / A.n_tiles) * A.fpi;
        das_tile<MODE, CPLX, EPI, SHAPE, true>(A, (int)(local % A.n_tiles), f0, -1,
                                               (int)min((int64_t)A.fpi, A.F - f0));
    }
}

template <bool CPLX, int SHAPE>
size_t smem_bytes(int64_t N, int64_t W) {
    constexpr int CG = Shape<SHAPE>::CG, KW = Shape<SHAPE>::KW;
    const int64_t NG = (N + CG - 1) / CG, NC = (W + KW - 1) / KW;
    return slot_buffer_bytes<CPLX>() + tile_tables(N, W, NG, NC, CG, KW).total;
}

// The stage shape a request runs with: ustb_das_geometry.stage_shape when given
// (1: waves outer 2 x 16, 2: channels outer 8 x 4, 3: channels outer 16 x 2),
// else the library's choice.  Returns the Shape<> index.
int shape_for(int dim, int32_t requested) {
    if (requested > 0) return requested - 1;
    switch (dim) {
        case USTB_DIM_RECEIVE: return 0;
        case USTB_DIM_BOTH: return kBothShape;
        default: return 1;
    }
}

template <int MODE, bool CPLX, bool EPI, int SHAPE>
int launch(const Params& A, int64_t n_tiles, int64_t F, cudaStream_t s) {
    const size_t smem = smem_bytes<CPLX, SHAPE>(A.N, A.W);
    int dev = 0, optin = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    USTB_REQUIRE(smem <= (size_t)optin, USTB_E_SHAPE,
                 "%lld channels / %lld waves need %zu bytes of shared memory per tile (limit %d)",
                 (long long)A.N, (long long)A.W, smem, optin);
    auto kern = das_fast_kernel<MODE, CPLX, EPI, SHAPE>;
    USTB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // dimension.both with few tiles (under 4 per SM): two CTAs per tile, each over half of
    // its stages, add their partial sums into the zeroed image, so the last wave of
    // tiles is half as long.  With many tiles the tail is already short.
    int sms = 0;
    USTB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    Params B = A;
    if (MODE != USTB_DIM_BOTH) B.split = 1;
    else if (B.split == 0) B.split = (n_tiles * F < 4 * (int64_t)sms) ? 2 : 1;
    if (B.split >= 2 && B.cube)
        USTB_CUDA(cudaMemsetAsync(B.cube, 0, (size_t)(B.P * F) * (CPLX ? 8 : 4), s));
    dim3 grid((unsigned)(n_tiles * B.split), (unsigned)F);
    kern<<<grid, kTile, smem, s>>>(B);
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}

template <int MODE, bool CPLX, bool EPI, int SHAPE>
int launch_batch(const Params* reqs, const int64_t* frames, int n, unsigned long long* counter, int max_ctas,
                 cudaStream_t s) {
    BatchParams B;
    B.n = n;
    B.counter = counter;
    B.first_item[0] = 0;
    int dev = 0, optin = 0, sms = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    USTB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t nct = max_ctas > 0 ? std::min(max_ctas, sms) : sms;
    size_t smem = 0;
    for (int i = 0; i < n; ++i) {
        B.req[i] = reqs[i];
        // frames per work item: up to 8, while every CTA keeps at least 8 items of the request
        const int64_t fpi = std::max<int64_t>(1, std::min<int64_t>(8, reqs[i].n_tiles * frames[i] / (8 * nct)));
        B.req[i].fpi = (int)fpi;
        B.first_item[i + 1] = B.first_item[i] + reqs[i].n_tiles * ((frames[i] + fpi - 1) / fpi);
        smem = std::max(smem, smem_bytes<CPLX, SHAPE>(reqs[i].N, reqs[i].W));
    }
    if (B.first_item[n] == 0) return USTB_OK;
    USTB_REQUIRE(smem <= (size_t)optin, USTB_E_SHAPE, "a request needs %zu bytes of shared memory per tile (limit %d)",
                 smem, optin);
    auto kern = das_fast_persistent<MODE, CPLX, EPI, SHAPE>;
    USTB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    USTB_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s));
    // one CTA per SM, or fewer (max_ctas) to leave SMs to launches on other streams
    const unsigned grid = (unsigned)std::min<int64_t>(B.first_item[n], nct);
    kern<<<grid, kTile, smem, s>>>(B);
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}

// Kernel variant of (dimension, epilogue, stage shape) for one request kind.
template <bool CPLX, bool BATCH>
int dispatch(int dim, int epi, int shape, const Params* reqs, const int64_t* frames, int n,
             unsigned long long* counter, int64_t nt, int64_t F, cudaStream_t s, int max_ctas = 0) {
#define USTB_RUN(M, E, S)                                                                      \
    return BATCH ? launch_batch<M, CPLX, E, S>(reqs, frames, n, counter, max_ctas, s)         \
                 : launch<M, CPLX, E, S>(reqs[0], nt, F, s)
    switch (dim) {
        case USTB_DIM_NONE:
            if (shape == 2) USTB_RUN(USTB_DIM_NONE, false, 2);
            USTB_RUN(USTB_DIM_NONE, false, 1);
        case USTB_DIM_RECEIVE: USTB_RUN(USTB_DIM_RECEIVE, false, 0);
        case USTB_DIM_TRANSMIT:
            if constexpr (CPLX)
                if (epi) {
                    if (shape == 2) USTB_RUN(USTB_DIM_TRANSMIT, true, 2);
                    USTB_RUN(USTB_DIM_TRANSMIT, true, 1);
                }
            if (shape == 2) USTB_RUN(USTB_DIM_TRANSMIT, false, 2);
            USTB_RUN(USTB_DIM_TRANSMIT, false, 1);
        default:
            if (shape == 0) USTB_RUN(USTB_DIM_BOTH, false, 0);
            if (shape == 2) USTB_RUN(USTB_DIM_BOTH, false, 2);
            USTB_RUN(USTB_DIM_BOTH, false, 1);
    }
#undef USTB_RUN
}

// ---- entries scratch ---------------------------------------------------------
int64_t entry_bytes(int64_t L, int64_t N, int64_t W, int64_t F, bool cplx) {
    return L * N * W * F * (cplx ? 16 : 8);
}

// A stream-ordered memory pool owned by the library (one per device) that keeps
// freed entry arrays for the next call instead of returning them to the driver.
cudaMemPool_t entry_pool(int dev) {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64) return nullptr;
    if (!pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        if (cudaMemPoolCreate(&p, &props) != cudaSuccess) return nullptr;
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        pools[dev] = p;
    }
    return pools[dev];
}

// Fill one request's entry array `dst` (entry_bytes(...) bytes of device memory).
int fill_entries(const void* ch, int32_t storage, bool cplx, int64_t L, int64_t N, int64_t W, int64_t F,
                 void* dst, cudaStream_t s) {
    int dev = 0, sms = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    USTB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t traces = N * W * F, total = traces * L;
    if (total == 0) return USTB_OK;
    const unsigned grid = (unsigned)std::min<int64_t>(traces, (int64_t)sms * 32);
    switch (storage * 2 + (cplx ? 1 : 0)) {
        case USTB_STORE_F32 * 2 + 1: build_entries_kernel<USTB_STORE_F32, true><<<grid, 256, 0, s>>>(ch, dst, L, L, traces); break;
        case USTB_STORE_F16 * 2 + 1: build_entries_kernel<USTB_STORE_F16, true><<<grid, 256, 0, s>>>(ch, dst, L, L, traces); break;
        case USTB_STORE_BF16 * 2 + 1: build_entries_kernel<USTB_STORE_BF16, true><<<grid, 256, 0, s>>>(ch, dst, L, L, traces); break;
        case USTB_STORE_F32 * 2: build_entries_kernel<USTB_STORE_F32, false><<<grid, 256, 0, s>>>(ch, dst, L, L, traces); break;
        case USTB_STORE_F16 * 2: build_entries_kernel<USTB_STORE_F16, false><<<grid, 256, 0, s>>>(ch, dst, L, L, traces); break;
        default: build_entries_kernel<USTB_STORE_BF16, false><<<grid, 256, 0, s>>>(ch, dst, L, L, traces); break;
    }
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}

// Allocate (stream-ordered, from the library pool) and fill one request's entries.
int build_entries(const void* ch, int32_t storage, bool cplx, int64_t L, int64_t N, int64_t W, int64_t F,
                  void** out, cudaStream_t s) {
    *out = nullptr;
    const int64_t bytes = entry_bytes(L, N, W, F, cplx);
    if (bytes == 0) return USTB_OK;
    int dev = 0;
    USTB_CUDA(cudaGetDevice(&dev));
    cudaMemPool_t pool = entry_pool(dev);
    USTB_REQUIRE(pool, USTB_E_CUDA, "could not create the entry memory pool on device %d", dev);
    const cudaError_t e = cudaMallocFromPoolAsync(out, (size_t)bytes, pool, s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        *out = nullptr;
        ustb::set_error("%lld bytes of interpolation entries: %s", (long long)bytes, cudaGetErrorString(e));
        return USTB_E_OOM;
    }
    return fill_entries(ch, storage, cplx, L, N, W, F, *out, s);
}

// Bytes of a caller workspace that holds the entries of every request of a batch
// (each request's array starts on a 256-byte boundary).
int64_t batch_workspace_bytes(const ustb_das_request* reqs, int32_t n) {
    int64_t total = 0;
    for (int i = 0; i < n; ++i) {
        const ustb_das_request& q = reqs[i];
        if (q.L <= 0 || q.N <= 0 || q.W <= 0 || q.F <= 0) continue;
        total += (entry_bytes(q.L, q.N, q.W, q.F, q.is_complex != 0) + 255) & ~int64_t(255);
    }
    return total;
}

}  // namespace

// Validate one request and fill its kernel parameters.  Returns USTB_OK, or a
// status; *empty is set when the request has no work (its outputs are already
// handled, e.g. zero-filled).
static int make_params(const void* ch, int32_t storage, int32_t is_complex, int64_t L, int64_t N, int64_t W,
                       int64_t F, const ustb_das_geometry* g, int32_t dimension, int32_t epilogue,
                       const ustb_das_outputs* out, uint32_t* flags, cudaStream_t s, Params& A, bool& empty) {
    empty = false;
    USTB_REQUIRE(g && out, USTB_E_ARG, "geometry and outputs must be given");
    USTB_REQUIRE(dimension >= 0 && dimension <= 3, USTB_E_ARG, "Unknown sum mode %d", (int)dimension);
    USTB_REQUIRE(storage >= 0 && storage <= 2, USTB_E_DTYPE, "unknown storage type %d", (int)storage);
    USTB_REQUIRE(is_complex == 0 || is_complex == 1, USTB_E_ARG, "is_complex must be 0 or 1");
    USTB_REQUIRE(L >= 0 && N >= 0 && W >= 0 && F >= 0, USTB_E_SHAPE, "negative size");
    USTB_REQUIRE(g->n_elements == N && g->n_waves == W, USTB_E_SHAPE,
                 "geometry has %lld elements / %lld waves, channel data %lld / %lld",
                 (long long)g->n_elements, (long long)g->n_waves, (long long)N, (long long)W);
    USTB_REQUIRE(is_complex || !(fabsf(g->fd) > 1e-6f), USTB_E_DTYPE,
                 "The modulation frequency > 0 but the input data is real. Check inputs.");
    USTB_REQUIRE(!epilogue || (dimension == USTB_DIM_TRANSMIT && is_complex), USTB_E_ARG,
                 "the coherence-factor / DMAS epilogue needs dimension.transmit and complex data");
    USTB_REQUIRE(flags, USTB_E_ARG, "flags pointer is NULL");
    USTB_REQUIRE(F <= 65535, USTB_E_SHAPE, "at most 65535 frames per call");
    USTB_REQUIRE(L <= INT32_MAX - 256, USTB_E_SHAPE, "L=%lld exceeds the 32-bit sample index", (long long)L);
    USTB_REQUIRE(N <= 1000000 && W <= 1000000, USTB_E_SHAPE, "N and W must be below 10^6");
    USTB_REQUIRE(g->n_tiles <= INT32_MAX, USTB_E_SHAPE, "too many tiles");
    USTB_REQUIRE(g->sound_speed > 0.f && g->fs > 0.f, USTB_E_ARG, "sound speed and fs must be > 0");
    if (g->n_tiles == 0 || F == 0 || g->n_pixels == 0) { empty = true; return USTB_OK; }
    USTB_REQUIRE(g->element_xyz && g->pixel_xyz && g->tile_pixels && (W == 0 || g->waves), USTB_E_ARG,
                 "a geometry pointer is NULL");
    USTB_REQUIRE(L == 0 || N == 0 || W == 0 || ch, USTB_E_ARG, "channel data pointer is NULL");
    USTB_REQUIRE(((uintptr_t)ch & 15) == 0, USTB_E_ARG, "channel data must be 16-byte aligned");
    const int64_t P = g->n_pixels;
    if (L == 0 || N == 0 || W == 0) {
        const int64_t nout = out_elems(dimension, P, N, W, F);
        if (out->cube && nout)
            USTB_CUDA(cudaMemsetAsync(out->cube, 0, (size_t)nout * (is_complex ? 8 : 4), s));
        empty = true;
        return USTB_OK;
    }
    A.entries = nullptr;  // built by the caller of make_params
    A.L = L; A.Lp = L; A.N = N; A.W = W; A.F = F; A.P = P;
    A.el = g->element_xyz;
    A.px = g->pixel_xyz;
    A.tiles = g->tile_pixels;
    A.n_tiles = g->n_tiles;
    A.waves = g->waves;
    A.tx_delay_tab = g->tx_delay_table;
    A.tx_apo_tab = g->tx_apo_table;
    A.rx_apo_tab = g->rx_apo_table;
    A.pix_phase = reinterpret_cast<const float2*>(g->pixel_phase);
    A.fs = g->fs; A.t0 = g->t0; A.fd = (fabsf(g->fd) > 1e-6f) ? g->fd : 0.f;
    A.inv_c = 1.f / g->sound_speed;
    A.lens = g->lens_delay;
    A.rx_window = g->rx_window;
    {
        const WinCoeffs wc = window_coeffs(g->rx_window);
        A.win_r1 = wc.r1; A.win_a = wc.a; A.win_e = wc.e; A.win_b = wc.b; A.win_c = wc.c; A.win_d = wc.d;
    }
    A.fnx = g->rx_f_number[0]; A.fny = g->rx_f_number[1];
    A.minx = g->rx_min_aperture[0]; A.miny = g->rx_min_aperture[1];
    A.maxx = g->rx_max_aperture[0]; A.maxy = g->rx_max_aperture[1];
    A.rx_origin = g->rx_use_origin;
    A.ox = g->rx_origin[0]; A.oy = g->rx_origin[1]; A.oz = g->rx_origin[2];
    A.cf_thr = g->cf_threshold;
    A.cube = out->cube;
    A.o_das = reinterpret_cast<float2*>(out->das);
    A.o_cf = out->cf;
    A.o_cfimg = reinterpret_cast<float2*>(out->cf_image);
    A.o_sdmas = out->sdmas;
    const OutStrides os = out_strides(dimension, P, N, W);
    A.rx_f = os.rx_f; A.w_f = os.w_f; A.f_f = os.f_f;
    A.flags = flags;
    USTB_REQUIRE(g->ctas_per_tile >= 0 && g->ctas_per_tile <= 4, USTB_E_ARG, "ctas_per_tile must be 0 to 4");
    A.split = g->ctas_per_tile;  // 0: chosen at launch
    USTB_REQUIRE(g->stage_shape >= 0 && g->stage_shape <= 3, USTB_E_ARG, "stage_shape must be 0, 1, 2 or 3");
    USTB_REQUIRE(g->stage_shape == 0 || dimension == USTB_DIM_BOTH ||
                     (dimension == USTB_DIM_RECEIVE) == (g->stage_shape == 1),
                 USTB_E_ARG, "stage_shape %d does not fit dimension %d (receive: 1; transmit/none: 2 or 3)",
                 (int)g->stage_shape, (int)dimension);
    A.shape = shape_for(dimension, g->stage_shape);
    A.fpi = 1;
    return USTB_OK;
}

extern "C" int ustb_das_fast(const void* ch, int32_t storage, int32_t is_complex, int64_t L, int64_t N,
                             int64_t W, int64_t F, const ustb_das_geometry* g, int32_t dimension,
                             int32_t epilogue, const ustb_das_outputs* out, uint32_t* flags, void* stream) {
    ustb::clear_error();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    USTB_REQUIRE(flags, USTB_E_ARG, "flags pointer is NULL");
    USTB_CUDA(cudaMemsetAsync(flags, 0, sizeof(uint32_t), s));
    Params A;
    bool empty = false;
    int rc = make_params(ch, storage, is_complex, L, N, W, F, g, dimension, epilogue, out, flags, s, A, empty);
    if (rc || empty) return rc;
    void* ent = nullptr;
    rc = build_entries(ch, storage, is_complex != 0, L, N, W, F, &ent, s);
    if (rc) return rc;
    A.entries = ent;
    const int64_t nt = g->n_tiles;
    rc = is_complex ? dispatch<true, false>(dimension, epilogue, A.shape, &A, nullptr, 1, nullptr, nt, F, s)
                    : dispatch<false, false>(dimension, 0, A.shape, &A, nullptr, 1, nullptr, nt, F, s);
    const cudaError_t fe = cudaFreeAsync(ent, s);
    if (rc) return rc;
    USTB_CUDA(fe);
    return USTB_OK;
}

extern "C" int64_t ustb_entries_bytes(int64_t L, int64_t N, int64_t W, int64_t F, int32_t is_complex) {
    if (L < 0 || N < 0 || W < 0 || F < 0) return 0;
    return entry_bytes(L, N, W, F, is_complex != 0);
}

extern "C" int ustb_build_entries(const void* ch, int32_t storage, int32_t is_complex, int64_t L, int64_t N,
                                  int64_t W, int64_t F, void* entries, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(storage >= 0 && storage <= 2, USTB_E_DTYPE, "unknown storage type %d", (int)storage);
    USTB_REQUIRE(L >= 0 && N >= 0 && W >= 0 && F >= 0, USTB_E_SHAPE, "negative size");
    USTB_REQUIRE(L <= INT32_MAX - 256, USTB_E_SHAPE, "L=%lld exceeds the 32-bit sample index", (long long)L);
    if (L == 0 || N == 0 || W == 0 || F == 0) return USTB_OK;
    USTB_REQUIRE(ch && entries, USTB_E_ARG, "NULL pointer");
    USTB_REQUIRE(((uintptr_t)entries & 15) == 0, USTB_E_ARG, "entries must be 16-byte aligned");
    return fill_entries(ch, storage, is_complex != 0, L, N, W, F, entries, static_cast<cudaStream_t>(stream));
}

extern "C" int ustb_das_fast_entries(const void* entries, int32_t is_complex, int64_t L, int64_t N, int64_t W,
                                     int64_t F, const ustb_das_geometry* g, int32_t dimension, int32_t epilogue,
                                     const ustb_das_outputs* out, uint32_t* flags, void* stream) {
    ustb::clear_error();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    USTB_REQUIRE(flags, USTB_E_ARG, "flags pointer is NULL");
    USTB_CUDA(cudaMemsetAsync(flags, 0, sizeof(uint32_t), s));
    Params A;
    bool empty = false;
    // make_params validates the request; the storage type is irrelevant for entries
    int rc = make_params(entries, USTB_STORE_F32, is_complex, L, N, W, F, g, dimension, epilogue, out, flags, s, A,
                         empty);
    if (rc || empty) return rc;
    USTB_REQUIRE(((uintptr_t)entries & 15) == 0, USTB_E_ARG, "entries must be 16-byte aligned");
    A.entries = entries;
    const int64_t nt = g->n_tiles;
    return is_complex ? dispatch<true, false>(dimension, epilogue, A.shape, &A, nullptr, 1, nullptr, nt, F, s)
                      : dispatch<false, false>(dimension, 0, A.shape, &A, nullptr, 1, nullptr, nt, F, s);
}

static int das_fast_batch_impl(const ustb_das_request* reqs, int32_t n, uint64_t* scratch, void* workspace,
                               int64_t workspace_bytes, int32_t max_ctas, void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(n >= 0 && (n == 0 || reqs), USTB_E_ARG, "bad request array");
    USTB_REQUIRE(max_ctas >= 0, USTB_E_ARG, "max_ctas must be >= 0 (0: one CTA per SM)");
    USTB_REQUIRE(scratch, USTB_E_ARG, "scratch pointer is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* flags = reinterpret_cast<uint32_t*>(scratch);
    USTB_CUDA(cudaMemsetAsync(scratch, 0, sizeof(uint64_t), s));
    if (n == 0) return USTB_OK;
    // validate all requests first, then launch one persistent kernel per kernel variant
    std::vector<Params> P(n);
    std::vector<int64_t> frames(n);
    std::vector<int> key(n, -1);
    for (int i = 0; i < n; ++i) {
        const ustb_das_request& q = reqs[i];
        bool empty = false;
        int rc = make_params(q.ch, q.storage, q.is_complex, q.L, q.N, q.W, q.F, q.geometry, q.dimension,
                             q.epilogue, q.out, flags, s, P[i], empty);
        if (rc) {
            char msg[1200];
            snprintf(msg, sizeof msg, "request %d: %s", i, ustb_last_error());
            ustb::set_error("%s", msg);
            return rc;
        }
        frames[i] = q.F;
        if (!empty) key[i] = ((q.dimension * 2 + q.is_complex) * 2 + (q.epilogue ? 1 : 0)) * 4 + P[i].shape;
    }
    // every request's entry array: carved from the caller's workspace, or allocated
    // from the library pool and freed (stream-ordered) after the launches
    std::vector<void*> ents;
    auto release = [&]() {
        for (void* e : ents) (void)cudaFreeAsync(e, s);
        ents.clear();
    };
    if (workspace) {
        const int64_t need = batch_workspace_bytes(reqs, n);
        USTB_REQUIRE(need <= workspace_bytes, USTB_E_SHAPE, "the workspace holds %lld bytes, the batch needs %lld",
                     (long long)workspace_bytes, (long long)need);
        USTB_REQUIRE(((uintptr_t)workspace & 255) == 0, USTB_E_ARG, "the workspace must be 256-byte aligned");
    }
    int64_t ws_off = 0;
    for (int i = 0; i < n; ++i) {
        if (key[i] < 0) continue;
        const ustb_das_request& q = reqs[i];
        void* ent = nullptr;
        int rc;
        if (workspace) {
            ent = static_cast<char*>(workspace) + ws_off;
            ws_off += (entry_bytes(q.L, q.N, q.W, q.F, q.is_complex != 0) + 255) & ~int64_t(255);
            rc = fill_entries(q.ch, q.storage, q.is_complex != 0, q.L, q.N, q.W, q.F, ent, s);
        } else {
            rc = build_entries(q.ch, q.storage, q.is_complex != 0, q.L, q.N, q.W, q.F, &ent, s);
            if (!rc) ents.push_back(ent);
        }
        if (rc) {
            release();
            return rc;
        }
        P[i].entries = ent;
    }
    int group = 0;
    std::vector<bool> done(n, false);
    for (int i = 0; i < n; ++i) {
        if (key[i] < 0 || done[i]) continue;
        std::vector<Params> gp;
        std::vector<int64_t> gf;
        for (int j = i; j < n; ++j)
            if (!done[j] && key[j] == key[i]) {
                gp.push_back(P[j]);
                gf.push_back(frames[j]);
                done[j] = true;
            }
        const ustb_das_request& q = reqs[i];
        for (size_t off = 0; off < gp.size(); off += kMaxBatch) {
            const int cnt = (int)std::min<size_t>(kMaxBatch, gp.size() - off);
            unsigned long long* counter = reinterpret_cast<unsigned long long*>(scratch + 1 + group);
            ++group;
            if (group > n) {
                release();
                ustb::set_error("scratch holds n + 1 words");
                return USTB_E_ARG;
            }
            const int rc = q.is_complex
                               ? dispatch<true, true>(q.dimension, q.epilogue, P[i].shape, gp.data() + off, gf.data() + off,
                                                      cnt, counter, 0, 0, s, max_ctas)
                               : dispatch<false, true>(q.dimension, 0, P[i].shape, gp.data() + off, gf.data() + off, cnt,
                                                       counter, 0, 0, s, max_ctas);
            if (rc) {
                release();
                return rc;
            }
        }
    }
    release();
    return USTB_OK;
}

extern "C" int ustb_das_fast_batch(const ustb_das_request* reqs, int32_t n, uint64_t* scratch, void* stream) {
    return das_fast_batch_impl(reqs, n, scratch, nullptr, 0, 0, stream);
}

extern "C" int ustb_das_fast_batch_ex(const ustb_das_request* reqs, int32_t n, uint64_t* scratch, void* workspace,
                                      int64_t workspace_bytes, int32_t max_ctas, void* stream) {
    return das_fast_batch_impl(reqs, n, scratch, workspace, workspace_bytes, max_ctas, stream);
}

extern "C" int64_t ustb_das_fast_workspace_bytes(const ustb_das_request* reqs, int32_t n) {
    if (n <= 0 || !reqs) return 0;
    return batch_workspace_bytes(reqs, n);
}

extern "C" int ustb_das_fast_batch_ws(const ustb_das_request* reqs, int32_t n, uint64_t* scratch, void* workspace,
                                      int64_t workspace_bytes, void* stream) {
    if (!workspace) {
        ustb::clear_error();
        ustb::set_error("workspace pointer is NULL (ustb_das_fast_batch allocates its own)");
        return USTB_E_ARG;
    }
    return das_fast_batch_impl(reqs, n, scratch, workspace, workspace_bytes, 0, stream);
}
