// Plain single-precision DAS on precomputed delay/apodization tables — the
// drop-in for the reference's das_c (+mex/source/das_c.cpp:355-409).
//
// One thread per pixel.  For the summing modes each thread keeps FC frame
// accumulators in registers and writes every output element exactly once, so
// the output needs no clearing.  Per unit the arithmetic follows das_c step by
// step in single precision, with the same roundings where they decide the
// result: delay = fl(tx + rx), s = fl(fl(delay - t0) * fs), n0 = trunc(s),
// b = s - floor(s), phase = fl(wd * delay).  Only the order of the final sums
// and FMA contraction in the interpolation/rotation differ (a few ulp).
//
// Loop order: for dimension.both/.receive, chunks of WC waves outer (their tx
// values in registers) and channels inner (rx values re-read once per chunk);
// for .transmit/.none, channels outer and wave chunks inner.
#include <mutex>

#include "common.cuh"
#include "phasor.cuh"

namespace {

constexpr int kThreads = 128;
constexpr double kRefPi = 3.14159265359;  // the PI das_c uses for wd (das_c.cpp:33,243)

struct TableArgs {
    const void* ch;
    int64_t L, N, W, F, P, LN, LNW;
    float fs, t0, wd;
    const float* apo_tx;
    const float* apo_rx;
    const float* d_tx;
    const float* d_rx;
    void* out;
    int64_t rx_f, w_f, f_f;
};

template <bool CPLX, int FC>
struct Acc {
    float re[FC];
    float im[FC];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int f = 0; f < FC; ++f) re[f] = im[f] = 0.f;
    }
};

template <bool CPLX, int FC>
__device__ __forceinline__ void store(const TableArgs& A, int64_t idx, int64_t f0, int nf,
                                      const Acc<CPLX, FC>& acc) {
#pragma unroll
    for (int f = 0; f < FC; ++f) {
        if (f < nf) {
            const int64_t o = idx + (f0 + f) * A.f_f;
            if (CPLX)
                reinterpret_cast<float2*>(A.out)[o] = make_float2(acc.re[f], acc.im[f]);
            else
                reinterpret_cast<float*>(A.out)[o] = acc.re[f];
        }
    }
}

// Waves are processed in chunks of WC whose tx delay/apodization sit in
// registers; for each channel the WC units of the chunk are independent.  They
// are evaluated branch-free: every unit loads from a safe sample index and an
// invalid or zero-apodization unit's contribution is selected away (not
// multiplied by zero, so non-finite samples behave as in das_c, which skips
// those units).  All WC sample loads are then in flight together.
constexpr int WC = 8;

// A table value that is read once per wave chunk: kept out of L1 so that it does not
// evict the channel-data lines the sample gathers reuse.
__device__ __forceinline__ float ld_stream(const float* p) {
    float v;
    asm volatile("ld.global.nc.L1::no_allocate.f32 %0, [%1];\n" : "=f"(v) : "l"(p));
    return v;
}

// das_c's n0 = (int)s and floor(s) (das_c.cpp:381-383).  For traces of at most 2^23
// samples the integer part comes from adding 2^23 with round-toward-zero: it equals
// (int)s for 0 <= s < 2^23, and negative, too large, NaN or infinite s give indices
// outside (0, L - 1), so those units stay invalid as in das_c; for the valid units
// (s >= 1) floor(s) = (int)s and the fraction s - floor(s) is the same float.
// Longer traces use the conversion instructions.
template <bool MAGIC>
__device__ __forceinline__ int trunc_floor(float s, float& fl) {
    if constexpr (MAGIC) {
        const float t = __fadd_rz(s, 8388608.0f);
        fl = __fsub_rn(t, 8388608.0f);
        return __float_as_int(t) - 0x4B000000;
    } else {
        fl = floorf(s);
        return __float2int_rz(s);
    }
}

// Prefetch into L1 the sample lines of one channel's WC units, so that their loads a
// channel later hit L1 instead of waiting on L2 (same index arithmetic as chunk_units).
template <bool CPLX, typename IDX, bool MAGIC>
__device__ __forceinline__ void prefetch_units(const TableArgs& A, IDX nL, const IDX* wbase, int wc, const float* txd,
                                               float rxd, float rxa) {
    if (rxa == 0.0f) return;
    const int Lm1 = (int)(A.L - 1);
#pragma unroll
    for (int k = 0; k < WC; ++k) {
        const float denay = __fmul_rn(__fsub_rn(__fadd_rn(txd[k], rxd), A.t0), A.fs);
        float fl;
        const int n0 = trunc_floor<MAGIC>(denay, fl);
        if (k < wc && n0 > 0 && n0 < Lm1) {
            const char* x = reinterpret_cast<const char*>(A.ch) + (size_t)(nL + wbase[k] + (IDX)n0) * (CPLX ? 8 : 4);
            asm volatile("prefetch.global.L1 [%0];\n" ::"l"(x));
        }
    }
}

// IDX: int32_t when every sample index of the call fits 31 bits, else int64_t.
// pf: also prefetch into L1 the next channel's sample line of each unit, at this unit's
// sample index shifted by dn, the receive-delay step to the next channel in samples
// (clamped into the trace; only where the lines are, not which units are valid).
template <bool CPLX, int FC, bool PER_WAVE, int NACC, typename IDX, bool MAGIC>
__device__ __forceinline__ void chunk_units(const TableArgs& A, IDX nL, const IDX* wbase, int wc, int64_t f0,
                                            int nf, const float* txd, const float* txa, float rxd, float rxa,
                                            Acc<CPLX, FC>* acc, bool pf = false, int dn = 0) {
    float a[WC], b[WC], wr[WC], wi[WC];
    IDX base[WC];
    bool ok[WC];
    const int Lm1 = (int)(A.L - 1);
#pragma unroll
    for (int k = 0; k < WC; ++k) {
        const float delay = __fadd_rn(txd[k], rxd);
        const float apo = __fmul_rn(txa[k], rxa);
        const float denay = __fmul_rn(__fsub_rn(delay, A.t0), A.fs);
        float fl;
        const int n0 = trunc_floor<MAGIC>(denay, fl);
        ok[k] = k < wc && txa[k] != 0.0f && rxa != 0.0f && n0 > 0 && n0 < Lm1;
        if (pf && k < wc) {
            const int m = min(max(n0 + dn, 1), Lm1 - 1);
            const char* x = reinterpret_cast<const char*>(A.ch) +
                            (size_t)(nL + (IDX)A.L + wbase[k] + (IDX)m) * (CPLX ? 8 : 4);
            asm volatile("prefetch.global.L1 [%0];\n" ::"l"(x));
        }
        b[k] = __fsub_rn(denay, fl);
        a[k] = __fsub_rn(1.0f, b[k]);
        base[k] = nL + wbase[k] + (IDX)(ok[k] ? n0 : 1);
        if (CPLX) {
            float c, s;
            ustb::expi_reduced(__fmul_rn(A.wd, delay), c, s);
            wr[k] = c * apo;
            wi[k] = s * apo;
        } else {
            wr[k] = apo;
            wi[k] = 0.f;
        }
    }
#pragma unroll
    for (int f = 0; f < FC; ++f) {
        if (f >= nf) continue;
#pragma unroll
        for (int k = 0; k < WC; ++k) {
            Acc<CPLX, FC>& ac = acc[PER_WAVE ? k : 0];
            if (CPLX) {
                const float2* x = reinterpret_cast<const float2*>(A.ch) + base[k] + f * A.LNW;
                const float2 x0 = __ldg(x), x1 = __ldg(x + 1);
                const float vr = fmaf(b[k], x1.x, a[k] * x0.x);
                const float vi = fmaf(b[k], x1.y, a[k] * x0.y);
                const float nr = fmaf(wr[k], vr, fmaf(-wi[k], vi, ac.re[f]));
                const float ni = fmaf(wr[k], vi, fmaf(wi[k], vr, ac.im[f]));
                ac.re[f] = ok[k] ? nr : ac.re[f];
                ac.im[f] = ok[k] ? ni : ac.im[f];
            } else {
                const float* x = reinterpret_cast<const float*>(A.ch) + base[k] + f * A.LNW;
                const float x0 = __ldg(x), x1 = __ldg(x + 1);
                const float nr = fmaf(wr[k], fmaf(b[k], x1, a[k] * x0), ac.re[f]);
                ac.re[f] = ok[k] ? nr : ac.re[f];
            }
        }
    }
}

// The index half of one channel's WC units (dimension both / receive): das_c's delay,
// the sample index and fraction, and which units are valid.  Formed one channel
// ahead, so that the same arithmetic also prefetches the channel's sample lines into
// L1, and carried to the next iteration, where unit_sum adds the units.
template <typename IDX>
struct UnitIdx {
    float delay[WC], b[WC];
    IDX base[WC];
    unsigned ok;  // bit k: unit k valid (k < wc, nonzero weights, 0 < n0 < L - 1)
};

template <bool CPLX, typename IDX, bool MAGIC>
__device__ __forceinline__ void unit_index(const TableArgs& A, IDX nL, const IDX* wbase, int wc, const float* txd,
                                           const float* txa, float rxd, float rxa, bool prefetch, UnitIdx<IDX>& u) {
    const unsigned Lm2 = (unsigned)(A.L - 2);  // L >= 3 here (the host zero-fills shorter traces)
    u.ok = 0u;
#pragma unroll
    for (int k = 0; k < WC; ++k) {
        const float delay = __fadd_rn(txd[k], rxd);
        const float denay = __fmul_rn(__fsub_rn(delay, A.t0), A.fs);
        float fl;
        const int n0 = trunc_floor<MAGIC>(denay, fl);
        const bool ok = k < wc && txa[k] != 0.0f && rxa != 0.0f && (unsigned)(n0 - 1) < Lm2;
        u.delay[k] = delay;
        u.b[k] = __fsub_rn(denay, fl);
        u.base[k] = nL + wbase[k] + (IDX)(ok ? n0 : 1);
        u.ok |= ok ? (1u << k) : 0u;
        if (prefetch && ok) {
            const char* x = reinterpret_cast<const char*>(A.ch) + (size_t)u.base[k] * (CPLX ? 8 : 4);
            asm volatile("prefetch.global.L1 [%0];\n" ::"l"(x));
        }
    }
}

template <bool CPLX, int FC, bool PER_WAVE, typename IDX>
__device__ __forceinline__ void unit_sum(const TableArgs& A, const UnitIdx<IDX>& u, const float* txa, float rxa,
                                         int nf, Acc<CPLX, FC>* acc) {
#pragma unroll
    for (int k = 0; k < WC; ++k) {
        const bool ok = (u.ok >> k) & 1u;
        const float apo = __fmul_rn(txa[k], rxa);
        const float b = u.b[k], a = __fsub_rn(1.0f, b);
        float wr = apo, wi = 0.f;
        if (CPLX) {
            float c, sn;
            ustb::expi_reduced(__fmul_rn(A.wd, u.delay[k]), c, sn);
            wr = c * apo;
            wi = sn * apo;
        }
#pragma unroll
        for (int f = 0; f < FC; ++f) {
            if (f >= nf) continue;
            Acc<CPLX, FC>& ac = acc[PER_WAVE ? k : 0];
            if (CPLX) {
                const float2* x = reinterpret_cast<const float2*>(A.ch) + u.base[k] + f * A.LNW;
                const float2 x0 = __ldg(x), x1 = __ldg(x + 1);
                const float vr = fmaf(b, x1.x, a * x0.x);
                const float vi = fmaf(b, x1.y, a * x0.y);
                const float nr = fmaf(wr, vr, fmaf(-wi, vi, ac.re[f]));
                const float ni = fmaf(wr, vi, fmaf(wi, vr, ac.im[f]));
                ac.re[f] = ok ? nr : ac.re[f];
                ac.im[f] = ok ? ni : ac.im[f];
            } else {
                const float* x = reinterpret_cast<const float*>(A.ch) + u.base[k] + f * A.LNW;
                const float x0 = __ldg(x), x1 = __ldg(x + 1);
                const float nr = fmaf(wr, fmaf(b, x1, a * x0), ac.re[f]);
                ac.re[f] = ok ? nr : ac.re[f];
            }
        }
    }
}

// Real data: at most 80 registers (6 CTAs of 128 threads per SM), with the carried unit
// indices; complex data: the phase of every unit needs more registers.
template <int MODE, bool CPLX, int FC, typename IDX, bool MAGIC>
__global__ void __launch_bounds__(kThreads, (CPLX ? 1 : 6)) das_table_kernel(const TableArgs A) {
    const int64_t p = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (p >= A.P) return;
    const int64_t P = A.P;
    constexpr bool PER_WAVE = (MODE == USTB_DIM_RECEIVE || MODE == USTB_DIM_NONE);
    constexpr int NACC = PER_WAVE ? WC : 1;
    Acc<CPLX, FC> acc[NACC];
    float txd[WC], txa[WC];
    auto load_tx = [&](int64_t w0, int wc) {
#pragma unroll
        for (int k = 0; k < WC; ++k) {
            txa[k] = k < wc ? __ldg(A.apo_tx + P * (w0 + k) + p) : 0.f;
            txd[k] = k < wc ? __ldg(A.d_tx + P * (w0 + k) + p) : 0.f;
        }
    };
    for (int64_t f0 = 0; f0 < A.F; f0 += FC) {
        const int nf = (int)min((int64_t)FC, A.F - f0);
        if (MODE == USTB_DIM_RECEIVE || MODE == USTB_DIM_BOTH) {
            if (MODE == USTB_DIM_BOTH) acc[0].zero();
            // the warp's channels with a nonzero receive weight lie in [nlo, nhi]: one scan
            // of the apodization column, so that every wave chunk reads the receive tables
            // of those channels only (the others are skipped per unit anyway)
            int nlo = (int)A.N, nhi = -1;
            for (int n = 0; n < (int)A.N; ++n)
                if (ld_stream(A.apo_rx + P * n + p) != 0.0f) {
                    nlo = min(nlo, n);
                    nhi = n;
                }
            const unsigned live = __activemask();
            nlo = __reduce_min_sync(live, nlo);
            nhi = __reduce_max_sync(live, nhi);
            for (int64_t w0 = 0; w0 < A.W; w0 += WC) {
                const int wc = (int)min((int64_t)WC, A.W - w0);
                load_tx(w0, wc);
                IDX wbase[WC];
#pragma unroll
                for (int k = 0; k < WC; ++k) wbase[k] = (IDX)(A.LN * (w0 + (k < wc ? k : 0)) + f0 * A.LNW);
                if (MODE == USTB_DIM_RECEIVE)
#pragma unroll
                    for (int k = 0; k < WC; ++k) acc[k].zero();
                // receive values are loaded two channels ahead and the next channel's
                // sample lines prefetched into L1 while this channel is computed
                // (no receive weight in this warp: nhi < nlo, the loop below runs no channel)
                const float* pa = A.apo_rx + P * max(nlo, 0) + p;
                const float* pd = A.d_rx + P * max(nlo, 0) + p;
                float rxa1 = 0.f, rxd1 = 0.f, rxa2 = 0.f, rxd2 = 0.f;
                if (nlo <= nhi) {
                    rxa1 = ld_stream(pa);
                    rxd1 = ld_stream(pd);
                }
                if (nlo + 1 <= nhi) {
                    rxa2 = ld_stream(pa + P);
                    rxd2 = ld_stream(pd + P);
                }
                pa += 2 * P;
                pd += 2 * P;
                IDX nL = (IDX)A.L * (IDX)nlo;
                if constexpr (CPLX) {
                    // complex: the register count left by the per-unit phase allows no
                    // carried indices; the next channel's lines are prefetched from this
                    // channel's indices shifted by the receive-delay step (the first
                    // channel, and lanes without a weight on this channel, form the next
                    // channel's indices for the prefetch)
                    if (FC == 1 && nlo <= nhi) prefetch_units<CPLX, IDX, MAGIC>(A, nL, wbase, wc, txd, rxd1, rxa1);
                    for (int n = nlo; n <= nhi; ++n, nL += (IDX)A.L) {
                        const float rxa = rxa1, rxd = rxd1;
                        rxa1 = rxa2;
                        rxd1 = rxd2;
                        if (n + 2 <= nhi) {
                            rxa2 = ld_stream(pa);
                            rxd2 = ld_stream(pd);
                            pa += P;
                            pd += P;
                        }
                        const bool pf = FC == 1 && n + 1 <= nhi && rxa1 != 0.0f;
                        if (rxa == 0.0f) {
                            if (pf) prefetch_units<CPLX, IDX, MAGIC>(A, nL + (IDX)A.L, wbase, wc, txd, rxd1, rxa1);
                            continue;
                        }
                        const int dn = __float2int_rn(__fmul_rn(__fsub_rn(rxd1, rxd), A.fs));
                        chunk_units<CPLX, FC, PER_WAVE, NACC, IDX, MAGIC>(A, nL, wbase, wc, f0, nf, txd, txa, rxd, rxa,
                                                                          acc, pf, dn);
                    }
                } else {
                // real: the indices formed with the prefetch are carried to the units
                UnitIdx<IDX> cur, nxt;
                if (nlo <= nhi) unit_index<CPLX, IDX, MAGIC>(A, nL, wbase, wc, txd, txa, rxd1, rxa1, FC == 1, cur);
                for (int n = nlo; n <= nhi; ++n, nL += (IDX)A.L) {
                    const float rxa = rxa1;
                    rxa1 = rxa2;
                    rxd1 = rxd2;
                    if (n + 2 <= nhi) {
                        rxa2 = ld_stream(pa);
                        rxd2 = ld_stream(pd);
                        pa += P;
                        pd += P;
                    }
                    if (n + 1 <= nhi)
                        unit_index<CPLX, IDX, MAGIC>(A, nL + (IDX)A.L, wbase, wc, txd, txa, rxd1, rxa1, FC == 1, nxt);
                    if (rxa != 0.0f) unit_sum<CPLX, FC, PER_WAVE, IDX>(A, cur, txa, rxa, nf, acc);
                    cur = nxt;
                }
                }
                if (MODE == USTB_DIM_RECEIVE)
#pragma unroll
                    for (int k = 0; k < WC; ++k)
                        if (k < wc) store<CPLX, FC>(A, p + A.w_f * (w0 + k), f0, nf, acc[k]);
            }
            if (MODE == USTB_DIM_BOTH) store<CPLX, FC>(A, p, f0, nf, acc[0]);
        } else {
            for (int64_t n = 0; n < A.N; ++n) {
                const float rxa = __ldg(A.apo_rx + P * n + p);
                const float rxd = __ldg(A.d_rx + P * n + p);
                if (MODE == USTB_DIM_TRANSMIT) acc[0].zero();
                for (int64_t w0 = 0; w0 < A.W; w0 += WC) {
                    const int wc = (int)min((int64_t)WC, A.W - w0);
                    load_tx(w0, wc);
                    IDX wbase[WC];
#pragma unroll
                    for (int k = 0; k < WC; ++k) wbase[k] = (IDX)(A.LN * (w0 + (k < wc ? k : 0)) + f0 * A.LNW);
                    if (MODE == USTB_DIM_NONE)
#pragma unroll
                        for (int k = 0; k < WC; ++k) acc[k].zero();
                    if (rxa != 0.0f)
                        chunk_units<CPLX, FC, PER_WAVE, NACC, IDX, MAGIC>(A, (IDX)(A.L * n), wbase, wc, f0, nf, txd, txa, rxd,
                                                                   rxa, acc);
                    if (MODE == USTB_DIM_NONE)
#pragma unroll
                        for (int k = 0; k < WC; ++k)
                            if (k < wc) store<CPLX, FC>(A, p + A.rx_f * n + A.w_f * (w0 + k), f0, nf, acc[k]);
                }
                if (MODE == USTB_DIM_TRANSMIT) store<CPLX, FC>(A, p + A.rx_f * n, f0, nf, acc[0]);
            }
        }
    }
}

template <int MODE, bool CPLX, typename IDX, bool MAGIC>
void launch_idx(const TableArgs& A, cudaStream_t s) {
    const unsigned grid = (unsigned)((A.P + kThreads - 1) / kThreads);
    if (A.F == 1)
        das_table_kernel<MODE, CPLX, 1, IDX, MAGIC><<<grid, kThreads, 0, s>>>(A);
    else if (A.F == 2)
        das_table_kernel<MODE, CPLX, 2, IDX, MAGIC><<<grid, kThreads, 0, s>>>(A);
    else
        das_table_kernel<MODE, CPLX, 4, IDX, MAGIC><<<grid, kThreads, 0, s>>>(A);
}

// 32-bit sample indices when every index of the call (and one past it) fits 31 bits;
// the float trick of trunc_floor for traces of at most 2^23 samples
template <int MODE, bool CPLX>
void launch_fc(const TableArgs& A, cudaStream_t s) {
    const bool short_traces = A.L <= ((int64_t)1 << 23);
    if (A.LNW * A.F < (int64_t)INT32_MAX - 1 && short_traces)
        launch_idx<MODE, CPLX, int32_t, true>(A, s);
    else if (short_traces)
        launch_idx<MODE, CPLX, int64_t, true>(A, s);
    else
        launch_idx<MODE, CPLX, int64_t, false>(A, s);
}

template <bool CPLX>
void launch_mode(int dim, const TableArgs& A, cudaStream_t s) {
    switch (dim) {
        case USTB_DIM_NONE: launch_fc<USTB_DIM_NONE, CPLX>(A, s); break;
        case USTB_DIM_RECEIVE: launch_fc<USTB_DIM_RECEIVE, CPLX>(A, s); break;
        case USTB_DIM_TRANSMIT: launch_fc<USTB_DIM_TRANSMIT, CPLX>(A, s); break;
        default: launch_fc<USTB_DIM_BOTH, CPLX>(A, s); break;
    }
}

int check_table_args(const void* ch, int32_t ch_complex, int64_t L, int64_t N, int64_t W, int64_t F,
                     float fd, int32_t dim, const void* apo_tx, const void* apo_rx,
                     const void* delay_tx, const void* delay_rx, int64_t P, const void* out) {
    USTB_REQUIRE(dim >= 0 && dim <= 3, USTB_E_ARG,
                 "Unknown sum mode %d. Available: 0 -> NONE, 1->RX, 2->TX, 3->BOTH", (int)dim);
    USTB_REQUIRE(L >= 0 && N >= 0 && W >= 0 && F >= 0 && P >= 0, USTB_E_SHAPE,
                 "negative size (L=%lld N=%lld W=%lld F=%lld P=%lld)", (long long)L, (long long)N,
                 (long long)W, (long long)F, (long long)P);
    USTB_REQUIRE(ch_complex == 0 || ch_complex == 1, USTB_E_ARG, "ch_complex must be 0 or 1");
    USTB_REQUIRE(ch_complex || !(fabsf(fd) > 1e-6f), USTB_E_DTYPE,
                 "The modulation frequency > 0 but the input data is real. Check inputs.");
    USTB_REQUIRE(L <= INT32_MAX, USTB_E_SHAPE, "L=%lld exceeds the 32-bit sample index", (long long)L);
    const bool empty_in = L == 0 || N == 0 || W == 0 || F == 0;
    USTB_REQUIRE(empty_in || ch, USTB_E_ARG, "channel data pointer is NULL");
    USTB_REQUIRE(P == 0 || (apo_tx && apo_rx && delay_tx && delay_rx), USTB_E_ARG,
                 "a delay/apodization table pointer is NULL");
    USTB_REQUIRE(out_elems(dim, P, N, W, F) == 0 || out, USTB_E_ARG, "output pointer is NULL");
    return USTB_OK;
}

// Byte counts of the host-pointer entries' device copies: channel data, one tx
// table, one rx table and the output.  Every product is checked for overflow, so
// a request whose sizes wrap 64 bits is rejected instead of under-allocated.
struct StagingBytes {
    size_t ch, tx, rx, out, total;
};

int staging_bytes(int32_t ch_complex, int64_t L, int64_t N, int64_t W, int64_t F, int64_t P, int32_t dim,
                  StagingBytes& b) {
    const uint64_t el = ch_complex ? 8 : 4;
    uint64_t ch = 0, tx = 0, rx = 0, out = 0, t = 0;
    const int64_t nk = (dim == USTB_DIM_NONE || dim == USTB_DIM_TRANSMIT) ? N : 1;
    const int64_t wk = (dim == USTB_DIM_NONE || dim == USTB_DIM_RECEIVE) ? W : 1;
    bool bad = __builtin_mul_overflow((uint64_t)L, (uint64_t)N, &t) || __builtin_mul_overflow(t, (uint64_t)W, &t) ||
               __builtin_mul_overflow(t, (uint64_t)F, &t) || __builtin_mul_overflow(t, el, &ch);
    bad = bad || __builtin_mul_overflow((uint64_t)P, (uint64_t)W, &t) || __builtin_mul_overflow(t, (uint64_t)4, &tx);
    bad = bad || __builtin_mul_overflow((uint64_t)P, (uint64_t)N, &t) || __builtin_mul_overflow(t, (uint64_t)4, &rx);
    bad = bad || __builtin_mul_overflow((uint64_t)P, (uint64_t)nk, &t) || __builtin_mul_overflow(t, (uint64_t)wk, &t) ||
          __builtin_mul_overflow(t, (uint64_t)F, &t) || __builtin_mul_overflow(t, el, &out);
    // each part is padded to 256 bytes; the sum of six padded parts must not wrap either
    const uint64_t lim = (UINT64_MAX >> 4) - 256;
    bad = bad || ch > lim || tx > lim || rx > lim || out > lim;
    USTB_REQUIRE(!bad, USTB_E_SHAPE, "the request's byte counts overflow 64 bits (L=%lld N=%lld W=%lld F=%lld P=%lld)",
                 (long long)L, (long long)N, (long long)W, (long long)F, (long long)P);
    auto align = [](uint64_t v) { return (v + 255) & ~uint64_t(255); };
    b.ch = (size_t)ch;
    b.tx = (size_t)tx;
    b.rx = (size_t)rx;
    b.out = (size_t)out;
    b.total = (size_t)(align(ch) + 2 * align(tx) + 2 * align(rx) + align(out));
    return USTB_OK;
}

// Makes `device` current for the lifetime of the guard and then restores the
// caller's current device, so the host-pointer entries leave the calling thread's
// CUDA state as they found it.
class DeviceGuard {
public:
    int enter(int device) {
        USTB_CUDA(cudaGetDevice(&prev_));
        if (prev_ != device) {
            USTB_CUDA(cudaSetDevice(device));
            restore_ = true;
        }
        return USTB_OK;
    }
    ~DeviceGuard() {
        if (restore_) (void)cudaSetDevice(prev_);
    }

private:
    int prev_ = 0;
    bool restore_ = false;
};

}  // namespace

extern "C" int ustb_das_table_f32(const void* ch, int32_t ch_complex, int64_t L, int64_t N,
                                  int64_t W, int64_t F, float fs, float t0, const float* apo_tx,
                                  const float* apo_rx, const float* delay_tx,
                                  const float* delay_rx, int64_t P, float fd, int32_t dimension,
                                  void* out, void* stream) {
    ustb::clear_error();
    int rc = check_table_args(ch, ch_complex, L, N, W, F, fd, dimension, apo_tx, apo_rx, delay_tx,
                              delay_rx, P, out);
    if (rc) return rc;
    const int64_t n_out = out_elems(dimension, P, N, W, F);
    if (n_out == 0) return USTB_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (L < 3 || N == 0 || W == 0) {
        // nothing to sum (a valid unit needs 0 < n0 < L - 1): das_c returns its
        // zero-initialised output
        USTB_CUDA(cudaMemsetAsync(out, 0, (size_t)n_out * (ch_complex ? 8 : 4), s));
        return USTB_OK;
    }
    TableArgs A;
    A.ch = ch;
    A.L = L; A.N = N; A.W = W; A.F = F; A.P = P;
    A.LN = L * N; A.LNW = L * N * W;
    A.fs = fs; A.t0 = t0;
    A.wd = 0.0f;
    if (fabsf(fd) > 1e-6f) A.wd = 2 * (float)kRefPi * fd;
    A.apo_tx = apo_tx; A.apo_rx = apo_rx; A.d_tx = delay_tx; A.d_rx = delay_rx;
    A.out = out;
    const OutStrides os = out_strides(dimension, P, N, W);
    A.rx_f = os.rx_f; A.w_f = os.w_f; A.f_f = os.f_f;
    if (ch_complex)
        launch_mode<true>(dimension, A, s);
    else
        launch_mode<false>(dimension, A, s);
    USTB_CUDA(cudaGetLastError());
    return USTB_OK;
}

extern "C" int ustb_das_table_f32_host(const void* ch, int32_t ch_complex, int64_t L, int64_t N,
                                       int64_t W, int64_t F, float fs, float t0,
                                       const float* apo_tx, const float* apo_rx,
                                       const float* delay_tx, const float* delay_rx, int64_t P,
                                       float fd, int32_t dimension, void* out, int32_t device) {
    ustb::clear_error();
    int rc = check_table_args(ch, ch_complex, L, N, W, F, fd, dimension, apo_tx, apo_rx, delay_tx,
                              delay_rx, P, out);
    if (rc) return rc;
    StagingBytes sb;
    rc = staging_bytes(ch_complex, L, N, W, F, P, dimension, sb);
    if (rc) return rc;
    DeviceGuard dg;
    rc = dg.enter(device);
    if (rc) return rc;
    const size_t ch_bytes = sb.ch, tx_bytes = sb.tx, rx_bytes = sb.rx, out_bytes = sb.out, total = sb.total;
    cudaStream_t s;
    USTB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    char* buf = nullptr;
    auto align = [](size_t v) { return (v + 255) & ~size_t(255); };
    cudaError_t e = cudaMallocAsync((void**)&buf, total ? total : 256, s);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return ustb::cuda_fail(e, "cudaMallocAsync", __FILE__, __LINE__);
    }
    char* p = buf;
    void* d_ch = p; p += align(ch_bytes);
    float* d_atx = (float*)p; p += align(tx_bytes);
    float* d_dtx = (float*)p; p += align(tx_bytes);
    float* d_arx = (float*)p; p += align(rx_bytes);
    float* d_drx = (float*)p; p += align(rx_bytes);
    void* d_out = p;
    rc = USTB_OK;
    do {
        if (ch_bytes && (e = cudaMemcpyAsync(d_ch, ch, ch_bytes, cudaMemcpyHostToDevice, s))) break;
        if (tx_bytes && (e = cudaMemcpyAsync(d_atx, apo_tx, tx_bytes, cudaMemcpyHostToDevice, s))) break;
        if (tx_bytes && (e = cudaMemcpyAsync(d_dtx, delay_tx, tx_bytes, cudaMemcpyHostToDevice, s))) break;
        if (rx_bytes && (e = cudaMemcpyAsync(d_arx, apo_rx, rx_bytes, cudaMemcpyHostToDevice, s))) break;
        if (rx_bytes && (e = cudaMemcpyAsync(d_drx, delay_rx, rx_bytes, cudaMemcpyHostToDevice, s))) break;
        rc = ustb_das_table_f32(d_ch, ch_complex, L, N, W, F, fs, t0, d_atx, d_arx, d_dtx, d_drx, P,
                                fd, dimension, d_out, s);
        if (rc) break;
        if (out_bytes && (e = cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, s))) break;
        e = cudaStreamSynchronize(s);
    } while (0);
    cudaFreeAsync(buf, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (rc) return rc;
    if (e != cudaSuccess) return ustb::cuda_fail(e, "host-pointer DAS copy/sync", __FILE__, __LINE__);
    return USTB_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free form of the host-pointer entry point.
//
// Staging buffers live in one file-scope device array instead of memory from
// cudaMalloc.  Host code may not use the array's name as a device address, so
// its address is looked up once per device with cudaGetSymbolAddress (with that
// device current) and cached.  All calls share the array.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[USTB_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// The scratch array's device address on the current device `device`.
int noalloc_scratch(int device, void** out) {
    USTB_REQUIRE(device >= 0 && device < kMaxDevices, USTB_E_ARG, "device %d out of range", device);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return ustb::cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
        g_noalloc_ptr[device] = p;
    }
    *out = g_noalloc_ptr[device];
    return USTB_OK;
}

}  // namespace

extern "C" int ustb_das_table_f32_host_noalloc(const void* ch, int32_t ch_complex, int64_t L, int64_t N,
                                               int64_t W, int64_t F, float fs, float t0,
                                               const float* apo_tx, const float* apo_rx,
                                               const float* delay_tx, const float* delay_rx, int64_t P,
                                               float fd, int32_t dimension, void* out, int32_t device) {
    ustb::clear_error();
    int rc = check_table_args(ch, ch_complex, L, N, W, F, fd, dimension, apo_tx, apo_rx, delay_tx,
                              delay_rx, P, out);
    if (rc) return rc;
    StagingBytes sb;
    rc = staging_bytes(ch_complex, L, N, W, F, P, dimension, sb);
    if (rc) return rc;
    const size_t ch_bytes = sb.ch, tx_bytes = sb.tx, rx_bytes = sb.rx, out_bytes = sb.out, total = sb.total;
    auto align = [](size_t v) { return (v + 255) & ~size_t(255); };
    USTB_REQUIRE(total <= (size_t)USTB_NOALLOC_SCRATCH_BYTES, USTB_E_SHAPE,
                 "this request needs %zu bytes of device scratch; the allocation-free entry point has "
                 "%zu (USTB_NOALLOC_SCRATCH_BYTES): use ustb_das_table_f32_host or split the pixels",
                 total, (size_t)USTB_NOALLOC_SCRATCH_BYTES);
    DeviceGuard dg;
    rc = dg.enter(device);
    if (rc) return rc;
    void* scratch = nullptr;
    rc = noalloc_scratch(device, &scratch);
    if (rc) return rc;
    char* p = static_cast<char*>(scratch);
    void* d_ch = p; p += align(ch_bytes);
    float* d_atx = (float*)p; p += align(tx_bytes);
    float* d_dtx = (float*)p; p += align(tx_bytes);
    float* d_arx = (float*)p; p += align(rx_bytes);
    float* d_drx = (float*)p; p += align(rx_bytes);
    void* d_out = p;
    // Every staged byte is overwritten below and the kernel writes every output
    // element, so nothing in the shared array needs clearing between calls.
    cudaStream_t s = cudaStreamPerThread;
    if (ch_bytes) USTB_CUDA(cudaMemcpyAsync(d_ch, ch, ch_bytes, cudaMemcpyHostToDevice, s));
    if (tx_bytes) USTB_CUDA(cudaMemcpyAsync(d_atx, apo_tx, tx_bytes, cudaMemcpyHostToDevice, s));
    if (tx_bytes) USTB_CUDA(cudaMemcpyAsync(d_dtx, delay_tx, tx_bytes, cudaMemcpyHostToDevice, s));
    if (rx_bytes) USTB_CUDA(cudaMemcpyAsync(d_arx, apo_rx, rx_bytes, cudaMemcpyHostToDevice, s));
    if (rx_bytes) USTB_CUDA(cudaMemcpyAsync(d_drx, delay_rx, rx_bytes, cudaMemcpyHostToDevice, s));
    rc = ustb_das_table_f32(d_ch, ch_complex, L, N, W, F, fs, t0, d_atx, d_arx, d_dtx, d_drx, P, fd,
                            dimension, d_out, s);
    if (rc) return rc;
    if (out_bytes) USTB_CUDA(cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, s));
    USTB_CUDA(cudaStreamSynchronize(s));
    return USTB_OK;
}
