// Resident plans: one acquisition's geometry copied to the device once, with a tile
// map planned here when the caller gives none.
//
// Tile planning (host): pixels are grouped into tiles of USTB_TILE_PIXELS so that
// every channel's and wave's sample window over a tile stays short.  On a pixel
// grid, the grid is cut into blocks whose physical extents are as even as the
// pixel spacings allow (product <= 512), and every block whose bounding-box
// diagonal exceeds kSpanLimit samples of one-way travel is halved along its longest
// axis until it fits.  Without a grid the pixels are ordered on a coarse spatial
// grid and cut into runs of 512 that are split the same way.  Tiles are then
// handed out most receive channels first (the kernel's own bounding-box rule for
// the receive window), and, when some waves take their delays from the table,
// tiles whose tabulated transmit delays span too many samples are halved again.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace {

constexpr int kTile = USTB_TILE_PIXELS;
constexpr double kSpanLimit = 74.0;  // samples of one-way travel across a tile

struct Pts {
    const float* xyz;
    double x(int64_t i, int a) const { return (double)xyz[3 * i + a]; }
};

// bounding-box diagonal of a set of pixels (m)
double diag(const Pts& p, const int32_t* idx, size_t n) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p.x(idx[i], a));
            hi[a] = std::max(hi[a], p.x(idx[i], a));
        }
    return std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                     (hi[2] - lo[2]) * (hi[2] - lo[2]));
}

// a box of pixel indices over the grid's axes (i, j, k), stored with the LAST axis
// fastest: this is also the order of the tile's lanes, so the warps of a 2D grid
// run along its lateral axis (warps along depth measured 17-20 % slower on the
// plane-wave and sector workloads)
struct Box {
    std::vector<int32_t> idx;
    int64_t d[3];
    int32_t at(int64_t i, int64_t j, int64_t k) const { return idx[(i * d[1] + j) * d[2] + k]; }
};

Box sub_box(const Box& b, int ax, int64_t from, int64_t to) {
    Box o;
    for (int a = 0; a < 3; ++a) o.d[a] = b.d[a];
    o.d[ax] = to - from;
    o.idx.reserve((size_t)(o.d[0] * o.d[1] * o.d[2]));
    for (int64_t i = 0; i < o.d[0]; ++i)
        for (int64_t j = 0; j < o.d[1]; ++j)
            for (int64_t k = 0; k < o.d[2]; ++k) {
                const int64_t c[3] = {i + (ax == 0 ? from : 0), j + (ax == 1 ? from : 0), k + (ax == 2 ? from : 0)};
                o.idx.push_back(b.at(c[0], c[1], c[2]));
            }
    return o;
}

// mean position of the slice at index s along axis ax
void slice_mean(const Pts& p, const Box& b, int ax, int64_t s, double m[3]) {
    m[0] = m[1] = m[2] = 0.0;
    int64_t n = 0;
    const int64_t e0 = ax == 0 ? 1 : b.d[0], e1 = ax == 1 ? 1 : b.d[1], e2 = ax == 2 ? 1 : b.d[2];
    for (int64_t k = 0; k < e2; ++k)
        for (int64_t j = 0; j < e1; ++j)
            for (int64_t i = 0; i < e0; ++i) {
                const int32_t q = b.at(ax == 0 ? s : i, ax == 1 ? s : j, ax == 2 ? s : k);
                for (int a = 0; a < 3; ++a) m[a] += p.x(q, a);
                ++n;
            }
    for (int a = 0; a < 3; ++a) m[a] /= (double)std::max<int64_t>(n, 1);
}

// halve boxes along their longest physical axis until each fits the span limit
void split_boxes(const Pts& p, Box root, double limit, std::vector<std::vector<int32_t>>& out) {
    std::vector<Box> stack;
    stack.push_back(std::move(root));
    while (!stack.empty()) {
        Box b = std::move(stack.back());
        stack.pop_back();
        if (b.idx.empty()) continue;
        if (b.idx.size() == 1 || diag(p, b.idx.data(), b.idx.size()) <= limit) {
            out.push_back(std::move(b.idx));
            continue;
        }
        int best = -1;
        double ext = -1.0;
        for (int ax = 0; ax < 3; ++ax) {
            if (b.d[ax] < 2) continue;
            double m0[3], m1[3];
            slice_mean(p, b, ax, 0, m0);
            slice_mean(p, b, ax, b.d[ax] - 1, m1);
            const double e = std::sqrt((m1[0] - m0[0]) * (m1[0] - m0[0]) + (m1[1] - m0[1]) * (m1[1] - m0[1]) +
                                       (m1[2] - m0[2]) * (m1[2] - m0[2]));
            if (e > ext) {
                ext = e;
                best = ax;
            }
        }
        if (best < 0) {  // no axis with a finite extent to halve: keep the box whole
            out.push_back(std::move(b.idx));
            continue;
        }
        const int64_t h = b.d[best] / 2;
        stack.push_back(sub_box(b, best, 0, h));
        stack.push_back(sub_box(b, best, h, b.d[best]));
    }
}

// block shape (product <= kTile) that balances the physical extents: double the
// axis whose extent is smallest while it fits the grid
void block_dims(const double sp[3], const int64_t shape[3], int64_t bd[3]) {
    bd[0] = bd[1] = bd[2] = 1;
    for (;;) {
        int bi = -1;
        double best = 0.0;
        for (int a = 0; a < 3; ++a) {
            if (bd[0] * bd[1] * bd[2] * 2 > kTile || bd[a] >= shape[a]) continue;
            const double e = (double)bd[a] * std::max(sp[a], 1e-12);
            if (bi < 0 || e < best) {
                best = e;
                bi = a;
            }
        }
        if (bi < 0) return;
        bd[bi] *= 2;
    }
}

std::vector<std::vector<int32_t>> plan_blocks(const Pts& p, int64_t P, const int64_t grid[3], double limit) {
    std::vector<std::vector<int32_t>> blocks;
    const bool have_grid = grid[0] > 0 && grid[1] > 0 && grid[2] > 0 && grid[0] * grid[1] * grid[2] == P;
    if (have_grid) {
        // spacing per axis: the largest neighbour distance along it (the outer
        // azimuth step of a sector, the pitch of a linear grid)
        double sp[3] = {0.0, 0.0, 0.0};
        const int64_t stride[3] = {1, grid[0], grid[0] * grid[1]};
        for (int a = 0; a < 3; ++a) {
            if (grid[a] < 2) continue;
            for (int64_t i = 0; i < P; ++i) {
                const int64_t c = (i / stride[a]) % grid[a];
                if (c + 1 >= grid[a]) continue;
                const int64_t q = i + stride[a];
                const double dx = p.x(q, 0) - p.x(i, 0), dy = p.x(q, 1) - p.x(i, 1), dz = p.x(q, 2) - p.x(i, 2);
                sp[a] = std::max(sp[a], std::sqrt(dx * dx + dy * dy + dz * dz));
            }
        }
        int64_t bd[3];
        block_dims(sp, grid, bd);
        for (int64_t i0 = 0; i0 < grid[0]; i0 += bd[0])
            for (int64_t j0 = 0; j0 < grid[1]; j0 += bd[1])
                for (int64_t k0 = 0; k0 < grid[2]; k0 += bd[2]) {
                    Box b;
                    b.d[0] = std::min(bd[0], grid[0] - i0);
                    b.d[1] = std::min(bd[1], grid[1] - j0);
                    b.d[2] = std::min(bd[2], grid[2] - k0);
                    b.idx.reserve((size_t)(b.d[0] * b.d[1] * b.d[2]));
                    for (int64_t i = 0; i < b.d[0]; ++i)
                        for (int64_t j = 0; j < b.d[1]; ++j)
                            for (int64_t k = 0; k < b.d[2]; ++k)
                                b.idx.push_back((int32_t)((i0 + i) + grid[0] * ((j0 + j) + grid[1] * (k0 + k))));
                    split_boxes(p, std::move(b), limit, blocks);
                }
        return blocks;
    }
    // no grid: order on a coarse spatial grid (cells of half the limit; y, then x,
    // then z), cut into runs of kTile and split those
    double lo[3] = {1e300, 1e300, 1e300};
    for (int64_t i = 0; i < P; ++i)
        for (int a = 0; a < 3; ++a) lo[a] = std::min(lo[a], p.x(i, a));
    const double cell = std::max(limit / 2, 1e-12);
    std::vector<int64_t> key((size_t)P * 3);
    for (int64_t i = 0; i < P; ++i)
        for (int a = 0; a < 3; ++a) key[3 * i + a] = (int64_t)std::floor((p.x(i, a) - lo[a]) / cell);
    std::vector<int32_t> order((size_t)P);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t u, int32_t v) {
        if (key[3 * u + 1] != key[3 * v + 1]) return key[3 * u + 1] < key[3 * v + 1];
        if (key[3 * u + 0] != key[3 * v + 0]) return key[3 * u + 0] < key[3 * v + 0];
        return key[3 * u + 2] < key[3 * v + 2];
    });
    for (int64_t s = 0; s < P; s += kTile) {
        Box b;
        b.d[0] = std::min<int64_t>(kTile, P - s);
        b.d[1] = b.d[2] = 1;
        b.idx.assign(order.begin() + s, order.begin() + s + b.d[0]);
        split_boxes(p, std::move(b), limit, blocks);
    }
    return blocks;
}

// split tiles whose tabulated transmit delays (waves of kind TABLE) span more than
// the limit, halving their pixel lists
void refine_by_table(std::vector<std::vector<int32_t>>& blocks, const ustb_das_geometry& g, int64_t P) {
    std::vector<int64_t> tw;
    for (int64_t w = 0; w < g.n_waves; ++w)
        if (g.waves[w].kind == USTB_WAVE_TABLE) tw.push_back(w);
    if (tw.empty()) return;
    std::vector<std::vector<int32_t>> out, stack(std::move(blocks));
    while (!stack.empty()) {
        std::vector<int32_t> b = std::move(stack.back());
        stack.pop_back();
        if (b.empty()) continue;
        double span = 0.0;
        for (int64_t w : tw) {
            double lo = 1e300, hi = -1e300;
            for (int32_t q : b) {
                const double t = (double)g.tx_delay_table[w * P + q] * g.fs;
                lo = std::min(lo, t);
                hi = std::max(hi, t);
            }
            span = std::max(span, hi - lo);
        }
        if (span <= kSpanLimit || b.size() == 1) {
            out.push_back(std::move(b));
            continue;
        }
        const size_t h = b.size() / 2;
        stack.emplace_back(b.begin(), b.begin() + h);
        stack.emplace_back(b.begin() + h, b.end());
    }
    blocks = std::move(out);
}

// most expensive tiles first: cost = channels whose receive window may be nonzero
// over the tile's bounding box (the kernel's rx_active rule)
void order_by_cost(std::vector<std::vector<int32_t>>& blocks, const ustb_das_geometry& g) {
    if (blocks.size() < 2 || g.rx_window == USTB_WIN_NONE || g.rx_apo_table || g.rx_use_origin) return;
    const Pts p{g.pixel_xyz};
    std::vector<int64_t> cost(blocks.size(), 0);
    for (size_t t = 0; t < blocks.size(); ++t) {
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int32_t q : blocks[t])
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], p.x(q, a));
                hi[a] = std::max(hi[a], p.x(q, a));
            }
        for (int64_t n = 0; n < g.n_elements; ++n) {
            const double ex = g.element_xyz[3 * n], ey = g.element_xyz[3 * n + 1], ez = g.element_xyz[3 * n + 2];
            const double xd = std::max(0.0, std::max(lo[0] - ex, ex - hi[0]));
            const double yd = std::max(0.0, std::max(lo[1] - ey, ey - hi[1]));
            const double zmax = std::max(std::fabs(lo[2] - ez), std::fabs(hi[2] - ez));
            const double zx = std::min(std::max(zmax, (double)g.rx_min_aperture[0] * g.rx_f_number[0]),
                                       (double)g.rx_max_aperture[0] * g.rx_f_number[0]);
            const double zy = std::min(std::max(zmax, (double)g.rx_min_aperture[1] * g.rx_f_number[1]),
                                       (double)g.rx_max_aperture[1] * g.rx_f_number[1]);
            const bool off = (zx > 0 && g.rx_f_number[0] * xd / zx > 0.5) || (zy > 0 && g.rx_f_number[1] * yd / zy > 0.5);
            cost[t] += off ? 0 : 1;
        }
    }
    std::vector<size_t> perm(blocks.size());
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<std::vector<int32_t>> o;
    o.reserve(blocks.size());
    for (size_t i : perm) o.push_back(std::move(blocks[i]));
    blocks = std::move(o);
}

// device copy of a host array (nullptr for a null source)
template <typename T>
int upload(const T* src, size_t n, T** dst, std::vector<void*>& owned) {
    *dst = nullptr;
    if (!src || n == 0) return USTB_OK;
    void* d = nullptr;
    USTB_CUDA(cudaMalloc(&d, n * sizeof(T)));
    owned.push_back(d);
    USTB_CUDA(cudaMemcpy(d, src, n * sizeof(T), cudaMemcpyHostToDevice));
    *dst = static_cast<T*>(d);
    return USTB_OK;
}

}  // namespace

struct ustb_plan_s {
    ustb_das_geometry g;  // device pointers
    int64_t L, F;
    int32_t storage, is_complex, dimension, epilogue;
    int device;
    std::vector<void*> owned;
    ~ustb_plan_s() {
        for (void* p : owned) cudaFree(p);
    }
};

// checks a descriptor and builds (or checks) its tile map; host only
static int plan_tiles(const ustb_plan_desc* d, std::vector<int32_t>& tiles, int64_t& T) {
    USTB_REQUIRE(d, USTB_E_ARG, "NULL pointer");
    const ustb_das_geometry& h = d->geometry;
    USTB_REQUIRE(h.element_xyz && h.pixel_xyz && h.waves, USTB_E_ARG, "geometry needs element, pixel and wave arrays");
    USTB_REQUIRE(h.n_elements >= 1 && h.n_pixels >= 1 && h.n_waves >= 1, USTB_E_SHAPE, "empty geometry");
    USTB_REQUIRE(h.n_pixels < INT32_MAX, USTB_E_SHAPE, "at most 2^31 - 1 pixels");
    USTB_REQUIRE(d->L >= 2 && d->F >= 1, USTB_E_SHAPE, "need L >= 2 samples and F >= 1 frames");
    USTB_REQUIRE(d->storage >= 0 && d->storage <= 2, USTB_E_DTYPE, "unknown storage type %d", (int)d->storage);
    USTB_REQUIRE(d->dimension >= 0 && d->dimension <= 3, USTB_E_ARG, "dimension must be in [0, 3]");
    USTB_REQUIRE(d->is_complex || h.fd == 0.f, USTB_E_DTYPE, "real channel data with a modulation frequency");
    USTB_REQUIRE(!d->epilogue || (d->is_complex && d->dimension == USTB_DIM_TRANSMIT), USTB_E_ARG,
                 "the epilogue needs complex data and dimension.transmit");
    USTB_REQUIRE(h.fs > 0.f && h.sound_speed > 0.f, USTB_E_ARG, "fs and sound speed must be > 0");
    for (int64_t i = 0; i < 3 * h.n_pixels; ++i)
        USTB_REQUIRE(std::isfinite(h.pixel_xyz[i]), USTB_E_ARG, "pixel %lld has a non-finite coordinate",
                     (long long)(i / 3));
    for (int64_t i = 0; i < 3 * h.n_elements; ++i)
        USTB_REQUIRE(std::isfinite(h.element_xyz[i]), USTB_E_ARG, "element %lld has a non-finite coordinate",
                     (long long)(i / 3));
    bool tables = false;
    for (int64_t w = 0; w < h.n_waves; ++w) {
        USTB_REQUIRE(h.waves[w].kind >= 0 && h.waves[w].kind <= 3, USTB_E_ARG, "wave %lld: unknown kind",
                     (long long)w);
        tables |= h.waves[w].kind == USTB_WAVE_TABLE;
    }
    USTB_REQUIRE(!tables || h.tx_delay_table, USTB_E_ARG, "table waves need tx_delay_table");
    const int64_t P = h.n_pixels;
    const int64_t* gr = d->pixel_grid;
    USTB_REQUIRE((gr[0] == 0 && gr[1] == 0 && gr[2] == 0) || (gr[0] > 0 && gr[1] > 0 && gr[2] > 0 && gr[0] * gr[1] * gr[2] == P),
                 USTB_E_SHAPE, "pixel_grid must multiply to n_pixels (or be all zero)");
    tiles.clear();
    T = 0;
    if (h.tile_pixels) {
        T = h.n_tiles;
        USTB_REQUIRE(T >= 1, USTB_E_SHAPE, "tile_pixels given with n_tiles < 1");
        tiles.assign(h.tile_pixels, h.tile_pixels + T * kTile);
        for (int64_t t = 0; t < T; ++t) {
            USTB_REQUIRE(tiles[t * kTile] >= 0 && tiles[t * kTile] < P, USTB_E_ARG, "tile %lld: lane 0 is idle",
                         (long long)t);
            for (int j = 0; j < kTile; ++j)
                USTB_REQUIRE(tiles[t * kTile + j] >= -1 && tiles[t * kTile + j] < P, USTB_E_ARG,
                             "tile %lld lane %d: pixel index out of range", (long long)t, j);
        }
        return USTB_OK;
    }
    const Pts p{h.pixel_xyz};
    const double limit = kSpanLimit * (double)h.sound_speed / (double)h.fs;
    std::vector<std::vector<int32_t>> blocks = plan_blocks(p, P, gr, limit);
    refine_by_table(blocks, h, P);
    order_by_cost(blocks, h);
    T = (int64_t)blocks.size();
    tiles.assign((size_t)(T * kTile), -1);
    for (int64_t t = 0; t < T; ++t) std::copy(blocks[t].begin(), blocks[t].end(), tiles.begin() + t * kTile);
    return USTB_OK;
}

extern "C" int64_t ustb_plan_tiles_host(const ustb_plan_desc* d, int32_t* out, int64_t capacity) {
    ustb::clear_error();
    std::vector<int32_t> tiles;
    int64_t T = 0;
    const int rc = plan_tiles(d, tiles, T);
    if (rc != USTB_OK) return -rc;
    if (out) std::copy(tiles.begin(), tiles.begin() + std::min(T, std::max<int64_t>(capacity, 0)) * kTile, out);
    return T;
}

extern "C" int ustb_plan_create(const ustb_plan_desc* d, ustb_plan* out) {
    ustb::clear_error();
    USTB_REQUIRE(d && out, USTB_E_ARG, "NULL pointer");
    *out = nullptr;
    std::vector<int32_t> tiles;
    int64_t T = 0;
    const int prc = plan_tiles(d, tiles, T);
    if (prc != USTB_OK) return prc;
    const ustb_das_geometry& h = d->geometry;
    const int64_t P = h.n_pixels, N = h.n_elements, W = h.n_waves;

    std::unique_ptr<ustb_plan_s> pl(new ustb_plan_s());
    USTB_CUDA(cudaGetDevice(&pl->device));
    pl->g = h;
    pl->L = d->L;
    pl->F = d->F;
    pl->storage = d->storage;
    pl->is_complex = d->is_complex;
    pl->dimension = d->dimension;
    pl->epilogue = d->epilogue;
    int rc;
    float* f = nullptr;
    if ((rc = upload(h.element_xyz, (size_t)(3 * N), &f, pl->owned))) return rc;
    pl->g.element_xyz = f;
    if ((rc = upload(h.pixel_xyz, (size_t)(3 * P), &f, pl->owned))) return rc;
    pl->g.pixel_xyz = f;
    int32_t* ti = nullptr;
    if ((rc = upload(tiles.data(), tiles.size(), &ti, pl->owned))) return rc;
    pl->g.tile_pixels = ti;
    pl->g.n_tiles = T;
    ustb_wave* wv = nullptr;
    if ((rc = upload(h.waves, (size_t)W, &wv, pl->owned))) return rc;
    pl->g.waves = wv;
    if ((rc = upload(h.tx_delay_table, h.tx_delay_table ? (size_t)(P * W) : 0, &f, pl->owned))) return rc;
    pl->g.tx_delay_table = f;
    if ((rc = upload(h.tx_apo_table, h.tx_apo_table ? (size_t)(P * W) : 0, &f, pl->owned))) return rc;
    pl->g.tx_apo_table = f;
    if ((rc = upload(h.rx_apo_table, h.rx_apo_table ? (size_t)(P * N) : 0, &f, pl->owned))) return rc;
    pl->g.rx_apo_table = f;
    if ((rc = upload(h.pixel_phase, h.pixel_phase ? (size_t)(2 * P) : 0, &f, pl->owned))) return rc;
    pl->g.pixel_phase = f;
    *out = pl.release();
    return USTB_OK;
}

extern "C" int ustb_plan_destroy(ustb_plan plan) {
    ustb::clear_error();
    USTB_REQUIRE(plan, USTB_E_ARG, "NULL plan");
    delete plan;
    return USTB_OK;
}

extern "C" int64_t ustb_plan_tiles(ustb_plan plan) {
    ustb::clear_error();
    USTB_REQUIRE(plan, -USTB_E_ARG, "NULL plan");
    return plan->g.n_tiles;
}

extern "C" int ustb_plan_execute(ustb_plan plan, const void* ch, const ustb_das_outputs* out, uint32_t* flags,
                                 void* stream) {
    ustb::clear_error();
    USTB_REQUIRE(plan && ch && out, USTB_E_ARG, "NULL pointer");
    return ustb_das_fast(ch, plan->storage, plan->is_complex, plan->L, plan->g.n_elements, plan->g.n_waves, plan->F,
                         &plan->g, plan->dimension, plan->epilogue, out, flags, stream);
}

// request description of a plan for a batched launch (used by the server)
namespace ustb {
void plan_request(ustb_plan plan, const void* ch, const ustb_das_outputs* out, ustb_das_request* r) {
    r->ch = ch;
    r->storage = plan->storage;
    r->is_complex = plan->is_complex;
    r->L = plan->L;
    r->N = plan->g.n_elements;
    r->W = plan->g.n_waves;
    r->F = plan->F;
    r->geometry = &plan->g;
    r->dimension = plan->dimension;
    r->epilogue = plan->epilogue;
    r->out = out;
}
}  // namespace ustb
