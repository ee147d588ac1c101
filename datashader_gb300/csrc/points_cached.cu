// points_cached.cu -- Canvas.points count() with a shared-memory cache of the
// hottest canvas tiles.
//
// A plain count() is one increment per kept row.  Done as L2 atomics it is
// bound by the L2 atomic rate (about 2.3e11 scattered 32-bit reductions per
// second on GB300), and clustered data concentrates those atomics on a few
// L2 slices.  This path absorbs the densest part of the canvas on chip:
//
//   sample  -- bin ~1% of the rows (evenly spaced chunks) into a histogram of
//              tiles (16x16 px, 32x32 or 64x64 for large canvases); the last
//              block to finish picks the K most populated tiles that fit in
//              shared memory (a uint32 counter per pixel) and writes
//              tile -> slot;
//   main    -- one CTA per SM streams x/y (float4 loads), bins each row
//              (binning.cuh: exact), and increments the tile's shared-memory
//              counter when the tile is cached, the output with an L2
//              reduction otherwise; at the end every CTA adds its cached
//              tile rows into the output with TMA bulk reductions
//              (cp.reduce.async.bulk .add.u32, one per 16-pixel row), or with
//              per-pixel atomics when the canvas rows are not 16-byte
//              aligned.
//
// Every result is exact: integer counts in any order.
#include "dsgb_internal.cuh"
#include "binning.cuh"

namespace dsgb {

constexpr int SMEM_BUDGET = 220 * 1024;     // dynamic shared memory of the main kernel
constexpr int MAX_TABLE_TILES = 8192;       // tile -> slot table entries (16 KB)
constexpr int SAMPLE_BLOCKS = 128;
constexpr int SAMPLE_THREADS = 1024;
constexpr int SAMPLE_CHUNK = 8192;          // rows per sample block: two float4 of x and of y per thread
constexpr int MIN_ROWS = 1 << 20;           // below this the single kernel is as fast

struct CachedParams {
    const float *xs, *ys;
    int64_t n;
    int32_t width, height;
    int32_t ts;                 // tile side = 1 << ts
    int32_t tiles_x, ntiles;
    int32_t K;                  // cached tiles
    BinAxis ax, ay;
    BinBounds bb;
    uint32_t *out;
    unsigned *hist;             // ntiles, then the sample blocks' done counter
    short *slot;                // ntiles
    int *slot_tile;             // K
    int32_t bulk_flush;         // canvas rows 16-byte aligned: flush with bulk reductions
    const double *vs;           // mean: the value column (float64, 16-byte aligned)
    double *sum_out;            // mean: the float64 sum base (out is the count base)
};

__device__ __forceinline__ int tile_cells(const CachedParams &p) { return 1 << (2 * p.ts); }

// ---- select: smallest T with #(count > T) <= K; those tiles get slots.
// Runs in the last sample block; the counts stay in registers (ntiles <=
// MAX_TABLE_TILES = 8 per thread) and each bisection step costs one barrier.
constexpr int SEL_PER_THREAD = MAX_TABLE_TILES / SAMPLE_THREADS;

__device__ void select_tiles(const CachedParams &p) {
    __shared__ unsigned part[2][32];
    __shared__ unsigned s_next;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned c[SEL_PER_THREAD];
    unsigned mx = 0;
#pragma unroll
    for (int k = 0; k < SEL_PER_THREAD; ++k) {
        const int i = threadIdx.x + k * blockDim.x;
        c[k] = i < p.ntiles ? __ldcg(&p.hist[i]) : 0u;
        mx = max(mx, c[k]);
    }
    for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) part[0][warp] = mx;
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    unsigned lo = 0, hi = 0;
    for (int w = 0; w < nw; ++w) hi = max(hi, part[0][w]);
    // every thread runs the same bisection on the same block-wide sums
    for (int it = 0; lo < hi && it < 40; ++it) {
        const unsigned mid = lo + (hi - lo) / 2;
        unsigned cnt = 0;
#pragma unroll
        for (int k = 0; k < SEL_PER_THREAD; ++k) cnt += c[k] > mid;
        for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        const int b = 1 - (it & 1);          // part[0] held the maxima: start on part[1]
        if (lane == 0) part[b][warp] = cnt;
        __syncthreads();
        unsigned t = 0;
        for (int w = 0; w < nw; ++w) t += part[b][w];
        if (t <= (unsigned)p.K) hi = mid; else lo = mid + 1;
    }
    const unsigned T = hi;
    for (int i = threadIdx.x; i < p.K; i += blockDim.x) p.slot_tile[i] = -1;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SEL_PER_THREAD; ++k) {
        const int i = threadIdx.x + k * blockDim.x;
        if (i >= p.ntiles) continue;
        short s = -1;
        if (c[k] > T) {
            const unsigned q = atomicAdd(&s_next, 1u);
            if (q < (unsigned)p.K) { s = (short)q; p.slot_tile[q] = i; }
        }
        p.slot[i] = s;
    }
}

// ---- sample: tile histogram of evenly spaced chunks (float4 loads, all
// issued before any is used), then the last block to finish selects.
__global__ void __launch_bounds__(SAMPLE_THREADS) cached_sample(const CachedParams p, int64_t chunk) {
    extern __shared__ unsigned sh_hist[];
    __shared__ bool s_last;
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x) sh_hist[i] = 0;
    __syncthreads();
    const int64_t start = ((p.n / gridDim.x) * blockIdx.x) & ~(int64_t)3;
    const int64_t end = start + chunk < p.n ? start + chunk : p.n;
    const float4 *x4 = (const float4 *)p.xs;
    const float4 *y4 = (const float4 *)p.ys;
    const int64_t v1 = end >> 2;             // whole float4s of the chunk (a sample: the ragged end is skipped)
    for (int64_t v = (start >> 2) + threadIdx.x; v < v1; v += 2 * (int64_t)blockDim.x) {
        const bool two = v + blockDim.x < v1;
        const float4 a0 = __ldg(x4 + v), b0 = __ldg(y4 + v);
        float4 a1 = make_float4(0.f, 0.f, 0.f, 0.f), b1 = a1;
        if (two) { a1 = __ldg(x4 + v + blockDim.x); b1 = __ldg(y4 + v + blockDim.x); }
        const float xs[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float ys[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (k >= 4 && !two) break;
            int xi, yi;
            const int r = bin_try_f32(xs[k], ys[k], p.bb, p.ax, p.ay, xi, yi);
            if (r == 2) bin_exact_f32(xs[k], ys[k], p.ax, p.ay, xi, yi);
            if (r) atomicAdd(&sh_hist[(yi >> p.ts) * p.tiles_x + (xi >> p.ts)], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x)
        if (sh_hist[i]) atomicAdd(&p.hist[i], sh_hist[i]);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&p.hist[p.ntiles], 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    select_tiles(p);
}

// ---- main
__device__ __forceinline__ void cached_emit(const CachedParams &p, const short *tab, unsigned *cache, int xi, int yi) {
    const int s = tab[(yi >> p.ts) * p.tiles_x + (xi >> p.ts)];
    if (s >= 0) {
        const int tm = (1 << p.ts) - 1;
        atomicAdd(&cache[((unsigned)s << (2 * p.ts)) + ((unsigned)(yi & tm) << p.ts) + (unsigned)(xi & tm)], 1u);
    } else {
        atomicAdd(&p.out[(int64_t)yi * p.width + xi], 1u);
    }
}

__global__ void __launch_bounds__(1024, 1) cached_main(const CachedParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    short *tab = (short *)smem;
    const int tab_bytes = ((p.ntiles * 2) + 15) & ~15;
    unsigned *cache = (unsigned *)(smem + tab_bytes);
    const int tc = tile_cells(p);
    const int cells = p.K * tc;
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x) tab[i] = p.slot[i];
    for (int i = threadIdx.x; i < cells; i += blockDim.x) cache[i] = 0;
    __syncthreads();
    const float4 *x4 = (const float4 *)p.xs;
    const float4 *y4 = (const float4 *)p.ys;
    const int64_t n4 = p.n >> 2;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n4; v += 2 * stride) {
        const bool two = v + stride < n4;
        const float4 a0 = __ldcs(x4 + v), b0 = __ldcs(y4 + v);
        float4 a1 = make_float4(0.f, 0.f, 0.f, 0.f), b1 = a1;
        if (two) { a1 = __ldcs(x4 + v + stride); b1 = __ldcs(y4 + v + stride); }
        const float xs[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float ys[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
        int xi[8], yi[8];
        unsigned in = 0, need = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int r = (k < 4 || two) ? bin_try_f32(xs[k], ys[k], p.bb, p.ax, p.ay, xi[k], yi[k]) : 0;
            in |= (unsigned)(r != 0) << k;
            need |= (unsigned)(r == 2) << k;
        }
        if (need) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if ((need >> k) & 1u) bin_exact_f32(xs[k], ys[k], p.ax, p.ay, xi[k], yi[k]);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if ((in >> k) & 1u) cached_emit(p, tab, cache, xi[k], yi[k]);
    }
    // rows past the last full float4
    for (int64_t i = 4 * n4 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += stride) {
        int xi, yi;
        const int r = bin_try_f32(p.xs[i], p.ys[i], p.bb, p.ax, p.ay, xi, yi);
        if (r == 2) bin_exact_f32(p.xs[i], p.ys[i], p.ax, p.ay, xi, yi);
        if (r) cached_emit(p, tab, cache, xi, yi);
    }
    __syncthreads();
    if (p.bulk_flush) {
        // Each cached tile row (16 B-aligned in shared and global memory, a
        // multiple of 16 B long) is added into the output by one bulk
        // reduction.  Every thread orders its shared-memory atomics before
        // the async proxy reads them.
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        const int side = 1 << p.ts;
        bool issued = false;
        for (int r = threadIdx.x; r < p.K * side; r += blockDim.x) {
            const int slot = r >> p.ts, ry = r & (side - 1);
            const int t = p.slot_tile[slot];
            if (t < 0) continue;
            const int yi = (t / p.tiles_x) * side + ry;
            const int x0 = (t % p.tiles_x) * side;
            if (yi >= p.height) continue;
            const int ncols = p.width - x0 < side ? p.width - x0 : side;   // a multiple of 4
            const unsigned *src = cache + ((unsigned)slot << (2 * p.ts)) + ((unsigned)ry << p.ts);
            unsigned any = 0;
            for (int c = 0; c < ncols; c += 4) {
                const uint4 q = *(const uint4 *)(src + c);
                any |= q.x | q.y | q.z | q.w;
            }
            if (!any) continue;
            const unsigned saddr = (unsigned)__cvta_generic_to_shared(src);
            asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.u32 [%0], [%1], %2;"
                         :: "l"(p.out + (int64_t)yi * p.width + x0), "r"(saddr), "r"(ncols * 4) : "memory");
            issued = true;
        }
        if (issued) {
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
        return;
    }
    for (int i = threadIdx.x; i < cells; i += blockDim.x) {
        const unsigned c = cache[i];
        if (!c) continue;
        const int t = p.slot_tile[i >> (2 * p.ts)];
        const int within = i & (tc - 1);
        const int yi = (t / p.tiles_x) * (1 << p.ts) + (within >> p.ts);
        const int xi = (t % p.tiles_x) * (1 << p.ts) + (within & ((1 << p.ts) - 1));
        atomicAdd(&p.out[(int64_t)yi * p.width + xi], c);
    }
}

// ---- mean(v): float64 sums and uint32 counts of the hottest tiles in shared
// memory (12 bytes a pixel, so about a third of the tiles of count()).
// Rows whose value is NaN add nothing (reductions.py:1280-1297 with
// _sum_zero and _count_ignore_antialiasing).
__device__ __forceinline__ void mean_emit(const CachedParams &p, const short *tab, double *ssum, unsigned *scnt,
                                          int xi, int yi, double v) {
    const int s = tab[(yi >> p.ts) * p.tiles_x + (xi >> p.ts)];
    if (s >= 0) {
        const int tm = (1 << p.ts) - 1;
        const unsigned c = ((unsigned)s << (2 * p.ts)) + ((unsigned)(yi & tm) << p.ts) + (unsigned)(xi & tm);
        atomicAdd(&ssum[c], v);
        atomicAdd(&scnt[c], 1u);
    } else {
        const int64_t pix = (int64_t)yi * p.width + xi;
        atomicAdd(&p.sum_out[pix], v);
        atomicAdd(&p.out[pix], 1u);
    }
}

__global__ void __launch_bounds__(1024, 1) cached_mean_main(const CachedParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    short *tab = (short *)smem;
    const int tab_bytes = ((p.ntiles * 2) + 15) & ~15;
    const int tc = tile_cells(p);
    const int cells = p.K * tc;
    double *ssum = (double *)(smem + tab_bytes);
    unsigned *scnt = (unsigned *)(ssum + cells);
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x) tab[i] = p.slot[i];
    for (int i = threadIdx.x; i < cells; i += blockDim.x) { ssum[i] = 0.0; scnt[i] = 0u; }
    __syncthreads();
    const float4 *x4 = (const float4 *)p.xs;
    const float4 *y4 = (const float4 *)p.ys;
    const double2 *v2 = (const double2 *)p.vs;
    const int64_t n4 = p.n >> 2;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n4; v += stride) {
        const float4 a = __ldcs(x4 + v), b = __ldcs(y4 + v);
        const double2 w0 = __ldcs(v2 + 2 * v), w1 = __ldcs(v2 + 2 * v + 1);
        const float xs[4] = {a.x, a.y, a.z, a.w};
        const float ys[4] = {b.x, b.y, b.z, b.w};
        const double vs[4] = {w0.x, w0.y, w1.x, w1.y};
        int xi[4], yi[4];
        unsigned in = 0, need = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int r = isnull(vs[k]) ? 0 : bin_try_f32(xs[k], ys[k], p.bb, p.ax, p.ay, xi[k], yi[k]);
            in |= (unsigned)(r != 0) << k;
            need |= (unsigned)(r == 2) << k;
        }
        if (need) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if ((need >> k) & 1u) bin_exact_f32(xs[k], ys[k], p.ax, p.ay, xi[k], yi[k]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if ((in >> k) & 1u) mean_emit(p, tab, ssum, scnt, xi[k], yi[k], vs[k]);
    }
    for (int64_t i = 4 * n4 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += stride) {
        const double vv = p.vs[i];
        if (isnull(vv)) continue;
        int xi, yi;
        const int r = bin_try_f32(p.xs[i], p.ys[i], p.bb, p.ax, p.ay, xi, yi);
        if (r == 2) bin_exact_f32(p.xs[i], p.ys[i], p.ax, p.ay, xi, yi);
        if (r) mean_emit(p, tab, ssum, scnt, xi, yi, vv);
    }
    __syncthreads();
    if (p.bulk_flush) {
        // one bulk reduction per cached tile row and array (add.f64 sums, add.u32 counts)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        const int side = 1 << p.ts;
        bool issued = false;
        for (int r = threadIdx.x; r < p.K * side; r += blockDim.x) {
            const int slot = r >> p.ts, ry = r & (side - 1);
            const int t = p.slot_tile[slot];
            if (t < 0) continue;
            const int yi = (t / p.tiles_x) * side + ry;
            const int x0 = (t % p.tiles_x) * side;
            if (yi >= p.height) continue;
            const int ncols = p.width - x0 < side ? p.width - x0 : side;   // a multiple of 4
            const unsigned off = ((unsigned)slot << (2 * p.ts)) + ((unsigned)ry << p.ts);
            unsigned any = 0;
            for (int c = 0; c < ncols; c += 4) {
                const uint4 q = *(const uint4 *)(scnt + off + c);
                any |= q.x | q.y | q.z | q.w;
            }
            if (!any) continue;
            const int64_t g = (int64_t)yi * p.width + x0;
            asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.u32 [%0], [%1], %2;"
                         :: "l"(p.out + g), "r"((unsigned)__cvta_generic_to_shared(scnt + off)), "r"(ncols * 4)
                         : "memory");
            asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f64 [%0], [%1], %2;"
                         :: "l"(p.sum_out + g), "r"((unsigned)__cvta_generic_to_shared(ssum + off)), "r"(ncols * 8)
                         : "memory");
            issued = true;
        }
        if (issued) {
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
        return;
    }
    for (int i = threadIdx.x; i < cells; i += blockDim.x) {
        const unsigned c = scnt[i];
        if (!c) continue;
        const int t = p.slot_tile[i >> (2 * p.ts)];
        const int within = i & (tc - 1);
        const int yi = (t / p.tiles_x) * (1 << p.ts) + (within >> p.ts);
        const int xi = (t % p.tiles_x) * (1 << p.ts) + (within & ((1 << p.ts) - 1));
        const int64_t pix = (int64_t)yi * p.width + xi;
        atomicAdd(&p.out[pix], c);
        atomicAdd(&p.sum_out[pix], ssum[i]);
    }
}

// ------------------------------------------------------------- host side

struct CachedLayout {
    int ts, tiles_x, ntiles, K, grid;
    size_t off_hist, off_slot, off_slot_tile, total;
};

static size_t align256(size_t v) { return (v + 255) / 256 * 256; }

static bool cached_layout(int64_t n, int width, int height, CachedLayout &L, int px_bytes = 4) {
    if (n < MIN_ROWS || width <= 0 || height <= 0) return false;
    int ts = 4;
    while (ts <= 6) {
        const int64_t tx = (width + (1 << ts) - 1) >> ts, ty = (height + (1 << ts) - 1) >> ts;
        if (tx * ty <= MAX_TABLE_TILES) break;
        ++ts;
    }
    if (ts > 6) return false;
    L.ts = ts;
    L.tiles_x = (width + (1 << ts) - 1) >> ts;
    L.ntiles = L.tiles_x * ((height + (1 << ts) - 1) >> ts);
    const int tab = ((L.ntiles * 2) + 15) & ~15;
    const int tile_bytes = (1 << (2 * ts)) * px_bytes;
    L.K = (SMEM_BUDGET - tab) / tile_bytes;
    if (L.K > L.ntiles) L.K = L.ntiles;
    if (L.K < 1) return false;
    const int sms = sm_count();
    L.grid = sms > 0 ? sms : 148;
    size_t o = 0;
    L.off_hist = o; o = align256(o + (size_t)L.ntiles * 4 + 4);     // + the done counter
    L.off_slot = o; o = align256(o + (size_t)L.ntiles * 2);
    L.off_slot_tile = o; o = align256(o + (size_t)L.K * 4);
    L.total = o;
    return true;
}

size_t cached_workspace_size(int64_t n, int width, int height) {
    CachedLayout L;
    return cached_layout(n, width, height, L) ? L.total : 0;
}

// DSGB_E_UNSUPPORTED when not eligible (the caller then runs the plain kernel).
int launch_points_cached(const ColumnRef &xc, const ColumnRef &yc, int64_t n, const dsgb_canvas *cv,
                         const BinAxis &ax, const BinAxis &ay, const BinBounds &bb,
                         uint32_t *out, bool accumulate, void *ws, size_t ws_bytes, cudaStream_t st) {
    if (xc.dtype != DSGB_F32 || yc.dtype != DSGB_F32) return DSGB_E_UNSUPPORTED;
    if (((uintptr_t)xc.data | (uintptr_t)yc.data) & 15u) return DSGB_E_UNSUPPORTED;
    if (!ws || ((uintptr_t)ws & 255u)) return DSGB_E_UNSUPPORTED;
    CachedLayout L;
    if (!cached_layout(n, cv->width, cv->height, L) || ws_bytes < L.total) return DSGB_E_UNSUPPORTED;
    CachedParams p;
    memset(&p, 0, sizeof(p));
    p.xs = (const float *)xc.data; p.ys = (const float *)yc.data; p.n = n;
    p.width = cv->width; p.height = cv->height;
    p.ts = L.ts; p.tiles_x = L.tiles_x; p.ntiles = L.ntiles; p.K = L.K;
    p.ax = ax; p.ay = ay; p.bb = bb;
    p.out = out;
    char *w = (char *)ws;
    p.hist = (unsigned *)(w + L.off_hist);
    p.slot = (short *)(w + L.off_slot);
    p.slot_tile = (int *)(w + L.off_slot_tile);
    p.bulk_flush = (cv->width % 4 == 0) && (((uintptr_t)out & 15u) == 0);
    cudaError_t e = cudaMemsetAsync(p.hist, 0, (size_t)L.ntiles * 4 + 4, st);
    if (e == cudaSuccess && !accumulate) e = cudaMemsetAsync(out, 0, (size_t)cv->width * cv->height * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "cached count memset");
    const int64_t chunk = SAMPLE_CHUNK < n / SAMPLE_BLOCKS ? SAMPLE_CHUNK : n / SAMPLE_BLOCKS;
    cached_sample<<<SAMPLE_BLOCKS, SAMPLE_THREADS, (size_t)L.ntiles * 4, st>>>(p, chunk);
    const size_t smem = (((size_t)L.ntiles * 2 + 15) & ~(size_t)15) + (size_t)L.K * (1 << (2 * L.ts)) * 4;
    e = cudaFuncSetAttribute(cached_main, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "cached count smem attribute");
    cached_main<<<L.grid, 1024, smem, st>>>(p);
    DSGB_CHECK_LAUNCH("cached count launch");
    return DSGB_OK;
}

}  // namespace dsgb

namespace dsgb {

// mean('v') of float32 coordinates and a float64 value column, all 16-byte
// aligned; `sum` and `count` are the SUM and COUNT bases.  The workspace of
// the count path is large enough (it keeps more tiles).
int launch_points_cached_mean(const ColumnRef &xc, const ColumnRef &yc, const ColumnRef &vc, int64_t n,
                              const dsgb_canvas *cv, const BinAxis &ax, const BinAxis &ay, const BinBounds &bb,
                              double *sum, uint32_t *count, bool accumulate, void *ws, size_t ws_bytes,
                              cudaStream_t st) {
    if (xc.dtype != DSGB_F32 || yc.dtype != DSGB_F32 || vc.dtype != DSGB_F64) return DSGB_E_UNSUPPORTED;
    if (((uintptr_t)xc.data | (uintptr_t)yc.data | (uintptr_t)vc.data) & 15u) return DSGB_E_UNSUPPORTED;
    if (!ws || ((uintptr_t)ws & 255u)) return DSGB_E_UNSUPPORTED;
    CachedLayout Lc, L;
    if (!cached_layout(n, cv->width, cv->height, Lc) || ws_bytes < Lc.total) return DSGB_E_UNSUPPORTED;
    if (!cached_layout(n, cv->width, cv->height, L, 12)) return DSGB_E_UNSUPPORTED;
    CachedParams p;
    memset(&p, 0, sizeof(p));
    p.xs = (const float *)xc.data; p.ys = (const float *)yc.data; p.vs = (const double *)vc.data; p.n = n;
    p.width = cv->width; p.height = cv->height;
    p.ts = L.ts; p.tiles_x = L.tiles_x; p.ntiles = L.ntiles; p.K = L.K;
    p.ax = ax; p.ay = ay; p.bb = bb;
    p.out = count;
    p.sum_out = sum;
    char *w = (char *)ws;
    p.hist = (unsigned *)(w + Lc.off_hist);
    p.slot = (short *)(w + Lc.off_slot);
    p.slot_tile = (int *)(w + Lc.off_slot_tile);
    p.bulk_flush = (cv->width % 4 == 0) && ((((uintptr_t)count | (uintptr_t)sum) & 15u) == 0);
    const size_t cells = (size_t)cv->width * cv->height;
    cudaError_t e = cudaMemsetAsync(p.hist, 0, (size_t)L.ntiles * 4 + 4, st);
    if (e == cudaSuccess && !accumulate) e = cudaMemsetAsync(count, 0, cells * 4, st);
    if (e == cudaSuccess && !accumulate) e = cudaMemsetAsync(sum, 0, cells * 8, st);
    if (e != cudaSuccess) return cuda_status(e, "cached mean memset");
    const int64_t chunk = SAMPLE_CHUNK < n / SAMPLE_BLOCKS ? SAMPLE_CHUNK : n / SAMPLE_BLOCKS;
    cached_sample<<<SAMPLE_BLOCKS, SAMPLE_THREADS, (size_t)L.ntiles * 4, st>>>(p, chunk);
    const size_t smem = (((size_t)L.ntiles * 2 + 15) & ~(size_t)15) + (size_t)L.K * (1 << (2 * L.ts)) * 12;
    e = cudaFuncSetAttribute(cached_mean_main, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "cached mean smem attribute");
    cached_mean_main<<<L.grid, 1024, smem, st>>>(p);
    DSGB_CHECK_LAUNCH("cached mean launch");
    return DSGB_OK;
}

}  // namespace dsgb
