// points_cached.cu -- Canvas.points count() with a shared-memory cache of the
// hottest canvas tiles.
//
// A plain count() is one increment per kept row.  Done as L2 atomics it is
// bound by the L2 atomic rate (about 2.3e11 scattered 32-bit reductions per
// second on GB300), and clustered data concentrates those atomics on a few
// L2 slices.  This path absorbs the densest part of the canvas on chip:
//
//   sample  -- bin ~1% of the rows (evenly spaced chunks) into a histogram of
//              tiles (16x16 px, 32x32 or 64x64 for large canvases);
//   select  -- one block picks the K most populated tiles that fit in shared
//              memory (a uint32 counter per pixel) and writes tile -> slot;
//   main    -- one CTA per SM streams x/y (float4 loads), bins each row
//              (binning.cuh: exact), and increments the tile's shared-memory
//              counter when the tile is cached, the output with an L2
//              reduction otherwise; at the end every CTA adds its non-zero
//              cached counters into the output.
//
// Every result is exact: integer counts in any order.
#include "dsgb_internal.cuh"
#include "binning.cuh"

namespace dsgb {

constexpr int SMEM_BUDGET = 220 * 1024;     // dynamic shared memory of the main kernel
constexpr int MAX_TABLE_TILES = 8192;       // tile -> slot table entries (16 KB)
constexpr int SAMPLE_BLOCKS = 128;
constexpr int SAMPLE_CHUNK = 8192;
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
    unsigned *hist;             // ntiles
    short *slot;                // ntiles
    int *slot_tile;             // K
};

__device__ __forceinline__ int tile_cells(const CachedParams &p) { return 1 << (2 * p.ts); }

// ---- sample: tile histogram of evenly spaced chunks
__global__ void __launch_bounds__(256) cached_sample(const CachedParams p, int64_t chunk) {
    extern __shared__ unsigned sh_hist[];
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x) sh_hist[i] = 0;
    __syncthreads();
    const int64_t start = (p.n / gridDim.x) * blockIdx.x;
    const int64_t end = start + chunk < p.n ? start + chunk : p.n;
    for (int64_t i = start + threadIdx.x; i < end; i += blockDim.x) {
        int xi, yi;
        const float x = p.xs[i], y = p.ys[i];
        int r = bin_try_f32(x, y, p.bb, p.ax, p.ay, xi, yi);
        if (r == 2) bin_exact_f32(x, y, p.ax, p.ay, xi, yi);
        if (r) atomicAdd(&sh_hist[(yi >> p.ts) * p.tiles_x + (xi >> p.ts)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x)
        if (sh_hist[i]) atomicAdd(&p.hist[i], sh_hist[i]);
}

// ---- select: smallest T with #(count > T) <= K; those tiles get slots
__global__ void __launch_bounds__(1024) cached_select(const CachedParams p) {
    __shared__ unsigned red[32];
    __shared__ unsigned s_lo, s_hi, s_next;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned mx = 0;
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x) mx = max(mx, p.hist[i]);
    for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) red[warp] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned m = 0;
        for (int w = 0; w < nw; ++w) m = max(m, red[w]);
        s_lo = 0; s_hi = m; s_next = 0;
    }
    __syncthreads();
    for (int it = 0; it < 40; ++it) {
        const unsigned lo = s_lo, hi = s_hi;
        if (lo >= hi) break;
        const unsigned mid = lo + (hi - lo) / 2;
        unsigned c = 0;
        for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x) c += p.hist[i] > mid;
        for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        __syncthreads();
        if (lane == 0) red[warp] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned t = 0;
            for (int w = 0; w < nw; ++w) t += red[w];
            if (t <= (unsigned)p.K) s_hi = mid; else s_lo = mid + 1;
        }
        __syncthreads();
    }
    const unsigned T = s_hi;
    for (int i = threadIdx.x; i < p.K; i += blockDim.x) p.slot_tile[i] = -1;
    __syncthreads();
    for (int i = threadIdx.x; i < p.ntiles; i += blockDim.x) {
        short s = -1;
        if (p.hist[i] > T) {
            const unsigned k = atomicAdd(&s_next, 1u);
            if (k < (unsigned)p.K) { s = (short)k; p.slot_tile[k] = i; }
        }
        p.slot[i] = s;
    }
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

// ------------------------------------------------------------- host side

struct CachedLayout {
    int ts, tiles_x, ntiles, K, grid;
    size_t off_hist, off_slot, off_slot_tile, total;
};

static size_t align256(size_t v) { return (v + 255) / 256 * 256; }

static bool cached_layout(int64_t n, int width, int height, CachedLayout &L) {
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
    const int tile_bytes = (1 << (2 * ts)) * 4;
    L.K = (SMEM_BUDGET - tab) / tile_bytes;
    if (L.K > L.ntiles) L.K = L.ntiles;
    if (L.K < 1) return false;
    const int sms = sm_count();
    L.grid = sms > 0 ? sms : 148;
    size_t o = 0;
    L.off_hist = o; o = align256(o + (size_t)L.ntiles * 4);
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
    cudaError_t e = cudaMemsetAsync(p.hist, 0, (size_t)L.ntiles * 4, st);
    if (e == cudaSuccess && !accumulate) e = cudaMemsetAsync(out, 0, (size_t)cv->width * cv->height * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "cached count memset");
    const int64_t chunk = SAMPLE_CHUNK < n / SAMPLE_BLOCKS ? SAMPLE_CHUNK : n / SAMPLE_BLOCKS;
    cached_sample<<<SAMPLE_BLOCKS, 256, (size_t)L.ntiles * 4, st>>>(p, chunk);
    cached_select<<<1, 1024, 0, st>>>(p);
    const size_t smem = (((size_t)L.ntiles * 2 + 15) & ~(size_t)15) + (size_t)L.K * (1 << (2 * L.ts)) * 4;
    e = cudaFuncSetAttribute(cached_main, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "cached count smem attribute");
    cached_main<<<L.grid, 1024, smem, st>>>(p);
    DSGB_CHECK_LAUNCH("cached count launch");
    return DSGB_OK;
}

}  // namespace dsgb
