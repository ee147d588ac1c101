// pyramid.cu -- a whole tile pyramid of Canvas.points count() and max(v).
//
// Every tile (z, tx, ty), zmin <= z <= zmax, of the square [x0, x1] x [y0, y1]
// is the aggregate of
//     Canvas(ts, ts, x_range=(lo(tx), lo(tx + 1)), y_range=(lo(ty), lo(ty + 1)))
//         .points(df, 'x', 'y', agg)           lo(t) = x0 + (x1 - x0) * (t / 2^z)
// with the reference's binning (datashader/glyphs/points.py:190-204:
// inclusive bounds, int() truncation, the upper edge clamped into the last
// pixel) and its scale / translate (core.py:62-81: s = ts / (hi - lo),
// t = -lo * s).  A point on the edge shared by two tiles is in both, exactly
// as two separate Canvas calls count it.  count() counts every point;
// max(v) skips NaN and reports NaN for empty pixels (reductions.py:1160-1227).
//
// Pipeline, one stream, capturable in a CUDA graph:
//   pyr_tables  -- per level, tile and axis: the tile's exact float64 bounds
//                  and binning axis, computed with the host's operations
//                  (IEEE float64, no contraction);
//   pyr_hist    -- the square is cut into 2^B x 2^B buckets, B = zmax + 1;
//                  each point falls in one bucket (a float32 estimate: the
//                  bucket is a work unit, not a result);
//   pyr_plan    -- one block: bucket offsets, work items (bucket, chunk,
//                  sub-bucket) and partial slots;
//   pyr_band / pyr_scatter
//               -- the points regrouped by bucket in two passes, first by
//                  bucket row (2^B bands) and then by bucket, so that every
//                  block writes runs of consecutive rows (block-aggregated
//                  reservations, two reads of the input per block);
//   pyr_render  -- persistent: each CTA takes work items off a queue.  The
//                  item's footprint at level z, (ts >> (B + split - z)) pixels
//                  on a side, is privatised in shared memory (uint32 count,
//                  uint32 order-preserving max key).  Each point is binned
//                  exactly into every tile of every level that holds it.
//                  The footprints partition every level, so the CTA that
//                  owns one writes it with plain stores (a bucket split into
//                  chunks combines its partials in the CTA of its last chunk).
//                  Contributions that land outside the item's footprint
//                  (edge duplicates in the neighbouring tile, or a bucket
//                  estimate off by one) are queued;
//   pyr_spill   -- applies the queued contributions with atomics.
// Dyadic squares (x0 = y0 = 0, power-of-two spans; checked by the host)
// have exact tile transforms at every level: a point's pixel at level z is
// its pixel at zmax shifted right by zmax - z.  There the render bins each
// point at zmax only and derives the coarser footprints in shared memory by
// 2x2 sums and maxima; only points on a tile edge (whose extra copies go to
// the queue) run the per-level code.
// The autotuned knobs are the shared-memory tile size (split: the finest
// footprint is ts/2 or ts/4 pixels on a side; a split bucket is rendered by
// 4 CTAs that each take their quarter of the bucket's points), the render
// CTA size and the chunk length.
#include "dsgb_internal.cuh"
#include "binning.cuh"

#include <mutex>

namespace dsgb {

constexpr int PYR_MAX_Z = 6;                  // 4^(zmax + 1) buckets <= 16384
constexpr int PYR_HIST_THREADS = 1024;
constexpr int PYR_SMEM_LIMIT = 220 * 1024;
constexpr int PYR_BAND_ROWS = 8;              // bucket rows per band of the first regroup pass
constexpr int PYR_SPILL_CAS_LIMIT = 1 << 20;

struct PyrEntry {                             // one tile of one level, one axis
    BinAxis ax;                               // exact binning into the tile's ts pixels
    float lo_f, hi_f;                         // exact float images of the inclusive bounds
};

struct PyrSpill {
    unsigned z, gx, gy;
    float v;                                  // NaN: count only
};

struct PyrCounters {
    unsigned queue;                           // next work item
    unsigned n_items;
    unsigned n_spill;
    unsigned flags;                           // bit 0: spill overflow, bit 1: CAS limit, bit 2: slots
    unsigned n_slots;                         // accumulation slots in use
};

struct PyrParams {
    const float *xs, *ys, *vs;                // input columns (vs may be null)
    int64_t n;
    int32_t zmin, zmax, ts, split;
    int32_t bls;                              // bucket level of the scatter (zmax + 1)
    int32_t nbk;                              // buckets per axis (1 << bls)
    int32_t nbuckets;
    int32_t chunk;
    int32_t vec;                              // columns 16-byte aligned
    double x0, x1, y0, y1;
    float x0f, y0f, bscale_x, bscale_y;       // bucket estimate
    PyrEntry *tab_x, *tab_y;                  // [(1 << z) - 1 + t]
    unsigned *bcount;                         // nbuckets
    unsigned *bstart;                         // nbuckets + 1
    unsigned *cursor;                         // nbuckets
    unsigned *band_cursor;                    // nbk (bucket rows)
    unsigned *item_base;                      // nbuckets + 1 (items before bucket b)
    unsigned *item_bucket;                    // n_items: the bucket of each work item
    unsigned *slot_base;                      // nbuckets (accumulation slot of b, when split in chunks)
    unsigned *done;                           // nbuckets << (2 * split)
    PyrCounters *ctr;
    float *sx, *sy, *sv;                      // points grouped by bucket
    float *bx_, *by_, *bv_;                   // points grouped by bucket row (first pass)
    int32_t dyadic;                           // exact nesting of the levels (see above)
    int32_t vec_out;                          // outputs 16-byte aligned: vector stores
    unsigned *partials;                       // slots x (2 * footprint) uint32: counts, then max keys
    int64_t slot_cap;
    PyrSpill *spill;
    int64_t spill_cap;
    int32_t footprint;                        // sum over levels of F_z^2, each rounded up to 4
    int32_t fp_off[PYR_MAX_Z + 2];            // offset of level z in the footprint (z - zmin)
    int64_t level_off[PYR_MAX_Z + 2];         // output offset of level z
    uint32_t *count_out;
    double *max_out;                          // may be null
};

// ---------------------------------------------------------------- helpers

__host__ __device__ __forceinline__ int ntab_of(int zmax) { return (1 << (zmax + 1)) - 1; }

// Order-preserving uint32 key of a float32 (0 = empty; -0.0 folded onto +0.0).
__device__ __forceinline__ unsigned fkey(float v) {
    unsigned b = __float_as_uint(v);
    if (b == 0x80000000u) b = 0u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fkey_value(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// The float64 bounds of tile t of level z, as the host computes them:
// lo(t) = x0 + (x1 - x0) * (t / 2^z).
__device__ __forceinline__ double tile_lo(double x0, double span, int z, int t) {
    return __dadd_rn(x0, __dmul_rn(span, ldexp((double)t, -z)));
}

__device__ float dev_float_ceil_of(double v) {
    float f = __double2float_rn(v);
    if ((double)f < v) f = nextafterf(f, INFINITY);
    return f;
}
__device__ float dev_float_floor_of(double v) {
    float f = __double2float_rn(v);
    if ((double)f > v) f = nextafterf(f, -INFINITY);
    return f;
}

// Device copy of the error bound of binning.cuh (binning_error_bound).
__device__ float dev_error_bound(double lo, double hi, double s, double t, int n) {
    if (!isfinite(lo) || !isfinite(hi) || !isfinite(s) || !isfinite(t)) return INFINITY;
    const double xm = fmax(fabs(lo), fabs(hi));
    const double sf = (double)__double2float_rn(s), tf = (double)__double2float_rn(t);
    const double mag = xm * fabs(s) + fabs(t) + (double)n + 1.0;
    if (!(mag < 1e6) || fabs(s) > 1e30 || xm > 1e30 || !isfinite(sf) || !isfinite(tf)) return INFINITY;
    const double e = xm * fabs(s - sf) + fabs(t - tf) + ldexp(1.0, -23) * xm * fabs(sf) +
                     ldexp(1.0, -24) * (xm * fabs(sf) + fabs(tf)) + ldexp(1.0, -52) * (xm * fabs(s) + fabs(t));
    return __double2float_ru(2.0 * e + 1e-30);
}

// Exact bin of a float32 coordinate inside a tile (the caller checked the bounds).
static __device__ __noinline__ int pyr_bin_exact(float x, double s, double t, int n) {
    return bin_exact64_st((double)x, s, t, n);
}
__device__ __forceinline__ int pyr_bin(float x, const BinAxis &a) {
    int r;
    if (fast_coord(__fmaf_rn(x, a.sf, a.tf), a, r)) return r;
    return pyr_bin_exact(x, a.s, a.t, a.n);
}

__device__ __forceinline__ int bucket_of(const PyrParams &p, const PyrEntry &dx, const PyrEntry &dy, float x, float y) {
    if (!(x >= dx.lo_f && x <= dx.hi_f && y >= dy.lo_f && y <= dy.hi_f)) return -1;
    int bx = (int)((x - p.x0f) * p.bscale_x);
    int by = (int)((y - p.y0f) * p.bscale_y);
    bx = bx < 0 ? 0 : (bx >= p.nbk ? p.nbk - 1 : bx);
    by = by < 0 ? 0 : (by >= p.nbk ? p.nbk - 1 : by);
    return by * p.nbk + bx;
}

// ---------------------------------------------------------------- tables

__global__ void pyr_tables(const PyrParams p) {
    const int ntab = ntab_of(p.zmax);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * ntab) return;
    const int axis = i / ntab, j = i % ntab;
    int z = 0;
    while (((1 << (z + 1)) - 1) <= j) ++z;
    const int t = j - ((1 << z) - 1);
    const double a0 = axis ? p.y0 : p.x0, a1 = axis ? p.y1 : p.x1;
    const double span = __dsub_rn(a1, a0);
    const double lo = tile_lo(a0, span, z, t), hi = tile_lo(a0, span, z, t + 1);
    PyrEntry e;
    const double s = __ddiv_rn((double)p.ts, __dsub_rn(hi, lo));
    const double tt = -__dmul_rn(lo, s);
    e.ax.s = s; e.ax.t = tt;
    e.ax.sf = __double2float_rn(s); e.ax.tf = __double2float_rn(tt);
    e.ax.n = p.ts;
    e.ax.e = dev_error_bound(lo, hi, s, tt, p.ts);
    if (!(e.ax.e < 0.01f)) e.ax.e = INFINITY;          // fast path off: every bin exact in float64
    e.lo_f = dev_float_ceil_of(lo);
    e.hi_f = dev_float_floor_of(hi);
    (axis ? p.tab_y : p.tab_x)[j] = e;
}

// ---------------------------------------------------------------- histogram

__global__ void __launch_bounds__(PYR_HIST_THREADS, 1) pyr_hist(const PyrParams p) {
    extern __shared__ unsigned h[];
    for (int i = threadIdx.x; i < p.nbuckets; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const PyrEntry dx = p.tab_x[0], dy = p.tab_y[0];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t done_rows = 0;
    if (p.vec) {
        const int64_t n4 = p.n >> 2;
        const float4 *x4 = (const float4 *)p.xs, *y4 = (const float4 *)p.ys;
        for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n4; v += stride) {
            const float4 a = __ldcs(x4 + v), b = __ldcs(y4 + v);
            const float xs[4] = {a.x, a.y, a.z, a.w}, ys[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int bk = bucket_of(p, dx, dy, xs[k], ys[k]);
                if (bk >= 0) atomicAdd(&h[bk], 1u);
            }
        }
        done_rows = 4 * n4;
    }
    for (int64_t i = done_rows + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += stride) {
        const int bk = bucket_of(p, dx, dy, p.xs[i], p.ys[i]);
        if (bk >= 0) atomicAdd(&h[bk], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < p.nbuckets; i += blockDim.x)
        if (h[i]) atomicAdd(&p.bcount[i], h[i]);
}

// ---------------------------------------------------------------- plan

// Block-wide exclusive scan of one value per thread (blockDim.x == 1024).
__device__ unsigned block_exclusive_scan(unsigned v, unsigned *total) {
    __shared__ unsigned warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        warp_sums[lane] = w;                  // inclusive over warps
    }
    __syncthreads();
    const unsigned before = warp ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[31];
    __syncthreads();
    return before + incl - v;
}

__host__ __device__ __forceinline__ unsigned chunks_of(unsigned cnt, int chunk) {
    return cnt == 0 ? 1u : (cnt + (unsigned)chunk - 1) / (unsigned)chunk;
}

__global__ void __launch_bounds__(1024) pyr_plan(const PyrParams p) {
    const int per = (p.nbuckets + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    const int nsub = 1 << (2 * p.split);
    unsigned s_cnt = 0, s_items = 0, s_slots = 0;
    for (int k = 0; k < per; ++k) {
        const int b = b0 + k;
        if (b >= p.nbuckets) break;
        const unsigned c = p.bcount[b], ch = chunks_of(c, p.chunk);
        s_cnt += c;
        s_items += ch * nsub;
        s_slots += ch > 1 ? (unsigned)nsub : 0u;
    }
    unsigned t_cnt, t_items, t_slots;
    unsigned o_cnt = block_exclusive_scan(s_cnt, &t_cnt);
    unsigned o_items = block_exclusive_scan(s_items, &t_items);
    unsigned o_slots = block_exclusive_scan(s_slots, &t_slots);
    for (int k = 0; k < per; ++k) {
        const int b = b0 + k;
        if (b >= p.nbuckets) break;
        const unsigned c = p.bcount[b], ch = chunks_of(c, p.chunk);
        p.bstart[b] = o_cnt;
        p.cursor[b] = o_cnt;
        if (b % (p.nbk * PYR_BAND_ROWS) == 0) p.band_cursor[b / (p.nbk * PYR_BAND_ROWS)] = o_cnt;
        p.item_base[b] = o_items;
        p.slot_base[b] = o_slots;
        for (unsigned i = 0; i < ch * nsub; ++i) p.item_bucket[o_items + i] = (unsigned)b;
        o_cnt += c;
        o_items += ch * nsub;
        o_slots += ch > 1 ? (unsigned)nsub : 0u;
        for (int q = 0; q < nsub; ++q) p.done[(int64_t)b * nsub + q] = 0;
    }
    if (threadIdx.x == 0) {
        p.bstart[p.nbuckets] = t_cnt;
        p.item_base[p.nbuckets] = t_items;
        p.ctr->queue = 0;
        p.ctr->n_items = t_items;
        p.ctr->n_spill = 0;
        p.ctr->flags = (int64_t)t_slots > p.slot_cap ? 4u : 0u;
        p.ctr->n_slots = t_slots;
    }
}

__global__ void pyr_zero_slots(const PyrParams p) {
    const unsigned ns = p.ctr->n_slots;
    const int64_t n4 = ((int64_t)(ns < p.slot_cap ? ns : p.slot_cap) * 2 * p.footprint) >> 2;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x)
        ((uint4 *)p.partials)[i] = make_uint4(0u, 0u, 0u, 0u);
}

// ---------------------------------------------------------------- scatter

// Warp-aggregated slot reservation: the lanes of a warp that share `key`
// (an index into h, or a value with bit 31 set for lanes that place
// nothing) take consecutive slots with one shared-memory atomic.
__device__ __forceinline__ unsigned warp_reserve(unsigned *h, unsigned key, bool live) {
    const int lane = threadIdx.x & 31;
    const unsigned k = live ? key : (0x80000000u | lane);
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    const int leader = __ffs(peers) - 1;
    unsigned base = 0;
    if (live && lane == leader) base = atomicAdd(&h[key], (unsigned)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

// Regroup passes.  A block takes PYR_STAGE_ROWS consecutive rows, ranks
// them by destination group in shared memory (warp-aggregated counters),
// reserves each group's range with one global atomic, stages the rows in
// shared memory in group order and writes them out as contiguous runs, so
// that global stores are coalesced instead of one sector per row.
constexpr int PYR_STAGE_THREADS = 512;
constexpr int PYR_STAGE_ITEMS = 8;
constexpr int PYR_STAGE_ROWS = PYR_STAGE_THREADS * PYR_STAGE_ITEMS;
constexpr int PYR_STAGE_MAX_GROUPS = 4096;    // 48 KB of counters + 64 KB of staged rows: two blocks an SM

struct StageIn {
    const float *x, *y, *v;       // v may be null
    int64_t r0, r1;               // the block's rows
};

// Dynamic shared memory: counters (ngroups), group offsets (ngroups + 1),
// global bases (ngroups), then the staged x, y, v (PYR_STAGE_ROWS each)
// and their group ids.  `group_of` maps (x, y) to a group in [0, ngroups)
// or -1 (dropped).
template <typename G>
__device__ void stage_and_write(const StageIn in, int ngroups, G group_of, unsigned *gcursor, float *ox,
                                float *oy, float *ov, unsigned char *sm) {
    unsigned *cnt = (unsigned *)sm;
    unsigned *off = cnt + ngroups;
    unsigned *gbase = off + ngroups + 1;
    float *sx = (float *)(gbase + ngroups);
    float *sy = sx + PYR_STAGE_ROWS;
    float *sv = sy + PYR_STAGE_ROWS;
    int *sg = (int *)(sv + PYR_STAGE_ROWS);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < ngroups; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    float xv[PYR_STAGE_ITEMS], yv[PYR_STAGE_ITEMS], vv[PYR_STAGE_ITEMS];
    int gv[PYR_STAGE_ITEMS];
    unsigned rk[PYR_STAGE_ITEMS];
#pragma unroll
    for (int k = 0; k < PYR_STAGE_ITEMS; ++k) {
        const int64_t i = in.r0 + (int64_t)(warp * PYR_STAGE_ITEMS + k) * 32 + lane;
        const bool live = i < in.r1;
        xv[k] = live ? __ldcs(in.x + i) : __int_as_float(0x7fc00000);
        yv[k] = live ? __ldcs(in.y + i) : 0.f;
        vv[k] = (live && in.v) ? __ldcs(in.v + i) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < PYR_STAGE_ITEMS; ++k) {
        gv[k] = group_of(xv[k], yv[k]);
        rk[k] = warp_reserve(cnt, gv[k] >= 0 ? (unsigned)gv[k] : 0u, gv[k] >= 0);
    }
    __syncthreads();
    {
        // exclusive scan of the group counts by the whole block: each thread
        // sums a run of consecutive groups, the runs are scanned across the
        // block (warp shuffles, then the warp totals), and each thread writes
        // its run's offsets
        __shared__ unsigned wsum[32];
        const int per = (ngroups + (int)blockDim.x - 1) / (int)blockDim.x;
        const int g0 = threadIdx.x * per;
        const int g1 = g0 + per < ngroups ? g0 + per : ngroups;
        unsigned own = 0;
        for (int g = g0; g < g1; ++g) own += cnt[g];
        unsigned incl = own;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const int nw = (int)blockDim.x >> 5;
            const unsigned w = lane < nw ? wsum[lane] : 0u;
            unsigned wi = w;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned u = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += u;
            }
            __syncwarp();
            if (lane < nw) wsum[lane] = wi - w;
            if (lane == nw - 1) off[ngroups] = wi;
        }
        __syncthreads();
        unsigned run = wsum[warp] + incl - own;
        for (int g = g0; g < g1; ++g) {
            off[g] = run;
            run += cnt[g];
        }
    }
    __syncthreads();
    for (int g = threadIdx.x; g < ngroups; g += blockDim.x)
        gbase[g] = (cnt[g] ? atomicAdd(&gcursor[g], cnt[g]) : 0u) - off[g];   // global base minus staged base
#pragma unroll
    for (int k = 0; k < PYR_STAGE_ITEMS; ++k) {
        if (gv[k] < 0) continue;
        const unsigned j = off[gv[k]] + rk[k];
        sx[j] = xv[k];
        sy[j] = yv[k];
        sv[j] = vv[k];
        sg[j] = gv[k];
    }
    __syncthreads();
    const int staged = (int)off[ngroups];
    for (int j = threadIdx.x; j < staged; j += blockDim.x) {
        const int g = sg[j];
        const unsigned pos = gbase[g] + (unsigned)j;
        ox[pos] = sx[j];
        oy[pos] = sy[j];
        if (ov) ov[pos] = sv[j];
    }
}

__host__ __device__ __forceinline__ size_t stage_smem_bytes(int ngroups) {
    return (size_t)(3 * ngroups + 1) * 4 + (size_t)PYR_STAGE_ROWS * 16;
}

// First pass: rows grouped by band (PYR_BAND_ROWS bucket rows).
__global__ void __launch_bounds__(PYR_STAGE_THREADS, 2) pyr_band(const PyrParams p) {
    extern __shared__ __align__(16) unsigned char smb[];
    const PyrEntry dx = p.tab_x[0], dy = p.tab_y[0];
    const int nbands = (p.nbk + PYR_BAND_ROWS - 1) / PYR_BAND_ROWS;
    const int band_div = p.nbk * PYR_BAND_ROWS;
    StageIn in;
    in.x = p.xs; in.y = p.ys; in.v = p.sv ? p.vs : nullptr;
    in.r0 = (int64_t)blockIdx.x * PYR_STAGE_ROWS;
    in.r1 = in.r0 + PYR_STAGE_ROWS < p.n ? in.r0 + PYR_STAGE_ROWS : p.n;
    stage_and_write(in, nbands, [&](float x, float y) {
        const int bk = bucket_of(p, dx, dy, x, y);
        return bk < 0 ? -1 : bk / band_div;
    }, p.band_cursor, p.bx_, p.by_, p.sv ? p.bv_ : nullptr, smb);
}

// Second pass: the banded copy grouped by bucket.  A block's rows come from
// a few consecutive bands, so its groups are only their buckets.
__global__ void __launch_bounds__(PYR_STAGE_THREADS, 2) pyr_scatter(const PyrParams p) {
    extern __shared__ __align__(16) unsigned char smb[];
    __shared__ int s_lo, s_hi;
    const PyrEntry dx = p.tab_x[0], dy = p.tab_y[0];
    const int64_t total = p.bstart[p.nbuckets];
    StageIn in;
    in.x = p.bx_; in.y = p.by_; in.v = p.sv ? p.bv_ : nullptr;
    in.r0 = (int64_t)blockIdx.x * PYR_STAGE_ROWS;
    in.r1 = in.r0 + PYR_STAGE_ROWS < total ? in.r0 + PYR_STAGE_ROWS : total;
    if (in.r0 >= in.r1) return;
    if (threadIdx.x == 0) {
        // the banded copy is ordered by band only: cover whole bands
        const int band_div = p.nbk * PYR_BAND_ROWS;
        s_lo = bucket_of(p, dx, dy, p.bx_[in.r0], p.by_[in.r0]) / band_div * band_div;
        const int hi = (bucket_of(p, dx, dy, p.bx_[in.r1 - 1], p.by_[in.r1 - 1]) / band_div + 1) * band_div;
        s_hi = hi < p.nbuckets ? hi : p.nbuckets;
    }
    __syncthreads();
    const int lo = s_lo;
    if (s_hi - s_lo > PYR_STAGE_MAX_GROUPS) {
        // a block spanning many sparse bands: place row by row
        for (int64_t i = in.r0 + threadIdx.x; i < in.r1; i += blockDim.x) {
            const float x = p.bx_[i], y = p.by_[i];
            const int bk = bucket_of(p, dx, dy, x, y);
            if (bk < 0) continue;
            const unsigned pos = atomicAdd(&p.cursor[bk], 1u);
            p.sx[pos] = x;
            p.sy[pos] = y;
            if (p.sv) p.sv[pos] = p.bv_[i];
        }
        return;
    }
    stage_and_write(in, s_hi - s_lo, [&](float x, float y) {
        const int bk = bucket_of(p, dx, dy, x, y);
        return bk < 0 ? -1 : bk - lo;
    }, p.cursor + lo, p.sx, p.sy, p.sv, smb);
}

// ---------------------------------------------------------------- render

struct PyrLevel {                 // per item and level, in shared memory
    PyrEntry hx, hy;              // home tiles of the item at this level
    int htx, hty;                 // their indices
    int f, lf;                    // footprint side and its log2
    int gx0, gy0;                 // footprint origin (global pixels of the level)
    int cf, cgx0, cgy0;           // the whole bucket's footprint (split > 0)
};

// The tiles of level z containing coordinate c (1 or 2) and the global pixel
// in each.  `home` is the item's home tile; anything else reads the table.
__device__ __forceinline__ int tiles_of(float c, const PyrEntry &home, int ht, const PyrEntry *tab, int z,
                                        int ts, float c0f, float span_inv_f, int g[2]) {
    const int nt = 1 << z;
    const PyrEntry *lvl = tab + (nt - 1);
    if (c >= home.lo_f && c <= home.hi_f) {
        int k = 0;
        g[k++] = ht * ts + pyr_bin(c, home.ax);
        if (c == home.lo_f && ht > 0) {
            const PyrEntry e = lvl[ht - 1];
            if (c <= e.hi_f) g[k++] = (ht - 1) * ts + pyr_bin(c, e.ax);
        } else if (c == home.hi_f && ht + 1 < nt) {
            const PyrEntry e = lvl[ht + 1];
            if (c >= e.lo_f) g[k++] = (ht + 1) * ts + pyr_bin(c, e.ax);
        }
        return k;
    }
    // not in the home tile (the bucket estimate was off): search around a new estimate
    // (g written with constant indices only, so that it stays in registers)
    int t = (int)((c - c0f) * span_inv_f * (float)nt);
    int k = 0;
#pragma unroll
    for (int d = -2; d <= 2; ++d) {
        const int u = t + d;
        if (k >= 2 || u < 0 || u >= nt) continue;
        const PyrEntry e = lvl[u];
        if (c >= e.lo_f && c <= e.hi_f) {
            const int gv = u * ts + pyr_bin(c, e.ax);
            if (k == 0) g[0] = gv; else g[1] = gv;
            ++k;
        }
    }
    return k;
}

__device__ __forceinline__ void pyr_queue(const PyrParams &p, int z, int gx, int gy, float v) {
    const unsigned si = atomicAdd(&p.ctr->n_spill, 1u);
    if ((int64_t)si < p.spill_cap) {
        PyrSpill s;
        s.z = (unsigned)z; s.gx = (unsigned)gx; s.gy = (unsigned)gy; s.v = v;
        p.spill[si] = s;
    } else {
        atomicOr(&p.ctr->flags, 1u);
    }
}

// Dyadic squares: a point on a tile edge (or outside its item's bucket)
// runs the per-level binning; every contribution other than the floor
// pixel already counted at zmax (gxp, gyp shifted to the level) is queued.
static __device__ __noinline__ void pyr_dyadic_edges(const PyrParams &p, const PyrLevel *L, int nlev, float x,
                                                     float y, float v, int gxp, int gyp, bool counted, float x0f,
                                                     float y0f, float span_inv_x, float span_inv_y) {
    for (int lz = 0; lz < nlev; ++lz) {
        const PyrLevel &l = L[lz];
        const int z = p.zmin + lz, k = p.zmax - z;
        int gx[2], gy[2];
        const int kx = tiles_of(x, l.hx, l.htx, p.tab_x, z, p.ts, x0f, span_inv_x, gx);
        const int ky = kx ? tiles_of(y, l.hy, l.hty, p.tab_y, z, p.ts, y0f, span_inv_y, gy) : 0;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                if (a >= kx || c >= ky) continue;
                if (counted && gx[a] == (gxp >> k) && gy[c] == (gyp >> k)) continue;
                pyr_queue(p, z, gx[a], gy[c], v);
            }
    }
}

__global__ void __launch_bounds__(1024, 1) pyr_render(const PyrParams p) {
    extern __shared__ __align__(16) unsigned char sm[];
    unsigned *scnt = (unsigned *)sm;
    unsigned *skey = scnt + p.footprint;
    __shared__ PyrLevel L[PYR_MAX_Z + 1];
    __shared__ unsigned s_q[2];                // this item and the next (ping-pong)
    __shared__ bool s_last;
    const int nlev = p.zmax - p.zmin + 1;
    const int nsub = 1 << (2 * p.split), sside = 1 << p.split;
    const int bl = p.bls + p.split;
    const float span_inv_x = 1.0f / (float)(p.x1 - p.x0), span_inv_y = 1.0f / (float)(p.y1 - p.y0);
    const float x0f = (float)p.x0, y0f = (float)p.y0;
    const unsigned n_items = p.ctr->n_items;
    if (threadIdx.x == 0) s_q[0] = atomicAdd(&p.ctr->queue, 1u);
    __syncthreads();
    for (unsigned it = 0;; ++it) {
        const unsigned item = s_q[it & 1];
        if (item >= n_items) break;
        // the next item is taken now (its slot was last read before the
        // previous iteration's final barrier); the atomic's latency hides
        // behind this item
        if (threadIdx.x == 0) s_q[(it + 1) & 1] = atomicAdd(&p.ctr->queue, 1u);
        const int b = (int)__ldg(&p.item_bucket[item]);
        const unsigned rel = item - __ldg(&p.item_base[b]);
        const unsigned j = rel / nsub, q = rel % nsub;
        const unsigned bcnt = p.bstart[b + 1] - p.bstart[b];
        const unsigned nch = chunks_of(bcnt, p.chunk);
        const int bx = ((b % p.nbk) << p.split) | (int)(q % sside);
        const int by = ((b / p.nbk) << p.split) | (int)(q / sside);
        if (threadIdx.x < nlev) {
            const int z = p.zmin + threadIdx.x;
            PyrLevel &l = L[threadIdx.x];
            l.f = p.ts >> (bl - z);
            l.lf = __ffs(l.f) - 1;
            l.gx0 = bx * l.f;
            l.gy0 = by * l.f;
            l.cf = l.f << p.split;
            l.cgx0 = (bx >> p.split) * l.cf;
            l.cgy0 = (by >> p.split) * l.cf;
            l.htx = l.gx0 / p.ts;
            l.hty = l.gy0 / p.ts;
            l.hx = p.tab_x[(1 << z) - 1 + l.htx];
            l.hy = p.tab_y[(1 << z) - 1 + l.hty];
        }
        if (p.dyadic) {
            // only the finest level accumulates; the coarser ones are derived
            const int o4 = p.fp_off[nlev - 1] >> 2, k4 = (p.footprint >> 2) - o4;
            for (int i = threadIdx.x; i < 2 * k4; i += blockDim.x) {
                const int j = i < k4 ? o4 + i : (p.footprint >> 2) + o4 + (i - k4);
                ((uint4 *)scnt)[j] = make_uint4(0u, 0u, 0u, 0u);
            }
        } else {
            const int n4 = (2 * p.footprint) >> 2;
            for (int i = threadIdx.x; i < n4; i += blockDim.x) ((uint4 *)scnt)[i] = make_uint4(0u, 0u, 0u, 0u);
        }
        __syncthreads();
        const unsigned s0 = p.bstart[b] + j * (unsigned)p.chunk;
        const unsigned s1 = s0 + (unsigned)p.chunk < p.bstart[b + 1] ? s0 + (unsigned)p.chunk : p.bstart[b + 1];
        constexpr int RI = 4;                 // rows per thread and iteration, loaded up front
        for (unsigned i0 = s0 + threadIdx.x; i0 < s1; i0 += RI * blockDim.x) {
          float xv[RI], yv[RI], vv[RI];
#pragma unroll
          for (int r = 0; r < RI; ++r) {
              const unsigned i = i0 + r * blockDim.x;
              const bool live = i < s1;
              xv[r] = live ? p.sx[i] : __int_as_float(0x7fc00000);
              yv[r] = live ? p.sy[i] : 0.f;
              vv[r] = (live && p.sv) ? p.sv[i] : __int_as_float(0x7fc00000);
          }
#pragma unroll 1
          for (int r = 0; r < RI; ++r) {
            if (i0 + r * blockDim.x >= s1) break;
            // take the front row and shift the rest down: constant indices
            // keep the rows in registers in this rolled loop
            const float x = xv[0], y = yv[0];
            const float v = vv[0];
#pragma unroll
            for (int u = 0; u + 1 < RI; ++u) { xv[u] = xv[u + 1]; yv[u] = yv[u + 1]; vv[u] = vv[u + 1]; }
            const bool hasv = !(v != v);
            const unsigned key = hasv ? fkey(v) : 0u;
            if (p.dyadic) {
                // bin at zmax only; the coarser footprints are derived below
                const PyrLevel &l = L[nlev - 1];
                int gx[2], gy[2];
                const int kx = tiles_of(x, l.hx, l.htx, p.tab_x, p.zmax, p.ts, x0f, span_inv_x, gx);
                const int ky = kx ? tiles_of(y, l.hy, l.hty, p.tab_y, p.zmax, p.ts, y0f, span_inv_y, gy) : 0;
                if (!kx || !ky) continue;
                // the floor pixel: on a tile edge the right / upper tile's first pixel
                const int gxp = kx == 2 ? max(gx[0], gx[1]) : gx[0];
                const int gyp = ky == 2 ? max(gy[0], gy[1]) : gy[0];
                const unsigned lx = (unsigned)(gxp - l.gx0), ly = (unsigned)(gyp - l.gy0);
                if (lx < (unsigned)l.f && ly < (unsigned)l.f) {
                    const int off = p.fp_off[nlev - 1] + (int)ly * l.f + (int)lx;
                    atomicAdd(&scnt[off], 1u);
                    if (hasv) atomicMax(&skey[off], key);
                }
                const bool in_bucket = (unsigned)(gxp - l.cgx0) < (unsigned)l.cf &&
                                       (unsigned)(gyp - l.cgy0) < (unsigned)l.cf;
                if (q == 0 && (!in_bucket || kx == 2 || ky == 2))
                    pyr_dyadic_edges(p, L, nlev, x, y, v, gxp, gyp, in_bucket, x0f, y0f, span_inv_x, span_inv_y);
                continue;
            }
            for (int lz = 0; lz < nlev; ++lz) {
                const PyrLevel &l = L[lz];
                const int z = p.zmin + lz;
                int gx[2], gy[2];
                const int kx = tiles_of(x, l.hx, l.htx, p.tab_x, z, p.ts, x0f, span_inv_x, gx);
                if (!kx) continue;
                const int ky = tiles_of(y, l.hy, l.hty, p.tab_y, z, p.ts, y0f, span_inv_y, gy);
#pragma unroll
                for (int a = 0; a < 2; ++a) {
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        if (a >= kx || c >= ky) continue;
                        const unsigned lx = (unsigned)(gx[a] - l.gx0), ly = (unsigned)(gy[c] - l.gy0);
                        if (lx < (unsigned)l.f && ly < (unsigned)l.f) {
                            const int off = p.fp_off[lz] + (int)ly * l.f + (int)lx;
                            atomicAdd(&scnt[off], 1u);
                            if (hasv) atomicMax(&skey[off], key);
                            continue;
                        }
                        if (p.split) {
                            // inside the bucket but outside this quarter: a sibling item takes it
                            const unsigned cx = (unsigned)(gx[a] - l.cgx0), cy = (unsigned)(gy[c] - l.cgy0);
                            if (cx < (unsigned)l.cf && cy < (unsigned)l.cf) continue;
                            if (q != 0) continue;     // one sibling queues what leaves the bucket
                        }
                        pyr_queue(p, z, gx[a], gy[c], v);
                    }
                }
            }
          }
        }
        __syncthreads();
        if (p.dyadic) {
            // level z from level z + 1: 2x2 sums of the counts, maxima of the keys
            for (int lz = nlev - 2; lz >= 0; --lz) {
                const int f = L[lz].f, fc = L[lz + 1].f;
                const int o = p.fp_off[lz], oc = p.fp_off[lz + 1];
                const int lf = L[lz].lf;
                for (int i = threadIdx.x; i < f * f; i += blockDim.x) {
                    const int r = i >> lf, c = i & (f - 1);
                    const int a = oc + 2 * r * fc + 2 * c;
                    scnt[o + i] = scnt[a] + scnt[a + 1] + scnt[a + fc] + scnt[a + fc + 1];
                    skey[o + i] = max(max(skey[a], skey[a + 1]), max(skey[a + fc], skey[a + fc + 1]));
                }
                __syncthreads();
            }
        }
        const unsigned *rc = scnt, *rk = skey;
        bool write = true;
        if (nch > 1) {
            // A bucket split into chunks: every chunk adds its footprint into the
            // bucket's zeroed slot with bulk reductions (add for counts, max for
            // keys); the chunk that finishes last reads the slot back and writes it.
            const int64_t slot = (int64_t)p.slot_base[b] + q;
            if (slot >= p.slot_cap) {
                write = false;                              // flagged by the plan (cannot happen)
            } else {
                unsigned *dst = p.partials + slot * 2 * p.footprint;
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncthreads();
                if (threadIdx.x == 0) {
                    const unsigned bytes = (unsigned)p.footprint * 4u;
                    const unsigned sa = (unsigned)__cvta_generic_to_shared(scnt);
                    const unsigned sk = (unsigned)__cvta_generic_to_shared(skey);
                    for (unsigned o = 0; o < bytes; o += 16384u) {
                        const unsigned sz = bytes - o < 16384u ? bytes - o : 16384u;
                        asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.u32 [%0], [%1], %2;"
                                     :: "l"((char *)dst + o), "r"(sa + o), "r"(sz) : "memory");
                        asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.max.u32 [%0], [%1], %2;"
                                     :: "l"((char *)(dst + p.footprint) + o), "r"(sk + o), "r"(sz) : "memory");
                    }
                    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
                    asm volatile("fence.proxy.async.global;" ::: "memory");
                    __threadfence();
                    s_last = atomicAdd(&p.done[(int64_t)b * nsub + q], 1u) == nch - 1;
                }
                __syncthreads();
                write = s_last;
                if (write) {
                    __threadfence();
                    const int n4 = (2 * p.footprint) >> 2;
                    for (int i = threadIdx.x; i < n4; i += blockDim.x)
                        ((uint4 *)scnt)[i] = __ldcg((const uint4 *)dst + i);
                    __syncthreads();
                }
            }
        }
        if (write) {
            const double qnan = __longlong_as_double(0x7ff8000000000000ll);
            for (int lz = 0; lz < nlev; ++lz) {
                const PyrLevel &l = L[lz];
                const int z = p.zmin + lz;
                const int row0 = l.gy0 - l.hty * p.ts, col0 = l.gx0 - l.htx * p.ts;
                const int64_t base = p.level_off[lz] +
                                     ((int64_t)((l.hty << z) + l.htx) * p.ts + row0) * p.ts + col0;
                const unsigned *cs = rc + p.fp_off[lz];
                const unsigned *ks = rk + p.fp_off[lz];
                if (l.f >= 4 && p.vec_out) {
                    // four consecutive pixels of a row per thread: one 16-byte count store,
                    // two 16-byte max stores (the offsets are multiples of 4 pixels)
                    const int q4 = (l.f * l.f) >> 2, lq = l.lf - 2;
                    for (int i = threadIdx.x; i < q4; i += blockDim.x) {
                        const int r = i >> lq, c = (i & ((l.f >> 2) - 1)) << 2;
                        const int off = (r << l.lf) + c;
                        const int64_t o = base + (int64_t)r * p.ts + c;
                        const uint4 cv = *(const uint4 *)(cs + off);
                        *(uint4 *)(p.count_out + o) = cv;
                        if (p.max_out) {
                            const uint4 kv = *(const uint4 *)(ks + off);
                            double2 m0, m1;
                            m0.x = kv.x ? f32_to_f64_exact(fkey_value(kv.x)) : qnan;
                            m0.y = kv.y ? f32_to_f64_exact(fkey_value(kv.y)) : qnan;
                            m1.x = kv.z ? f32_to_f64_exact(fkey_value(kv.z)) : qnan;
                            m1.y = kv.w ? f32_to_f64_exact(fkey_value(kv.w)) : qnan;
                            *(double2 *)(p.max_out + o) = m0;
                            *(double2 *)(p.max_out + o + 2) = m1;
                        }
                    }
                } else {
                    for (int i = threadIdx.x; i < l.f * l.f; i += blockDim.x) {
                        const int r = i >> l.lf, c = i & (l.f - 1);
                        const int64_t o = base + (int64_t)r * p.ts + c;
                        p.count_out[o] = cs[i];
                        if (p.max_out) {
                            const unsigned k = ks[i];
                            p.max_out[o] = k ? f32_to_f64_exact(fkey_value(k)) : qnan;
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- spill

__global__ void pyr_spill(const PyrParams p) {
    const int64_t ns = p.ctr->n_spill < p.spill_cap ? (int64_t)p.ctr->n_spill : p.spill_cap;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += (int64_t)gridDim.x * blockDim.x) {
        const PyrSpill s = p.spill[i];
        const int lz = (int)s.z - p.zmin;
        const int tx = (int)s.gx / p.ts, ty = (int)s.gy / p.ts;
        const int64_t o = p.level_off[lz] + ((int64_t)((ty << s.z) + tx) * p.ts + (s.gy % p.ts)) * p.ts +
                          (s.gx % p.ts);
        atomicAdd(&p.count_out[o], 1u);
        if (p.max_out && !(s.v != s.v)) {
            const double v = (double)(s.v == 0.0f ? 0.0f : s.v);
            unsigned long long *a = (unsigned long long *)(p.max_out + o);
            unsigned long long old = *(volatile unsigned long long *)a;
            int it = 0;
            for (; it < PYR_SPILL_CAS_LIMIT; ++it) {
                const double cur = __longlong_as_double((long long)old);
                if (!(cur != cur) && cur >= v) break;
                const unsigned long long got = atomicCAS(a, old, (unsigned long long)__double_as_longlong(v));
                if (got == old) break;
                old = got;
            }
            if (it == PYR_SPILL_CAS_LIMIT) atomicOr(&p.ctr->flags, 2u);
        }
    }
}

// ---------------------------------------------------------------- host side

struct PyrLayout {
    int bls, nbk, nbuckets, nsub, footprint, ntab;
    int64_t fp_bytes, slot_cap, spill_cap;
    size_t off_tab_x, off_tab_y, off_bcount, off_bstart, off_cursor, off_item_base, off_item_bucket, off_slot_base,
        off_done,
        off_ctr, off_sx, off_sy, off_sv, off_bx, off_by, off_bv, off_band, off_partials, off_spill, total;
};

static size_t pyr_align(size_t v) { return (v + 255) / 256 * 256; }

static int pyr_layout(int64_t n, bool has_v, const dsgb_pyramid_config *c, PyrLayout &L) {
    if (!c || n < 0 || n >= (int64_t)0xF0000000ll) return DSGB_E_INVALID;
    if (c->zmin < 0 || c->zmax < c->zmin || c->zmax > PYR_MAX_Z) return DSGB_E_UNSUPPORTED;
    if (c->tile_size < 1 || c->tile_size > 4096 || (c->tile_size & (c->tile_size - 1))) return DSGB_E_UNSUPPORTED;
    if (c->split < 0 || c->split > 2 || c->chunk < 256) return DSGB_E_INVALID;
    if (c->threads != 256 && c->threads != 512 && c->threads != 1024) return DSGB_E_INVALID;
    L.bls = c->zmax + 1;
    const int bl = L.bls + c->split;
    if ((c->tile_size >> (bl - c->zmin)) < 1) return DSGB_E_UNSUPPORTED;     // footprint below one pixel
    L.nbk = 1 << L.bls;
    L.nbuckets = L.nbk * L.nbk;
    L.nsub = 1 << (2 * c->split);
    L.ntab = ntab_of(c->zmax);
    int64_t fp = 0;
    for (int z = c->zmin; z <= c->zmax; ++z) {
        const int64_t f = c->tile_size >> (bl - z);
        fp += (f * f + 3) & ~(int64_t)3;          // every level starts on a 16-byte boundary
    }
    if (fp * 8 > PYR_SMEM_LIMIT) return DSGB_E_UNSUPPORTED;
    L.footprint = (int)fp;
    L.fp_bytes = fp * 8;
    L.slot_cap = (n / c->chunk + 1) * L.nsub;       // a bucket is split only if it holds > chunk rows
    L.spill_cap = n / 64 + (1 << 20);
    size_t o = 0;
    L.off_tab_x = o; o = pyr_align(o + (size_t)L.ntab * sizeof(PyrEntry));
    L.off_tab_y = o; o = pyr_align(o + (size_t)L.ntab * sizeof(PyrEntry));
    L.off_bcount = o; o = pyr_align(o + (size_t)L.nbuckets * 4);
    L.off_bstart = o; o = pyr_align(o + (size_t)(L.nbuckets + 1) * 4);
    L.off_cursor = o; o = pyr_align(o + (size_t)L.nbuckets * 4);
    L.off_item_base = o; o = pyr_align(o + (size_t)(L.nbuckets + 1) * 4);
    // items = sum over buckets of max(1, ceil(count / chunk)) * nsub <= (n / chunk + nbuckets) * nsub
    L.off_item_bucket = o; o = pyr_align(o + ((size_t)(n / c->chunk) + (size_t)L.nbuckets) * L.nsub * 4);
    L.off_slot_base = o; o = pyr_align(o + (size_t)L.nbuckets * 4);
    L.off_done = o; o = pyr_align(o + (size_t)L.nbuckets * L.nsub * 4);
    L.off_ctr = o; o = pyr_align(o + sizeof(PyrCounters));
    L.off_sx = o; o = pyr_align(o + (size_t)n * 4);
    L.off_sy = o; o = pyr_align(o + (size_t)n * 4);
    L.off_sv = o; o = pyr_align(o + (has_v ? (size_t)n * 4 : 0));
    L.off_bx = o; o = pyr_align(o + (size_t)n * 4);
    L.off_by = o; o = pyr_align(o + (size_t)n * 4);
    L.off_bv = o; o = pyr_align(o + (has_v ? (size_t)n * 4 : 0));
    L.off_band = o; o = pyr_align(o + (size_t)L.nbk * 4);
    L.off_partials = o; o = pyr_align(o + (size_t)L.slot_cap * L.fp_bytes);
    L.off_spill = o; o = pyr_align(o + (size_t)L.spill_cap * sizeof(PyrSpill));
    L.total = o;
    return DSGB_OK;
}

// One-time per device: the dynamic shared-memory limits of the kernels and
// the render occupancy for each CTA size (kept out of stream capture).
struct PyrDeviceInfo {
    bool ready = false;
    int sms = 0;
};
static std::mutex g_pyr_mu;
static PyrDeviceInfo g_pyr_dev[64];

static int pyr_device_setup(int &sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "dsgb_pyramid: cudaGetDevice");
    if (dev < 0 || dev >= 64) { set_error("dsgb_pyramid: device ordinal %d out of range", dev); return DSGB_E_INVALID; }
    std::lock_guard<std::mutex> lock(g_pyr_mu);
    PyrDeviceInfo &d = g_pyr_dev[dev];
    if (!d.ready) {
        e = cudaFuncSetAttribute(pyr_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(pyr_band, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)stage_smem_bytes(1 << (PYR_MAX_Z + 1)));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(pyr_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)stage_smem_bytes(PYR_STAGE_MAX_GROUPS));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(pyr_render, cudaFuncAttributeMaxDynamicSharedMemorySize, PYR_SMEM_LIMIT);
        if (e != cudaSuccess) return cuda_status(e, "dsgb_pyramid: cudaFuncSetAttribute");
        d.sms = sm_count();
        if (d.sms <= 0) d.sms = 148;
        d.ready = true;
    }
    sms = d.sms;
    return DSGB_OK;
}

}  // namespace dsgb

using namespace dsgb;

extern "C" int64_t dsgb_pyramid_tile_offset(int32_t zmin, int32_t z, int32_t tile_size) {
    int64_t off = 0;
    for (int32_t k = zmin; k < z; ++k) off += ((int64_t)1 << (2 * k)) * tile_size * tile_size;
    return off;
}

extern "C" size_t dsgb_pyramid_workspace_size(int64_t n, int32_t has_v, const dsgb_pyramid_config *config) {
    PyrLayout L;
    return pyr_layout(n, has_v != 0, config, L) == DSGB_OK ? L.total : 0;
}

extern "C" int dsgb_pyramid(const dsgb_column *cols, int32_t ncols, int64_t n, int32_t x_col, int32_t y_col,
                            int32_t v_col, const dsgb_pyramid_config *config, uint32_t *counts, double *max_out,
                            void *workspace, size_t workspace_bytes, uint32_t flags, void *stream) {
    const int cap_shift = (int)((flags >> 8) & 31u);
    if (!cols || !config || !counts || x_col < 0 || y_col < 0 || x_col >= ncols || y_col >= ncols ||
        v_col >= ncols || (v_col >= 0 && !max_out)) {
        set_error("dsgb_pyramid: invalid arguments");
        return DSGB_E_INVALID;
    }
    if (cols[x_col].dtype != DSGB_F32 || cols[y_col].dtype != DSGB_F32 || (v_col >= 0 && cols[v_col].dtype != DSGB_F32)) {
        set_error("dsgb_pyramid: x, y and v must be float32 columns");
        return DSGB_E_UNSUPPORTED;
    }
    if (!(config->x1 > config->x0) || !(config->y1 > config->y0) || !std::isfinite(config->x0) ||
        !std::isfinite(config->x1) || !std::isfinite(config->y0) || !std::isfinite(config->y1)) {
        set_error("dsgb_pyramid: the square must be finite with x1 > x0 and y1 > y0");
        return DSGB_E_INVALID;
    }
    PyrLayout L;
    int rc = pyr_layout(n, v_col >= 0, config, L);
    if (rc) {
        set_error("dsgb_pyramid: unsupported configuration (zmax <= %d, power-of-two tile size, split 0..2, "
                  "threads 256/512/1024, chunk >= 256, footprint <= %d bytes of shared memory)",
                  PYR_MAX_Z, PYR_SMEM_LIMIT);
        return rc;
    }
    if (!workspace || ((uintptr_t)workspace & 255u) || workspace_bytes < L.total) {
        set_error("dsgb_pyramid: workspace must be 256-byte aligned and at least %zu bytes", L.total);
        return DSGB_E_NOSPACE;
    }
    int sms = 0;
    rc = pyr_device_setup(sms);
    if (rc) return rc;
    PyrParams p;
    memset(&p, 0, sizeof(p));
    p.xs = (const float *)cols[x_col].data;
    p.ys = (const float *)cols[y_col].data;
    p.vs = v_col >= 0 ? (const float *)cols[v_col].data : nullptr;
    p.n = n;
    p.zmin = config->zmin; p.zmax = config->zmax; p.ts = config->tile_size; p.split = config->split;
    p.bls = L.bls; p.nbk = L.nbk; p.nbuckets = L.nbuckets; p.chunk = config->chunk;
    p.vec = (((uintptr_t)p.xs | (uintptr_t)p.ys) & 15u) == 0;
    p.x0 = config->x0; p.x1 = config->x1; p.y0 = config->y0; p.y1 = config->y1;
    p.x0f = (float)p.x0; p.y0f = (float)p.y0;
    p.bscale_x = (float)L.nbk / (float)(p.x1 - p.x0);
    p.bscale_y = (float)L.nbk / (float)(p.y1 - p.y0);
    char *w = (char *)workspace;
    p.tab_x = (PyrEntry *)(w + L.off_tab_x);
    p.tab_y = (PyrEntry *)(w + L.off_tab_y);
    p.bcount = (unsigned *)(w + L.off_bcount);
    p.bstart = (unsigned *)(w + L.off_bstart);
    p.cursor = (unsigned *)(w + L.off_cursor);
    p.item_base = (unsigned *)(w + L.off_item_base);
    p.item_bucket = (unsigned *)(w + L.off_item_bucket);
    p.slot_base = (unsigned *)(w + L.off_slot_base);
    p.done = (unsigned *)(w + L.off_done);
    p.ctr = (PyrCounters *)(w + L.off_ctr);
    p.sx = (float *)(w + L.off_sx);
    p.sy = (float *)(w + L.off_sy);
    p.sv = v_col >= 0 ? (float *)(w + L.off_sv) : nullptr;
    p.bx_ = (float *)(w + L.off_bx);
    p.by_ = (float *)(w + L.off_by);
    p.bv_ = v_col >= 0 ? (float *)(w + L.off_bv) : nullptr;
    p.band_cursor = (unsigned *)(w + L.off_band);
    {
        int ex = 0, ey = 0;
        const double mx = frexp(config->x1 - config->x0, &ex), my = frexp(config->y1 - config->y0, &ey);
        p.dyadic = config->x0 == 0.0 && config->y0 == 0.0 && mx == 0.5 && my == 0.5 &&
                   ex > -100 && ex < 100 && ey > -100 && ey < 100;
    }
    p.partials = (unsigned *)(w + L.off_partials);
    p.slot_cap = L.slot_cap >> cap_shift;
    p.spill = (PyrSpill *)(w + L.off_spill);
    p.spill_cap = L.spill_cap >> cap_shift;
    p.footprint = L.footprint;
    const int bl = L.bls + p.split;
    int fo = 0;
    for (int z = p.zmin; z <= p.zmax; ++z) {
        p.fp_off[z - p.zmin] = fo;
        const int f = p.ts >> (bl - z);
        fo += (f * f + 3) & ~3;
        p.level_off[z - p.zmin] = dsgb_pyramid_tile_offset(p.zmin, z, p.ts);
    }
    p.count_out = counts;
    p.max_out = v_col >= 0 ? max_out : nullptr;
    p.vec_out = ((uintptr_t)counts & 15u) == 0 && ((uintptr_t)p.max_out & 15u) == 0;

    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(p.bcount, 0, (size_t)L.nbuckets * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "dsgb_pyramid memset");
    pyr_tables<<<(2 * L.ntab + 127) / 128, 128, 0, st>>>(p);
    DSGB_CHECK_LAUNCH("pyr_tables");
    pyr_hist<<<sms, PYR_HIST_THREADS, (size_t)L.nbuckets * 4, st>>>(p);
    DSGB_CHECK_LAUNCH("pyr_hist");
    pyr_plan<<<1, 1024, 0, st>>>(p);
    DSGB_CHECK_LAUNCH("pyr_plan");
    pyr_zero_slots<<<sms * 4, 256, 0, st>>>(p);
    DSGB_CHECK_LAUNCH("pyr_zero_slots");
    const int64_t sblocks = (n + PYR_STAGE_ROWS - 1) / PYR_STAGE_ROWS;
    if (sblocks > 0) {
        const int nbands = (L.nbk + PYR_BAND_ROWS - 1) / PYR_BAND_ROWS;
        pyr_band<<<(unsigned)sblocks, PYR_STAGE_THREADS, stage_smem_bytes(nbands), st>>>(p);
        DSGB_CHECK_LAUNCH("pyr_band");
        const int ng = L.nbuckets < PYR_STAGE_MAX_GROUPS ? L.nbuckets : PYR_STAGE_MAX_GROUPS;
        pyr_scatter<<<(unsigned)sblocks, PYR_STAGE_THREADS, stage_smem_bytes(ng), st>>>(p);
        DSGB_CHECK_LAUNCH("pyr_scatter");
    }
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pyr_render, config->threads, (size_t)L.fp_bytes);
    if (e != cudaSuccess) return cuda_status(e, "dsgb_pyramid occupancy");
    if (per_sm < 1) {
        set_error("dsgb_pyramid: the render kernel does not fit on an SM with %d threads", config->threads);
        return DSGB_E_UNSUPPORTED;
    }
    const int grid = sms * per_sm;
    pyr_render<<<grid, config->threads, (size_t)L.fp_bytes, st>>>(p);
    DSGB_CHECK_LAUNCH("pyr_render");
    pyr_spill<<<sms * 2, 256, 0, st>>>(p);
    DSGB_CHECK_LAUNCH("pyr_spill");
    return DSGB_OK;
}

extern "C" int dsgb_pyramid_status(const void *workspace, int64_t n, int32_t has_v,
                                   const dsgb_pyramid_config *config, uint32_t *flags_out, void *stream) {
    PyrLayout L;
    if (!workspace || !flags_out || pyr_layout(n, has_v != 0, config, L) != DSGB_OK) {
        set_error("dsgb_pyramid_status: invalid arguments");
        return DSGB_E_INVALID;
    }
    const PyrCounters *c = (const PyrCounters *)((const char *)workspace + L.off_ctr);
    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaMemcpyAsync(flags_out, &c->flags, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e, "dsgb_pyramid_status");
    return DSGB_OK;
}
