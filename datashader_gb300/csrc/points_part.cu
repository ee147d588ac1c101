// points_part.cu -- Canvas.points for plans of several bases over float32
// coordinates (a summary of count / sum / mean / min / max / first / last /
// where / by): rows partitioned by canvas block, each block aggregated in
// shared memory.
//
// Replaces Point._build_extend (datashader/glyphs/points.py:182-242) with the
// fused append of compiler.make_append (datashader/compiler.py:321-475) for
// these plans.  With one L2 atomic per base and row, such a plan is bound by
// the L2 atomic rate (about 2e11 a second on GB300: 8 bases over 1e8 rows take
// 4 ms).  Here the atomics move into shared memory:
//
//   part_sample  -- bin one tile of 1,024 rows in eight (the exact binning of
//                   binning.cuh) and count them per canvas block (a power-of-two
//                   rectangle of pixels sized so that every base of the plan
//                   fits in shared memory for the whole block);
//   part_plan1   -- one CTA: each block's room, the scaled-up sample count plus
//                   a margin of six standard deviations and 64 rows, laid out
//                   by an exclusive scan;
//   part_scatter -- bin every row (the same function as the sample) and write
//                   one 16-byte record per row {value, row, pixel in the block,
//                   category} into its block's room: a CTA ranks a batch of
//                   2048 rows by block in shared memory and writes each block's
//                   run contiguously; a row that finds the room full (a sample
//                   far off; rare) goes straight into the bases with L2 atomics;
//   part_plan2   -- one CTA: the rows each block holds, split into work items
//                   of at most 2^18;
//   part_reduce  -- persistent CTAs take work items; each initialises every
//                   base over its block in shared memory, applies the item's
//                   records with shared-memory atomics, and adds the block into
//                   the bases: plain read-modify-write when the block is one
//                   item (no other CTA touches it), atomics otherwise.
//
// Every base combines order-independently (counts and sums add, min / max /
// first / last / where keep the smaller row on ties: reductions.py:1178-1182,
// 1223-1227), so the result is the reference's; float64 sums add in another
// order than the reference's row loop (the 1e-12 tolerance of every atomic
// sum).  Rows are processed in chunks of 2^27 so that a record's row fits in
// 32 bits and the records take at most 2 GiB of workspace.
#include "points_params.cuh"

namespace dsgb {
namespace part {

constexpr int HIST_THREADS = 256;
constexpr int SC_THREADS = 512;
constexpr int SC_BATCH = 4 * SC_THREADS;        // rows a scatter CTA ranks at once
constexpr int RD_THREADS = 1024;
constexpr int PLAN_THREADS = 1024;
constexpr int MAX_BLOCKS = 16384;
constexpr int64_t CHUNK = (int64_t)1 << 27;
constexpr int64_t ITEM = (int64_t)1 << 18;
constexpr int64_t MAX_ITEMS = CHUNK / ITEM + MAX_BLOCKS + 1;
constexpr int64_t MIN_ROWS = (int64_t)1 << 20;
constexpr int SAMPLE_LOG = 3;                    // part_sample bins one tile of rows in 2^SAMPLE_LOG
constexpr int SAMPLE_TILE = 256;                 // float4 groups of a sampled tile (1,024 rows)
constexpr int STATE_BUDGET = 200 * 1024;         // shared memory for the bases of one block
constexpr uint8_t CAT_NONE = 0xff;

struct Rec {                                     // 16 bytes
    double v;
    uint32_t row;                                // row within the chunk
    uint16_t lpix;                               // pixel within the block
    uint8_t cat;                                 // category code, CAT_NONE when invalid
    uint8_t pad;
};

struct PBase {
    int32_t op, has_col, has_cat, ncat;
    int32_t off;                                 // byte offset of its block state in shared memory
    int32_t esize;
    int32_t key_off;                             // >= 0: max / min taken from the key of this where() pair state
    void *agg;
};

struct Params {
    const float *xs, *ys;                        // the chunk's first row
    ColumnRef vcol, ccol;                        // value / category column at the chunk's first row (data null: none)
    int64_t n, row0;                             // rows of the chunk, global row of its first row
    int W, H, bw_log, bh_log, bx, nblk;
    int ncat;                                    // categories of the record's code (0: no category column)
    BinAxis ax, ay;
    BinBounds bb;
    // integer classification of the float32 image (when edges_ok holds for both axes)
    int lean;
    float sxf, txf, syf, tyf, exlo, exhi, eylo, eyhi;
    double sx, tx, sy, ty, xmin, xmax, ymin, ymax;
    uint32_t *blk_count, *blk_start, *blk_cursor, *blk_end;
    int64_t rec_cap;                             // records the workspace holds
    Rec *recs;
    int4 *items;                                 // {block, begin, end, owned}
    uint32_t *counters;                          // [0] items, [1] next item
    int nbases, state_bytes;
    PBase bases[MAX_BASES];
    // The common bases by kind, applied by straight-line code: a bit of
    // fast_mask and the shared-memory offset of each; the other bases
    // (rest) take the generic loop.
    unsigned fast_mask;
    int fast_off[16];
    int fast_ncat;                               // categories of KF_COUNT_C
    int nrest;
    int rest[MAX_BASES];
};

enum FastKind {
    KF_COUNT = 0,                                // count() of every row
    KF_COUNT_V,                                  // count('v'): rows with a value
    KF_SUM_V, KF_MAX_V, KF_MIN_V,
    KF_MINROW_V, KF_MAXROW_V,                    // first / last
    KF_ARGMAX_V, KF_ARGMIN_V,                    // where(max / min)
    KF_COUNT_C,                                  // by(cat, count())
    KF_N
};

// The reference formula for a row the float32 image cannot decide: the
// inclusive bounds, then int(x * s + t) in float64 clamped (points.py:199-203);
// packed (xi, yi), or ~0 outside the bounds.
static __device__ __noinline__ unsigned long long exact_xy(float x, float y, const Params *pp) {
    const Params &p = *pp;
    const double dx = (double)x, dy = (double)y;
    if (!(p.xmin <= dx && dx <= p.xmax && p.ymin <= dy && dy <= p.ymax)) return ~0ull;
    const unsigned xi = (unsigned)bin_exact64_st(dx, p.sx, p.tx, p.W);
    const unsigned yi = (unsigned)bin_exact64_st(dy, p.sy, p.ty, p.H);
    return (unsigned long long)xi | ((unsigned long long)yi << 32);
}

// Both passes bin every row with this one function, so they agree on its
// block.  Lean form (the hot-tile kernels' classification, exact under
// edges_ok): v = fma32(x, sf, tf); k = floor(v) by the 1.5 * 2^23 addition
// rounded toward zero; both k in [0, n) with the fraction inside the window
// (E, 1 - E) decide the pixel; a k outside [-1, n] is outside the bounds;
// anything else takes the float64 formula.  Otherwise binning.cuh's bounds
// test and fast path.
__device__ __forceinline__ bool bin_row(const Params &p, float x, float y, int &xi, int &yi) {
    if (p.lean) {
        const float vx = __fmaf_rn(x, p.sxf, p.txf), vy = __fmaf_rn(y, p.syf, p.tyf);
        const float tx = __fadd_rz(vx, 12582912.0f), ty = __fadd_rz(vy, 12582912.0f);
        const int kx = __float_as_int(tx) - 0x4B400000, ky = __float_as_int(ty) - 0x4B400000;
        const float fx = __fsub_rn(vx, __fsub_rn(tx, 12582912.0f)), fy = __fsub_rn(vy, __fsub_rn(ty, 12582912.0f));
        if ((unsigned)kx < (unsigned)p.W && (unsigned)ky < (unsigned)p.H && fx > p.exlo && fx < p.exhi &&
            fy > p.eylo && fy < p.eyhi) {
            xi = kx;
            yi = ky;
            return true;
        }
        if (!((unsigned)(kx + 1) < (unsigned)(p.W + 2) && (unsigned)(ky + 1) < (unsigned)(p.H + 2))) return false;
        const unsigned long long r = exact_xy(x, y, &p);
        if (r == ~0ull) return false;
        xi = (int)(unsigned)r;
        yi = (int)(unsigned)(r >> 32);
        return true;
    }
    const int r = bin_try_f32(x, y, p.bb, p.ax, p.ay, xi, yi);
    if (r == 2) bin_exact_f32(x, y, p.ax, p.ay, xi, yi);
    return r != 0;
}

__device__ __forceinline__ int block_of(const Params &p, int xi, int yi) {
    return (yi >> p.bh_log) * p.bx + (xi >> p.bw_log);
}

__device__ __forceinline__ unsigned local_pixel(const Params &p, int xi, int yi) {
    return ((unsigned)(yi & ((1 << p.bh_log) - 1)) << p.bw_log) | (unsigned)(xi & ((1 << p.bw_log) - 1));
}

// ------------------------------------------------------------ part_sample
// Rows per block, estimated from one tile of 1,024 consecutive rows in every
// 2^SAMPLE_LOG (whole cache lines); part_plan1 gives each block room for the
// estimate and a margin, and part_scatter applies the rows that do not fit
// straight to the bases.
__global__ void __launch_bounds__(HIST_THREADS) part_sample(const __grid_constant__ Params p) {
    extern __shared__ unsigned hist[];
    for (int i = threadIdx.x; i < p.nblk; i += HIST_THREADS) hist[i] = 0;
    __syncthreads();
    const int64_t n4 = p.n >> 2;
    const int64_t ns = ((n4 >> SAMPLE_LOG) / SAMPLE_TILE) * SAMPLE_TILE;     // sampled groups
    const float4 *x4 = (const float4 *)p.xs, *y4 = (const float4 *)p.ys;
    for (int64_t k = (int64_t)blockIdx.x * HIST_THREADS + threadIdx.x; k < ns; k += (int64_t)gridDim.x * HIST_THREADS) {
        const int64_t g = ((k / SAMPLE_TILE) << SAMPLE_LOG) * SAMPLE_TILE + k % SAMPLE_TILE;
        const float4 a = __ldcs(x4 + g), b = __ldcs(y4 + g);
        const float xs[4] = {a.x, a.y, a.z, a.w}, ys[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int xi, yi;
            if (bin_row(p, xs[j], ys[j], xi, yi)) atomicAdd(&hist[block_of(p, xi, yi)], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < p.nblk; i += HIST_THREADS)
        if (hist[i]) atomicAdd(&p.blk_count[i], hist[i]);
}

// Exclusive scan of one value per thread over the CTA; returns the prefix
// and leaves the total in *total.
template <int T>
__device__ __forceinline__ unsigned block_scan(unsigned v, unsigned *warp_sums, unsigned *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < T / 32 ? warp_sums[lane] : 0u;
        unsigned wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += t;
        }
        if (lane < T / 32) warp_sums[lane] = wi - w;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    return warp_sums[warp] + incl - v;
}

// ------------------------------------------------------------ part_plan1
// One CTA, blocks in rounds of PLAN_THREADS: each block's room is its
// estimated rows (the sampled count scaled up) plus a margin of six standard
// deviations of the estimate and 64 rows; the rooms are laid out by an
// exclusive scan.  Room past the workspace's records is cut to nothing (those
// rows then take the direct path).
__device__ __forceinline__ unsigned block_room(unsigned sampled) {
    const double est = (double)sampled * (double)(1 << SAMPLE_LOG);
    return (unsigned)(est + 6.0 * sqrt(est * (double)((1 << SAMPLE_LOG) - 1)) + 64.0);
}

__global__ void __launch_bounds__(PLAN_THREADS) part_plan1(const __grid_constant__ Params p) {
    __shared__ unsigned ws1[32];
    __shared__ unsigned tot1;
    unsigned long long carry = 0;
    for (int r0 = 0; r0 < p.nblk; r0 += PLAN_THREADS) {
        const int b = r0 + threadIdx.x;
        const unsigned cap = b < p.nblk ? block_room(p.blk_count[b]) : 0u;
        const unsigned o = block_scan<PLAN_THREADS>(cap, ws1, &tot1);
        if (b < p.nblk) {
            const unsigned long long start = carry + o;
            const unsigned long long end = start + cap;
            const unsigned s0 = (unsigned)min(start, (unsigned long long)p.rec_cap);
            p.blk_start[b] = s0;
            p.blk_cursor[b] = s0;
            p.blk_end[b] = (unsigned)min(end, (unsigned long long)p.rec_cap);
        }
        carry += tot1;
    }
}

// ------------------------------------------------------------ part_plan2
// One CTA: the rows each block holds (its cursor, at most its room) split
// into work items of at most ITEM rows, ceil(c / m) each.
__global__ void __launch_bounds__(PLAN_THREADS) part_plan2(const __grid_constant__ Params p) {
    __shared__ unsigned ws2[32];
    __shared__ unsigned tot2;
    unsigned carry2 = 0;
    for (int r0 = 0; r0 < p.nblk; r0 += PLAN_THREADS) {
        const int b = r0 + threadIdx.x;
        unsigned c = 0, o1 = 0;
        if (b < p.nblk) {
            o1 = p.blk_start[b];
            c = min(p.blk_cursor[b], p.blk_end[b]) - o1;
        }
        const unsigned m = (unsigned)((c + (unsigned)ITEM - 1) / (unsigned)ITEM);
        const unsigned o2 = block_scan<PLAN_THREADS>(m, ws2, &tot2) + carry2;
        if (b < p.nblk) {
            const unsigned sz = m ? (c + m - 1) / m : 0u;
            for (unsigned j = 0; j < m; ++j) {
                const unsigned lo = j * sz, hi = min(c, lo + sz);
                p.items[o2 + j] = make_int4(b, (int)(o1 + lo), (int)(o1 + hi), m == 1 ? 1 : 0);
            }
        }
        carry2 += tot2;
    }
    if (threadIdx.x == 0) {
        p.counters[0] = carry2;
        p.counters[1] = 0;
    }
}

__device__ __forceinline__ Rec decode(const uint4 q) {
    Rec r;
    r.v = __longlong_as_double((long long)(((unsigned long long)q.y << 32) | q.x));
    r.row = q.z;
    r.lpix = (uint16_t)(q.w & 0xffffu);
    r.cat = (uint8_t)((q.w >> 16) & 0xffu);
    r.pad = 0;
    return r;
}

// A row whose block has no room left: its appends go straight into the bases
// with L2 atomics, as the generic kernel does (reductions combine in any
// order, so the result does not depend on which rows take this path).
static __device__ __noinline__ void apply_direct(const Params *pp, int blk, uint4 q) {
    const Params &p = *pp;
    const Rec r = decode(q);
    const unsigned lx = r.lpix & ((1u << p.bw_log) - 1), ly = (unsigned)r.lpix >> p.bw_log;
    const int64_t gpix = (int64_t)(((blk / p.bx) << p.bh_log) + (int)ly) * p.W + ((blk % p.bx) << p.bw_log) + lx;
    const bool has = !isnull(r.v);
    const long long key = f64_key(r.v);
    const long long row = p.row0 + (long long)r.row;
    for (int b = 0; b < p.nbases; ++b) {
        const PBase &B = p.bases[b];
        if (B.has_col && !has) continue;
        int64_t cell = gpix;
        if (B.has_cat) {
            if (r.cat == CAT_NONE) continue;
            cell = gpix * B.ncat + r.cat;
        }
        switch (B.op) {
        case DSGB_BASE_COUNT: atomicAdd((unsigned *)B.agg + cell, 1u); break;
        case DSGB_BASE_ANY: ((volatile uint8_t *)B.agg)[cell] = 1; break;
        case DSGB_BASE_SUM: atomicAdd((double *)B.agg + cell, r.v); break;
        case DSGB_BASE_MAX: atomic_max_key((long long *)B.agg + cell, key); break;
        case DSGB_BASE_MIN: atomic_min_key((long long *)B.agg + cell, key); break;
        case DSGB_BASE_MIN_ROW: atomic_min_key((long long *)B.agg + cell, row); break;
        case DSGB_BASE_MAX_ROW: atomic_max_key((long long *)B.agg + cell, row); break;
        case DSGB_BASE_ARGMAX: pair_update<true>((long long *)B.agg + 2 * cell, key, row); break;
        case DSGB_BASE_ARGMIN: pair_update<false>((long long *)B.agg + 2 * cell, key, row); break;
        default: break;
        }
    }
}

// ------------------------------------------------------------ part_scatter
__device__ __forceinline__ double load_value(const Params &p, int64_t i) {
    return p.vcol.data ? load_f64(p.vcol, i) : 0.0;
}

__device__ __forceinline__ uint8_t load_code(const Params &p, int64_t i) {
    if (!p.ccol.data) return CAT_NONE;
    long long c = load_i64(p.ccol, i);
    if (c < 0) c += p.ncat;                       // compiler.py:379-390: negative codes wrap
    return (c < 0 || c >= p.ncat) ? CAT_NONE : (uint8_t)c;
}

// Value loads: VK 0 no value column, 1 float64 column (16-byte aligned: two
// double2 per four rows), 2 any other (load_f64).  Code loads: CK 0 none,
// 1 int8 / uint8 (4-byte aligned: one word per four rows), 2 any other.
template <int VK>
__device__ __forceinline__ void load_values4(const Params &p, int64_t g, double (&v)[4]) {
    if (VK == 1) {
        const double2 *v2 = (const double2 *)p.vcol.data;
        const double2 a = __ldcs(v2 + 2 * g), b = __ldcs(v2 + 2 * g + 1);
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = VK == 2 ? load_f64(p.vcol, 4 * g + k) : 0.0;
    }
}

__device__ __forceinline__ unsigned wrap_code(const Params &p, long long c) {
    if (c < 0) c += p.ncat;                       // compiler.py:379-390: negative codes wrap
    return (c < 0 || c >= p.ncat) ? CAT_NONE : (unsigned)c;
}

template <int CK>
__device__ __forceinline__ unsigned load_codes4(const Params &p, int64_t g) {
    if (CK == 0) return 0xffffffffu;
    if (CK == 1) {
        const unsigned w = __ldcs((const unsigned *)p.ccol.data + g);
        const bool sgn = p.ccol.dtype == DSGB_I8;
        unsigned out = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned b = (w >> (8 * k)) & 0xffu;
            const long long c = sgn ? (long long)(int8_t)b : (long long)b;
            out |= wrap_code(p, c) << (8 * k);
        }
        return out;
    }
    unsigned out = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) out |= wrap_code(p, load_i64(p.ccol, 4 * g + k)) << (8 * k);
    return out;
}

template <int VK, int CK>
__global__ void __launch_bounds__(SC_THREADS, 2) part_scatter(const __grid_constant__ Params p) {
    extern __shared__ __align__(16) unsigned char sm[];
    uint4 *stage = (uint4 *)sm;                                   // SC_BATCH records
    uint16_t *sblk = (uint16_t *)(sm + SC_BATCH * sizeof(Rec));   // block of each staged record
    unsigned *hist = (unsigned *)(sm + SC_BATCH * (sizeof(Rec) + 2));   // counts, then staging offsets
    unsigned *delta = hist + p.nblk;                              // record index - staging index of a block's run
    __shared__ unsigned warp_sums[32];
    __shared__ unsigned s_total;
    for (int i = threadIdx.x; i < p.nblk; i += SC_THREADS) hist[i] = 0;
    __syncthreads();
    const int64_t n4 = p.n >> 2;
    const int64_t g0 = n4 * blockIdx.x / gridDim.x, g1 = n4 * (blockIdx.x + 1) / gridDim.x;
    const float4 *x4 = (const float4 *)p.xs, *y4 = (const float4 *)p.ys;
    const int per = (p.nblk + SC_THREADS - 1) / SC_THREADS;       // scan entries per thread
    // the next batch's columns are loaded while this one is ranked and written
    float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nb = na;
    double nv[4] = {0.0, 0.0, 0.0, 0.0};
    unsigned ncodes = 0xffffffffu;
    if (g0 + threadIdx.x < g1) {
        na = __ldcs(x4 + g0 + threadIdx.x);
        nb = __ldcs(y4 + g0 + threadIdx.x);
        load_values4<VK>(p, g0 + threadIdx.x, nv);
        ncodes = load_codes4<CK>(p, g0 + threadIdx.x);
    }
    for (int64_t base = g0; base < g1; base += SC_THREADS) {
        const int64_t g = base + threadIdx.x;
        const bool live = g < g1;
        int blk[4];
        unsigned lp[4], rank[4];
        const float4 a = na, b = nb;
        const double v[4] = {nv[0], nv[1], nv[2], nv[3]};
        const unsigned codes = ncodes;
        if (g + SC_THREADS < g1) {
            na = __ldcs(x4 + g + SC_THREADS);
            nb = __ldcs(y4 + g + SC_THREADS);
            load_values4<VK>(p, g + SC_THREADS, nv);
            ncodes = load_codes4<CK>(p, g + SC_THREADS);
        }
        const float xs[4] = {a.x, a.y, a.z, a.w}, ys[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            int xi, yi;
            blk[k] = -1;
            if (live && bin_row(p, xs[k], ys[k], xi, yi)) {
                blk[k] = block_of(p, xi, yi);
                lp[k] = local_pixel(p, xi, yi);
            }
            if (blk[k] >= 0) rank[k] = atomicAdd(&hist[blk[k]], 1u);
        }
        __syncthreads();
        // offsets of the blocks in the staging area, and their runs' places in the records
        const int e0 = threadIdx.x * per;
        {
            unsigned s = 0;
            for (int j = 0; j < per; ++j) {
                const int e = e0 + j;
                if (e < p.nblk) s += hist[e];
            }
            unsigned o = block_scan<SC_THREADS>(s, warp_sums, &s_total);
            for (int j = 0; j < per; ++j) {
                const int e = e0 + j;
                if (e >= p.nblk) break;
                const unsigned h = hist[e];
                hist[e] = o;
                if (h) delta[e] = atomicAdd(&p.blk_cursor[e], h) - o;
                o += h;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (blk[k] < 0) continue;
            const unsigned pos = hist[blk[k]] + rank[k];
            if (pos >= (unsigned)SC_BATCH) { raise_status(DSGB_STATUS_INDEX); continue; }
            const unsigned long long vb = (unsigned long long)__double_as_longlong(v[k]);
            stage[pos] = make_uint4((unsigned)vb, (unsigned)(vb >> 32), (unsigned)(4 * g + k),
                                    lp[k] | (((codes >> (8 * k)) & 0xffu) << 16));
            sblk[pos] = (uint16_t)blk[k];
        }
        __syncthreads();
        const unsigned total = s_total;
        for (unsigned i = threadIdx.x; i < total; i += SC_THREADS) {
            const uint4 q = stage[i];
            const unsigned e = sblk[i];
            if (e >= (unsigned)p.nblk) { raise_status(DSGB_STATUS_INDEX); continue; }
            const unsigned dst = delta[e] + i;
            if (dst < __ldg(p.blk_end + e)) __stcg((uint4 *)(p.recs + dst), q);
            else apply_direct(&p, e, q);          // the block's room is full
        }
        for (int j = 0; j < per; ++j) {
            const int e = e0 + j;
            if (e < p.nblk) hist[e] = 0;
        }
        __syncthreads();
    }
    if (blockIdx.x == gridDim.x - 1) {
        // the rows after the last float4 (at most 3)
        for (int64_t i = 4 * n4 + threadIdx.x; i < p.n; i += SC_THREADS) {
            int xi, yi;
            if (!bin_row(p, p.xs[i], p.ys[i], xi, yi)) continue;
            const int e = block_of(p, xi, yi);
            Rec r;
            r.v = load_value(p, i);
            r.row = (uint32_t)i;
            r.lpix = (uint16_t)local_pixel(p, xi, yi);
            r.cat = load_code(p, i);
            r.pad = 0;
            const unsigned dst = atomicAdd(&p.blk_cursor[e], 1u);
            if (dst < p.blk_end[e]) p.recs[dst] = r;
            else apply_direct(&p, e, make_uint4((unsigned)__double_as_longlong(r.v),
                                                (unsigned)((unsigned long long)__double_as_longlong(r.v) >> 32),
                                                r.row, (unsigned)r.lpix | ((unsigned)r.cat << 16)));
        }
    }
}

// ------------------------------------------------------------ part_reduce

__device__ __forceinline__ void cas128_shared(unsigned addr, long long cmp_lo, long long cmp_hi, long long new_lo,
                                              long long new_hi, long long &old_lo, long long &old_hi) {
    asm volatile(
        "{\n\t.reg .b128 d, c, n;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 n, {%4, %5};\n\t"
        "atom.shared.cas.b128 d, [%6], c, n;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(old_lo), "=l"(old_hi)
        : "l"(cmp_lo), "l"(cmp_hi), "l"(new_lo), "l"(new_hi), "r"(addr)
        : "memory");
}

// pair_update (dsgb_internal.cuh) on a shared-memory pair.
template <bool MAX>
__device__ __forceinline__ void pair_update_shared(long long *slot, long long key, long long row) {
    // the pre-check may read a stale key: keys only improve, so a stale key
    // strictly better than ours still proves the slot better
    long long ok = slot[0];
    if (MAX ? (ok > key) : (ok < key)) return;
    long long orow = ((volatile long long *)slot)[1];
    ok = ((volatile long long *)slot)[0];
    const unsigned addr = (unsigned)__cvta_generic_to_shared(slot);
    for (int guard = 0; guard < (1 << 24); ++guard) {
        long long rk, rr;
        if (!pair_better<MAX>(key, row, ok, orow)) {
            cas128_shared(addr, ok, orow, ok, orow, rk, rr);
            if (rk == ok && rr == orow) return;
        } else {
            cas128_shared(addr, ok, orow, key, row, rk, rr);
            if (rk == ok && rr == orow) return;
        }
        ok = rk; orow = rr;
    }
    raise_status(DSGB_STATUS_CAS_GUARD);
}

__device__ __forceinline__ void init_state(const Params &p, unsigned char *sm, int px) {
    for (int b = 0; b < p.nbases; ++b) {
        const PBase &B = p.bases[b];
        const int cells = px * (B.has_cat ? B.ncat : 1);
        unsigned char *s = sm + B.off;
        switch (B.op) {
        case DSGB_BASE_COUNT:
            for (int i = threadIdx.x; i < cells; i += RD_THREADS) ((unsigned *)s)[i] = 0u;
            break;
        case DSGB_BASE_ANY:
            for (int i = threadIdx.x; i < cells; i += RD_THREADS) s[i] = 0;
            break;
        case DSGB_BASE_SUM:
            for (int i = threadIdx.x; i < cells; i += RD_THREADS) ((double *)s)[i] = 0.0;
            break;
        case DSGB_BASE_MAX:
            for (int i = threadIdx.x; i < cells; i += RD_THREADS) ((long long *)s)[i] = KEY_EMPTY_MAX;
            break;
        case DSGB_BASE_MIN:
            for (int i = threadIdx.x; i < cells; i += RD_THREADS) ((long long *)s)[i] = KEY_EMPTY_MIN;
            break;
        case DSGB_BASE_MIN_ROW:
            for (int i = threadIdx.x; i < cells; i += RD_THREADS) ((long long *)s)[i] = ROW_EMPTY_MIN;
            break;
        case DSGB_BASE_MAX_ROW:
            for (int i = threadIdx.x; i < cells; i += RD_THREADS) ((long long *)s)[i] = -1;
            break;
        case DSGB_BASE_ARGMAX: case DSGB_BASE_ARGMIN: {
            const long long k0 = B.op == DSGB_BASE_ARGMAX ? KEY_EMPTY_MAX : KEY_EMPTY_MIN;
            for (int i = threadIdx.x; i < cells; i += RD_THREADS) {
                ((long long *)s)[2 * i] = k0;
                ((long long *)s)[2 * i + 1] = ROW_EMPTY_MIN;
            }
            break;
        }
        default: break;
        }
    }
}


// One record into every base's block state: the common kinds first, by
// warp-uniform tests of fast_mask, then the rest by the generic loop.
__device__ __forceinline__ void apply(const Params &p, unsigned char *sm, const Rec &r) {
    if (r.lpix >= (1u << (p.bw_log + p.bh_log)) || (r.cat != CAT_NONE && r.cat >= p.ncat)) {
        raise_status(DSGB_STATUS_INDEX);        // a record outside its block: never written by part_scatter
        return;
    }
    const bool has = !isnull(r.v);
    const long long key = f64_key(r.v);
    const long long row = p.row0 + (long long)r.row;
    const unsigned m = p.fast_mask;
    const unsigned lp = r.lpix;
    if (m & (1u << KF_COUNT)) atomicAdd((unsigned *)(sm + p.fast_off[KF_COUNT]) + lp, 1u);
    if ((m & (1u << KF_COUNT_C)) && r.cat != CAT_NONE)
        atomicAdd((unsigned *)(sm + p.fast_off[KF_COUNT_C]) + lp * (unsigned)p.fast_ncat + r.cat, 1u);
    if (has) {
        if (m & (1u << KF_COUNT_V)) atomicAdd((unsigned *)(sm + p.fast_off[KF_COUNT_V]) + lp, 1u);
        if (m & (1u << KF_SUM_V)) atomicAdd((double *)(sm + p.fast_off[KF_SUM_V]) + lp, r.v);
        // pre-checks read without ordering: keys and rows only improve, so a
        // stale read costs at most a redundant atomic
        if (m & (1u << KF_MAX_V)) {
            long long *q = (long long *)(sm + p.fast_off[KF_MAX_V]) + lp;
            if (*q < key) atomicMax(q, key);
        }
        if (m & (1u << KF_MIN_V)) {
            long long *q = (long long *)(sm + p.fast_off[KF_MIN_V]) + lp;
            if (*q > key) atomicMin(q, key);
        }
        if (m & (1u << KF_MINROW_V)) {
            long long *q = (long long *)(sm + p.fast_off[KF_MINROW_V]) + lp;
            if (*q > row) atomicMin(q, row);
        }
        if (m & (1u << KF_MAXROW_V)) {
            long long *q = (long long *)(sm + p.fast_off[KF_MAXROW_V]) + lp;
            if (*q < row) atomicMax(q, row);
        }
        if (m & (1u << KF_ARGMAX_V))
            pair_update_shared<true>((long long *)(sm + p.fast_off[KF_ARGMAX_V]) + 2 * lp, key, row);
        if (m & (1u << KF_ARGMIN_V))
            pair_update_shared<false>((long long *)(sm + p.fast_off[KF_ARGMIN_V]) + 2 * lp, key, row);
    }
#pragma unroll 1
    for (int j = 0; j < p.nrest; ++j) {
        const PBase &B = p.bases[p.rest[j]];
        if (B.has_col && !has) continue;
        unsigned cell = r.lpix;
        if (B.has_cat) {
            if (r.cat == CAT_NONE) continue;
            cell = cell * (unsigned)B.ncat + r.cat;
        }
        unsigned char *s = sm + B.off;
        switch (B.op) {
        case DSGB_BASE_COUNT: atomicAdd((unsigned *)s + cell, 1u); break;
        case DSGB_BASE_ANY: s[cell] = 1; break;
        case DSGB_BASE_SUM: atomicAdd((double *)s + cell, r.v); break;
        case DSGB_BASE_MAX: {
            long long *q = (long long *)s + cell;
            if (*q < key) atomicMax(q, key);
            break;
        }
        case DSGB_BASE_MIN: {
            long long *q = (long long *)s + cell;
            if (*q > key) atomicMin(q, key);
            break;
        }
        case DSGB_BASE_MIN_ROW: {
            long long *q = (long long *)s + cell;
            if (*q > row) atomicMin(q, row);
            break;
        }
        case DSGB_BASE_MAX_ROW: {
            long long *q = (long long *)s + cell;
            if (*q < row) atomicMax(q, row);
            break;
        }
        case DSGB_BASE_ARGMAX: pair_update_shared<true>((long long *)s + 2 * cell, key, row); break;
        case DSGB_BASE_ARGMIN: pair_update_shared<false>((long long *)s + 2 * cell, key, row); break;
        default: break;
        }
    }
}

// The block's state into the bases: read-modify-write when this CTA owns
// the block, atomics otherwise.  A thread takes a pixel and every base's
// cells of it; pixels that no record reached (a zero count() when the plan
// has one) and cells holding the identity are skipped.
__device__ __forceinline__ void flush_state(const Params &p, const unsigned char *sm, int blk, bool owned) {
    const int x0 = (blk % p.bx) << p.bw_log, y0 = (blk / p.bx) << p.bh_log;
    const int w = min(1 << p.bw_log, p.W - x0), h = min(1 << p.bh_log, p.H - y0);
    const int npx = h << p.bw_log;
    const bool counted = (p.fast_mask & (1u << KF_COUNT)) != 0;
    const unsigned *cnt = (const unsigned *)(sm + p.fast_off[KF_COUNT]);
    for (int q = threadIdx.x; q < npx; q += RD_THREADS) {
        const int lx = q & ((1 << p.bw_log) - 1), ly = q >> p.bw_log;
        if (lx >= w) continue;
        if (counted && cnt[q] == 0) continue;
        const int64_t gpix = (int64_t)(y0 + ly) * p.W + (x0 + lx);
#pragma unroll 1
        for (int b = 0; b < p.nbases; ++b) {
            const PBase &B = p.bases[b];
            const int nc = B.ncat;
            const unsigned char *s = sm + B.off;
#pragma unroll 1
            for (int c = 0; c < nc; ++c) {
                const int lc = q * nc + c;
                const int64_t gc = gpix * nc + c;
                switch (B.op) {
                case DSGB_BASE_COUNT: {
                    const unsigned v = ((const unsigned *)s)[lc];
                    if (!v) break;
                    unsigned *d = (unsigned *)B.agg + gc;
                    if (owned) *d += v; else atomicAdd(d, v);
                    break;
                }
                case DSGB_BASE_ANY:
                    if (s[lc]) ((uint8_t *)B.agg)[gc] = 1;
                    break;
                case DSGB_BASE_SUM: {
                    const double v = ((const double *)s)[lc];
                    if (v == 0.0) break;
                    double *d = (double *)B.agg + gc;
                    if (owned) *d += v; else atomicAdd(d, v);
                    break;
                }
                case DSGB_BASE_MAX: case DSGB_BASE_MAX_ROW: {
                    const long long v = B.key_off >= 0 ? ((const long long *)(sm + B.key_off))[2 * lc]
                                                       : ((const long long *)s)[lc];
                    if (v == (B.op == DSGB_BASE_MAX ? KEY_EMPTY_MAX : -1ll)) break;
                    long long *d = (long long *)B.agg + gc;
                    if (owned) { if (v > *d) *d = v; }
                    else atomic_max_key(d, v);
                    break;
                }
                case DSGB_BASE_MIN: case DSGB_BASE_MIN_ROW: {
                    const long long v = B.key_off >= 0 ? ((const long long *)(sm + B.key_off))[2 * lc]
                                                       : ((const long long *)s)[lc];
                    if (v == KEY_EMPTY_MIN) break;             // == ROW_EMPTY_MIN
                    long long *d = (long long *)B.agg + gc;
                    if (owned) { if (v < *d) *d = v; }
                    else atomic_min_key(d, v);
                    break;
                }
                case DSGB_BASE_ARGMAX: case DSGB_BASE_ARGMIN: {
                    const bool mx = B.op == DSGB_BASE_ARGMAX;
                    const long long k = ((const long long *)s)[2 * lc], r = ((const long long *)s)[2 * lc + 1];
                    if (r == ROW_EMPTY_MIN) break;
                    long long *d = (long long *)B.agg + 2 * gc;
                    if (owned) {
                        if (mx ? pair_better<true>(k, r, d[0], d[1]) : pair_better<false>(k, r, d[0], d[1])) {
                            d[0] = k;
                            d[1] = r;
                        }
                    } else if (mx) {
                        pair_update<true>(d, k, r);
                    } else {
                        pair_update<false>(d, k, r);
                    }
                    break;
                }
                default: break;
                }
            }
        }
    }
}

__global__ void __launch_bounds__(RD_THREADS, 1) part_reduce(const __grid_constant__ Params p) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ int s_item;
    const int px = 1 << (p.bw_log + p.bh_log);
    const unsigned nitems = p.counters[0];
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(&p.counters[1], 1u);
        __syncthreads();
        const int it = s_item;
        if ((unsigned)it >= nitems) break;
        const int4 item = p.items[it];
        if (item.x < 0 || item.x >= p.nblk || item.y < 0 || item.y > item.z || (int64_t)item.z > p.rec_cap) {
            raise_status(DSGB_STATUS_INDEX);
            __syncthreads();
            continue;
        }
        init_state(p, sm, px);
        __syncthreads();
        const uint4 *src = (const uint4 *)p.recs;
        // four records a thread in flight: the loads are issued before the
        // shared-memory updates of any of them
        int64_t i = (int64_t)item.y + threadIdx.x;
        for (; i + 3 * RD_THREADS < item.z; i += 4 * RD_THREADS) {
            uint4 q[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) q[k] = __ldcs(src + i + k * RD_THREADS);
#pragma unroll
            for (int k = 0; k < 4; ++k) apply(p, sm, decode(q[k]));
        }
        for (; i < item.z; i += RD_THREADS) apply(p, sm, decode(__ldcs(src + i)));
        __syncthreads();
        flush_state(p, sm, item.x, item.w != 0);
        __syncthreads();
    }
}

// ------------------------------------------------------------ host

static int elem_size(int op) {
    switch (op) {
    case DSGB_BASE_COUNT: return 4;
    case DSGB_BASE_ANY: return 1;
    case DSGB_BASE_SUM: case DSGB_BASE_MAX: case DSGB_BASE_MIN: case DSGB_BASE_MIN_ROW: case DSGB_BASE_MAX_ROW:
        return 8;
    case DSGB_BASE_ARGMAX: case DSGB_BASE_ARGMIN: return 16;
    default: return 0;
    }
}

// Shared-memory bytes of one pixel over all bases (0: a base this path does
// not serve, or columns it cannot share).
static int pixel_bytes(const dsgb_base *bases, int nbases, int &vcol, int &ccol, int &ncat) {
    vcol = -1; ccol = -1; ncat = 0;
    int total = 0;
    for (int b = 0; b < nbases; ++b) {
        const dsgb_base &B = bases[b];
        const int es = elem_size(B.op);
        if (!es) return 0;
        if (B.col >= 0) {
            if (vcol >= 0 && vcol != B.col) return 0;       // one value column
            vcol = B.col;
        }
        if (B.cat_col >= 0) {
            if ((ccol >= 0 && (ccol != B.cat_col || ncat != B.ncat)) || B.ncat < 1 || B.ncat > 255) return 0;
            ccol = B.cat_col;
            ncat = B.ncat;
        }
        total += es * (B.cat_col >= 0 ? B.ncat : 1);
    }
    return total;
}

// Block geometry: the most pixels (a power of two, at most 2^16 so that a
// pixel fits the record's 16 bits) whose state fits the budget; 64 pixels
// wide at most.
static bool geometry(int bpp, int W, int H, int &bw_log, int &bh_log, int &bx, int &nblk) {
    if (bpp <= 0) return false;
    int lg = 0;
    while (lg < 16 && ((int64_t)bpp << (lg + 1)) + 16 * MAX_BASES <= STATE_BUDGET) ++lg;
    if (lg < 6) return false;
    bw_log = std::min(lg, 6);
    bh_log = lg - bw_log;
    bx = (W + (1 << bw_log) - 1) >> bw_log;
    const int by = (H + (1 << bh_log) - 1) >> bh_log;
    if ((int64_t)bx * by > MAX_BLOCKS) return false;
    nblk = bx * by;
    return true;
}

static size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

// Records the workspace holds for a pass of `rows` rows over `nblk` blocks:
// the rows, plus the blocks' margins (six standard deviations of a sampled
// estimate and 64 rows each, at most 6 * sqrt(7 * nblk * rows) + 64 * nblk
// together), plus 1/16 for the sampling error of the estimates' sum.
static int64_t record_room(int64_t rows, int nblk) {
    return rows + rows / 16 + 64 * (int64_t)nblk +
           (int64_t)(6.0 * sqrt(7.0 * (double)nblk * (double)rows)) + 1024;
}

constexpr size_t BLK_ARRAYS = (size_t)4 * MAX_BLOCKS * 4;     // count, start, cursor, end

}  // namespace part

// Workspace of the partitioned path for n rows (0 when the bases are not served).
size_t part_workspace_size(int64_t n, const dsgb_canvas *cv, const dsgb_base *bases, int32_t nbases) {
    using namespace part;
    if (n < MIN_ROWS || !cv || nbases < 1) return 0;
    int vcol, ccol, ncat, bwl, bhl, bx, nblk;
    const int bpp = pixel_bytes(bases, nbases, vcol, ccol, ncat);
    if (!geometry(bpp, cv->width, cv->height, bwl, bhl, bx, nblk)) return 0;
    const int64_t rows = std::min(n, CHUNK);
    return align16((size_t)record_room(rows, nblk) * sizeof(Rec)) + align16((size_t)MAX_ITEMS * sizeof(int4)) +
           BLK_ARRAYS + 16;
}

// DSGB_E_UNSUPPORTED when the case is not served (the caller takes the
// generic kernels).  The bases hold their initial values (or a previous
// call's, when accumulating); the call adds the rows into them.
int launch_points_part(const PointsParams &pp, const dsgb_base *bases, void *ws, size_t ws_bytes, cudaStream_t st) {
    using namespace part;
    if (!ws || pp.n < MIN_ROWS) return DSGB_E_UNSUPPORTED;
    const ColumnRef &xc = pp.cols[pp.x_col], &yc = pp.cols[pp.y_col];
    if (xc.dtype != DSGB_F32 || yc.dtype != DSGB_F32 || (((uintptr_t)xc.data | (uintptr_t)yc.data) & 15u))
        return DSGB_E_UNSUPPORTED;
    if (pp.x_log || pp.y_log || !fast_path_ok(pp.ax, pp.ay)) return DSGB_E_UNSUPPORTED;
    int vcol, ccol, ncat;
    const int bpp = pixel_bytes(bases, pp.nbases, vcol, ccol, ncat);
    Params p;
    memset(&p, 0, sizeof(p));
    if (!geometry(bpp, pp.width, pp.height, p.bw_log, p.bh_log, p.bx, p.nblk)) return DSGB_E_UNSUPPORTED;
    const int64_t rows = std::min(pp.n, CHUNK);
    p.rec_cap = record_room(rows, p.nblk);
    const size_t rec_bytes = align16((size_t)p.rec_cap * sizeof(Rec));
    const size_t item_bytes = align16((size_t)MAX_ITEMS * sizeof(int4));
    const size_t need = rec_bytes + item_bytes + BLK_ARRAYS + 16;
    if (ws_bytes < need || ((uintptr_t)ws & 15u)) return DSGB_E_UNSUPPORTED;
    unsigned char *w = (unsigned char *)ws;
    p.recs = (Rec *)w;
    p.items = (int4 *)(w + rec_bytes);
    p.blk_count = (uint32_t *)(w + rec_bytes + item_bytes);
    p.blk_start = p.blk_count + MAX_BLOCKS;
    p.blk_cursor = p.blk_start + MAX_BLOCKS;
    p.blk_end = p.blk_cursor + MAX_BLOCKS;
    p.counters = (uint32_t *)(w + rec_bytes + item_bytes + BLK_ARRAYS);
    p.W = pp.width; p.H = pp.height;
    p.ax = pp.ax; p.ay = pp.ay; p.bb = pp.bb;
    p.lean = edges_ok(pp.bb.xminf, pp.bb.xmaxf, pp.sx, pp.tx, pp.width) &&
             edges_ok(pp.bb.yminf, pp.bb.ymaxf, pp.sy, pp.ty, pp.height);
    p.sxf = pp.ax.sf; p.txf = pp.ax.tf; p.syf = pp.ay.sf; p.tyf = pp.ay.tf;
    p.exlo = float_ceil_of((double)pp.ax.e); p.exhi = float_floor_of(1.0 - (double)pp.ax.e);
    p.eylo = float_ceil_of((double)pp.ay.e); p.eyhi = float_floor_of(1.0 - (double)pp.ay.e);
    p.sx = pp.sx; p.tx = pp.tx; p.sy = pp.sy; p.ty = pp.ty;
    p.xmin = pp.xmin; p.xmax = pp.xmax; p.ymin = pp.ymin; p.ymax = pp.ymax;
    p.ncat = ncat;
    p.nbases = pp.nbases;
    const int px = 1 << (p.bw_log + p.bh_log);
    int off = 0;
    for (int b = 0; b < pp.nbases; ++b) {
        const dsgb_base &B = bases[b];
        PBase &q = p.bases[b];
        q.op = B.op;
        q.has_col = B.col >= 0;
        q.has_cat = B.cat_col >= 0;
        q.ncat = B.cat_col >= 0 ? B.ncat : 1;
        q.esize = elem_size(B.op);
        q.off = off;
        q.agg = B.agg;
        off += (int)align16((size_t)px * q.ncat * q.esize);
    }
    p.state_bytes = off;
    for (int b = 0; b < pp.nbases; ++b) {
        const PBase &q = p.bases[b];
        int k = -1;
        if (!q.has_cat) {
            switch (q.op) {
            case DSGB_BASE_COUNT: k = q.has_col ? KF_COUNT_V : KF_COUNT; break;
            case DSGB_BASE_SUM: k = q.has_col ? KF_SUM_V : -1; break;
            case DSGB_BASE_MAX: k = q.has_col ? KF_MAX_V : -1; break;
            case DSGB_BASE_MIN: k = q.has_col ? KF_MIN_V : -1; break;
            case DSGB_BASE_MIN_ROW: k = q.has_col ? KF_MINROW_V : -1; break;
            case DSGB_BASE_MAX_ROW: k = q.has_col ? KF_MAXROW_V : -1; break;
            case DSGB_BASE_ARGMAX: k = q.has_col ? KF_ARGMAX_V : -1; break;
            case DSGB_BASE_ARGMIN: k = q.has_col ? KF_ARGMIN_V : -1; break;
            default: break;
            }
        } else if (q.op == DSGB_BASE_COUNT && !q.has_col) {
            k = KF_COUNT_C;
            p.fast_ncat = q.ncat;
        }
        if (k >= 0 && !(p.fast_mask & (1u << k))) {
            p.fast_mask |= 1u << k;
            p.fast_off[k] = q.off;
        } else {
            p.rest[p.nrest++] = b;
        }
    }
    // max('v') beside where(max('v')) (and min beside where(min)): the pair's
    // key is the maximum, so the max base is not updated per row and its flush
    // reads the pair's key
    for (int b = 0; b < pp.nbases; ++b) p.bases[b].key_off = -1;
    const int pairs[2][2] = {{KF_MAX_V, KF_ARGMAX_V}, {KF_MIN_V, KF_ARGMIN_V}};
    for (const auto &pr : pairs) {
        if ((p.fast_mask & (1u << pr[0])) && (p.fast_mask & (1u << pr[1]))) {
            for (int b = 0; b < pp.nbases; ++b)
                if (p.bases[b].off == p.fast_off[pr[0]]) p.bases[b].key_off = p.fast_off[pr[1]];
            p.fast_mask &= ~(1u << pr[0]);
        }
    }
    const int sms = sm_count();
    if (sms <= 0) return cuda_status(cudaErrorNoDevice, "points part: device");
    const size_t sc_smem = (size_t)SC_BATCH * (sizeof(Rec) + 2) + (size_t)2 * p.nblk * 4;
    // value and code load forms (the chunk starts keep the columns' alignment: 2^27 rows)
    const int VK = vcol < 0 ? 0 : (pp.cols[vcol].dtype == DSGB_F64 && !((uintptr_t)pp.cols[vcol].data & 15u)) ? 1 : 2;
    const int CK = ccol < 0 ? 0
                 : ((pp.cols[ccol].dtype == DSGB_I8 || pp.cols[ccol].dtype == DSGB_U8) &&
                    !((uintptr_t)pp.cols[ccol].data & 3u)) ? 1 : 2;
    void (*scatter)(Params) = nullptr;
#define DSGB_SC(V, C) if (VK == V && CK == C) scatter = part_scatter<V, C>;
    DSGB_SC(0, 0) DSGB_SC(0, 1) DSGB_SC(0, 2) DSGB_SC(1, 0) DSGB_SC(1, 1) DSGB_SC(1, 2)
    DSGB_SC(2, 0) DSGB_SC(2, 1) DSGB_SC(2, 2)
#undef DSGB_SC
    cudaError_t e = cudaFuncSetAttribute(part_reduce, cudaFuncAttributeMaxDynamicSharedMemorySize, p.state_bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc_smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(part_sample, cudaFuncAttributeMaxDynamicSharedMemorySize, p.nblk * 4);
    if (e != cudaSuccess) return cuda_status(e, "points part: shared memory attribute");
    int sc_per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sc_per_sm, scatter, SC_THREADS, sc_smem);
    if (e != cudaSuccess || sc_per_sm < 1) return cuda_status(e, "points part: scatter occupancy");
    for (int64_t c0 = 0; c0 < pp.n; c0 += CHUNK) {
        const int64_t m = std::min(CHUNK, pp.n - c0);
        p.n = m;
        p.row0 = pp.row_offset + c0;
        p.xs = (const float *)xc.data + c0;
        p.ys = (const float *)yc.data + c0;
        p.vcol.data = nullptr;
        p.ccol.data = nullptr;
        if (vcol >= 0) {
            p.vcol.dtype = pp.cols[vcol].dtype;
            p.vcol.data = (const unsigned char *)pp.cols[vcol].data + c0 * dtype_size(p.vcol.dtype);
        }
        if (ccol >= 0) {
            p.ccol.dtype = pp.cols[ccol].dtype;
            p.ccol.data = (const unsigned char *)pp.cols[ccol].data + c0 * dtype_size(p.ccol.dtype);
        }
        e = cudaMemsetAsync(p.blk_count, 0, (size_t)p.nblk * 4, st);
        if (e != cudaSuccess) return cuda_status(e, "points part: memset");
        const int64_t n4 = m >> 2;
        const int64_t ns = n4 >> SAMPLE_LOG;
        const int sample_grid =
            (int)std::min<int64_t>((int64_t)sms * 8, std::max<int64_t>(1, (ns + HIST_THREADS - 1) / HIST_THREADS));
        part_sample<<<sample_grid, HIST_THREADS, (size_t)p.nblk * 4, st>>>(p);
        part_plan1<<<1, PLAN_THREADS, 0, st>>>(p);
        const int sc_grid = (int)std::min<int64_t>((int64_t)sms * sc_per_sm, std::max<int64_t>(1, n4 / SC_THREADS));
        scatter<<<sc_grid, SC_THREADS, sc_smem, st>>>(p);
        part_plan2<<<1, PLAN_THREADS, 0, st>>>(p);
        part_reduce<<<sms, RD_THREADS, p.state_bytes, st>>>(p);
        DSGB_CHECK_LAUNCH("points part: launch");
    }
    return DSGB_OK;
}

DSGB_STATUS_READER(status_points_part)

}  // namespace dsgb
