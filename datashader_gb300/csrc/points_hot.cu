// points_hot.cu -- Canvas.points count() of float32 coordinates on GB300.
//
// Replaces Point._build_extend (datashader/glyphs/points.py:182-242) with
// the count append (reductions.py:580-584) for the common case: float32 x/y,
// a linear canvas of at most 8192 16x16-pixel tiles, at least 2^20 rows.
//
// One CTA of 1024 threads per SM streams a contiguous share of the rows.
//   prologue -- the CTA bins 4096 of its own rows (one float4 of x and of y
//               per thread, spread over its share) into a tile histogram in
//               shared memory and keeps the K most populated tiles (K ~ 430)
//               as 16-bit counters, one per pixel;
//   main     -- four rows per thread per step, each binned and counted by an
//               inline-PTX body: the float32 binning of binning.cuh, a
//               classification on the integer bins (fast / exact path / out of
//               bounds), the tile lookup, and one predicated increment: a
//               shared-memory atomic on the pixel's 16-bit counter or an L2
//               reduction on the output.  Rows the float32 image cannot decide
//               take the float64 formula out of line;
//   flush    -- the counters are widened to 32 bits in place, a tile at a
//               time, and added into the output by a TMA tensor reduction
//               (one 16x16 box per tile).
//
// 16-bit counters double the pixels a CTA keeps on chip.  They stay exact:
// an increment returns the old word; a thread that saw a half at or above
// 0x8000 moves 0x8000 of it to the output with a CAS before its next batch
// of increments.  Each thread adds at most 4 between checks, so a half can
// exceed 0x8000 by at most 4 * 1024 before a correction lands and never
// carries into its neighbour (see fix_words).  Results are bit-identical to
// the reference.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "dsgb_internal.cuh"
#include "binning.cuh"

namespace dsgb {
namespace hot {

constexpr int THREADS = 1024;
constexpr int TS = 4;                       // tiles of 16x16 pixels
constexpr int TILE_PX = 1 << (2 * TS);
constexpr int MAX_TILES = 8192;             // tile -> slot table (int16)
constexpr int MAX_SLOTS = 512;
constexpr int DYN_SMEM = 232448 - 2048;     // dynamic shared memory; the static arrays take the rest
constexpr int64_t MIN_ROWS = 1 << 20;
constexpr int SAMPLE_GROUPS = 1;            // float4 groups of x / y a thread samples for the tile choice (count)
constexpr int MEAN_SAMPLE_GROUPS = 2;       // the same for mean
constexpr float MAGIC = 12582912.0f;        // 1.5 * 2^23
constexpr int MAGIC_BITS = 0x4B400000;

struct Params {
    const float *xs, *ys;
    int64_t n, n4;
    int W, H, tiles_x, ntiles, K;
    float sxf, txf, syf, tyf;
    float ex_lo, ex_hi, ey_lo, ey_hi;       // window of the fractional part that proves a bin
    float xminf, xmaxf, yminf, ymaxf;       // float32 images of the inclusive bounds
    double sx, tx, sy, ty;
    double xmin, xmax, ymin, ymax;          // the inclusive bounds (the exact path's test)
    int coord64;                            // x / y are float64 columns
    uint32_t *out;                          // count (the COUNT base of mean)
    const double *vs;                       // mean: the value column
    double *sum_out;                        // mean: the float64 SUM base
    int use_tma;
    int cnt_off, tab_off, st_off;           // byte offsets of the 16-bit counters, tile table, slot list
};

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// ---- tile selection: the smallest T with #(count > T) <= K; those tiles,
// then ties at T while slots remain, get slots.  One LDS + REDUX a step.
__device__ void select_tiles(const Params &p, const unsigned *hist, short *tab, short *slot_tile) {
    __shared__ unsigned part[2][32];
    __shared__ unsigned s_next;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int PER = MAX_TILES / THREADS;
    unsigned c[PER];
    unsigned mx = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int i = threadIdx.x + k * THREADS;
        c[k] = i < p.ntiles ? hist[i] : 0u;
        mx = max(mx, c[k]);
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    if (lane == 0) part[0][warp] = mx;
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    unsigned lo = 0, hi = __reduce_max_sync(0xffffffffu, part[0][lane]);
    for (int it = 0; lo < hi && it < 40; ++it) {
        const unsigned mid = lo + (hi - lo) / 2;
        unsigned cnt = 0;
#pragma unroll
        for (int k = 0; k < PER; ++k) cnt += c[k] > mid;
        cnt = __reduce_add_sync(0xffffffffu, cnt);
        const int b = 1 - (it & 1);
        if (lane == 0) part[b][warp] = cnt;
        __syncthreads();
        const unsigned t = __reduce_add_sync(0xffffffffu, part[b][lane]);
        if (t <= (unsigned)p.K) hi = mid; else lo = mid + 1;
    }
    const unsigned T = hi;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int i = threadIdx.x + k * THREADS;
        if (i >= p.ntiles) continue;
        short s = -1;
        if (c[k] > T) {
            const unsigned q = atomicAdd(&s_next, 1u);
            s = (short)q;
            slot_tile[q] = (short)i;
        }
        tab[i] = s;
    }
    __syncthreads();
    if (T > 0) {
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int i = threadIdx.x + k * THREADS;
            if (i >= p.ntiles || c[k] != T) continue;
            const unsigned q = atomicAdd(&s_next, 1u);
            if (q < (unsigned)p.K) { tab[i] = (short)q; slot_tile[q] = (short)i; }
        }
    }
    __syncthreads();
    const unsigned used = min(s_next, (unsigned)p.K);
    for (int q = used + threadIdx.x; q < p.K; q += THREADS) slot_tile[q] = -1;
}

// ---- per-row body
struct RowConsts {
    float sxf, txf, syf, tyf, exlo, exhi, eylo, eyhi;
    unsigned W, H, W2, H2, tx2, tab, cache;
    unsigned long long out;
};

// One row: classify and count.  fast (both fractional parts inside the
// window, both bins inside the canvas): add one to the pixel's 16-bit
// counter (atom, old word ORed into ovf) when its tile has a slot, else an
// L2 reduction on the output.  Not fast but both bins within one of the
// canvas (k + 1 in [0, n + 1]): the row may be inside the bounds; its bit
// goes into slowm for the exact path.  Anything else is outside the bounds.
__device__ __forceinline__ void count_row(const RowConsts &k, float x, float y, unsigned bit, unsigned &slowm,
                                          unsigned &ovf) {
    asm volatile(
        "{\n\t"
        ".reg .f32 vx, vy, tx, ty, kxf, kyf, fx, fy;\n\t"
        ".reg .b32 kx, ky, a, b, t, s, c, pix, inc, old;\n\t"
        ".reg .b64 ga;\n\t"
        ".reg .pred pw, pf, pm, ps, pc, pu;\n\t"
        "fma.rn.f32 vx, %2, %4, %5;\n\t"
        "fma.rn.f32 vy, %3, %6, %7;\n\t"
        "add.rz.f32 tx, vx, 0f4B400000;\n\t"
        "add.rz.f32 ty, vy, 0f4B400000;\n\t"
        "sub.rn.f32 kxf, tx, 0f4B400000;\n\t"
        "sub.rn.f32 kyf, ty, 0f4B400000;\n\t"
        "sub.rn.f32 fx, vx, kxf;\n\t"
        "sub.rn.f32 fy, vy, kyf;\n\t"
        "setp.gt.f32 pw, fx, %8;\n\t"
        "setp.lt.and.f32 pw, fx, %9, pw;\n\t"
        "setp.gt.and.f32 pw, fy, %10, pw;\n\t"
        "setp.lt.and.f32 pw, fy, %11, pw;\n\t"
        "mov.b32 kx, tx;\n\t"
        "mov.b32 ky, ty;\n\t"
        "sub.s32 kx, kx, 0x4B400000;\n\t"
        "sub.s32 ky, ky, 0x4B400000;\n\t"
        "setp.lt.u32 pf, kx, %12;\n\t"
        "setp.lt.and.u32 pf, ky, %13, pf;\n\t"
        "add.s32 a, kx, 1;\n\t"
        "add.s32 b, ky, 1;\n\t"
        "setp.lt.u32 pm, a, %14;\n\t"
        "setp.lt.and.u32 pm, b, %15, pm;\n\t"
        "and.pred pf, pf, pw;\n\t"
        "not.pred ps, pf;\n\t"
        "and.pred ps, ps, pm;\n\t"
        "@ps or.b32 %0, %0, %20;\n\t"
        "shr.u32 a, ky, 4;\n\t"
        "shr.u32 b, kx, 4;\n\t"
        "mad.lo.u32 t, a, %16, %17;\n\t"
        "mad.lo.u32 t, b, 2, t;\n\t"
        "@!pf mov.u32 t, %17;\n\t"
        "ld.shared.s16 s, [t];\n\t"
        "setp.ge.and.s32 pc, s, 0, pf;\n\t"
        "setp.lt.and.s32 pu, s, 0, pf;\n\t"
        "and.b32 a, ky, 15;\n\t"
        "and.b32 b, kx, 15;\n\t"
        "mad.lo.u32 c, a, 16, b;\n\t"
        "mad.lo.u32 c, s, 256, c;\n\t"
        "and.b32 inc, c, 1;\n\t"
        "mad.lo.u32 inc, inc, 65535, 1;\n\t"
        "and.b32 c, c, -2;\n\t"
        "mad.lo.u32 c, c, 2, %18;\n\t"
        "@pc atom.shared.add.u32 old, [c], inc;\n\t"
        "@pc or.b32 %1, %1, old;\n\t"
        "mad.lo.u32 pix, ky, %12, kx;\n\t"
        "mad.wide.u32 ga, pix, 4, %19;\n\t"
        "@pu red.global.add.u32 [ga], 1;\n\t"
        "}"
        : "+r"(slowm), "+r"(ovf)
        : "f"(x), "f"(y), "f"(k.sxf), "f"(k.txf), "f"(k.syf), "f"(k.tyf), "f"(k.exlo), "f"(k.exhi),
          "f"(k.eylo), "f"(k.eyhi), "r"(k.W), "r"(k.H), "r"(k.W2), "r"(k.H2), "r"(k.tx2), "r"(k.tab),
          "r"(k.cache), "l"(k.out), "r"(bit)
        : "memory");
}

// The reference formula (bounds, then int(x*sx + tx) in float64, clamp) for
// one row; returns packed (xi, yi) or ~0 when outside the bounds.
static __device__ __noinline__ unsigned long long exact_bin(int64_t row, const Params *pp) {
    const Params &p = *pp;
    const double x = p.coord64 ? ((const double *)p.xs)[row] : (double)p.xs[row];
    const double y = p.coord64 ? ((const double *)p.ys)[row] : (double)p.ys[row];
    if (!(p.xmin <= x && x <= p.xmax && p.ymin <= y && y <= p.ymax)) return ~0ull;
    const unsigned xi = (unsigned)bin_exact64_st(x, p.sx, p.tx, p.W);
    const unsigned yi = (unsigned)bin_exact64_st(y, p.sy, p.ty, p.H);
    return (unsigned long long)xi | ((unsigned long long)yi << 32);
}

// float32 image of a float64 coordinate by mantissa truncation (integer
// operations): within 2^-23 relative, the truncation term of the error bound
// E; magnitudes below the float32 normal range become +-0 (an absolute
// error far below E), above it +-inf, NaN stays NaN.
__device__ __forceinline__ float trunc_f32(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    if (e >= 1 && e <= 254) return __uint_as_float(sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffu));
    if (e > 254) return __uint_as_float(sign | 0x7f800000u | (((b << 12) != 0) ? 0x400000u : 0u));
    return __uint_as_float(sign);
}

__device__ __forceinline__ unsigned half_index(int s, int xi, int yi) {
    return ((unsigned)s << (2 * TS)) | ((unsigned)(yi & 15) << TS) | (unsigned)(xi & 15);
}

// Exact path of one row: count it like the fast path; returns the old word
// of a shared increment (0 for an L2 one or an outside row).
static __device__ __noinline__ unsigned slow_row(const Params *pp, const short *tab, unsigned *cw, int64_t row) {
    const Params &p = *pp;
    const unsigned long long r = exact_bin(row, pp);
    if (r == ~0ull) return 0u;
    const int xi = (int)(unsigned)r, yi = (int)(unsigned)(r >> 32);
    const int s = tab[(yi >> TS) * p.tiles_x + (xi >> TS)];
    if (s >= 0) {
        const unsigned h = half_index(s, xi, yi);
        return atomicAdd(&cw[h >> 1], (h & 1u) ? 0x10000u : 1u);
    }
    atomicAdd(&p.out[(int64_t)yi * p.W + xi], 1u);
    return 0u;
}

// Correction of the 16-bit halves of the words that rows [row0, row0 + 4)
// touched: a half at or above 0x8000 gives 0x8000 to the output by CAS.
// Any thread may correct any word; only halves >= 0x8000 lose 0x8000, so no
// half goes negative, and a thread that saw such a half corrects it before
// it adds again.  The CAS retries only when another thread changed the word
// (finitely often); the iteration guard raises DSGB_STATUS_CAS_GUARD.
static __device__ __noinline__ void fix_words(const Params *pp, const short *tab, const short *slot_tile,
                                              unsigned *cw, int64_t row0) {
    const Params &p = *pp;
    for (int k = 0; k < 4; ++k) {
        const int64_t row = row0 + k;
        if (row >= p.n) continue;
        const unsigned long long r = exact_bin(row, pp);
        if (r == ~0ull) continue;
        const int xi = (int)(unsigned)r, yi = (int)(unsigned)(r >> 32);
        const int s = tab[(yi >> TS) * p.tiles_x + (xi >> TS)];
        if (s < 0) continue;
        const unsigned hb = half_index(s, xi, yi) & ~1u;
        unsigned *w = &cw[hb >> 1];
        bool done = false;
        for (int guard = 0; guard < (1 << 22) && !done; ++guard) {
            const unsigned cur = *(volatile unsigned *)w;
            const unsigned sub = (cur & 0x80000000u) | (cur & 0x8000u);
            if (!sub) { done = true; break; }
            if (atomicCAS(w, cur, cur - sub) == cur) {
                const int t = slot_tile[s];
                const int y0 = (t / p.tiles_x) << TS, x0 = (t % p.tiles_x) << TS;
                for (int half = 0; half < 2; ++half) {
                    if (!(sub & (half ? 0x80000000u : 0x8000u))) continue;
                    const unsigned hh = (hb | (unsigned)half) & (TILE_PX - 1);
                    atomicAdd(&p.out[(int64_t)(y0 + (hh >> TS)) * p.W + x0 + (hh & 15)], 0x8000u);
                }
                done = true;
            }
        }
        if (!done) raise_status(DSGB_STATUS_CAS_GUARD);
    }
}

__device__ __forceinline__ void tma_reduce_tile(const CUtensorMap *map, int tile, int tiles_x, unsigned src) {
    const int y0 = (tile / tiles_x) << TS, x0 = (tile % tiles_x) << TS;
    asm volatile("cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];"
                 :: "l"(map), "r"(x0), "r"(y0), "r"(src) : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Rows 4g .. 4g+3 of x and y as float32 images (float64 columns truncated).
template <bool C64, bool STREAM>
__device__ __forceinline__ void load_rows4(const Params &p, int64_t g, float4 &a, float4 &b) {
    if (C64) {
        const double2 *x2 = (const double2 *)p.xs, *y2 = (const double2 *)p.ys;
        const double2 u0 = STREAM ? __ldcs(x2 + 2 * g) : __ldg(x2 + 2 * g);
        const double2 u1 = STREAM ? __ldcs(x2 + 2 * g + 1) : __ldg(x2 + 2 * g + 1);
        const double2 w0 = STREAM ? __ldcs(y2 + 2 * g) : __ldg(y2 + 2 * g);
        const double2 w1 = STREAM ? __ldcs(y2 + 2 * g + 1) : __ldg(y2 + 2 * g + 1);
        a = make_float4(trunc_f32(u0.x), trunc_f32(u0.y), trunc_f32(u1.x), trunc_f32(u1.y));
        b = make_float4(trunc_f32(w0.x), trunc_f32(w0.y), trunc_f32(w1.x), trunc_f32(w1.y));
    } else {
        const float4 *x4 = (const float4 *)p.xs, *y4 = (const float4 *)p.ys;
        a = STREAM ? __ldcs(x4 + g) : __ldg(x4 + g);
        b = STREAM ? __ldcs(y4 + g) : __ldg(y4 + g);
    }
}

template <bool C64>
__global__ void __launch_bounds__(THREADS, 1) hot_count_kernel(const __grid_constant__ Params p,
                                                               const __grid_constant__ CUtensorMap tmap) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned *cw = (unsigned *)smem;                          // K tiles of 16-bit counters
    short *tab = (short *)(smem + p.tab_off);
    short *slot_tile = (short *)(smem + p.st_off);
    const int64_t g0 = p.n4 * blockIdx.x / gridDim.x, g1 = p.n4 * (blockIdx.x + 1) / gridDim.x;
    const int64_t full = g0 + ((g1 - g0) / THREADS) * THREADS;

    // ---- prologue: tile histogram of a sample of this CTA's rows (in the cache area)
    unsigned *hist = cw;
    for (int i = threadIdx.x; i < p.ntiles; i += THREADS) hist[i] = 0;
    __syncthreads();
    if (g1 > g0) {
#pragma unroll
        for (int j = 0; j < SAMPLE_GROUPS; ++j) {
            const int64_t g = g0 + (g1 - g0) * (threadIdx.x + j * THREADS) / (SAMPLE_GROUPS * THREADS);
            float4 a, b;
            load_rows4<C64, false>(p, g, a, b);
            const float xs[4] = {a.x, a.y, a.z, a.w};
            const float ys[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float x = xs[k], y = ys[k];
                if (!(x >= p.xminf && x <= p.xmaxf && y >= p.yminf && y <= p.ymaxf)) continue;
                const int xi = min(max(__float_as_int(__fadd_rz(__fmaf_rn(x, p.sxf, p.txf), MAGIC)) - MAGIC_BITS, 0),
                                   p.W - 1);
                const int yi = min(max(__float_as_int(__fadd_rz(__fmaf_rn(y, p.syf, p.tyf), MAGIC)) - MAGIC_BITS, 0),
                                   p.H - 1);
                atomicAdd(&hist[(yi >> TS) * p.tiles_x + (xi >> TS)], 1u);
            }
        }
    }
    __syncthreads();
    select_tiles(p, hist, tab, slot_tile);
    {
        uint4 *c4 = (uint4 *)cw;
        for (int i = threadIdx.x; i < p.K * (TILE_PX / 8); i += THREADS) c4[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();

    // ---- main loop: four rows per thread per step
    RowConsts rk;
    rk.sxf = p.sxf; rk.txf = p.txf; rk.syf = p.syf; rk.tyf = p.tyf;
    rk.exlo = p.ex_lo; rk.exhi = p.ex_hi; rk.eylo = p.ey_lo; rk.eyhi = p.ey_hi;
    rk.W = p.W; rk.H = p.H; rk.W2 = p.W + 2; rk.H2 = p.H + 2; rk.tx2 = 2 * p.tiles_x;
    rk.tab = smem_addr(tab); rk.cache = smem_addr(cw);
    rk.out = (unsigned long long)p.out;
    for (int64_t g = g0 + threadIdx.x; g < full; g += THREADS) {
        float4 a, b;
        load_rows4<C64, true>(p, g, a, b);
        unsigned slowm = 0, ovf = 0;
        count_row(rk, a.x, b.x, 1u, slowm, ovf);
        count_row(rk, a.y, b.y, 2u, slowm, ovf);
        count_row(rk, a.z, b.z, 4u, slowm, ovf);
        count_row(rk, a.w, b.w, 8u, slowm, ovf);
        if (slowm) {
#pragma unroll 1
            for (int k = 0; k < 4; ++k)
                if ((slowm >> k) & 1u) ovf |= slow_row(&p, tab, cw, 4 * g + k);
        }
        if (ovf & 0x80008000u) fix_words(&p, tab, slot_tile, cw, 4 * g);
    }
    // the ragged end of this CTA's share, and (last CTA) the rows after the last float4
    for (int64_t row = 4 * full + threadIdx.x; row < 4 * g1; row += THREADS) {
        if (slow_row(&p, tab, cw, row) & 0x80008000u) fix_words(&p, tab, slot_tile, cw, row & ~(int64_t)3);
    }
    if (blockIdx.x == gridDim.x - 1) {
        for (int64_t row = 4 * p.n4 + threadIdx.x; row < p.n; row += THREADS) {
            const unsigned long long r = exact_bin(row, &p);
            if (r != ~0ull) atomicAdd(&p.out[(int64_t)(unsigned)(r >> 32) * p.W + (unsigned)r], 1u);
        }
    }
    __syncthreads();

    // ---- flush: every slot pair is 1 KB of 16-bit counters; a warp holds
    // both tiles in registers, writes the first as 32-bit counters over the
    // pair, reduces it into the output, then the second.
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (p.use_tma) {
        for (int j = warp; 2 * j < p.K; j += THREADS / 32) {
            unsigned char *region = (unsigned char *)cw + (size_t)j * 1024;
            const uint4 q0 = *(const uint4 *)(region + 16 * lane);
            const uint4 q1 = *(const uint4 *)(region + 512 + 16 * lane);
            __syncwarp();
            const int t0 = slot_tile[2 * j];
            const int t1 = 2 * j + 1 < p.K ? slot_tile[2 * j + 1] : -1;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint4 q = h ? q1 : q0;
                const int t = h ? t1 : t0;
                if (t < 0) continue;            // warp-uniform
                *(uint4 *)(region + 32 * lane) = make_uint4(q.x & 0xffffu, q.x >> 16, q.y & 0xffffu, q.y >> 16);
                *(uint4 *)(region + 32 * lane + 16) = make_uint4(q.z & 0xffffu, q.z >> 16, q.w & 0xffffu, q.w >> 16);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) tma_reduce_tile(&tmap, t, p.tiles_x, smem_addr(region));
                __syncwarp();
            }
        }
        return;
    }
    // canvas rows not 16-byte aligned: per-pixel atomics
    for (int i = threadIdx.x; i < p.K * TILE_PX; i += THREADS) {
        const unsigned c = (cw[i >> 1] >> ((i & 1) * 16)) & 0xffffu;
        if (!c) continue;
        const int t = slot_tile[i >> (2 * TS)];
        if (t < 0) continue;
        const int within = i & (TILE_PX - 1);
        const int yi = ((t / p.tiles_x) << TS) + (within >> TS);
        const int xi = ((t % p.tiles_x) << TS) + (within & 15);
        atomicAdd(&p.out[(int64_t)yi * p.W + xi], c);
    }
}


// ================================================================== mean('v')
// The same pass for mean('v') (reductions.py:1280-1297: bases _sum_zero and
// _count_ignore_antialiasing, rows with a NaN value add nothing): per cached
// pixel a float64 sum (shared-memory add) beside the 16-bit count; other rows
// add their value and one into the output bases by L2 reductions.
__device__ __forceinline__ void mean_row(const RowConsts &k, unsigned sums, unsigned long long sout, float x,
                                         float y, double v, unsigned bit, unsigned &slowm, unsigned &ovf) {
    asm volatile(
        "{\n\t"
        ".reg .f32 vx, vy, tx, ty, kxf, kyf, fx, fy;\n\t"
        ".reg .b32 kx, ky, a, b, t, s, c, pix, inc, old, cs;\n\t"
        ".reg .b64 ga, gs;\n\t"
        ".reg .pred pw, pf, pm, ps, pc, pu, pn;\n\t"
        "testp.notanumber.f64 pn, %21;\n\t"
        "fma.rn.f32 vx, %2, %4, %5;\n\t"
        "fma.rn.f32 vy, %3, %6, %7;\n\t"
        "add.rz.f32 tx, vx, 0f4B400000;\n\t"
        "add.rz.f32 ty, vy, 0f4B400000;\n\t"
        "sub.rn.f32 kxf, tx, 0f4B400000;\n\t"
        "sub.rn.f32 kyf, ty, 0f4B400000;\n\t"
        "sub.rn.f32 fx, vx, kxf;\n\t"
        "sub.rn.f32 fy, vy, kyf;\n\t"
        "setp.gt.f32 pw, fx, %8;\n\t"
        "setp.lt.and.f32 pw, fx, %9, pw;\n\t"
        "setp.gt.and.f32 pw, fy, %10, pw;\n\t"
        "setp.lt.and.f32 pw, fy, %11, pw;\n\t"
        "mov.b32 kx, tx;\n\t"
        "mov.b32 ky, ty;\n\t"
        "sub.s32 kx, kx, 0x4B400000;\n\t"
        "sub.s32 ky, ky, 0x4B400000;\n\t"
        "setp.lt.u32 pf, kx, %12;\n\t"
        "setp.lt.and.u32 pf, ky, %13, pf;\n\t"
        "add.s32 a, kx, 1;\n\t"
        "add.s32 b, ky, 1;\n\t"
        "setp.lt.u32 pm, a, %14;\n\t"
        "setp.lt.and.u32 pm, b, %15, pm;\n\t"
        "and.pred pf, pf, pw;\n\t"
        "not.pred ps, pf;\n\t"
        "and.pred ps, ps, pm;\n\t"
        "not.pred pn, pn;\n\t"
        "and.pred ps, ps, pn;\n\t"
        "and.pred pf, pf, pn;\n\t"
        "@ps or.b32 %0, %0, %20;\n\t"
        "shr.u32 a, ky, 4;\n\t"
        "shr.u32 b, kx, 4;\n\t"
        "mad.lo.u32 t, a, %16, %17;\n\t"
        "mad.lo.u32 t, b, 2, t;\n\t"
        "@!pf mov.u32 t, %17;\n\t"
        "ld.shared.s16 s, [t];\n\t"
        "setp.ge.and.s32 pc, s, 0, pf;\n\t"
        "setp.lt.and.s32 pu, s, 0, pf;\n\t"
        "and.b32 a, ky, 15;\n\t"
        "and.b32 b, kx, 15;\n\t"
        "mad.lo.u32 c, a, 16, b;\n\t"
        "mad.lo.u32 c, s, 256, c;\n\t"
        "mad.lo.u32 cs, c, 8, %22;\n\t"
        "@pc red.shared.add.f64 [cs], %21;\n\t"
        "and.b32 inc, c, 1;\n\t"
        "mad.lo.u32 inc, inc, 65535, 1;\n\t"
        "and.b32 c, c, -2;\n\t"
        "mad.lo.u32 c, c, 2, %18;\n\t"
        "@pc atom.shared.add.u32 old, [c], inc;\n\t"
        "@pc or.b32 %1, %1, old;\n\t"
        "mad.lo.u32 pix, ky, %12, kx;\n\t"
        "mad.wide.u32 ga, pix, 4, %19;\n\t"
        "mad.wide.u32 gs, pix, 8, %23;\n\t"
        "@pu red.global.add.f64 [gs], %21;\n\t"
        "@pu red.global.add.u32 [ga], 1;\n\t"
        "}"
        : "+r"(slowm), "+r"(ovf)
        : "f"(x), "f"(y), "f"(k.sxf), "f"(k.txf), "f"(k.syf), "f"(k.tyf), "f"(k.exlo), "f"(k.exhi),
          "f"(k.eylo), "f"(k.eyhi), "r"(k.W), "r"(k.H), "r"(k.W2), "r"(k.H2), "r"(k.tx2), "r"(k.tab),
          "r"(k.cache), "l"(k.out), "r"(bit), "d"(v), "r"(sums), "l"(sout)
        : "memory");
}

// Exact path of one mean row; returns the old count word of a shared increment.
static __device__ __noinline__ unsigned slow_row_mean(const Params *pp, const short *tab, double *sums,
                                                      unsigned *cw, int64_t row) {
    const Params &p = *pp;
    const double v = p.vs[row];
    if (isnull(v)) return 0u;
    const unsigned long long r = exact_bin(row, pp);
    if (r == ~0ull) return 0u;
    const int xi = (int)(unsigned)r, yi = (int)(unsigned)(r >> 32);
    const int s = tab[(yi >> TS) * p.tiles_x + (xi >> TS)];
    if (s >= 0) {
        const unsigned h = half_index(s, xi, yi);
        atomicAdd(&sums[h], v);
        return atomicAdd(&cw[h >> 1], (h & 1u) ? 0x10000u : 1u);
    }
    const int64_t pix = (int64_t)yi * p.W + xi;
    atomicAdd(&p.sum_out[pix], v);
    atomicAdd(&p.out[pix], 1u);
    return 0u;
}

__global__ void __launch_bounds__(THREADS, 1) hot_mean_kernel(const __grid_constant__ Params p,
                                                              const __grid_constant__ CUtensorMap tmap) {
    extern __shared__ __align__(1024) unsigned char smem[];
    double *sums = (double *)smem;                            // K tiles of float64 sums
    unsigned *cw = (unsigned *)(smem + p.cnt_off);            // K tiles of 16-bit counts
    short *tab = (short *)(smem + p.tab_off);
    short *slot_tile = (short *)(smem + p.st_off);
    const float4 *x4 = (const float4 *)p.xs;
    const float4 *y4 = (const float4 *)p.ys;
    const double2 *v2 = (const double2 *)p.vs;
    const int64_t g0 = p.n4 * blockIdx.x / gridDim.x, g1 = p.n4 * (blockIdx.x + 1) / gridDim.x;

    unsigned *hist = (unsigned *)smem;
    for (int i = threadIdx.x; i < p.ntiles; i += THREADS) hist[i] = 0;
    __syncthreads();
    if (g1 > g0) {
#pragma unroll
        for (int j = 0; j < MEAN_SAMPLE_GROUPS; ++j) {
            const int64_t g = g0 + (g1 - g0) * (threadIdx.x + j * THREADS) / (MEAN_SAMPLE_GROUPS * THREADS);
            const float4 a = __ldg(x4 + g), b = __ldg(y4 + g);
            const float xs[4] = {a.x, a.y, a.z, a.w};
            const float ys[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float x = xs[k], y = ys[k];
                if (!(x >= p.xminf && x <= p.xmaxf && y >= p.yminf && y <= p.ymaxf)) continue;
                const int xi = min(max(__float_as_int(__fadd_rz(__fmaf_rn(x, p.sxf, p.txf), MAGIC)) - MAGIC_BITS, 0),
                                   p.W - 1);
                const int yi = min(max(__float_as_int(__fadd_rz(__fmaf_rn(y, p.syf, p.tyf), MAGIC)) - MAGIC_BITS, 0),
                                   p.H - 1);
                atomicAdd(&hist[(yi >> TS) * p.tiles_x + (xi >> TS)], 1u);
            }
        }
    }
    __syncthreads();
    select_tiles(p, hist, tab, slot_tile);
    {
        uint4 *c4 = (uint4 *)smem;
        const int words = p.cnt_off / 16 + p.K * (TILE_PX / 8);
        for (int i = threadIdx.x; i < words; i += THREADS) c4[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();

    RowConsts rk;
    rk.sxf = p.sxf; rk.txf = p.txf; rk.syf = p.syf; rk.tyf = p.tyf;
    rk.exlo = p.ex_lo; rk.exhi = p.ex_hi; rk.eylo = p.ey_lo; rk.eyhi = p.ey_hi;
    rk.W = p.W; rk.H = p.H; rk.W2 = p.W + 2; rk.H2 = p.H + 2; rk.tx2 = 2 * p.tiles_x;
    rk.tab = smem_addr(tab); rk.cache = smem_addr(cw);
    rk.out = (unsigned long long)p.out;
    const unsigned sums_s = smem_addr(sums);
    const unsigned long long sout = (unsigned long long)p.sum_out;
    for (int64_t g = g0 + threadIdx.x; g < g1; g += THREADS) {
        const float4 a = __ldcs(x4 + g), b = __ldcs(y4 + g);
        const double2 c0 = __ldcs(v2 + 2 * g), c1 = __ldcs(v2 + 2 * g + 1);
        unsigned slowm = 0, ovf = 0;
        mean_row(rk, sums_s, sout, a.x, b.x, c0.x, 1u, slowm, ovf);
        mean_row(rk, sums_s, sout, a.y, b.y, c0.y, 2u, slowm, ovf);
        mean_row(rk, sums_s, sout, a.z, b.z, c1.x, 4u, slowm, ovf);
        mean_row(rk, sums_s, sout, a.w, b.w, c1.y, 8u, slowm, ovf);
        if (slowm) {
#pragma unroll 1
            for (int k = 0; k < 4; ++k)
                if ((slowm >> k) & 1u) ovf |= slow_row_mean(&p, tab, sums, cw, 4 * g + k);
        }
        if (ovf & 0x80008000u) fix_words(&p, tab, slot_tile, cw, 4 * g);
    }
    if (blockIdx.x == gridDim.x - 1) {
        for (int64_t row = 4 * p.n4 + threadIdx.x; row < p.n; row += THREADS) {
            const double v = p.vs[row];
            if (isnull(v)) continue;
            const unsigned long long r = exact_bin(row, &p);
            if (r == ~0ull) continue;
            const int64_t pix = (int64_t)(unsigned)(r >> 32) * p.W + (unsigned)r;
            atomicAdd(&p.sum_out[pix], v);
            atomicAdd(&p.out[pix], 1u);
        }
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (p.use_tma) {
        // sums: one bulk float64 reduction per tile row (16 values, 128 bytes)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        bool issued = false;
        for (int r = threadIdx.x; r < p.K * 16; r += THREADS) {
            const int slot = r >> 4, ry = r & 15;
            const int t = slot_tile[slot];
            if (t < 0) continue;
            const int yi = (t / p.tiles_x) * 16 + ry, x0 = (t % p.tiles_x) * 16;
            if (yi >= p.H) continue;
            const int ncols = p.W - x0 < 16 ? p.W - x0 : 16;       // even: W is a multiple of 4 here
            const double *src = sums + (size_t)slot * TILE_PX + ry * 16;
            asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f64 [%0], [%1], %2;"
                         :: "l"(p.sum_out + (int64_t)yi * p.W + x0), "r"(smem_addr(src)), "r"(ncols * 8)
                         : "memory");
            issued = true;
        }
        if (issued) asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        // counts: 16-bit pairs widened in place, a tensor reduction per tile
        for (int j = warp; 2 * j < p.K; j += THREADS / 32) {
            unsigned char *region = (unsigned char *)cw + (size_t)j * 1024;
            const uint4 q0 = *(const uint4 *)(region + 16 * lane);
            const uint4 q1 = *(const uint4 *)(region + 512 + 16 * lane);
            __syncwarp();
            const int t0 = slot_tile[2 * j];
            const int t1 = 2 * j + 1 < p.K ? slot_tile[2 * j + 1] : -1;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint4 q = h ? q1 : q0;
                const int t = h ? t1 : t0;
                if (t < 0) continue;
                *(uint4 *)(region + 32 * lane) = make_uint4(q.x & 0xffffu, q.x >> 16, q.y & 0xffffu, q.y >> 16);
                *(uint4 *)(region + 32 * lane + 16) = make_uint4(q.z & 0xffffu, q.z >> 16, q.w & 0xffffu, q.w >> 16);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) tma_reduce_tile(&tmap, t, p.tiles_x, smem_addr(region));
                __syncwarp();
            }
        }
        if (issued) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        return;
    }
    for (int i = threadIdx.x; i < p.K * TILE_PX; i += THREADS) {
        const unsigned c = (cw[i >> 1] >> ((i & 1) * 16)) & 0xffffu;
        if (!c) continue;
        const int t = slot_tile[i >> (2 * TS)];
        if (t < 0) continue;
        const int within = i & (TILE_PX - 1);
        const int64_t pix = (int64_t)(((t / p.tiles_x) << TS) + (within >> TS)) * p.W + ((t % p.tiles_x) << TS) +
                            (within & 15);
        atomicAdd(&p.out[pix], c);
        atomicAdd(&p.sum_out[pix], sums[i]);
    }
}

// ------------------------------------------------------------------ host

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
    }
    return fn;
}

// edges_ok (binning.cuh) for float64 coordinates: the bounds themselves and
// the doubles next to them.
static double image64d(double v, double s, double t) {
    volatile double a = v * s;
    volatile double b = a + t;
    return b;
}
static bool edges_ok64(double lo, double hi, double s, double t, int n) {
    if (!(s > 0.0) || !std::isfinite(lo) || !std::isfinite(hi) || !(hi >= lo)) return false;
    return image64d(nextafter(lo, -INFINITY), s, t) <= 0.0 && image64d(lo, s, t) >= 0.0 &&
           image64d(hi, s, t) < n + 0.5 && image64d(nextafter(hi, INFINITY), s, t) >= (double)n;
}

// Common set-up of both kernels; px_bytes is the shared memory a cached
// pixel takes (2: count; 10: mean's float64 sum and 16-bit count).
static int hot_setup(const ColumnRef &xc, const ColumnRef &yc, int64_t n, const dsgb_canvas *cv, const BinAxis &ax,
                     const BinAxis &ay, const BinBounds &bb, uint32_t *out, int px_bytes, Params &p, int &smem,
                     CUtensorMap &tmap) {
    const bool c64 = xc.dtype == DSGB_F64 && yc.dtype == DSGB_F64;
    if (!(c64 || (xc.dtype == DSGB_F32 && yc.dtype == DSGB_F32)) || n < MIN_ROWS) return DSGB_E_UNSUPPORTED;
    if (((uintptr_t)xc.data | (uintptr_t)yc.data) & 15u) return DSGB_E_UNSUPPORTED;
    if (cv->x_log || cv->y_log || !fast_path_ok(ax, ay)) return DSGB_E_UNSUPPORTED;
    const int W = cv->width, H = cv->height;
    const int tiles_x = (W + 15) >> 4, tiles_y = (H + 15) >> 4;
    if ((int64_t)tiles_x * tiles_y > MAX_TILES) return DSGB_E_UNSUPPORTED;
    const bool edges = c64 ? edges_ok64(cv->xmin, cv->xmax, cv->sx, cv->tx, W) &&
                                 edges_ok64(cv->ymin, cv->ymax, cv->sy, cv->ty, H)
                           : edges_ok(bb.xminf, bb.xmaxf, cv->sx, cv->tx, W) &&
                                 edges_ok(bb.yminf, bb.ymaxf, cv->sy, cv->ty, H);
    if (!edges) return DSGB_E_UNSUPPORTED;
    memset(&p, 0, sizeof(p));
    p.xs = (const float *)xc.data; p.ys = (const float *)yc.data; p.n = n; p.n4 = n / 4;
    p.W = W; p.H = H; p.tiles_x = tiles_x; p.ntiles = tiles_x * tiles_y;
    p.sxf = ax.sf; p.txf = ax.tf; p.syf = ay.sf; p.tyf = ay.tf;
    p.ex_lo = float_ceil_of((double)ax.e); p.ex_hi = float_floor_of(1.0 - (double)ax.e);
    p.ey_lo = float_ceil_of((double)ay.e); p.ey_hi = float_floor_of(1.0 - (double)ay.e);
    p.xminf = bb.xminf; p.xmaxf = bb.xmaxf; p.yminf = bb.yminf; p.ymaxf = bb.ymaxf;
    p.sx = cv->sx; p.tx = cv->tx; p.sy = cv->sy; p.ty = cv->ty;
    p.xmin = cv->xmin; p.xmax = cv->xmax; p.ymin = cv->ymin; p.ymax = cv->ymax;
    p.coord64 = c64;
    p.out = out;
    const int tab_bytes = (p.ntiles * 2 + 127) & ~127;
    const int st_bytes = MAX_SLOTS * 2;
    int K = (DYN_SMEM - tab_bytes - st_bytes - 1024) / (TILE_PX * px_bytes);
    K = std::min(K, MAX_SLOTS);
    K = std::min(K, p.ntiles);
    K &= ~1;                                          // slot pairs in the flush
    if (K < 2) return DSGB_E_UNSUPPORTED;
    p.K = K;
    const int sum_bytes = px_bytes > 2 ? K * TILE_PX * 8 : 0;
    p.cnt_off = sum_bytes;                            // multiples of 1 KB
    int cache_bytes = sum_bytes + K * TILE_PX * 2;
    if (cache_bytes < p.ntiles * 4) cache_bytes = (p.ntiles * 4 + 1023) & ~1023;   // the prologue's histogram
    p.tab_off = cache_bytes;
    p.st_off = cache_bytes + tab_bytes;
    smem = p.st_off + st_bytes;
    if (smem > DYN_SMEM) return DSGB_E_UNSUPPORTED;
    memset(&tmap, 0, sizeof(tmap));
    if ((W % 4) == 0 && (((uintptr_t)out) & 15u) == 0) {
        auto fn = encode_fn();
        if (fn) {
            cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
            cuuint64_t strides[1] = {(cuuint64_t)W * 4};
            cuuint32_t box[2] = {16, 16};
            cuuint32_t es[2] = {1, 1};
            if (fn(&tmap, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, out, dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
                p.use_tma = 1;
        }
    }
    return DSGB_OK;
}

}  // namespace hot

// DSGB_E_UNSUPPORTED when the case is not covered (the caller then takes
// another path).  No workspace.
int launch_points_hot(const ColumnRef &xc, const ColumnRef &yc, int64_t n, const dsgb_canvas *cv,
                      const BinAxis &ax, const BinAxis &ay, const BinBounds &bb, uint32_t *out, bool accumulate,
                      cudaStream_t st) {
    using namespace hot;
    Params p;
    int smem = 0;
    CUtensorMap tmap;
    int rc = hot_setup(xc, yc, n, cv, ax, ay, bb, out, 2, p, smem, tmap);
    if (rc) return rc;
    const int sms = sm_count();
    if (sms <= 0) return cuda_status(cudaErrorNoDevice, "points hot: device");
    cudaError_t e = cudaSuccess;
    if (!accumulate) e = cudaMemsetAsync(out, 0, (size_t)p.W * p.H * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "points hot: memset");
    if (p.coord64) {
        e = cudaFuncSetAttribute(hot_count_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return cuda_status(e, "points hot: shared memory attribute");
        hot_count_kernel<true><<<sms, THREADS, smem, st>>>(p, tmap);
    } else {
        e = cudaFuncSetAttribute(hot_count_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return cuda_status(e, "points hot: shared memory attribute");
        hot_count_kernel<false><<<sms, THREADS, smem, st>>>(p, tmap);
    }
    DSGB_CHECK_LAUNCH("points hot: launch");
    return DSGB_OK;
}

// mean('v') of float32 x/y and a float64 value column: sum into the SUM base,
// non-NaN count into the COUNT base.
int launch_points_hot_mean(const ColumnRef &xc, const ColumnRef &yc, const ColumnRef &vc, int64_t n,
                           const dsgb_canvas *cv, const BinAxis &ax, const BinAxis &ay, const BinBounds &bb,
                           double *sum, uint32_t *count, bool accumulate, cudaStream_t st) {
    using namespace hot;
    if (vc.dtype != DSGB_F64 || ((uintptr_t)vc.data & 15u) || (((uintptr_t)sum) & 15u) || (cv->width & 1))
        return DSGB_E_UNSUPPORTED;
    Params p;
    int smem = 0;
    CUtensorMap tmap;
    int rc = hot_setup(xc, yc, n, cv, ax, ay, bb, count, 10, p, smem, tmap);
    if (rc) return rc;
    if (p.coord64) return DSGB_E_UNSUPPORTED;         // float32 coordinates only
    p.vs = (const double *)vc.data;
    p.sum_out = sum;
    const int sms = sm_count();
    if (sms <= 0) return cuda_status(cudaErrorNoDevice, "points hot mean: device");
    const size_t cells = (size_t)p.W * p.H;
    cudaError_t e = cudaSuccess;
    if (!accumulate) e = cudaMemsetAsync(count, 0, cells * 4, st);
    if (e == cudaSuccess && !accumulate) e = cudaMemsetAsync(sum, 0, cells * 8, st);
    if (e != cudaSuccess) return cuda_status(e, "points hot mean: memset");
    e = cudaFuncSetAttribute(hot_mean_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return cuda_status(e, "points hot mean: shared memory attribute");
    hot_mean_kernel<<<sms, THREADS, smem, st>>>(p, tmap);
    DSGB_CHECK_LAUNCH("points hot mean: launch");
    return DSGB_OK;
}

DSGB_STATUS_READER(status_points_hot)

}  // namespace dsgb
