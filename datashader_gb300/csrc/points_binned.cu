// points_binned.cu -- Canvas.points count() without global atomics.
//
// Scattered global atomics top out near 2.3e11 per second on GB300, and the
// 5-Gaussian workload concentrates them on a few L2 slices, so a count over
// 1e8 points bound by L2 atomics runs near 1 ms.  This path keeps every
// increment on chip instead:
//
//   pass 1 (bin)   -- stream x/y (float4 loads), bin each row exactly as
//                     points.py:190-204 (float32 fast path + exact float64
//                     fallback, shared with points.cu), and, per round of
//                     8192 rows, sort the 16-bit band-local pixel index of
//                     each kept row by row band in shared memory; write the
//                     sorted round (16 KB, coalesced) and its per-band
//                     (offset, count) directory to the workspace.
//   plan           -- one block turns the per-band totals into work items
//                     (band, range of rounds) of similar size.
//   pass 2 (accum) -- one CTA per work item holds its band of the canvas
//                     (R rows x W uint32) in shared memory, adds every entry
//                     of its rounds with shared-memory atomics, then adds the
//                     band into the output with one TMA bulk reduction
//                     (cp.reduce.async.bulk .add.u32).
//
// HBM traffic: 8 B/row read + 2 B/row written + 2 B/row read, plus the
// directory; the count is exact (integer adds in any order).
#include "dsgb_internal.cuh"

#include <cmath>

namespace dsgb {

constexpr int ROUND = 8192;           // rows per round (1024 threads x 8 rows)
constexpr int MAX_BANDS = 256;
constexpr int ROUND_CAP = 10240;      // entry slots per round: 8192 + padding of every band to 8
constexpr int MAX_BAND_CELLS = 49152; // band-local index < 65535 (0xFFFF pads a run)
constexpr uint16_t PAD = 0xFFFFu;

struct BinnedParams {
    const float *xs32, *ys32;         // float32 coordinates (or null)
    const double *xs64, *ys64;        // float64 coordinates (or null)
    int64_t n;
    int32_t width, height;
    int32_t rows_per_band, nbands;
    int64_t nrounds;
    double sx, tx, sy, ty;
    float xminf, xmaxf, yminf, ymaxf, sxf, txf, syf, tyf, ex, ey;
    long long kxmin, kxmax, kymin, kymax;
    uint16_t *entries;                // nrounds * ROUND_CAP
    uint32_t *dir;                    // nrounds * nbands: (offset in 8-entry units << 16) | count
    unsigned long long *totals;       // nbands
    int4 *items;                      // (band, r0, r1, -)
    int *nitems;
    int *status;                      // 0, or 1 when a bounded wait gave up
    uint32_t *out;                    // height * width counts
};

// ---- mbarrier / bulk-copy helpers (sm_90+ PTX)
__device__ __forceinline__ unsigned smem_addr(const void *ptr) {
    return (unsigned)__cvta_generic_to_shared(ptr);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    unsigned long long state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state) : "r"(smem_addr(bar)), "r"(bytes) : "memory");
    (void)state;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
// Wait for the phase with the given parity; false when the limit runs out.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity) {
    for (int it = 0; it < (1 << 20); ++it) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// ---- binning (the same arithmetic as points.cu; see its header comment)
__device__ __forceinline__ int bb_exact(double m, double s, double t, int n) {
    double v = __dadd_rn(__dmul_rn(m, s), t);
    long long xx = __double2ll_rz(v);
    if (xx >= n) xx = n - 1;
    if (xx < 0) xx += n;
    if (xx < 0) xx = 0;
    return (int)xx;
}
__device__ __forceinline__ int bb_fast(float xf, double xd, float sf, float tf, float e, double s, double t, int n) {
    float v = __fmaf_rn(xf, sf, tf);
    float fl = floorf(v);
    float d = fminf(v - fl, (fl + 1.0f) - v);
    if (d > e) {
        int xx = __float2int_rz(v);
        if (xx >= n) xx = n - 1;
        if (xx < 0) xx += n;
        if (xx < 0) xx = 0;
        return xx;
    }
    return bb_exact(xd, s, t, n);
}
__device__ __forceinline__ bool bb_f32(const BinnedParams &p, float x, float y, int &xi, int &yi) {
    if (!(x >= p.xminf && x <= p.xmaxf && y >= p.yminf && y <= p.ymaxf)) return false;
    xi = bb_fast(x, (double)x, p.sxf, p.txf, p.ex, p.sx, p.tx, p.width);
    yi = bb_fast(y, (double)y, p.syf, p.tyf, p.ey, p.sy, p.ty, p.height);
    return true;
}
__device__ __forceinline__ bool bb_trunc(double x, float &out) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if ((b << 1) == 0) { out = 0.0f; return true; }
    int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    if (e <= 0 || e >= 255) return false;
    out = __uint_as_float(((unsigned)(b >> 63) << 31) | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffu));
    return true;
}
__device__ __forceinline__ long long bb_key(double v) {
    long long b = __double_as_longlong(v);
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}
__device__ __forceinline__ bool bb_f64(const BinnedParams &p, double x, double y, int &xi, int &yi) {
    long long kx = bb_key(x), ky = bb_key(y);
    if (!(kx >= p.kxmin && kx <= p.kxmax && ky >= p.kymin && ky <= p.kymax)) return false;
    float xf, yf;
    xi = bb_trunc(x, xf) ? bb_fast(xf, x, p.sxf, p.txf, p.ex, p.sx, p.tx, p.width) : bb_exact(x, p.sx, p.tx, p.width);
    yi = bb_trunc(y, yf) ? bb_fast(yf, y, p.syf, p.tyf, p.ey, p.sy, p.ty, p.height) : bb_exact(y, p.sy, p.ty, p.height);
    return true;
}

// ---- pass 1
template <bool F64>
__global__ void __launch_bounds__(1024, 1) binned_pass1(const BinnedParams p) {
    __shared__ __align__(16) uint16_t stage[ROUND_CAP];
    __shared__ unsigned hist[MAX_BANDS];
    __shared__ unsigned offs[MAX_BANDS];
    __shared__ unsigned wsum[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int B = p.nbands;
    for (int b = threadIdx.x; b < B; b += blockDim.x) hist[b] = 0;
    unsigned long long my_total = 0;          // per-band totals kept by thread b (b < B)
    __syncthreads();
    for (int64_t r = blockIdx.x; r < p.nrounds; r += gridDim.x) {
        const int64_t row0 = r * ROUND;
        int band[8];
        int local[8];
        int rank[8];
        // rows row0 + h*4096 + tid*4 + k (h < 2, k < 4): all loads issued first
        if (!F64) {
            float xf[8], yf[8];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t i0 = row0 + (int64_t)h * 4096 + (int64_t)threadIdx.x * 4;
                if (i0 + 3 < p.n) {
                    float4 a = __ldcs((const float4 *)(p.xs32 + i0));
                    float4 c = __ldcs((const float4 *)(p.ys32 + i0));
                    xf[4 * h + 0] = a.x; xf[4 * h + 1] = a.y; xf[4 * h + 2] = a.z; xf[4 * h + 3] = a.w;
                    yf[4 * h + 0] = c.x; yf[4 * h + 1] = c.y; yf[4 * h + 2] = c.z; yf[4 * h + 3] = c.w;
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        xf[4 * h + k] = i0 + k < p.n ? p.xs32[i0 + k] : __int_as_float(0x7fc00000);
                        yf[4 * h + k] = i0 + k < p.n ? p.ys32[i0 + k] : 0.0f;
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                int xi, yi, bnd = -1, loc = 0;
                if (bb_f32(p, xf[k], yf[k], xi, yi)) {
                    bnd = yi / p.rows_per_band;
                    loc = (yi - bnd * p.rows_per_band) * p.width + xi;
                }
                band[k] = bnd;
                local[k] = loc;
            }
        } else {
            double xd[8], yd[8];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t i0 = row0 + (int64_t)h * 4096 + (int64_t)threadIdx.x * 4;
                if (i0 + 3 < p.n) {
                    double2 a0 = __ldcs((const double2 *)(p.xs64 + i0)), a1 = __ldcs((const double2 *)(p.xs64 + i0 + 2));
                    double2 c0 = __ldcs((const double2 *)(p.ys64 + i0)), c1 = __ldcs((const double2 *)(p.ys64 + i0 + 2));
                    xd[4 * h + 0] = a0.x; xd[4 * h + 1] = a0.y; xd[4 * h + 2] = a1.x; xd[4 * h + 3] = a1.y;
                    yd[4 * h + 0] = c0.x; yd[4 * h + 1] = c0.y; yd[4 * h + 2] = c1.x; yd[4 * h + 3] = c1.y;
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        xd[4 * h + k] = i0 + k < p.n ? p.xs64[i0 + k] : __longlong_as_double(0x7ff8000000000000ll);
                        yd[4 * h + k] = i0 + k < p.n ? p.ys64[i0 + k] : 0.0;
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                int xi, yi, bnd = -1, loc = 0;
                if (bb_f64(p, xd[k], yd[k], xi, yi)) {
                    bnd = yi / p.rows_per_band;
                    loc = (yi - bnd * p.rows_per_band) * p.width + xi;
                }
                band[k] = bnd;
                local[k] = loc;
            }
        }
        // ranks within (round, band): one shared atomic per distinct band per warp slot
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int bnd = band[k];
            const unsigned peers = __match_any_sync(0xffffffffu, bnd);
            const int leader = __ffs(peers) - 1;
            unsigned base = 0;
            if (lane == leader && bnd >= 0) base = atomicAdd(&hist[bnd], (unsigned)__popc(peers));
            base = __shfl_sync(0xffffffffu, base, leader);
            rank[k] = (int)(base + __popc(peers & ((1u << lane) - 1u)));
        }
        __syncthreads();
        // exclusive scan of the band runs padded to 8 entries (B <= 256)
        {
            const unsigned cnt = threadIdx.x < (unsigned)B ? hist[threadIdx.x] : 0u;
            const unsigned v = (cnt + 7u) & ~7u;
            unsigned s = v;
            for (int o = 1; o < 32; o <<= 1) {
                unsigned t = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += t;
            }
            if (lane == 31) wsum[warp] = s;
            __syncthreads();
            if (warp == 0) {
                unsigned w = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0u;
                for (int o = 1; o < 32; o <<= 1) {
                    unsigned t = __shfl_up_sync(0xffffffffu, w, o);
                    if (lane >= o) w += t;
                }
                wsum[lane] = w;
            }
            __syncthreads();
            const unsigned excl = s - v + (warp > 0 ? wsum[warp - 1] : 0u);
            if (threadIdx.x < (unsigned)B) {
                offs[threadIdx.x] = excl;
                p.dir[r * B + threadIdx.x] = ((excl >> 3) << 16) | cnt;
                my_total += cnt;
                for (unsigned j = excl + cnt; j < excl + v; ++j) stage[j] = PAD;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (band[k] >= 0) stage[offs[band[k]] + rank[k]] = (uint16_t)local[k];
        __syncthreads();
        // the sorted, padded round (coalesced uint4 stores)
        const unsigned total = wsum[31];
        uint4 *dst = (uint4 *)(p.entries + r * ROUND_CAP);
        const uint4 *src = (const uint4 *)stage;
        for (unsigned v = threadIdx.x; v < total / 8; v += blockDim.x) __stcs(dst + v, src[v]);
        for (int b = threadIdx.x; b < B; b += blockDim.x) hist[b] = 0;
        __syncthreads();
    }
    if (threadIdx.x < (unsigned)B && my_total) atomicAdd(&p.totals[threadIdx.x], my_total);
}

// float32 coordinates: the rounds stream in through a two-slot TMA bulk-copy
// ring (x and y, 32 KB each per round) so that HBM reads overlap the binning
// and sorting of the previous round.
__global__ void __launch_bounds__(1024, 1) binned_pass1_tma(const BinnedParams p) {
    extern __shared__ __align__(128) unsigned char dyn[];
    float *xb = (float *)dyn;                       // [2][ROUND]
    float *yb = xb + 2 * ROUND;                     // [2][ROUND]
    uint16_t *stage = (uint16_t *)(yb + 2 * ROUND); // [ROUND_CAP]
    __shared__ unsigned hist[MAX_BANDS];
    __shared__ unsigned offs[MAX_BANDS];
    __shared__ unsigned wsum[32];
    __shared__ __align__(8) unsigned long long bar[2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int B = p.nbands;
    const int64_t nfull = p.n / ROUND;              // rounds fully inside the columns
    for (int b = tid; b < B; b += blockDim.x) hist[b] = 0;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int64_t r, int slot) {
        if (r < nfull) {
            mbar_expect_tx(&bar[slot], 2u * ROUND * 4u);
            bulk_g2s(xb + slot * ROUND, p.xs32 + r * ROUND, ROUND * 4u, &bar[slot]);
            bulk_g2s(yb + slot * ROUND, p.ys32 + r * ROUND, ROUND * 4u, &bar[slot]);
        }
    };
    if (tid == 0) {
        issue(blockIdx.x, 0);
        issue(blockIdx.x + gridDim.x, 1);
    }
    unsigned parity[2] = {0u, 0u};
    unsigned long long my_total = 0;
    int i = 0;
    for (int64_t r = blockIdx.x; r < p.nrounds; r += gridDim.x, ++i) {
        const int slot = i & 1;
        const int64_t row0 = r * ROUND;
        float xf[8], yf[8];
        if (r < nfull) {
            const bool ok = mbar_wait_bounded(&bar[slot], parity[slot]);
            parity[slot] ^= 1u;
            if (__syncthreads_or(!ok)) {
                // a bulk copy did not land within the limit: report and stop
                if (tid == 0) atomicExch(p.status, 1);
                return;
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                xf[k] = xb[slot * ROUND + tid + 1024 * k];
                yf[k] = yb[slot * ROUND + tid + 1024 * k];
            }
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int64_t ii = row0 + tid + 1024 * k;
                xf[k] = ii < p.n ? p.xs32[ii] : __int_as_float(0x7fc00000);
                yf[k] = ii < p.n ? p.ys32[ii] : 0.0f;
            }
        }
        int band[8], local[8], rank[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int xi, yi, bnd = -1, loc = 0;
            if (bb_f32(p, xf[k], yf[k], xi, yi)) {
                bnd = yi / p.rows_per_band;
                loc = (yi - bnd * p.rows_per_band) * p.width + xi;
            }
            band[k] = bnd;
            local[k] = loc;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int bnd = band[k];
            const unsigned peers = __match_any_sync(0xffffffffu, bnd);
            const int leader = __ffs(peers) - 1;
            unsigned base = 0;
            if (lane == leader && bnd >= 0) base = atomicAdd(&hist[bnd], (unsigned)__popc(peers));
            base = __shfl_sync(0xffffffffu, base, leader);
            rank[k] = (int)(base + __popc(peers & ((1u << lane) - 1u)));
        }
        __syncthreads();   // hist complete; every thread is done with this slot's buffers
        if (tid == 0) issue(r + 2 * (int64_t)gridDim.x, slot);
        {
            const unsigned cnt = tid < B ? hist[tid] : 0u;
            const unsigned v = (cnt + 7u) & ~7u;
            unsigned sc = v;
            for (int o = 1; o < 32; o <<= 1) {
                unsigned t = __shfl_up_sync(0xffffffffu, sc, o);
                if (lane >= o) sc += t;
            }
            if (lane == 31) wsum[warp] = sc;
            __syncthreads();
            if (warp == 0) {
                unsigned w = wsum[lane];
                for (int o = 1; o < 32; o <<= 1) {
                    unsigned t = __shfl_up_sync(0xffffffffu, w, o);
                    if (lane >= o) w += t;
                }
                wsum[lane] = w;
            }
            __syncthreads();
            const unsigned excl = sc - v + (warp > 0 ? wsum[warp - 1] : 0u);
            if (tid < B) {
                offs[tid] = excl;
                p.dir[r * B + tid] = ((excl >> 3) << 16) | cnt;
                my_total += cnt;
                for (unsigned j = excl + cnt; j < excl + v; ++j) stage[j] = PAD;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (band[k] >= 0) stage[offs[band[k]] + rank[k]] = (uint16_t)local[k];
        __syncthreads();
        const unsigned total = wsum[31];
        uint4 *dst = (uint4 *)(p.entries + r * ROUND_CAP);
        const uint4 *src = (const uint4 *)stage;
        for (unsigned v = tid; v < total / 8; v += blockDim.x) __stcs(dst + v, src[v]);
        if (tid < B) hist[tid] = 0;
        __syncthreads();
    }
    if (tid < B && my_total) atomicAdd(&p.totals[tid], my_total);
}

// ---- plan: work items of similar size
__global__ void __launch_bounds__(256) binned_plan(const BinnedParams p, int target_items) {
    __shared__ unsigned long long s_all[8];
    __shared__ int s_k[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned long long t = tid < p.nbands ? p.totals[tid] : 0ull;
    unsigned long long a = t;
    for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) s_all[warp] = a;
    __syncthreads();
    unsigned long long all = 0;
    for (int w = 0; w < 8; ++w) all += s_all[w];
    long long k = 0;
    if (t) {
        k = (long long)((t * (unsigned long long)target_items + all - 1) / all);
        if (k < 1) k = 1;
        if (k > p.nrounds) k = p.nrounds;
    }
    int inc = (int)k;
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) s_k[warp] = inc;
    __syncthreads();
    int base = inc - (int)k;
    for (int w = 0; w < warp; ++w) base += s_k[w];
    for (long long j = 0; j < k; ++j) {
        const int r0 = (int)(p.nrounds * j / k), r1 = (int)(p.nrounds * (j + 1) / k);
        p.items[base + j] = make_int4(tid, r0, r1, 0);
    }
    if (tid == 255) *p.nitems = base + (int)k;
}

// ---- pass 2
__global__ void __launch_bounds__(512) binned_pass2(const BinnedParams p) {
    extern __shared__ __align__(128) uint32_t band_sm[];
    const int item = blockIdx.x;
    if (item >= *p.nitems) return;
    const int4 it = p.items[item];
    const int b = it.x;
    const int rows = min(p.rows_per_band, p.height - b * p.rows_per_band);
    const int cells = rows * p.width;
    for (int i = threadIdx.x; i < cells; i += blockDim.x) band_sm[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const uint4 *ent = (const uint4 *)p.entries;
    // 32 rounds per warp step: lane j owns round rbase + j; the runs of the 32
    // rounds are flattened into one index space of 8-entry vectors.
    for (int rbase = it.y + warp * 32; rbase < it.z; rbase += nwarps * 32) {
        const int r = rbase + lane;
        const uint32_t d = r < it.z ? __ldg(&p.dir[(int64_t)r * p.nbands + b]) : 0u;
        const unsigned nv = ((d & 0xffffu) + 7u) >> 3;
        const unsigned offv = d >> 16;
        unsigned incl = nv;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const unsigned excl = incl - nv;
        const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
        for (unsigned vb = 0; vb < total; vb += 32) {
            const unsigned e = vb + lane;
            int j = 0;
#pragma unroll
            for (int st = 16; st >= 1; st >>= 1) {
                const unsigned x = __shfl_sync(0xffffffffu, excl, j + st);
                if (x <= e) j += st;
            }
            const unsigned offj = __shfl_sync(0xffffffffu, offv, j);
            const unsigned exj = __shfl_sync(0xffffffffu, excl, j);
            if (e < total) {
                const uint4 q = __ldcs(ent + (int64_t)(rbase + j) * (ROUND_CAP / 8) + offj + (e - exj));
                const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const unsigned lo = w[k] & 0xffffu, hi = w[k] >> 16;
                    if (lo != PAD) atomicAdd(&band_sm[lo], 1u);
                    if (hi != PAD) atomicAdd(&band_sm[hi], 1u);
                }
            }
        }
    }
    __syncthreads();
    // add the band into the output with TMA bulk reductions (16-byte granules);
    // every thread orders its shared-memory writes before the async proxy reads
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t *gdst = p.out + (int64_t)b * p.rows_per_band * p.width;
        const unsigned bytes = (unsigned)cells * 4u;
        const unsigned chunk = 16384u;
        for (unsigned o = 0; o < bytes; o += chunk) {
            unsigned sz = bytes - o < chunk ? bytes - o : chunk;
            unsigned saddr = (unsigned)__cvta_generic_to_shared((char *)band_sm + o);
            asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.u32 [%0], [%1], %2;"
                         :: "l"((char *)gdst + o), "r"(saddr), "r"(sz) : "memory");
        }
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    }
    __syncthreads();
}

// ------------------------------------------------------------- host side

struct BinnedLayout {
    int rows_per_band, nbands;
    int64_t nrounds;
    size_t off_entries, off_dir, off_totals, off_items, off_nitems, off_status, total;
};

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

static bool binned_layout(int64_t n, int width, int height, int target_items, BinnedLayout &L) {
    if (width <= 0 || height <= 0 || width > MAX_BAND_CELLS || (width % 4) != 0) return false;
    // rows per band: about 16K cells (64 KB of shared memory, several CTAs per
    // SM in pass 2), more when needed to keep at most MAX_BANDS bands
    int rpb = 16384 / width;
    if (rpb < 1) rpb = 1;
    while ((height + rpb - 1) / rpb > MAX_BANDS && (int64_t)(rpb + 1) * width <= MAX_BAND_CELLS) ++rpb;
    if (rpb > height) rpb = height;
    int nb = (height + rpb - 1) / rpb;
    if (nb > MAX_BANDS) return false;
    L.rows_per_band = rpb;
    L.nbands = nb;
    L.nrounds = (n + ROUND - 1) / ROUND;
    size_t o = 0;
    L.off_entries = o; o = align_up(o + (size_t)L.nrounds * ROUND_CAP * 2, 256);
    L.off_dir = o; o = align_up(o + (size_t)L.nrounds * nb * 4, 256);
    L.off_totals = o; o = align_up(o + (size_t)nb * 8, 256);
    L.off_items = o; o = align_up(o + (size_t)(nb + target_items + 8) * 16, 256);
    L.off_nitems = o; o = align_up(o + 16, 256);
    L.off_status = o; o = align_up(o + 16, 256);
    L.total = o;
    return true;
}

static int target_items_for_device() {
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    return sms * 3;
}

size_t binned_workspace_size(int64_t n, int width, int height) {
    BinnedLayout L;
    if (!binned_layout(n, width, height, target_items_for_device(), L)) return 0;
    return L.total;
}

// Returns DSGB_E_UNSUPPORTED when the call is not eligible (the caller then
// uses the single-pass path).
int launch_points_binned(const ColumnRef &xc, const ColumnRef &yc, int64_t n, const dsgb_canvas *cv,
                         float xminf, float xmaxf, float yminf, float ymaxf, float ex, float ey,
                         long long kx0, long long kx1, long long ky0, long long ky1,
                         uint32_t *out, bool accumulate, void *ws, size_t ws_bytes, cudaStream_t st) {
    const bool f32 = xc.dtype == DSGB_F32 && yc.dtype == DSGB_F32;
    const bool f64 = xc.dtype == DSGB_F64 && yc.dtype == DSGB_F64;
    if (!(f32 || f64)) return DSGB_E_UNSUPPORTED;
    if (((uintptr_t)xc.data | (uintptr_t)yc.data) & 15u) return DSGB_E_UNSUPPORTED;
    if (((uintptr_t)out & 15u) || ((uintptr_t)ws & 255u)) return DSGB_E_UNSUPPORTED;
    const int target = target_items_for_device();
    BinnedLayout L;
    if (!binned_layout(n, cv->width, cv->height, target, L)) return DSGB_E_UNSUPPORTED;
    if (!ws || ws_bytes < L.total) return DSGB_E_UNSUPPORTED;
    BinnedParams p;
    memset(&p, 0, sizeof(p));
    if (f32) { p.xs32 = (const float *)xc.data; p.ys32 = (const float *)yc.data; }
    else { p.xs64 = (const double *)xc.data; p.ys64 = (const double *)yc.data; }
    p.n = n; p.width = cv->width; p.height = cv->height;
    p.rows_per_band = L.rows_per_band; p.nbands = L.nbands; p.nrounds = L.nrounds;
    p.sx = cv->sx; p.tx = cv->tx; p.sy = cv->sy; p.ty = cv->ty;
    p.xminf = xminf; p.xmaxf = xmaxf; p.yminf = yminf; p.ymaxf = ymaxf;
    p.sxf = (float)cv->sx; p.txf = (float)cv->tx; p.syf = (float)cv->sy; p.tyf = (float)cv->ty;
    p.ex = ex; p.ey = ey;
    p.kxmin = kx0; p.kxmax = kx1; p.kymin = ky0; p.kymax = ky1;
    char *w = (char *)ws;
    p.entries = (uint16_t *)(w + L.off_entries);
    p.dir = (uint32_t *)(w + L.off_dir);
    p.totals = (unsigned long long *)(w + L.off_totals);
    p.items = (int4 *)(w + L.off_items);
    p.nitems = (int *)(w + L.off_nitems);
    p.status = (int *)(w + L.off_status);
    p.out = out;
    cudaError_t e = cudaMemsetAsync(p.totals, 0, (size_t)L.nbands * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.status, 0, 16, st);
    if (e == cudaSuccess && !accumulate) e = cudaMemsetAsync(out, 0, (size_t)cv->width * cv->height * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "binned memset");
    if (n == 0) return DSGB_OK;
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    int64_t g1 = (int64_t)sms;
    if (g1 > L.nrounds) g1 = L.nrounds;
    if (f32) {
        const size_t smem1 = (size_t)4 * ROUND * 4 + (size_t)ROUND_CAP * 2;
        e = cudaFuncSetAttribute(binned_pass1_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
        if (e != cudaSuccess) return cuda_status(e, "binned pass1 smem attribute");
        binned_pass1_tma<<<(unsigned)g1, 1024, smem1, st>>>(p);
    } else {
        binned_pass1<true><<<(unsigned)g1, 1024, 0, st>>>(p);
    }
    binned_plan<<<1, 256, 0, st>>>(p, target);
    const size_t smem = (size_t)L.rows_per_band * cv->width * 4;
    e = cudaFuncSetAttribute(binned_pass2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "binned pass2 smem attribute");
    binned_pass2<<<(unsigned)(L.nbands + target + 8), 512, smem, st>>>(p);
    DSGB_CHECK_LAUNCH("binned count launch");
    return DSGB_OK;
}

}  // namespace dsgb
