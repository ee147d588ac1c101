// points_det.cu -- deterministic sum / mean for Canvas.points.
//
// The reference's CPU loop adds a pixel's values in row order
// (reductions.py:1054-1063 for sum, :938-996 for the _sum_zero base of
// mean).  Float64 atomics add them in arrival order, so the last bits of a
// sum can differ from run to run.  With DSGB_FLAG_DETERMINISTIC the SUM
// bases are computed instead by
//
//   det_keys     -- the cell of every row (pixel, or pixel * ncat + category;
//                   `invalid` for rows outside the canvas);
//   det_count / det_scan_* / det_scatter
//                -- a stable LSD radix sort of (cell, row) pairs, 8-bit
//                   digits: per tile of 2048 rows a digit histogram, an
//                   exclusive scan of all histograms in digit-major order,
//                   then each tile places its rows in row order (ranks from
//                   a warp match per digit and per-warp digit counts);
//   det_segsum   -- one thread per cell adds the cell's values in row order,
//                   starting from 0.0 and skipping NaN, like _sum_zero.
//
// The result is bit-identical to the reference's sequential loop and to
// every other run.
#include "points_params.cuh"

namespace dsgb {

constexpr int DET_THREADS = 256;
constexpr int DET_ITEMS = 8;
constexpr int DET_TILE = DET_THREADS * DET_ITEMS;
constexpr int DET_WARPS = DET_THREADS / 32;
constexpr int DET_SCAN_CHUNK = 4096;        // entries per scan block (1024 threads x 4)

__device__ __forceinline__ bool det_bin(const PointsParams &p, int64_t i, bool fast, int &xi, int &yi) {
    const int xdt = p.cols[p.x_col].dtype, ydt = p.cols[p.y_col].dtype;
    if (fast && xdt == DSGB_F32 && ydt == DSGB_F32) {
        const float x = ((const float *)p.cols[p.x_col].data)[i], y = ((const float *)p.cols[p.y_col].data)[i];
        return bin_point_f32(x, y, p.bb, p.ax, p.ay, xi, yi);
    }
    if (fast && xdt == DSGB_F64 && ydt == DSGB_F64) {
        const double x = ((const double *)p.cols[p.x_col].data)[i], y = ((const double *)p.cols[p.y_col].data)[i];
        return bin_point_f64(x, y, p.bb, p.ax, p.ay, xi, yi);
    }
    return bin_exact_xy(p, load_f64(p.cols[p.x_col], i), load_f64(p.cols[p.y_col], i), xi, yi);
}

__global__ void det_keys(const PointsParams p, bool fast, int cat_col, int ncat, unsigned invalid,
                         unsigned *key, unsigned *idx) {
    for (int64_t i = gtid(); i < p.n; i += gstride()) {
        int xi, yi;
        unsigned k = invalid;
        if (det_bin(p, i, fast, xi, yi)) {
            k = (unsigned)yi * (unsigned)p.width + (unsigned)xi;
            if (cat_col >= 0) {
                long long c = load_i64(p.cols[cat_col], i);
                if (c < 0) c += ncat;                   // numba's negative index (compiler.py:379-390)
                k = (c < 0 || c >= ncat) ? invalid : k * (unsigned)ncat + (unsigned)c;
            }
        }
        key[i] = k;
        idx[i] = (unsigned)i;
    }
}

__global__ void __launch_bounds__(DET_THREADS) det_count(const unsigned *key, int64_t n, int shift,
                                                         unsigned *counts, int64_t ntiles) {
    __shared__ unsigned h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * DET_TILE;
    for (int k = 0; k < DET_ITEMS; ++k) {
        const int64_t row = base + k * DET_THREADS + threadIdx.x;
        if (row < n) atomicAdd(&h[(key[row] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of m uint32 in place: per-block scan + block totals ...
__global__ void __launch_bounds__(1024) det_scan_blocks(unsigned *a, int64_t m, unsigned *block_sums) {
    __shared__ unsigned ws[32];
    const int64_t b0 = (int64_t)blockIdx.x * DET_SCAN_CHUNK + threadIdx.x * 4;
    unsigned v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = b0 + k < m ? a[b0 + k] : 0u;
        s += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        ws[lane] = w;
    }
    __syncthreads();
    unsigned off = (warp ? ws[warp - 1] : 0u) + incl - s;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (b0 + k < m) a[b0 + k] = off;
        off += v[k];
    }
    if (threadIdx.x == blockDim.x - 1) block_sums[blockIdx.x] = ws[31];
}

// ... one block scans the block totals (nb <= 1024 * 64) ...
__global__ void __launch_bounds__(1024) det_scan_sums(unsigned *s, int64_t nb) {
    __shared__ unsigned ws[32];
    const int per = (int)((nb + blockDim.x - 1) / blockDim.x);
    const int64_t b0 = (int64_t)threadIdx.x * per;
    unsigned mine = 0;
    for (int k = 0; k < per && b0 + k < nb; ++k) mine += s[b0 + k];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        ws[lane] = w;
    }
    __syncthreads();
    unsigned off = (warp ? ws[warp - 1] : 0u) + incl - mine;
    for (int k = 0; k < per && b0 + k < nb; ++k) {
        const unsigned c = s[b0 + k];
        s[b0 + k] = off;
        off += c;
    }
}

// ... and every block adds its offset.
__global__ void __launch_bounds__(1024) det_scan_add(unsigned *a, int64_t m, const unsigned *block_sums) {
    const unsigned add = block_sums[blockIdx.x];
    const int64_t b0 = (int64_t)blockIdx.x * DET_SCAN_CHUNK + threadIdx.x * 4;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (b0 + k < m) a[b0 + k] += add;
}

__global__ void __launch_bounds__(DET_THREADS) det_scatter(const unsigned *key_in, const unsigned *idx_in,
                                                           unsigned *key_out, unsigned *idx_out, int64_t n,
                                                           int shift, const unsigned *offsets, int64_t ntiles) {
    __shared__ unsigned run[256];
    __shared__ unsigned wc[DET_WARPS][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    run[threadIdx.x] = offsets[(int64_t)threadIdx.x * ntiles + blockIdx.x];
    const int64_t base = (int64_t)blockIdx.x * DET_TILE;
    const unsigned lt = (1u << lane) - 1u;
    for (int k = 0; k < DET_ITEMS; ++k) {
        for (int j = threadIdx.x; j < DET_WARPS * 256; j += DET_THREADS) (&wc[0][0])[j] = 0u;
        __syncthreads();
        const int64_t row = base + k * DET_THREADS + threadIdx.x;
        const bool valid = row < n;
        const unsigned kv = valid ? key_in[row] : 0u;
        const unsigned d = (kv >> shift) & 255u;
        const unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 0x100u + lane);
        const unsigned lrank = __popc(peers & lt);
        if (valid && lrank == 0) wc[warp][d] = __popc(peers);
        __syncthreads();
        {
            unsigned acc = run[threadIdx.x];
#pragma unroll
            for (int w = 0; w < DET_WARPS; ++w) {
                const unsigned c = wc[w][threadIdx.x];
                wc[w][threadIdx.x] = acc;
                acc += c;
            }
            run[threadIdx.x] = acc;
        }
        __syncthreads();
        if (valid) {
            const unsigned pos = wc[warp][d] + lrank;
            key_out[pos] = kv;
            idx_out[pos] = idx_in[row];
        }
        __syncthreads();
    }
}

__global__ void det_segsum(const unsigned *key, const unsigned *idx, int64_t n, unsigned invalid, ColumnRef v,
                           double *sum_out) {
    for (int64_t j = gtid(); j < n; j += gstride()) {
        const unsigned k = key[j];
        if (k == invalid || (j > 0 && key[j - 1] == k)) continue;
        double acc = 0.0;
        for (int64_t m = j; m < n && key[m] == k; ++m) {
            const double x = load_f64(v, idx[m]);
            if (!isnull(x)) acc = __dadd_rn(acc, x);
        }
        sum_out[k] = acc;
    }
}

// ------------------------------------------------------------- host side

struct DetLayout {
    int64_t ntiles, m, nscan;
    size_t off_k0, off_i0, off_k1, off_i1, off_counts, off_sums, total;
};

static size_t det_align(size_t v) { return (v + 255) / 256 * 256; }

static DetLayout det_layout(int64_t n) {
    DetLayout L;
    L.ntiles = (n + DET_TILE - 1) / DET_TILE;
    L.m = 256 * L.ntiles;
    L.nscan = (L.m + DET_SCAN_CHUNK - 1) / DET_SCAN_CHUNK;
    size_t o = 0;
    L.off_k0 = o; o = det_align(o + (size_t)n * 4);
    L.off_i0 = o; o = det_align(o + (size_t)n * 4);
    L.off_k1 = o; o = det_align(o + (size_t)n * 4);
    L.off_i1 = o; o = det_align(o + (size_t)n * 4);
    L.off_counts = o; o = det_align(o + (size_t)L.m * 4);
    L.off_sums = o; o = det_align(o + (size_t)L.nscan * 4);
    L.total = o;
    return L;
}

size_t det_workspace_size(int64_t n) { return n > 0 ? det_layout(n).total : 0; }

// Computes every SUM base of `p` deterministically (the bases are
// initialised; the other bases are left to the caller).
int det_sums(const PointsParams &p, bool fast, void *ws, size_t ws_bytes, cudaStream_t st) {
    if (p.n <= 0) return DSGB_OK;
    if (p.n >= (int64_t)0xF0000000ll) {
        set_error("dsgb_points: the deterministic mode handles fewer than 2^32 - 2^28 rows");
        return DSGB_E_UNSUPPORTED;
    }
    const DetLayout L = det_layout(p.n);
    if (!ws || ((uintptr_t)ws & 255u) || ws_bytes < L.total) {
        set_error("dsgb_points: the deterministic mode needs a 256-byte aligned workspace of %zu bytes", L.total);
        return DSGB_E_NOSPACE;
    }
    if (L.nscan > 1024 * 64) {
        set_error("dsgb_points: too many rows for the deterministic scan");
        return DSGB_E_UNSUPPORTED;
    }
    char *w = (char *)ws;
    unsigned *k0 = (unsigned *)(w + L.off_k0), *i0 = (unsigned *)(w + L.off_i0);
    unsigned *k1 = (unsigned *)(w + L.off_k1), *i1 = (unsigned *)(w + L.off_i1);
    unsigned *counts = (unsigned *)(w + L.off_counts), *sums = (unsigned *)(w + L.off_sums);
    const int64_t ncells = (int64_t)p.width * p.height;
    int sorted_cat = -2, sorted_ncat = 0;
    const unsigned *ks = k0, *is = i0;
    for (int b = 0; b < p.nbases; ++b) {
        const BaseDev &B = p.bases[b];
        if (B.op != DSGB_BASE_SUM) continue;
        const int64_t cells = ncells * (B.cat_col >= 0 ? B.ncat : 1);
        if (cells >= (int64_t)0xFFFFFFFFll) {
            set_error("dsgb_points: the deterministic mode handles fewer than 2^32 cells");
            return DSGB_E_UNSUPPORTED;
        }
        const unsigned invalid = (unsigned)cells;
        if (B.cat_col != sorted_cat || (B.cat_col >= 0 && B.ncat != sorted_ncat)) {
            det_keys<<<grid_of(p.n), 256, 0, st>>>(p, fast, B.cat_col, B.ncat, invalid, k0, i0);
            DSGB_CHECK_LAUNCH("det_keys");
            int bits = 1;
            while (bits < 32 && ((uint64_t)1 << bits) <= (uint64_t)invalid) ++bits;
            unsigned *kin = k0, *iin = i0, *kout = k1, *iout = i1;
            for (int shift = 0; shift < bits; shift += 8) {
                det_count<<<(unsigned)L.ntiles, DET_THREADS, 0, st>>>(kin, p.n, shift, counts, L.ntiles);
                det_scan_blocks<<<(unsigned)L.nscan, 1024, 0, st>>>(counts, L.m, sums);
                det_scan_sums<<<1, 1024, 0, st>>>(sums, L.nscan);
                det_scan_add<<<(unsigned)L.nscan, 1024, 0, st>>>(counts, L.m, sums);
                det_scatter<<<(unsigned)L.ntiles, DET_THREADS, 0, st>>>(kin, iin, kout, iout, p.n, shift, counts,
                                                                      L.ntiles);
                DSGB_CHECK_LAUNCH("det radix pass");
                unsigned *t = kin; kin = kout; kout = t;
                t = iin; iin = iout; iout = t;
            }
            ks = kin; is = iin;
            sorted_cat = B.cat_col;
            sorted_ncat = B.ncat;
        }
        det_segsum<<<grid_of(p.n), 256, 0, st>>>(ks, is, p.n, invalid, p.cols[B.col], (double *)B.agg);
        DSGB_CHECK_LAUNCH("det_segsum");
    }
    return DSGB_OK;
}

}  // namespace dsgb
