// serve.cu -- the resident, spatially bucketed store behind viewport requests.
//
// A viewport request aggregates only the points inside its ranges.  To read
// only those, the store keeps every column regrouped by a G x G grid of
// buckets over a domain square (row-major bucket order, then an "outside"
// bucket for points beyond the domain or with NaN coordinates).  A
// viewport's points then lie in one contiguous row segment per bucket row,
// which dsgb_points_segments aggregates in one launch.
//
//   bs_hist    -- per-block shared-memory histogram of bucket ids;
//   bs_scan    -- one block: exclusive scan into bucket_start (int64) and
//                 the scatter cursors;
//   bs_scatter -- block-aggregated placement (one global reservation per
//                 non-empty bucket and block), every column copied.
//
// Bucket ids come from a float64 estimate; a caller widens a viewport's
// bucket range by one bucket on each side, so no point inside the viewport
// can fall outside the rows it reads.  No reference counterpart: the
// reference rescans the whole frame for every Canvas call.
#include "dsgb_internal.cuh"

namespace dsgb {

constexpr int BS_MAX_GRID = 128;              // 16384 buckets + 1 outside
constexpr int BS_THREADS = 1024;
constexpr int BS_ROWS = 32768;                // rows per scatter block

struct BsParams {
    ColumnRef in[MAX_COLS];
    void *out[MAX_COLS];
    int32_t esize[MAX_COLS];
    int32_t ncols, x_col, y_col;
    int64_t n;
    int32_t grid, nb;                         // nb = grid * grid + 1
    double x0, x1, y0, y1, sx, sy;
    int32_t f32;                              // x and y float32: the estimate in float32
    float x0f, x1f, y0f, y1f, sxf, syf;
    unsigned *count;                          // nb
    unsigned *cursor;                         // nb
    int64_t *start;                           // nb + 1
};

// The bucket is an estimate (readers widen by one bucket and always read the
// outside bucket), so float32 columns are bucketed in float32: GB300 issues
// float64 at a small fraction of the float32 rate.
__device__ __forceinline__ int bs_bucket(const BsParams &p, int64_t i) {
    int bx, by;
    if (p.f32) {
        const float x = __ldg((const float *)p.in[p.x_col].data + i), y = __ldg((const float *)p.in[p.y_col].data + i);
        if (!(x >= p.x0f && x <= p.x1f && y >= p.y0f && y <= p.y1f)) return p.nb - 1;
        bx = (int)((x - p.x0f) * p.sxf);
        by = (int)((y - p.y0f) * p.syf);
    } else {
        const double x = load_f64(p.in[p.x_col], i), y = load_f64(p.in[p.y_col], i);
        if (!(x >= p.x0 && x <= p.x1 && y >= p.y0 && y <= p.y1)) return p.nb - 1;
        bx = (int)((x - p.x0) * p.sx);
        by = (int)((y - p.y0) * p.sy);
    }
    bx = bx < 0 ? 0 : (bx >= p.grid ? p.grid - 1 : bx);
    by = by < 0 ? 0 : (by >= p.grid ? p.grid - 1 : by);
    return by * p.grid + bx;
}

__global__ void __launch_bounds__(BS_THREADS, 1) bs_hist(const BsParams p) {
    extern __shared__ unsigned h[];
    for (int i = threadIdx.x; i < p.nb; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&h[bs_bucket(p, i)], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < p.nb; i += blockDim.x)
        if (h[i]) atomicAdd(&p.count[i], h[i]);
}

__global__ void __launch_bounds__(1024) bs_scan(const BsParams p) {
    __shared__ unsigned long long warp_sums[32];
    const int per = (p.nb + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    unsigned long long mine = 0;
    for (int k = 0; k < per && b0 + k < p.nb; ++k) mine += p.count[b0 + k];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    unsigned long long off = (warp ? warp_sums[warp - 1] : 0ull) + incl - mine;
    for (int k = 0; k < per && b0 + k < p.nb; ++k) {
        p.start[b0 + k] = (int64_t)off;
        p.cursor[b0 + k] = (unsigned)off;
        off += p.count[b0 + k];
    }
    if (threadIdx.x == blockDim.x - 1) p.start[p.nb] = (int64_t)warp_sums[31];
}

__device__ __forceinline__ void copy_elem(const void *src, void *dst, int64_t i, int64_t j, int esize) {
    switch (esize) {
    case 1: ((uint8_t *)dst)[j] = ((const uint8_t *)src)[i]; break;
    case 2: ((uint16_t *)dst)[j] = ((const uint16_t *)src)[i]; break;
    case 4: ((uint32_t *)dst)[j] = ((const uint32_t *)src)[i]; break;
    default: ((uint64_t *)dst)[j] = ((const uint64_t *)src)[i]; break;
    }
}

__global__ void __launch_bounds__(BS_THREADS, 1) bs_scatter(const BsParams p) {
    extern __shared__ unsigned h[];
    for (int i = threadIdx.x; i < p.nb; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const int64_t r0 = (int64_t)blockIdx.x * BS_ROWS;
    const int64_t r1 = r0 + BS_ROWS < p.n ? r0 + BS_ROWS : p.n;
    for (int64_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) atomicAdd(&h[bs_bucket(p, i)], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < p.nb; i += blockDim.x) {
        const unsigned c = h[i];
        if (c) h[i] = atomicAdd(&p.cursor[i], c);
    }
    __syncthreads();
    for (int64_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const unsigned pos = atomicAdd(&h[bs_bucket(p, i)], 1u);
        for (int c = 0; c < p.ncols; ++c) copy_elem(p.in[c].data, p.out[c], i, pos, p.esize[c]);
    }
}

}  // namespace dsgb

using namespace dsgb;

extern "C" size_t dsgb_bucket_sort_workspace_size(int32_t grid) {
    if (grid < 1 || grid > BS_MAX_GRID) return 0;
    const size_t nb = (size_t)grid * grid + 1;
    return ((nb * 4 + 255) / 256) * 256 * 2;
}

extern "C" int dsgb_bucket_sort(const dsgb_column *cols, int32_t ncols, int64_t n, int32_t x_col, int32_t y_col,
                                const double *domain, int32_t grid, void *const *out_data, int64_t *bucket_start,
                                void *workspace, size_t workspace_bytes, void *stream) {
    if (!cols || !domain || !out_data || !bucket_start || ncols < 1 || ncols > MAX_COLS || n < 0 ||
        n >= (int64_t)0xF0000000ll || x_col < 0 || x_col >= ncols || y_col < 0 || y_col >= ncols ||
        grid < 1 || grid > BS_MAX_GRID) {
        set_error("dsgb_bucket_sort: invalid arguments (ncols=%d, n=%lld, grid=%d; grid <= %d, n < 2^32 - 2^28)",
                  ncols, (long long)n, grid, BS_MAX_GRID);
        return DSGB_E_INVALID;
    }
    if (!(domain[1] > domain[0]) || !(domain[3] > domain[2])) {
        set_error("dsgb_bucket_sort: empty domain");
        return DSGB_E_INVALID;
    }
    const size_t need = dsgb_bucket_sort_workspace_size(grid);
    if (!workspace || ((uintptr_t)workspace & 255u) || workspace_bytes < need) {
        set_error("dsgb_bucket_sort: workspace must be 256-byte aligned and at least %zu bytes", need);
        return DSGB_E_NOSPACE;
    }
    BsParams p;
    memset(&p, 0, sizeof(p));
    for (int c = 0; c < ncols; ++c) {
        const int es = dtype_size(cols[c].dtype);
        if (es == 0 || (n > 0 && (!cols[c].data || !out_data[c]))) {
            set_error("dsgb_bucket_sort: column %d has bad dtype or null data", c);
            return DSGB_E_INVALID;
        }
        p.in[c] = ColumnRef{cols[c].data, cols[c].dtype};
        p.out[c] = out_data[c];
        p.esize[c] = es;
    }
    p.ncols = ncols; p.x_col = x_col; p.y_col = y_col; p.n = n;
    p.grid = grid; p.nb = grid * grid + 1;
    p.x0 = domain[0]; p.x1 = domain[1]; p.y0 = domain[2]; p.y1 = domain[3];
    p.sx = grid / (p.x1 - p.x0);
    p.sy = grid / (p.y1 - p.y0);
    p.f32 = cols[x_col].dtype == DSGB_F32 && cols[y_col].dtype == DSGB_F32;
    p.x0f = (float)p.x0; p.x1f = (float)p.x1; p.y0f = (float)p.y0; p.y1f = (float)p.y1;
    p.sxf = (float)p.sx; p.syf = (float)p.sy;
    const size_t half = need / 2;
    p.count = (unsigned *)workspace;
    p.cursor = (unsigned *)((char *)workspace + half);
    p.start = bucket_start;
    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(p.count, 0, (size_t)p.nb * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "dsgb_bucket_sort memset");
    const size_t smem = (size_t)p.nb * 4;
    e = cudaFuncSetAttribute(bs_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, 66 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(bs_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, 66 * 1024);
    if (e != cudaSuccess) return cuda_status(e, "dsgb_bucket_sort attributes");
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    bs_hist<<<sms, BS_THREADS, smem, st>>>(p);
    DSGB_CHECK_LAUNCH("bs_hist");
    bs_scan<<<1, 1024, 0, st>>>(p);
    DSGB_CHECK_LAUNCH("bs_scan");
    const int64_t blocks = (n + BS_ROWS - 1) / BS_ROWS;
    if (blocks > 0) {
        bs_scatter<<<(unsigned)blocks, BS_THREADS, smem, st>>>(p);
        DSGB_CHECK_LAUNCH("bs_scatter");
    }
    return DSGB_OK;
}
