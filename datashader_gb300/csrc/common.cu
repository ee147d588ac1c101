// common.cu -- error reporting, base initialisation, finalize, autorange.
//
// bases_init restates the initial values of Reduction._create_*
// (datashader/reductions.py:397-472) in their GPU base forms; finalize
// restates the _finalize functions (reductions.py: sum 1091-1096, mean
// 1290-1296, first/last 1369-1373, where 2152-2162) and make_finalize
// (datashader/compiler.py:510-536).
#include "dsgb_internal.cuh"

#include <stdarg.h>
#include <cmath>

namespace dsgb {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char *what) {
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    return DSGB_E_CUDA;
}

int sm_count() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    return n;
}

// ------------------------------------------------------------------ init


static unsigned grid_for(int64_t n, int threads = 256) {
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    int64_t g = (n + threads - 1) / threads;
    int64_t cap = (int64_t)sms * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (unsigned)g;
}

// Every base's initial value in one launch: a base is a byte range filled
// with a 16-byte pattern (two 64-bit words; 8-byte values repeat).
constexpr int INIT_BATCH = 16;
struct InitBatch {
    int32_t count;
    int64_t chunks;                     // 16-byte chunks of the largest base
    unsigned char *ptr[INIT_BATCH];
    int64_t bytes[INIT_BATCH];
    unsigned long long lo[INIT_BATCH], hi[INIT_BATCH];
};

__global__ void init_kernel(const __grid_constant__ InitBatch b) {
    for (int64_t i = gtid(); i < b.chunks; i += gstride()) {
#pragma unroll 1
        for (int k = 0; k < b.count; ++k) {
            const int64_t off = 16 * i;
            if (off + 16 <= b.bytes[k] && !((uintptr_t)b.ptr[k] & 15u)) {
                *(ulonglong2 *)(b.ptr[k] + off) = make_ulonglong2(b.lo[k], b.hi[k]);
            } else if (off < b.bytes[k]) {
                const int64_t end = off + 16 < b.bytes[k] ? off + 16 : b.bytes[k];
                for (int64_t j = off; j < end; ++j)
                    b.ptr[k][j] = (unsigned char)((j & 8 ? b.hi[k] : b.lo[k]) >> (8 * (j & 7)));
            }
        }
    }
}

int bases_init(const dsgb_base *bases, int32_t nbases, int64_t ncells, cudaStream_t st) {
    InitBatch ib;
    memset(&ib, 0, sizeof(ib));
    auto flush = [&]() -> int {
        if (!ib.count) return DSGB_OK;
        init_kernel<<<grid_for(ib.chunks), 256, 0, st>>>(ib);
        DSGB_CHECK_LAUNCH("dsgb_bases_init");
        ib.count = 0;
        ib.chunks = 0;
        return DSGB_OK;
    };
    for (int b = 0; b < nbases; ++b) {
        const dsgb_base &B = bases[b];
        const int64_t n = ncells * (B.ncat < 1 ? 1 : B.ncat);
        if (!B.agg) { set_error("dsgb_bases_init: base %d has null agg", b); return DSGB_E_INVALID; }
        unsigned long long lo = 0, hi = 0;
        int64_t bytes = 0;
        switch (B.op) {
        case DSGB_BASE_COUNT: case DSGB_BASE_AA_CNT0: bytes = n * 4; break;
        case DSGB_BASE_ANY: bytes = n; break;
        case DSGB_BASE_SUM: case DSGB_BASE_AA_SUM: bytes = n * 8; break;
        case DSGB_BASE_MAX: case DSGB_BASE_AA_MAX:
            bytes = n * 8; lo = hi = (unsigned long long)KEY_EMPTY_MAX; break;
        case DSGB_BASE_MIN: bytes = n * 8; lo = hi = (unsigned long long)KEY_EMPTY_MIN; break;
        case DSGB_BASE_MIN_ROW: bytes = n * 8; lo = hi = (unsigned long long)ROW_EMPTY_MIN; break;
        case DSGB_BASE_MAX_ROW: bytes = n * 8; lo = hi = ~0ull; break;          // -1
        case DSGB_BASE_ARGMAX: case DSGB_BASE_AA_ARGMAX:
            bytes = n * 16; lo = (unsigned long long)KEY_EMPTY_MAX; hi = (unsigned long long)ROW_EMPTY_MIN; break;
        case DSGB_BASE_ARGMIN:
            bytes = n * 16; lo = (unsigned long long)KEY_EMPTY_MIN; hi = (unsigned long long)ROW_EMPTY_MIN; break;
        default:
            set_error("dsgb_bases_init: unknown base op %d", B.op);
            return DSGB_E_INVALID;
        }
        ib.ptr[ib.count] = (unsigned char *)B.agg;
        ib.bytes[ib.count] = bytes;
        ib.lo[ib.count] = lo;
        ib.hi[ib.count] = hi;
        ++ib.count;
        const int64_t ch = (bytes + 15) / 16;
        if (ch > ib.chunks) ib.chunks = ch;
        if (ib.count == INIT_BATCH) {
            const int rc = flush();
            if (rc) return rc;
        }
    }
    return flush();
}

// -------------------------------------------------------------- finalize

struct FinArgs {
    int32_t op;
    int32_t b0op, b1op;
    const void *b0, *b1;
    ColumnRef col;
    int64_t row_offset;
    int64_t ncol_rows;
    void *out;
    int64_t n;
    int32_t out_bytes;
};

__device__ __forceinline__ double nan_d() { return __longlong_as_double(0x7ff8000000000000ll); }

// Row index held by a row-valued base, or -1.
__device__ __forceinline__ long long base_row(int op, const void *b, int64_t i) {
    const long long *q = (const long long *)b;
    switch (op) {
    case DSGB_BASE_MIN_ROW: { long long r = q[i]; return r == ROW_EMPTY_MIN ? -1 : r; }
    case DSGB_BASE_MAX_ROW: return q[i];
    case DSGB_BASE_ARGMAX: case DSGB_BASE_ARGMIN: case DSGB_BASE_AA_ARGMAX: {
        long long r = q[2 * i + 1]; return r == ROW_EMPTY_MIN ? -1 : r; }
    default: return -1;
    }
}

// Key held by a key-valued base, with empty = false.
__device__ __forceinline__ bool base_key(int op, const void *b, int64_t i, long long &k) {
    const long long *q = (const long long *)b;
    switch (op) {
    case DSGB_BASE_MAX: case DSGB_BASE_AA_MAX: k = q[i]; return k != KEY_EMPTY_MAX;
    case DSGB_BASE_MIN: k = q[i]; return k != KEY_EMPTY_MIN;
    case DSGB_BASE_ARGMAX: case DSGB_BASE_AA_ARGMAX: k = q[2 * i]; return k != KEY_EMPTY_MAX;
    case DSGB_BASE_ARGMIN: k = q[2 * i]; return k != KEY_EMPTY_MIN;
    default: return false;
    }
}

// Whether something landed in cell i, from a count/any base.
__device__ __forceinline__ bool base_hit(int op, const void *b, int64_t i, unsigned &cnt) {
    if (op == DSGB_BASE_ANY) { cnt = ((const uint8_t *)b)[i]; return cnt != 0; }
    cnt = ((const unsigned *)b)[i];
    return cnt != 0;
}

__device__ __forceinline__ void finalize_cell(const FinArgs &a, int64_t i) {
    {
        switch (a.op) {
        case DSGB_FIN_SUM_NAN: {
            unsigned c; bool hit = base_hit(a.b1op, a.b1, i, c);
            ((double *)a.out)[i] = hit ? ((const double *)a.b0)[i] : nan_d();
            break; }
        case DSGB_FIN_SUM_F32: {
            unsigned c; bool hit = base_hit(a.b1op, a.b1, i, c);
            ((float *)a.out)[i] = hit ? (float)((const double *)a.b0)[i] : __int_as_float(0x7fc00000);
            break; }
        case DSGB_FIN_MEAN: {
            unsigned c; base_hit(a.b1op, a.b1, i, c);
            // reductions.py:1293-1296: where(counts > 0, sums/counts, nan)
            ((double *)a.out)[i] = c > 0 ? ((const double *)a.b0)[i] / (double)c : nan_d();
            break; }
        case DSGB_FIN_KEY_F64: {
            long long k; bool ok = base_key(a.b0op, a.b0, i, k);
            ((double *)a.out)[i] = ok ? key_f64(k) : nan_d();
            break; }
        case DSGB_FIN_KEY_F32: {
            long long k; bool ok = base_key(a.b0op, a.b0, i, k);
            ((float *)a.out)[i] = ok ? (float)key_f64(k) : __int_as_float(0x7fc00000);
            break; }
        case DSGB_FIN_ROW:
            ((long long *)a.out)[i] = base_row(a.b0op, a.b0, i);
            break;
        case DSGB_FIN_GATHER: {
            long long r = base_row(a.b0op, a.b0, i);
            long long j = r - a.row_offset;
            ((double *)a.out)[i] = (r >= 0 && j >= 0 && j < a.ncol_rows) ? load_f64(a.col, j) : nan_d();
            break; }
        case DSGB_FIN_COPY: {
            if (a.out_bytes == 4) ((unsigned *)a.out)[i] = ((const unsigned *)a.b0)[i];
            else if (a.out_bytes == 1) ((uint8_t *)a.out)[i] = ((const uint8_t *)a.b0)[i];
            else ((unsigned long long *)a.out)[i] = ((const unsigned long long *)a.b0)[i];
            break; }
        default: break;
        }
    }
}

// Every output of a plan in one launch: a thread finalizes cell i of each
// output that has one.
constexpr int FIN_BATCH = 16;
struct FinBatch {
    int32_t count;
    int64_t n;                      // the largest output
    FinArgs a[FIN_BATCH];
};

__global__ void finalize_kernel(const __grid_constant__ FinBatch b) {
    for (int64_t i = gtid(); i < b.n; i += gstride()) {
#pragma unroll 1
        for (int k = 0; k < b.count; ++k)
            if (i < b.a[k].n) finalize_cell(b.a[k], i);
    }
}

// Gather over row partitions (dask.py:102-117 numbers each partition's rows
// from its own offset): the row that the combined row-index base selected
// is looked up in the partition that holds it.
constexpr int FIN_MAX_PARTS = 64;
struct GatherParts {
    int32_t nparts, b0op;
    const void *b0;
    void *out;
    int64_t n;
    ColumnRef col[FIN_MAX_PARTS];
    int64_t first[FIN_MAX_PARTS], rows[FIN_MAX_PARTS];
};

__global__ void gather_parts_kernel(const __grid_constant__ GatherParts g) {
    for (int64_t i = gtid(); i < g.n; i += gstride()) {
        const long long r = base_row(g.b0op, g.b0, i);
        double v = nan_d();
        if (r >= 0) {
            for (int p = 0; p < g.nparts; ++p) {
                const long long j = r - g.first[p];
                if (j >= 0 && j < g.rows[p]) { v = load_f64(g.col[p], j); break; }
            }
        }
        ((double *)g.out)[i] = v;
    }
}

// Cross-process form: partition p looked its gather up itself (vals[p], one
// float64 per cell, NaN where empty); the owner of the selected row gives
// the value.  A cell that no partition selected reads partition 0 (NaN).
struct SelectParts {
    int32_t nparts, b0op;
    const void *b0;
    double *out;
    int64_t n;
    const double *vals[FIN_MAX_PARTS];
    int64_t first[FIN_MAX_PARTS], rows[FIN_MAX_PARTS];
};

__global__ void select_owner_kernel(const __grid_constant__ SelectParts g) {
    for (int64_t i = gtid(); i < g.n; i += gstride()) {
        const long long r = base_row(g.b0op, g.b0, i);
        int owner = 0;
        if (r >= 0) {
            for (int p = 0; p < g.nparts; ++p) {
                const long long j = r - g.first[p];
                if (j >= 0 && j < g.rows[p]) { owner = p; break; }
            }
        }
        g.out[i] = g.vals[owner][i];
    }
}

static int base_elem_bytes(int op) {
    switch (op) {
    case DSGB_BASE_COUNT: case DSGB_BASE_AA_CNT0: return 4;
    case DSGB_BASE_ANY: return 1;
    case DSGB_BASE_ARGMAX: case DSGB_BASE_ARGMIN: case DSGB_BASE_AA_ARGMAX: return 16;
    default: return 8;
    }
}

int finalize_outputs(const dsgb_column *cols, int32_t ncols, int64_t row_offset,
                     const dsgb_base *bases, int32_t nbases, const dsgb_output *outs, int32_t nouts,
                     int64_t ncells, cudaStream_t st, int64_t ncol_rows) {
    NvtxRange range("dsgb finalize");
    FinBatch batch;
    memset(&batch, 0, sizeof(batch));
    for (int o = 0; o < nouts; ++o) {
        const dsgb_output &O = outs[o];
        if (!O.out || O.base0 < 0 || O.base0 >= nbases) {
            set_error("dsgb_finalize: output %d invalid", o);
            return DSGB_E_INVALID;
        }
        FinArgs a;
        memset(&a, 0, sizeof(a));
        a.op = O.op;
        const dsgb_base &B0 = bases[O.base0];
        a.b0op = B0.op; a.b0 = B0.agg;
        if (O.op == DSGB_FIN_SUM_NAN || O.op == DSGB_FIN_MEAN || O.op == DSGB_FIN_SUM_F32) {
            if (O.base1 < 0 || O.base1 >= nbases) { set_error("dsgb_finalize: output %d needs base1", o); return DSGB_E_INVALID; }
            a.b1op = bases[O.base1].op; a.b1 = bases[O.base1].agg;
        }
        if (O.op == DSGB_FIN_GATHER) {
            if (O.col < 0 || O.col >= ncols || !cols) { set_error("dsgb_finalize: output %d gather column", o); return DSGB_E_INVALID; }
            a.col.data = cols[O.col].data; a.col.dtype = cols[O.col].dtype;
        }
        if (O.op < DSGB_FIN_SUM_NAN || O.op > DSGB_FIN_COPY) { set_error("dsgb_finalize: bad op %d", O.op); return DSGB_E_INVALID; }
        a.row_offset = row_offset;
        a.ncol_rows = ncol_rows;
        a.out = O.out;
        a.n = ncells * (B0.ncat < 1 ? 1 : B0.ncat);
        a.out_bytes = base_elem_bytes(B0.op);
        batch.a[batch.count++] = a;
        if (a.n > batch.n) batch.n = a.n;
        if (batch.count == FIN_BATCH || o == nouts - 1) {
            finalize_kernel<<<grid_for(batch.n), 256, 0, st>>>(batch);
            DSGB_CHECK_LAUNCH("finalize kernel");
            batch.count = 0;
            batch.n = 0;
        }
    }
    return DSGB_OK;
}

// Compatibility overload used by the glyph entry points: the gather bound
// is the number of rows of the call.
int finalize_outputs(const dsgb_column *cols, int32_t ncols, int64_t row_offset,
                     const dsgb_base *bases, int32_t nbases, const dsgb_output *outs, int32_t nouts,
                     int64_t ncells, cudaStream_t st) {
    return finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st,
                            (int64_t)1 << 62);
}

// ------------------------------------------------------------- autorange

__device__ __forceinline__ unsigned long long ord_u64(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double unord_u64(unsigned long long u) {
    unsigned long long b = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)b);
}

// glyph.py:66-78: NaN-skipping min/max.  mm[0] = ordered min, mm[1] = ordered max.
__global__ void bounds_kernel(const ColumnRef c, int64_t n, unsigned long long *mm) {
    unsigned long long lo = ~0ull, hi = 0ull;
    for (int64_t i = gtid(); i < n; i += gstride()) {
        double v = load_f64(c, i);
        if (v == v) {
            unsigned long long u = ord_u64(v);
            lo = u < lo ? u : lo;
            hi = u > hi ? u : hi;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o);
        unsigned long long h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    if ((threadIdx.x & 31) == 0) {
        if (lo != ~0ull) atomicMin(&mm[0], lo);
        if (hi != 0ull) atomicMax(&mm[1], hi);
    }
}

__global__ void bounds_finish_kernel(unsigned long long *mm, double *out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        unsigned long long lo = mm[0], hi = mm[1];
        double a = (lo == ~0ull) ? __longlong_as_double(0x7ff0000000000000ll) : unord_u64(lo);
        double b = (hi == 0ull) ? __longlong_as_double((long long)0xfff0000000000000ull) : unord_u64(hi);
        out[0] = a;
        out[1] = b;
    }
}

__global__ void bounds_init_kernel(unsigned long long *mm) {
    if (threadIdx.x == 0 && blockIdx.x == 0) { mm[0] = ~0ull; mm[1] = 0ull; }
}

}  // namespace dsgb

using namespace dsgb;

extern "C" int dsgb_abi_version(void) { return DSGB_ABI_VERSION; }
extern "C" const char *dsgb_last_error(void) { return g_err; }
namespace dsgb {
int status_points(unsigned *bits, bool clear);
int status_line(unsigned *bits, bool clear);
int status_points_hot(unsigned *bits, bool clear);
int status_points_part(unsigned *bits, bool clear);
}

extern "C" int dsgb_device_status(uint32_t *bits, int32_t clear) {
    if (!bits) {
        set_error("dsgb_device_status: null bits");
        return DSGB_E_INVALID;
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_status(e, "dsgb_device_status synchronize");
    unsigned v = 0;
    int rc = status_points(&v, clear != 0);
    if (rc == DSGB_OK) rc = status_line(&v, clear != 0);
    if (rc == DSGB_OK) rc = status_points_hot(&v, clear != 0);
    if (rc == DSGB_OK) rc = status_points_part(&v, clear != 0);
    if (rc != DSGB_OK) return rc;
    *bits |= v;
    return DSGB_OK;
}

extern "C" int dsgb_device_sm_count(void) {
    int n = sm_count();
    if (n < 0) { set_error("no CUDA device"); return DSGB_E_CUDA; }
    return n;
}

// ---- combine: partial bases of two row partitions (datashader's dask
// combine, dask.py:86-219 with each reduction's _combine).  Rows carry
// their global index (row_offset), so row-index bases combine by min / max
// and {key,row} pairs by the same order as the append.
__global__ void combine_kernel(int op, void *dst, const void *src, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        switch (op) {
        case DSGB_BASE_COUNT: case DSGB_BASE_AA_CNT0: ((unsigned *)dst)[i] += ((const unsigned *)src)[i]; break;
        case DSGB_BASE_ANY: ((uint8_t *)dst)[i] |= ((const uint8_t *)src)[i]; break;
        case DSGB_BASE_SUM: case DSGB_BASE_AA_SUM: ((double *)dst)[i] += ((const double *)src)[i]; break;
        case DSGB_BASE_MAX: case DSGB_BASE_MAX_ROW: case DSGB_BASE_AA_MAX: {
            long long *d = (long long *)dst;
            const long long v = ((const long long *)src)[i];
            if (v > d[i]) d[i] = v;
            break;
        }
        case DSGB_BASE_MIN: case DSGB_BASE_MIN_ROW: {
            long long *d = (long long *)dst;
            const long long v = ((const long long *)src)[i];
            if (v < d[i]) d[i] = v;
            break;
        }
        case DSGB_BASE_ARGMAX: case DSGB_BASE_ARGMIN: case DSGB_BASE_AA_ARGMAX: {
            long long *d = (long long *)dst + 2 * i;
            const long long *q = (const long long *)src + 2 * i;
            const bool better = op != DSGB_BASE_ARGMIN ? pair_better<true>(q[0], q[1], d[0], d[1])
                                                       : pair_better<false>(q[0], q[1], d[0], d[1]);
            if (better) { d[0] = q[0]; d[1] = q[1]; }
            break;
        }
        default: break;
        }
    }
}

extern "C" int dsgb_combine(const dsgb_base *dst, const dsgb_base *src, int32_t nbases, int64_t ncells,
                            void *stream) {
    if ((nbases > 0 && (!dst || !src)) || nbases < 0 || ncells < 0) {
        set_error("dsgb_combine: bad arguments");
        return DSGB_E_INVALID;
    }
    cudaStream_t st = as_stream(stream);
    for (int b = 0; b < nbases; ++b) {
        const dsgb_base &D = dst[b], &S = src[b];
        if (D.op != S.op || D.ncat != S.ncat || !D.agg || !S.agg) {
            set_error("dsgb_combine: base %d differs between the partials", b);
            return DSGB_E_INVALID;
        }
        if (D.op < DSGB_BASE_COUNT || D.op > DSGB_BASE_AA_ARGMAX) {
            set_error("dsgb_combine: unknown base op %d", D.op);
            return DSGB_E_INVALID;
        }
        const int64_t n = ncells * (D.ncat > 0 ? D.ncat : 1);
        if (n == 0) continue;
        combine_kernel<<<grid_for(n), 256, 0, st>>>(D.op, D.agg, S.agg, n);
        DSGB_CHECK_LAUNCH("dsgb_combine");
    }
    return DSGB_OK;
}

extern "C" int dsgb_bases_init(const dsgb_base *bases, int32_t nbases, int64_t ncells, void *stream) {
    if ((nbases > 0 && !bases) || nbases < 0 || ncells < 0) { set_error("dsgb_bases_init: bad args"); return DSGB_E_INVALID; }
    return bases_init(bases, nbases, ncells, as_stream(stream));
}

extern "C" int dsgb_finalize(const dsgb_column *cols, int32_t ncols, int64_t row_offset,
                             const dsgb_base *bases, int32_t nbases,
                             const dsgb_output *outs, int32_t nouts, int64_t ncells, void *stream) {
    if ((nbases > 0 && !bases) || (nouts > 0 && !outs) || ncells < 0) { set_error("dsgb_finalize: bad args"); return DSGB_E_INVALID; }
    return finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, as_stream(stream));
}

extern "C" int dsgb_select_by_owner(const dsgb_base *row_base, int32_t nparts, const int64_t *part_first,
                                    const int64_t *part_rows, const double *const *part_vals, double *out,
                                    int64_t ncells, void *stream) {
    if (!row_base || !row_base->agg || !part_first || !part_rows || !part_vals || !out || ncells < 0 ||
        nparts < 1) {
        set_error("dsgb_select_by_owner: bad args");
        return DSGB_E_INVALID;
    }
    if (nparts > FIN_MAX_PARTS) {
        set_error("dsgb_select_by_owner: at most %d partitions", FIN_MAX_PARTS);
        return DSGB_E_UNSUPPORTED;
    }
    const int op = row_base->op;
    if (op != DSGB_BASE_MIN_ROW && op != DSGB_BASE_MAX_ROW && op != DSGB_BASE_ARGMAX && op != DSGB_BASE_ARGMIN &&
        op != DSGB_BASE_AA_ARGMAX) {
        set_error("dsgb_select_by_owner: base op %d carries no row", op);
        return DSGB_E_INVALID;
    }
    SelectParts g;
    memset(&g, 0, sizeof(g));
    g.nparts = nparts;
    g.b0op = op;
    g.b0 = row_base->agg;
    g.out = out;
    g.n = ncells * (row_base->ncat < 1 ? 1 : row_base->ncat);
    for (int p = 0; p < nparts; ++p) {
        if (!part_vals[p]) { set_error("dsgb_select_by_owner: partition %d values null", p); return DSGB_E_INVALID; }
        g.vals[p] = part_vals[p];
        g.first[p] = part_first[p];
        g.rows[p] = part_rows[p];
    }
    if (g.n > 0) select_owner_kernel<<<grid_for(g.n), 256, 0, as_stream(stream)>>>(g);
    DSGB_CHECK_LAUNCH("dsgb_select_by_owner");
    return DSGB_OK;
}

// dsgb_finalize for bases combined from row partitions: every output but the
// gathers as dsgb_finalize with partition 0's columns; a gather reads its row
// from the partition [first, first + rows) that holds it (NaN if none).
extern "C" int dsgb_finalize_partitioned(const dsgb_column *part_cols, int32_t ncols, int32_t nparts,
                                         const int64_t *part_first, const int64_t *part_rows,
                                         const dsgb_base *bases, int32_t nbases, const dsgb_output *outs,
                                         int32_t nouts, int64_t ncells, void *stream) {
    if ((nbases > 0 && !bases) || (nouts > 0 && !outs) || ncells < 0 || nparts < 1 || ncols < 0 ||
        (ncols > 0 && !part_cols) || !part_first || !part_rows) {
        set_error("dsgb_finalize_partitioned: bad args");
        return DSGB_E_INVALID;
    }
    if (nparts > FIN_MAX_PARTS) {
        set_error("dsgb_finalize_partitioned: at most %d partitions", FIN_MAX_PARTS);
        return DSGB_E_UNSUPPORTED;
    }
    cudaStream_t st = as_stream(stream);
    for (int o = 0; o < nouts; ++o) {
        const dsgb_output &O = outs[o];
        if (O.op != DSGB_FIN_GATHER) {
            const int rc = finalize_outputs(part_cols, ncols, part_first[0], bases, nbases, &O, 1, ncells, st);
            if (rc) return rc;
            continue;
        }
        if (!O.out || O.base0 < 0 || O.base0 >= nbases || O.col < 0 || O.col >= ncols) {
            set_error("dsgb_finalize_partitioned: output %d invalid", o);
            return DSGB_E_INVALID;
        }
        GatherParts g;
        memset(&g, 0, sizeof(g));
        g.nparts = nparts;
        g.b0op = bases[O.base0].op;
        g.b0 = bases[O.base0].agg;
        g.out = O.out;
        g.n = ncells * (bases[O.base0].ncat < 1 ? 1 : bases[O.base0].ncat);
        for (int p = 0; p < nparts; ++p) {
            const dsgb_column &c = part_cols[(int64_t)p * ncols + O.col];
            g.col[p] = ColumnRef{c.data, c.dtype};
            g.first[p] = part_first[p];
            g.rows[p] = part_rows[p];
        }
        if (g.n > 0) gather_parts_kernel<<<grid_for(g.n), 256, 0, st>>>(g);
        DSGB_CHECK_LAUNCH("dsgb_finalize_partitioned gather");
    }
    return DSGB_OK;
}

// The min/max travel as order-preserving uint64 in the first 16 bytes of
// out_minmax (used as scratch), then are decoded in place.
extern "C" int dsgb_bounds(const dsgb_column *col, int64_t n, double *out_minmax, void *stream) {
    if (!col || !out_minmax || n < 0 || dtype_size(col->dtype) == 0 || (n > 0 && !col->data)) {
        set_error("dsgb_bounds: bad args");
        return DSGB_E_INVALID;
    }
    cudaStream_t st = as_stream(stream);
    unsigned long long *mm = (unsigned long long *)out_minmax;
    bounds_init_kernel<<<1, 32, 0, st>>>(mm);
    ColumnRef c{col->data, col->dtype};
    if (n > 0) bounds_kernel<<<grid_for(n), 256, 0, st>>>(c, n, mm);
    bounds_finish_kernel<<<1, 32, 0, st>>>(mm, out_minmax);
    DSGB_CHECK_LAUNCH("dsgb_bounds");
    return DSGB_OK;
}
