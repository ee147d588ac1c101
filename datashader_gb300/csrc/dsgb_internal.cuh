// dsgb_internal.cuh -- shared device/host helpers of libdsgb (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "../../include/dsgb.h"

namespace dsgb {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *what);
int sm_count();

#define DSGB_CHECK_LAUNCH(what)                                   \
    do {                                                          \
        cudaError_t _e = cudaGetLastError();                      \
        if (_e != cudaSuccess) return ::dsgb::cuda_status(_e, what); \
    } while (0)

static inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// An NVTX range over one host-side stage of an entry point (plan, launch,
// finalize); free when no profiler is attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Blocks of 256 threads for a grid-stride loop over n items (at most 16 per SM).
static inline unsigned grid_of(int64_t n) {
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    int64_t g = (n + 255) / 256;
    if (g > (int64_t)sms * 16) g = (int64_t)sms * 16;
    if (g < 1) g = 1;
    return (unsigned)g;
}

static inline int dtype_size(int32_t dt) {
    switch (dt) {
    case DSGB_F32: case DSGB_I32: case DSGB_U32: return 4;
    case DSGB_F64: case DSGB_I64: return 8;
    case DSGB_I8: case DSGB_U8: case DSGB_BOOL: return 1;
    case DSGB_I16: return 2;
    default: return 0;
    }
}

// ------------------------------------------------------- device status
// Kernels never trap: a condition that a correct input cannot produce (a CAS
// retry loop that reached its iteration guard, an aggregate index outside
// its base in debug mode) sets a bit in a device status word, which
// dsgb_device_status reads.  Each translation unit is its own device module
// and keeps its own word (a static __device__ variable); the units that can
// raise a bit expose it through DSGB_STATUS_READER.
static __device__ unsigned g_unit_status;
__device__ __forceinline__ void raise_status(unsigned bits) { atomicOr(&g_unit_status, bits); }

static inline int unit_status_take(unsigned *bits, bool clear) {
    unsigned v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_unit_status, sizeof(v));
    if (e == cudaSuccess && clear && v) {
        const unsigned zero = 0;
        e = cudaMemcpyToSymbol(g_unit_status, &zero, sizeof(zero));
    }
    if (e != cudaSuccess) return cuda_status(e, "device status word");
    *bits |= v;
    return DSGB_OK;
}
#define DSGB_STATUS_READER(name) \
    int name(unsigned *bits, bool clear) { return unit_status_take(bits, clear); }

// ------------------------------------------------------- device helpers
constexpr int MAX_BASES = 16;
constexpr int MAX_COLS = 16;

struct ColumnRef {
    const void *data;
    int32_t dtype;
};

struct BaseDev {
    int32_t op, col, cat_col, ncat, flags;
    void *agg;
};

// Work order of the antialiased LineAxis0 segments (line.cu): segment
// indices counting-sorted by an estimate of their pixel work, so that the
// lanes of a warp draw segments of similar size.  Shared by the forward and
// the adjoint.  Returns the order (n - 1 entries inside the workspace) or
// null when the workspace is missing or too small (callers then draw in
// row order).
struct LineWorkArgs {
    ColumnRef X, Y;
    int64_t n;
    double sx, sy, line_width;
};
size_t line_work_order_bytes(int64_t n);
const unsigned *build_line_work_order(const LineWorkArgs &a, void *workspace, size_t ws_bytes, cudaStream_t st);

// Load element i of a column as float64 (the promotion numba applies when a
// column meets a float64 scale or aggregate).  Integers never read as NaN.
__device__ __forceinline__ double load_f64(const ColumnRef &c, int64_t i) {
    switch (c.dtype) {
    case DSGB_F32: return (double)__ldg((const float *)c.data + i);
    case DSGB_F64: return __ldg((const double *)c.data + i);
    case DSGB_I8: return (double)((const int8_t *)c.data)[i];
    case DSGB_U8: case DSGB_BOOL: return (double)((const uint8_t *)c.data)[i];
    case DSGB_I16: return (double)((const int16_t *)c.data)[i];
    case DSGB_I32: return (double)__ldg((const int32_t *)c.data + i);
    case DSGB_I64: return (double)__ldg((const long long *)c.data + i);
    case DSGB_U32: return (double)__ldg((const unsigned int *)c.data + i);
    default: return __longlong_as_double(0x7ff8000000000000ll);
    }
}

__device__ __forceinline__ int64_t load_i64(const ColumnRef &c, int64_t i) {
    switch (c.dtype) {
    case DSGB_I8: return ((const int8_t *)c.data)[i];
    case DSGB_U8: case DSGB_BOOL: return ((const uint8_t *)c.data)[i];
    case DSGB_I16: return ((const int16_t *)c.data)[i];
    case DSGB_I32: return __ldg((const int32_t *)c.data + i);
    case DSGB_I64: return __ldg((const long long *)c.data + i);
    case DSGB_U32: return __ldg((const unsigned int *)c.data + i);
    case DSGB_F32: return (int64_t)__ldg((const float *)c.data + i);
    case DSGB_F64: return (int64_t)__ldg((const double *)c.data + i);
    default: return 0;
    }
}

// utils.py:598-603 -- isnull(v) = not (v <= 0 or v > 0), true exactly for
// NaN.  Tested on the bit pattern (exponent all ones, mantissa non-zero):
// integer ALU work instead of two float64 compares, which GB300 issues at a
// small fraction of its integer rate.
__device__ __forceinline__ bool isnull(double v) {
    return ((unsigned long long)__double_as_longlong(v) << 1) > 0xffe0000000000000ull;
}

// Order-preserving int64 image of a non-NaN double: key(a) < key(b) <=> a < b,
// except that -0.0 orders just below +0.0.
__host__ __device__ __forceinline__ long long f64_key(double v) {
#ifdef __CUDA_ARCH__
    long long b = __double_as_longlong(v);
#else
    long long b; memcpy(&b, &v, 8);
#endif
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}
__host__ __device__ __forceinline__ double key_f64(long long k) {
    long long b = k >= 0 ? k : (k ^ 0x7fffffffffffffffll);
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double v; memcpy(&v, &b, 8); return v;
#endif
}
constexpr long long KEY_EMPTY_MAX = (long long)0x8000000000000000ull;  // below every key
constexpr long long KEY_EMPTY_MIN = 0x7fffffffffffffffll;              // above every key
constexpr long long ROW_EMPTY_MIN = 0x7fffffffffffffffll;

// 128-bit compare-and-swap on a {key, row} pair (sm_90+ atom.cas.b128).
__device__ __forceinline__ void cas128(long long *addr, long long cmp_lo, long long cmp_hi,
                                       long long new_lo, long long new_hi,
                                       long long &old_lo, long long &old_hi) {
    asm volatile(
        "{\n\t.reg .b128 d, c, n;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 n, {%4, %5};\n\t"
        "atom.global.cas.b128 d, [%6], c, n;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(old_lo), "=l"(old_hi)
        : "l"(cmp_lo), "l"(cmp_hi), "l"(new_lo), "l"(new_hi), "l"(addr)
        : "memory");
}

// {key,row} "better" order: larger key wins (argmax) / smaller key wins
// (argmin); equal keys keep the smaller row (the first row in row order).
template <bool MAX>
__device__ __forceinline__ bool pair_better(long long k, long long r, long long ok, long long orow) {
    if (MAX) return k > ok || (k == ok && r < orow);
    return k < ok || (k == ok && r < orow);
}

template <bool MAX>
__device__ __forceinline__ void pair_update(long long *slot, long long key, long long row) {
    // Pre-check on the key word alone: keys only improve, so a key read that
    // is strictly better than ours proves that the slot is better.  The two
    // words are not read as one atomic unit, so every other decision is taken
    // on a pair that a 128-bit CAS returned atomically.
    volatile long long *v = slot;
    long long ok = v[0];
    if (MAX ? (ok > key) : (ok < key)) return;
    long long orow = v[1];
    // Each failed CAS observes a strictly better pair written by another
    // thread; improvements are bounded by the rows landing on this slot, so
    // the loop ends.  The iteration limit is a guard, not a wait: reaching it
    // leaves this row's update undone and raises DSGB_STATUS_CAS_GUARD.
    for (int guard = 0; guard < (1 << 24); ++guard) {
        long long rk, rr;
        if (!pair_better<MAX>(key, row, ok, orow)) {
            // confirm the snapshot atomically (writes back the same pair)
            cas128(slot, ok, orow, ok, orow, rk, rr);
            if (rk == ok && rr == orow) return;
        } else {
            cas128(slot, ok, orow, key, row, rk, rr);
            if (rk == ok && rr == orow) return;
        }
        ok = rk; orow = rr;
    }
    raise_status(DSGB_STATUS_CAS_GUARD);
}

__device__ __forceinline__ void atomic_max_key(long long *slot, long long key) {
    if (*(volatile long long *)slot < key) atomicMax(slot, key);
}
__device__ __forceinline__ void atomic_min_key(long long *slot, long long key) {
    if (*(volatile long long *)slot > key) atomicMin(slot, key);
}

// Exact float32 -> float64 widening with integer operations only.  GB300
// runs the float conversion instruction on its narrow float64 pipe; this
// form keeps bulk conversions on the integer ALU.  A normal float keeps its
// sign and mantissa (shifted up by 29 bits) and its exponent is rebiased by
// 1023 - 127 = 896; zero, subnormals (normalised by their leading bit),
// infinities and NaNs take the rare branch.
__device__ __forceinline__ double f32_to_f64_exact(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu, m = b & 0x7fffffu, sign = b & 0x80000000u;
    unsigned hi, lo;
    if (e - 1u < 254u) {                       // normal: 1 <= e <= 254
        hi = sign | (((b & 0x7fffffffu) >> 3) + (896u << 20));
        lo = b << 29;
    } else if (e == 0xffu) {                   // inf / NaN: exponent all ones, payload shifted
        hi = sign | 0x7ff00000u | (m >> 3);
        lo = m << 29;
    } else if (m == 0u) {                      // +-0
        hi = sign;
        lo = 0u;
    } else {                                   // subnormal: m * 2^-149, leading bit at p
        const int p = 31 - __clz((int)m);
        const unsigned long long frac = ((unsigned long long)m << (52 - p)) & 0xfffffffffffffull;
        hi = sign | ((unsigned)(p - 149 + 1023) << 20) | (unsigned)(frac >> 32);
        lo = (unsigned)frac;
    }
    return __hiloint2double((int)hi, (int)lo);
}

// Grid-stride helpers.
__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t gstride() { return (int64_t)gridDim.x * blockDim.x; }

}  // namespace dsgb
