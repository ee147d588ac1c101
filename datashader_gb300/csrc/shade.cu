// shade.cu -- tf.shade(how='linear' | 'log' | 'cbrt') of a 2-D aggregate.
//
// Restates datashader/transfer_functions/__init__.py:
//   _interpolate_lookup (220-223): linear = d, log = log1p(d), cbrt = d**(1/3)
//       on the unmasked values;
//   _interpolate (251-356): mask = data == 0 (uint) / isnan (float); with no
//       span, offset = min of the unmasked values and span = (min, max) of
//       the transformed values; with a span, the unmasked values are clipped
//       into it, offset = span[0] and span = f([0, span[1] - span[0]]);
//       list colormap: interp(data, linspace(span, ncolors), channel,
//       left=255), NaN -> 0, astype(uint8), alpha where not NaN; single colour:
//       r, g, b constant, alpha = interp(data, linspace(span, n_alpha),
//       arange(min_alpha, alpha + 1), left=0, right=255);
//       everything masked -> a zero image.
// uint32 aggregates subtract the offset in uint32 and transform in float64
// (numpy promotes with the NaN); float64 aggregates stay float64.  The
// transforms call CUDA's log1p and pow(x, 1/3), numpy the C library's: they
// can differ by an ulp, so log and cbrt colours can differ by one step
// where a value sits on a colour boundary; linear is bit-identical.
//
// Three launches: offset (min/max of the unmasked values), span of the
// transformed values, apply.
#include "dsgb_internal.cuh"
#include "shade_common.cuh"

#include <cmath>

namespace dsgb {

enum ShadeHow { SHADE_LINEAR = 0, SHADE_LOG = 1, SHADE_CBRT = 2 };

struct ShadeHeader {
    unsigned long long lo, hi;       // ordered min / max of the unmasked values (before the offset)
    unsigned long long tlo, thi;     // ordered min / max of the transformed values
    unsigned long long total;        // unmasked count
};

struct ShadeArgs {
    int how;
    int has_span;
    double span0, span1;
    int cmap_kind;                   // 0 = list of colours, 1 = single colour + alpha ramp
    int ncolors;                     // list: colours; single: alpha steps (alpha - min_alpha + 1)
    double r[256], g[256], b[256];   // list colours, float64 channels as given (a tuple may hold floats)
    int alpha, min_alpha;
    int sr, sg, sb;                  // single colour
};

template <typename T> __device__ __forceinline__ bool s_masked(T v);
template <> __device__ __forceinline__ bool s_masked<unsigned int>(unsigned int v) { return v == 0u; }
template <> __device__ __forceinline__ bool s_masked<double>(double v) { return v != v; }

template <typename T> __device__ __forceinline__ unsigned long long s_key(T v);
template <> __device__ __forceinline__ unsigned long long s_key<unsigned int>(unsigned int v) { return v; }
template <> __device__ __forceinline__ unsigned long long s_key<double>(double v) { return ord64(v); }

template <typename T> __device__ __forceinline__ T s_unkey(unsigned long long k);
template <> __device__ __forceinline__ unsigned int s_unkey<unsigned int>(unsigned long long k) { return (unsigned)k; }
template <> __device__ __forceinline__ double s_unkey<double>(unsigned long long k) { return unord64(k); }

__device__ __forceinline__ double s_transform(int how, double d) {
    if (how == SHADE_LOG) return log1p(d);
    if (how == SHADE_CBRT) return pow(d, 1.0 / 3.0);
    return d;
}

// The offset and the clipping of one unmasked value, in the data's type.
template <typename T>
__device__ __forceinline__ double s_value(const ShadeArgs &a, T v, T offset, T clo, T chi) {
    if (a.has_span) v = v < clo ? clo : (v > chi ? chi : v);
    if (sizeof(T) == 4) return (double)(unsigned)((unsigned)v - (unsigned)offset);
    return __dsub_rn((double)v, (double)offset);
}

__global__ void shade_init(ShadeHeader *h) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        h->lo = ~0ull; h->hi = 0ull; h->tlo = ~0ull; h->thi = 0ull; h->total = 0ull;
    }
}

template <typename T>
__global__ void shade_minmax(const T *data, int64_t n, ShadeHeader *h) {
    unsigned long long lo = ~0ull, hi = 0ull, cnt = 0;
    for (int64_t i = gtid(); i < n; i += gstride()) {
        const T v = data[i];
        if (s_masked<T>(v)) continue;
        const unsigned long long u = s_key<T>(v);
        lo = u < lo ? u : lo;
        hi = u > hi ? u : hi;
        ++cnt;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    if ((threadIdx.x & 31) == 0 && cnt) {
        atomicMin(&h->lo, lo);
        atomicMax(&h->hi, hi);
        atomicAdd(&h->total, cnt);
    }
}

template <typename T>
__device__ __forceinline__ void s_offsets(const ShadeArgs &a, const ShadeHeader &h, T &offset, T &clo, T &chi) {
    if (a.has_span) {
        if (sizeof(T) == 4) {
            // np.array(span, dtype=uint32)[0]; the clip bounds in the data's type
            offset = (T)(unsigned)(long long)a.span0;
            clo = (T)(unsigned)(long long)a.span0;
            chi = (T)(unsigned)(long long)a.span1;
        } else {
            offset = (T)a.span0; clo = (T)a.span0; chi = (T)a.span1;
        }
    } else {
        offset = s_unkey<T>(h.lo); clo = offset; chi = s_unkey<T>(h.hi);
    }
}

template <typename T>
__global__ void shade_span(const T *data, int64_t n, const __grid_constant__ ShadeArgs a, ShadeHeader *hp) {
    const ShadeHeader h = *hp;
    if (h.total == 0 || a.has_span) return;
    T offset, clo, chi;
    s_offsets<T>(a, h, offset, clo, chi);
    unsigned long long lo = ~0ull, hi = 0ull;
    for (int64_t i = gtid(); i < n; i += gstride()) {
        const T v = data[i];
        if (s_masked<T>(v)) continue;
        const double t = s_transform(a.how, s_value<T>(a, v, offset, clo, chi));
        if (t != t) continue;                          // nanmin / nanmax
        const unsigned long long u = ord64(t);
        lo = u < lo ? u : lo;
        hi = u > hi ? u : hi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    if ((threadIdx.x & 31) == 0 && lo != ~0ull) {
        atomicMin(&hp->tlo, lo);
        atomicMax(&hp->thi, hi);
    }
}

__device__ __forceinline__ uint32_t s_u8(double x) { return (uint32_t)(uint8_t)(int)x; }

template <typename T>
__global__ void __launch_bounds__(256) shade_apply(const T *data, int64_t n, const __grid_constant__ ShadeArgs a,
                                                   const ShadeHeader *hp, uint32_t *rgba) {
    const ShadeHeader h = *hp;
    if (h.total == 0) {                              // everything masked: a zero image
        for (int64_t i = gtid(); i < n; i += gstride()) rgba[i] = 0u;
        return;
    }
    T offset, clo, chi;
    s_offsets<T>(a, h, offset, clo, chi);
    double s0, s1;
    if (a.has_span) {
        // interpolater([0, span[1] - span[0]], 0), in float64
        s0 = s_transform(a.how, 0.0);
        s1 = s_transform(a.how, __dsub_rn(a.span1, a.span0));
    } else {
        s0 = unord64(h.tlo);
        s1 = unord64(h.thi);
    }
    // np.linspace(span, num), the alpha ramp and the colours, shared by the block
    __shared__ double xs[256], ramp[256], cr[256], cg[256], cb[256];
    const int m = a.ncolors < 256 ? a.ncolors : 256;
    {
        const int div = m - 1;
        const double delta = __dsub_rn(s1, s0);
        const double step = div > 0 ? __ddiv_rn(delta, (double)div) : 0.0;
        for (int k = threadIdx.x; k < m; k += blockDim.x) {
            double y;
            if (div > 0 && step == 0.0) y = __dmul_rn(__ddiv_rn((double)k, (double)div), delta);
            else y = __dmul_rn((double)k, step);
            xs[k] = (div > 0 && k == div) ? s1 : __dadd_rn(y, s0);
            ramp[k] = (double)(a.min_alpha + k);
            if (a.cmap_kind == 0) { cr[k] = a.r[k]; cg[k] = a.g[k]; cb[k] = a.b[k]; }
        }
    }
    __syncthreads();
    for (int64_t i = gtid(); i < n; i += gstride()) {
        const T v = data[i];
        double t = dnan();
        if (!s_masked<T>(v)) t = s_transform(a.how, s_value<T>(a, v, offset, clo, chi));
        uint32_t px;
        if (a.cmap_kind == 0) {
            px = 0u;
            if (t == t) {
                const double r = np_interp(t, xs, cr, m, 255.0, cr[m - 1]);
                const double g = np_interp(t, xs, cg, m, 255.0, cg[m - 1]);
                const double b = np_interp(t, xs, cb, m, 255.0, cb[m - 1]);
                px = s_u8(r) | (s_u8(g) << 8) | (s_u8(b) << 16) | ((uint32_t)(uint8_t)a.alpha << 24);
            }
        } else {
            // alpha ramp: interp(data, span, arange(min_alpha, alpha + 1), left=0, right=255),
            // NaN -> 0 (numpy's nan_to_num)
            const double al = t == t ? np_interp(t, xs, ramp, m, 0.0, 255.0) : 0.0;
            px = (uint32_t)(uint8_t)a.sr | ((uint32_t)(uint8_t)a.sg << 8) | ((uint32_t)(uint8_t)a.sb << 16) |
                 (s_u8(al) << 24);
        }
        rgba[i] = px;
    }
}

static unsigned s_grid(int64_t n) {
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    int64_t g = (n + 255) / 256;
    if (g > (int64_t)sms * 8) g = (int64_t)sms * 8;
    return (unsigned)(g < 1 ? 1 : g);
}

template <typename T>
static int shade_impl(const T *data, int64_t n, int32_t how, const double *span, const double *cmap_rgb,
                      int32_t ncolors, const uint8_t *single_rgb, int32_t alpha, int32_t min_alpha, uint32_t *rgba,
                      void *ws, size_t ws_bytes, void *stream) {
    if (n < 0 || (n > 0 && (!data || !rgba)) || how < 0 || how > 2 || alpha < 0 || alpha > 255 || min_alpha < 0 ||
        min_alpha > alpha) {
        set_error("dsgb_shade: invalid arguments");
        return DSGB_E_INVALID;
    }
    if (!ws || ws_bytes < sizeof(ShadeHeader) || ((uintptr_t)ws & 255u)) {
        set_error("dsgb_shade: workspace must be 256-byte aligned and at least %zu bytes", sizeof(ShadeHeader));
        return DSGB_E_NOSPACE;
    }
    ShadeArgs a;
    memset(&a, 0, sizeof(a));
    a.how = how;
    a.alpha = alpha;
    a.min_alpha = min_alpha;
    if (span) {
        a.has_span = 1;
        a.span0 = span[0];
        a.span1 = span[1];
    }
    if (single_rgb) {
        a.cmap_kind = 1;
        a.sr = single_rgb[0]; a.sg = single_rgb[1]; a.sb = single_rgb[2];
        a.ncolors = alpha - min_alpha + 1;
    } else {
        if (!cmap_rgb || ncolors < 1 || ncolors > 256) {
            set_error("dsgb_shade: a list colormap has 1..256 colours");
            return DSGB_E_INVALID;
        }
        a.ncolors = ncolors;
        for (int k = 0; k < ncolors; ++k) {
            a.r[k] = cmap_rgb[3 * k]; a.g[k] = cmap_rgb[3 * k + 1]; a.b[k] = cmap_rgb[3 * k + 2];
        }
    }
    cudaStream_t st = as_stream(stream);
    ShadeHeader *h = (ShadeHeader *)ws;
    shade_init<<<1, 32, 0, st>>>(h);
    if (n > 0) {
        shade_minmax<T><<<s_grid(n), 256, 0, st>>>(data, n, h);
        shade_span<T><<<s_grid(n), 256, 0, st>>>(data, n, a, h);
        shade_apply<T><<<s_grid(n), 256, 0, st>>>(data, n, a, h, rgba);
    }
    DSGB_CHECK_LAUNCH("dsgb_shade");
    return DSGB_OK;
}

// ---- compositing (datashader/composite.py:31-127): uint32 RGBA pixels,
// components as float64 byte / 255, recombined by truncating component * 255
// and capping at 255; an alpha of 0 gives the pixel 0.  Every float64
// operation is an explicit round-to-nearest intrinsic in the reference's
// order (numba emits no FMA), so results are bit-identical.
enum CompOp { COMP_SOURCE = 0, COMP_OVER = 1, COMP_ADD = 2, COMP_SATURATE = 3 };

__device__ __forceinline__ double comp_scaled(uint32_t x, int shift) {
    return __ddiv_rn((double)((x >> shift) & 255u), 255.0);
}
__device__ __forceinline__ uint32_t comp_byte(double c) {
    const uint32_t u = __double2uint_rz(__dmul_rn(c, 255.0));
    return u < 255u ? u : 255u;
}

__device__ __forceinline__ uint32_t composite_px(uint32_t src, uint32_t dst, int op) {
    if (op == COMP_SOURCE) return (src & 0xff000000u) ? src : dst;
    const double sr = comp_scaled(src, 0), sg = comp_scaled(src, 8), sb = comp_scaled(src, 16),
                 sa = comp_scaled(src, 24);
    const double dr = comp_scaled(dst, 0), dg = comp_scaled(dst, 8), db = comp_scaled(dst, 16),
                 da = comp_scaled(dst, 24);
    double a, r, g, b;
    if (op == COMP_OVER) {
        const double factor = __dsub_rn(1.0, sa);
        a = __dadd_rn(sa, __dmul_rn(da, factor));
        if (a == 0.0) return 0u;
        r = __ddiv_rn(__dadd_rn(__dmul_rn(sr, sa), __dmul_rn(__dmul_rn(dr, da), factor)), a);
        g = __ddiv_rn(__dadd_rn(__dmul_rn(sg, sa), __dmul_rn(__dmul_rn(dg, da), factor)), a);
        b = __ddiv_rn(__dadd_rn(__dmul_rn(sb, sa), __dmul_rn(__dmul_rn(db, da), factor)), a);
    } else {
        const double sum = __dadd_rn(sa, da);
        a = sum < 1.0 ? sum : 1.0;
        if (a == 0.0) return 0u;
        if (op == COMP_ADD) {
            r = __ddiv_rn(__dadd_rn(__dmul_rn(sr, sa), __dmul_rn(dr, da)), a);
            g = __ddiv_rn(__dadd_rn(__dmul_rn(sg, sa), __dmul_rn(dg, da)), a);
            b = __ddiv_rn(__dadd_rn(__dmul_rn(sb, sa), __dmul_rn(db, da)), a);
        } else {
            const double rest = __dsub_rn(1.0, da);
            const double factor = sa < rest ? sa : rest;
            r = __ddiv_rn(__dadd_rn(__dmul_rn(factor, sr), __dmul_rn(dr, da)), a);
            g = __ddiv_rn(__dadd_rn(__dmul_rn(factor, sg), __dmul_rn(dg, da)), a);
            b = __ddiv_rn(__dadd_rn(__dmul_rn(factor, sb), __dmul_rn(db, da)), a);
        }
    }
    return (comp_byte(a) << 24) | (comp_byte(b) << 16) | (comp_byte(g) << 8) | comp_byte(r);
}

// Four pixels a thread when the buffers are 16-byte aligned (uint4 loads and stores).
__global__ void __launch_bounds__(256) composite_kernel(const uint32_t *src, const uint32_t *dst, uint32_t dst_value,
                                                        uint32_t *out, int64_t n, int op, int vec) {
    if (vec) {
        const int64_t n4 = n >> 2;
        for (int64_t i = gtid(); i < n4; i += gstride()) {
            const uint4 s = ((const uint4 *)src)[i];
            const uint4 d = dst ? ((const uint4 *)dst)[i] : make_uint4(dst_value, dst_value, dst_value, dst_value);
            ((uint4 *)out)[i] = make_uint4(composite_px(s.x, d.x, op), composite_px(s.y, d.y, op),
                                           composite_px(s.z, d.z, op), composite_px(s.w, d.w, op));
        }
        for (int64_t i = 4 * n4 + gtid(); i < n; i += gstride())
            out[i] = composite_px(src[i], dst ? dst[i] : dst_value, op);
        return;
    }
    for (int64_t i = gtid(); i < n; i += gstride()) out[i] = composite_px(src[i], dst ? dst[i] : dst_value, op);
}

}  // namespace dsgb

using namespace dsgb;

extern "C" int dsgb_composite(const uint32_t *src, const uint32_t *dst, uint32_t dst_value, int64_t n, int32_t op,
                              uint32_t *out, void *stream) {
    if (n < 0 || (n > 0 && (!src || !out)) || op < COMP_SOURCE || op > COMP_SATURATE) {
        set_error("dsgb_composite: invalid arguments");
        return DSGB_E_INVALID;
    }
    if (n == 0) return DSGB_OK;
    const int vec = ((((uintptr_t)src | (uintptr_t)dst | (uintptr_t)out) & 15u) == 0);
    composite_kernel<<<grid_of(n), 256, 0, as_stream(stream)>>>(src, dst, dst_value, out, n, op, vec);
    DSGB_CHECK_LAUNCH("dsgb_composite");
    return DSGB_OK;
}

extern "C" size_t dsgb_shade_workspace_size(void) { return 256; }

extern "C" int dsgb_shade_u32(const uint32_t *data, int64_t n, int32_t how, const double *span,
                              const double *cmap_rgb, int32_t ncolors, const uint8_t *single_rgb, int32_t alpha,
                              int32_t min_alpha, uint32_t *rgba, void *workspace, size_t workspace_bytes,
                              void *stream) {
    return shade_impl<unsigned int>((const unsigned int *)data, n, how, span, cmap_rgb, ncolors, single_rgb, alpha,
                                    min_alpha, rgba, workspace, workspace_bytes, stream);
}

extern "C" int dsgb_shade_f64(const double *data, int64_t n, int32_t how, const double *span,
                              const double *cmap_rgb, int32_t ncolors, const uint8_t *single_rgb, int32_t alpha,
                              int32_t min_alpha, uint32_t *rgba, void *workspace, size_t workspace_bytes,
                              void *stream) {
    return shade_impl<double>(data, n, how, span, cmap_rgb, ncolors, single_rgb, alpha, min_alpha, rgba, workspace,
                              workspace_bytes, stream);
}
