// eq_hist.cu -- histogram equalisation (tf.shade(how='eq_hist')) on GB300.
//
// Restates datashader/transfer_functions/__init__.py:
//   _interpolate prologue (251-297): mask = data == 0 (uint) / isnan (float),
//       offset = min of the unmasked values, data -= offset;
//   eq_hist (148-223): integer data with ptp < nbins -> exact per-value
//       counts over [vmin, vmax]; otherwise numpy.histogram(data, nbins)
//       with empty bins dropped; cdf = cumsum / total; np.interp(data,
//       bin_centers, cdf); masked -> NaN; discrete_levels = #non-empty bins;
//   span / _rescale_discrete_levels (299-316, 234-248) and the list-colormap
//       RGBA branch (317-351).
//
// numpy.histogram's bin assignment (numpy/lib/_histograms_impl.py: estimate
// from (x - first) / (last - first) * nbins, then correct against the
// linspace edges) and numpy.linspace's edges (i*step + start, last = stop)
// are reproduced exactly, so the histogram is bit-identical.
//
// Four launches: min/max, histogram (shared-memory privatised low bins),
// one-block scan (cdf, levels, span), apply (cdf lookup / interp + RGBA).
#include <cuda.h>
#include <cudaTypedefs.h>

#include "dsgb_internal.cuh"
#include "shade_common.cuh"

#include <cmath>
#include <mutex>

namespace dsgb {

struct EqHeader {
    unsigned long long lo, hi;     // ordered min / max of the unmasked values
    unsigned long long total;      // unmasked count
    long long levels;
    int32_t path;                  // 0 = no data, 1 = integer counts, 2 = binned
    int32_t nkept;                 // float path: non-empty bins
    double first, last, step;      // float path: outer edges and linspace step
    double span0, span1;           // colormap span
    double offset;                 // offset (float data)
    double dmax;                   // largest unmasked value after the offset
    unsigned int uoffset;          // offset (uint32 data)
    unsigned int ptp;
    double cdf_total;              // integer path: the divisor of the cumulative counts
};

constexpr int SMEM_BINS = 8192;
constexpr size_t HDR_BYTES = 256;
static_assert(sizeof(EqHeader) <= HDR_BYTES, "header");

struct EqLayout {
    EqHeader *hdr;
    unsigned int *hist;   // nbins
    double *cdf;          // nbins
    double *centers;      // nbins (float path, compacted)
};

static size_t ws_bytes(int nbins) {
    return HDR_BYTES + (size_t)nbins * (4 + 8 + 8) + 64;
}

static EqLayout layout(void *ws, int nbins) {
    char *b = (char *)ws;
    EqLayout L;
    L.hdr = (EqHeader *)b;
    L.hist = (unsigned int *)(b + HDR_BYTES);
    size_t off = HDR_BYTES + (((size_t)nbins * 4 + 15) & ~(size_t)15);
    L.cdf = (double *)(b + off);
    L.centers = (double *)(b + off + (size_t)nbins * 8);
    return L;
}



template <typename T> __device__ __forceinline__ bool masked(T v);
template <> __device__ __forceinline__ bool masked<unsigned int>(unsigned int v) { return v == 0u; }
template <> __device__ __forceinline__ bool masked<double>(double v) { return v != v; }

__global__ void eqh_init(EqHeader *h) {
    if (threadIdx.x == 0) {
        memset(h, 0, sizeof(EqHeader));
        h->lo = ~0ull;
        h->hi = 0ull;
    }
}

template <typename T>
__global__ void eqh_minmax(const T *data, int64_t n, EqHeader *h) {
    unsigned long long lo = ~0ull, hi = 0ull, cnt = 0;
    for (int64_t i = gtid(); i < n; i += gstride()) {
        T v = data[i];
        if (masked<T>(v)) continue;
        unsigned long long u = sizeof(T) == 4 ? (unsigned long long)v : ord64((double)v);
        lo = u < lo ? u : lo;
        hi = u > hi ? u : hi;
        ++cnt;
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o);
        unsigned long long h2 = __shfl_xor_sync(0xffffffffu, hi, o);
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

// numpy.linspace(first, last, nbins+1)[j] (function_base.py: i*step + start,
// the endpoint set to stop; a zero step falls back to i/div*delta).
__device__ __forceinline__ double lin_edge(const EqHeader &h, int j, int nbins) {
    if (j >= nbins) return h.last;
    if (h.step == 0.0) return __dadd_rn(__dmul_rn(__ddiv_rn((double)j, (double)nbins), h.last - h.first), h.first);
    return __dadd_rn(__dmul_rn((double)j, h.step), h.first);
}

// numpy.histogram uniform-bin index of x (within [first, last]).
__device__ __forceinline__ int np_hist_index(const EqHeader &h, double x, int nbins) {
    double denom = __dsub_rn(h.last, h.first);
    double f = __dmul_rn(__ddiv_rn(__dsub_rn(x, h.first), denom), (double)nbins);
    long long idx = (long long)f;
    if (idx == nbins) idx -= 1;
    if (idx < 0) idx = 0;
    if (idx > nbins - 1) idx = nbins - 1;
    if (x < lin_edge(h, (int)idx, nbins)) idx -= 1;
    if (idx < 0) idx = 0;
    if (idx != nbins - 1 && x >= lin_edge(h, (int)idx + 1, nbins)) idx += 1;
    return (int)idx;
}

// Decide the path and the float-path edges (one thread).
template <typename T>
__global__ void eqh_plan(EqHeader *h, int nbins) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (h->total == 0) { h->path = 0; return; }
    if (sizeof(T) == 4) {
        unsigned int lo = (unsigned int)h->lo, hi = (unsigned int)h->hi;
        h->uoffset = lo;
        h->ptp = hi - lo;
        if ((long long)(hi - lo) < (long long)nbins) { h->path = 1; return; }
        // binned path on uint32: edges over [0, ptp] in float64
        h->first = 0.0;
        h->last = (double)(hi - lo);
        h->dmax = h->last;
    } else {
        double lo = unord64(h->lo), hi = unord64(h->hi);
        h->offset = lo;
        // data -= offset happens elementwise: the extremes become these
        h->first = __dsub_rn(lo, lo);
        h->last = __dsub_rn(hi, lo);
        h->dmax = h->last;
    }
    if (h->first == h->last) { h->first = h->first - 0.5; h->last = h->last + 0.5; }
    h->step = __ddiv_rn(__dsub_rn(h->last, h->first), (double)nbins);
    h->path = 2;
}

template <typename T>
__device__ __forceinline__ double shifted(const EqHeader &h, T v) {
    if (sizeof(T) == 4) return (double)(unsigned int)((unsigned int)v - h.uoffset);
    return __dsub_rn((double)v, h.offset);
}

template <typename T>
__global__ void __launch_bounds__(512) eqh_hist(const T *data, int64_t n, const EqHeader *hp,
                                                unsigned int *hist, int nbins) {
    __shared__ unsigned int sh[SMEM_BINS];
    const EqHeader h = *hp;
    if (h.path == 0) return;
    for (int j = threadIdx.x; j < SMEM_BINS; j += blockDim.x) sh[j] = 0;
    __syncthreads();
    for (int64_t i = gtid(); i < n; i += gstride()) {
        T v = data[i];
        if (masked<T>(v)) continue;
        int bin;
        if (h.path == 1) bin = (int)((unsigned int)v - h.uoffset);
        else bin = np_hist_index(h, shifted<T>(h, v), nbins);
        if (bin < SMEM_BINS) atomicAdd(&sh[bin], 1u);
        else atomicAdd(&hist[bin], 1u);
    }
    __syncthreads();
    const int lim = nbins < SMEM_BINS ? nbins : SMEM_BINS;
    for (int j = threadIdx.x; j < lim; j += blockDim.x)
        if (sh[j]) atomicAdd(&hist[j], sh[j]);
}

// One block: cumulative sums, cdf, levels, the float-path compaction and the span.
__global__ void __launch_bounds__(1024) eqh_scan(EqHeader *hp, const unsigned int *hist, double *cdf,
                                                 double *centers, int nbins, int rescale) {
    __shared__ unsigned long long wsum[32];
    __shared__ int wkept[32];
    EqHeader &h = *hp;
    if (h.path == 0) return;
    const int path = h.path;
    const int nb = path == 1 ? (int)h.ptp + 1 : nbins;
    const int per = (nb + blockDim.x - 1) / blockDim.x;
    const int j0 = threadIdx.x * per;
    const int j1 = min(nb, j0 + per);
    unsigned long long s = 0;
    int kept = 0;
    for (int j = j0; j < j1; ++j) { s += hist[j]; kept += hist[j] != 0; }
    // block exclusive scan of (s, kept)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long xs = s;
    int xk = kept;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long t = __shfl_up_sync(0xffffffffu, xs, o);
        int tk = __shfl_up_sync(0xffffffffu, xk, o);
        if (lane >= o) { xs += t; xk += tk; }
    }
    if (lane == 31) { wsum[warp] = xs; wkept[warp] = xk; }
    __syncthreads();
    if (warp == 0) {
        unsigned long long a = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
        int ak = lane < (int)(blockDim.x >> 5) ? wkept[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long t = __shfl_up_sync(0xffffffffu, a, o);
            int tk = __shfl_up_sync(0xffffffffu, ak, o);
            if (lane >= o) { a += t; ak += tk; }
        }
        wsum[lane] = a;
        wkept[lane] = ak;
    }
    __syncthreads();
    unsigned long long run = xs - s + (warp > 0 ? wsum[warp - 1] : 0);
    int krun = xk - kept + (warp > 0 ? wkept[warp - 1] : 0);
    const unsigned long long total = wsum[31];
    const int nkept = wkept[31];
    const double ftotal = (double)total;
    for (int j = j0; j < j1; ++j) {
        unsigned int c = hist[j];
        run += c;
        if (path == 1) {
            cdf[j] = (double)run;                             // divided by eqh_div (:200-201)
        } else if (c) {
            cdf[krun] = __ddiv_rn((double)run, ftotal);
            double e0 = lin_edge(h, j, nbins), e1 = lin_edge(h, j + 1, nbins);
            centers[krun] = __ddiv_rn(__dadd_rn(e0, e1), 2.0);  // (:194)
            ++krun;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        h.levels = (long long)nkept;
        h.nkept = nkept;
        // span = (min, max) of the equalised unmasked values: the output is
        // monotone in the value, so they are the images of the extremes.
        double s0, s1;
        if (path == 1) {
            h.cdf_total = ftotal;
            s0 = __ddiv_rn(cdf[0], ftotal);
            s1 = __ddiv_rn(cdf[h.ptp], ftotal);
        } else {
            // the shifted extremes of the unmasked data are 0 and dmax
            s0 = np_interp(0.0, centers, cdf, nkept, cdf[0], cdf[nkept - 1]);
            s1 = np_interp(h.dmax, centers, cdf, nkept, cdf[0], cdf[nkept - 1]);
        }
        if (rescale) {
            // _rescale_discrete_levels (:234-248)
            double m = __ddiv_rn(-0.5, 98.0);
            double c = __dsub_rn(1.5, __dmul_rn(2.0, m));
            double multiple = __dadd_rn(__dmul_rn(m, (double)h.levels), c);
            if (multiple > 1) {
                double lower = __dsub_rn(s1, __dmul_rn(multiple, __dsub_rn(s1, s0)));
                s0 = lower > 0 ? lower : 0;
                s1 = 1;
            }
        }
        h.span0 = s0;
        h.span1 = s1;
    }
}

// Integer path: cdf = cumsum / cumsum[-1] (:200-201), one correctly rounded
// division per bin, spread over the GPU (a float64 division is dozens of
// operations on GB300's float64 pipe; one CTA took ~50 us for 20,000 bins).
__global__ void eqh_div(const EqHeader *hp, double *cdf) {
    const EqHeader &h = *hp;
    if (h.path != 1) return;
    const int64_t nb = (int64_t)h.ptp + 1;
    const double t = h.cdf_total;
    for (int64_t j = gtid(); j < nb; j += gstride()) cdf[j] = __ddiv_rn(cdf[j], t);
}

struct Cmap {
    double r[256], g[256], b[256];   // float64 channels as given (a tuple may hold floats)
    int n;
    int alpha;
};

// np.interp of one x against the three colour channels: one interval search
// and, per channel, numpy's slope (fp[j+1] - fp[j]) / (xp[j+1] - xp[j])
// (compiled_base.c arr_interp, which also precomputes the slopes when the
// table is not longer than x) taken from a per-block table, then
// slope * (x - xp[j]) + fp[j] with numpy's NaN fallbacks: the same operations
// in the same order as np_interp per channel.
__device__ __forceinline__ void np_interp_rgb(double x, const double *xp, const double (*fp)[256],
                                              const double (*sl)[256], int len, double left, double out[3]) {
    if (x > xp[len - 1]) {
        for (int c = 0; c < 3; ++c) out[c] = fp[c][len - 1];
        return;
    }
    if (x < xp[0]) {
        for (int c = 0; c < 3; ++c) out[c] = left;
        return;
    }
    int lo = 0, hi = len - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (xp[mid] <= x) lo = mid; else hi = mid;
    }
    int j = lo;
    if (x >= xp[len - 1]) j = len - 1;
    if (j == len - 1 || xp[j] == x) {
        for (int c = 0; c < 3; ++c) out[c] = fp[c][j];
        return;
    }
    const double dx = __dsub_rn(x, xp[j]);
    for (int c = 0; c < 3; ++c) {
        const double slope = sl[c][j];
        double r = __dadd_rn(__dmul_rn(slope, dx), fp[c][j]);
        if (r != r) {
            r = __dadd_rn(__dmul_rn(slope, __dsub_rn(x, xp[j + 1])), fp[c][j + 1]);
            if (r != r && fp[c][j] == fp[c][j + 1]) r = fp[c][j];
        }
        out[c] = r;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) eqh_apply(const T *data, int64_t n, const EqHeader *hp,
                                                 const double *cdf, const double *centers, double *out,
                                                 uint32_t *rgba, const __grid_constant__ Cmap cm, int nbins) {
    const EqHeader h = *hp;
    // np.linspace(span0, span1, ncolors) (:320), the colours and their slopes, shared by the block
    __shared__ double xs[256], ch[3][256], sl[3][256];
    if (rgba) {
        const int div = cm.n - 1;
        const double delta = __dsub_rn(h.span1, h.span0);
        const double step = div > 0 ? __ddiv_rn(delta, (double)div) : 0.0;
        for (int k = threadIdx.x; k < cm.n; k += blockDim.x) {
            double y;
            if (div > 0 && step == 0.0) y = __dmul_rn(__ddiv_rn((double)k, (double)div), delta);
            else y = __dmul_rn((double)k, step);
            xs[k] = (div > 0 && k == div) ? h.span1 : __dadd_rn(y, h.span0);
            ch[0][k] = cm.r[k]; ch[1][k] = cm.g[k]; ch[2][k] = cm.b[k];
        }
        __syncthreads();
        for (int k = threadIdx.x; k < 3 * (cm.n - 1); k += blockDim.x) {
            const int c = k / (cm.n - 1), j = k % (cm.n - 1);
            sl[c][j] = __ddiv_rn(__dsub_rn(ch[c][j + 1], ch[c][j]), __dsub_rn(xs[j + 1], xs[j]));
        }
    }
    __syncthreads();
    for (int64_t i = gtid(); i < n; i += gstride()) {
        T v = data[i];
        double o;
        if (h.path == 0 || masked<T>(v)) {
            o = dnan();
        } else if (h.path == 1) {
            o = cdf[(unsigned int)v - h.uoffset];
        } else {
            o = np_interp(shifted<T>(h, v), centers, cdf, h.nkept, cdf[0], cdf[h.nkept - 1]);
        }
        out[i] = o;
        if (rgba) {
            uint32_t px = 0;
            if (o == o) {
                // interp(data, span, chan, left=255), nan_to_num, astype(uint8)
                double c[3];
                np_interp_rgb(o, xs, ch, sl, cm.n, 255.0, c);
                px = (uint32_t)(uint8_t)(int)c[0] | ((uint32_t)(uint8_t)(int)c[1] << 8) |
                     ((uint32_t)(uint8_t)(int)c[2] << 16) | ((uint32_t)(uint8_t)cm.alpha << 24);
            }
            rgba[i] = px;
        }
    }
}

__global__ void eqh_levels(const EqHeader *h, long long *levels) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *levels = h->path == 0 ? 0 : h->levels;
}

static unsigned grid_cap(int64_t n, int threads, int mult) {
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    int64_t g = (n + threads - 1) / threads;
    if (g > (int64_t)sms * mult) g = (int64_t)sms * mult;
    if (g < 1) g = 1;
    return (unsigned)g;
}

template <typename T>
static int eq_hist_impl(const T *data, int64_t n, int32_t nbins, double *out, int64_t *levels,
                        uint32_t *rgba, const double *cmap_rgb, int32_t ncolors, int32_t alpha,
                        int32_t rescale, void *workspace, size_t wsb, void *stream) {
    if ((!data && n > 0) || n < 0 || !out || !levels || nbins < 1 || nbins > (1 << 24) || !workspace) {
        set_error("dsgb_eq_hist: invalid arguments");
        return DSGB_E_INVALID;
    }
    if (wsb < ws_bytes(nbins)) {
        set_error("dsgb_eq_hist: workspace of %zu bytes, %zu needed", wsb, ws_bytes(nbins));
        return DSGB_E_NOSPACE;
    }
    if (rgba && (!cmap_rgb || ncolors < 1 || ncolors > 256)) {
        set_error("dsgb_eq_hist: colormap must have 1..256 colours");
        return DSGB_E_INVALID;
    }
    Cmap cm;
    memset(&cm, 0, sizeof(cm));
    if (rgba) {
        cm.n = ncolors;
        for (int k = 0; k < ncolors; ++k) {
            cm.r[k] = cmap_rgb[3 * k]; cm.g[k] = cmap_rgb[3 * k + 1]; cm.b[k] = cmap_rgb[3 * k + 2];
        }
        cm.alpha = alpha;
    }
    cudaStream_t st = as_stream(stream);
    EqLayout L = layout(workspace, nbins);
    eqh_init<<<1, 32, 0, st>>>(L.hdr);
    cudaError_t e = cudaMemsetAsync(L.hist, 0, (size_t)nbins * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "dsgb_eq_hist memset");
    if (n > 0) eqh_minmax<T><<<grid_cap(n, 256, 4), 256, 0, st>>>(data, n, L.hdr);
    eqh_plan<T><<<1, 32, 0, st>>>(L.hdr, nbins);
    if (n > 0) eqh_hist<T><<<grid_cap(n, 512, 2), 512, 0, st>>>(data, n, L.hdr, L.hist, nbins);
    eqh_scan<<<1, 1024, 0, st>>>(L.hdr, L.hist, L.cdf, L.centers, nbins, rescale);
    eqh_div<<<grid_cap(nbins, 256, 1), 256, 0, st>>>(L.hdr, L.cdf);
    if (n > 0) eqh_apply<T><<<grid_cap(n, 256, 2), 256, 0, st>>>(data, n, L.hdr, L.cdf, L.centers, out, rgba, cm, nbins);
    eqh_levels<<<1, 32, 0, st>>>(L.hdr, (long long *)levels);
    DSGB_CHECK_LAUNCH("dsgb_eq_hist");
    return DSGB_OK;
}

// ---- allocation-free variant --------------------------------------------
//
// Some callers cannot allocate device memory at the moment they need an
// equalised image: a host thread with a latency budget (cudaMalloc may
// synchronise the whole device), code that runs where allocation is not
// allowed (inside a stream callback or another library's allocator hook),
// or a plugin whose host process owns every device allocation.  For them
// the scratch of eq_hist lives in this file-scope device array instead of a
// caller workspace.  It is sized for the largest histogram the reference
// uses (nbins = 65536, about 1.25 MiB); every GPU that loads the library
// holds it until the process exits.
constexpr int STATIC_MAX_BINS = 65536;
static __device__ __align__(256) unsigned char g_eq_hist_scratch[HDR_BYTES + (size_t)STATIC_MAX_BINS * 20 + 64];
static_assert(sizeof(g_eq_hist_scratch) >= HDR_BYTES + (size_t)STATIC_MAX_BINS * 20 + 64, "scratch size");

// In host code `g_eq_hist_scratch` names a host-side shadow, not device
// memory, so the device address is looked up with the device current and
// cached per device together with the context it belongs to: after a
// cudaDeviceReset the device has a new primary context, the module is
// loaded again, and the address is looked up again.
static std::mutex g_scratch_mu;
static void *g_scratch_ptr[128];
static CUcontext g_scratch_ctx[128];

static PFN_cuCtxGetCurrent_v4000 ctx_current_fn() {
    static PFN_cuCtxGetCurrent_v4000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuCtxGetCurrent_v4000)f;
    }
    return fn;
}

static int static_scratch(void **ptr) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "dsgb_eq_hist_u32_static: cudaGetDevice");
    if (dev < 0 || dev >= 128) { set_error("dsgb_eq_hist_u32_static: device ordinal %d out of range", dev); return DSGB_E_INVALID; }
    CUcontext ctx = nullptr;                // null before the runtime made a context current: look up again
    auto fn = ctx_current_fn();
    if (fn && fn(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev] || !ctx || ctx != g_scratch_ctx[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_eq_hist_scratch);
        if (e != cudaSuccess) return cuda_status(e, "dsgb_eq_hist_u32_static: cudaGetSymbolAddress");
        g_scratch_ptr[dev] = p;
        g_scratch_ctx[dev] = ctx;
    }
    *ptr = g_scratch_ptr[dev];
    return DSGB_OK;
}

}  // namespace dsgb

using namespace dsgb;

extern "C" int dsgb_eq_hist_u32_static(const uint32_t *data, int64_t n, int32_t nbins, double *out,
                                       int64_t *levels, uint32_t *rgba, const double *cmap_rgb,
                                       int32_t ncolors, int32_t alpha, int32_t rescale, void *stream) {
    if (nbins < 1 || nbins > STATIC_MAX_BINS) {
        set_error("dsgb_eq_hist_u32_static: nbins=%d is outside 1..%d, the size of the static scratch",
                  nbins, STATIC_MAX_BINS);
        return DSGB_E_INVALID;
    }
    void *scratch = nullptr;
    int rc = static_scratch(&scratch);
    if (rc) return rc;
    return eq_hist_impl<unsigned int>((const unsigned int *)data, n, nbins, out, levels, rgba, cmap_rgb,
                                      ncolors, alpha, rescale, scratch, sizeof(g_eq_hist_scratch), stream);
}

extern "C" size_t dsgb_eq_hist_workspace_size(int32_t nbins) { return ws_bytes(nbins < 1 ? 1 : nbins); }

extern "C" int dsgb_eq_hist_u32(const uint32_t *data, int64_t n, int32_t nbins, double *out, int64_t *levels,
                                uint32_t *rgba, const double *cmap_rgb, int32_t ncolors, int32_t alpha,
                                int32_t rescale, void *workspace, size_t wsb, void *stream) {
    return eq_hist_impl<unsigned int>((const unsigned int *)data, n, nbins, out, levels, rgba, cmap_rgb,
                                      ncolors, alpha, rescale, workspace, wsb, stream);
}

extern "C" int dsgb_eq_hist_f64(const double *data, int64_t n, int32_t nbins, double *out, int64_t *levels,
                                uint32_t *rgba, const double *cmap_rgb, int32_t ncolors, int32_t alpha,
                                int32_t rescale, void *workspace, size_t wsb, void *stream) {
    return eq_hist_impl<double>(data, n, nbins, out, levels, rgba, cmap_rgb, ncolors, alpha, rescale,
                                workspace, wsb, stream);
}
