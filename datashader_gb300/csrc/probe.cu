// probe.cu -- a float64 throughput probe for the roofline of the float64-bound
// kernels (antialiased line coverage).  No counterpart in the reference.
//
// Every thread runs 8 independent chains of float64 FMAs; the caller times
// one launch with CUDA events: FLOP/s = 2 * 8 * iters * blocks * threads / s.
#include "dsgb_internal.cuh"

namespace dsgb {

constexpr int PROBE_CHAINS = 8;
constexpr int PROBE_THREADS = 256;

__global__ void __launch_bounds__(PROBE_THREADS) fp64_probe_kernel(double *sink, int iters, double a, double b) {
    double c[PROBE_CHAINS];
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) c[k] = (double)(threadIdx.x + k) * 1e-9;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < PROBE_CHAINS; ++k) c[k] = __fma_rn(c[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) s += c[k];
    if (s == 1234.5) sink[0] = s;          // keeps the chains live; never true for the probe's inputs
}

}  // namespace dsgb

using namespace dsgb;

extern "C" int dsgb_fp64_probe(double *sink, int32_t iters, int32_t blocks_per_sm, int64_t *flops, void *stream) {
    if (!sink || !flops || iters <= 0 || blocks_per_sm <= 0) {
        set_error("dsgb_fp64_probe: invalid arguments");
        return DSGB_E_INVALID;
    }
    const int sms = sm_count();
    if (sms <= 0) return cuda_status(cudaErrorNoDevice, "dsgb_fp64_probe: device");
    const int blocks = sms * blocks_per_sm;
    fp64_probe_kernel<<<blocks, PROBE_THREADS, 0, as_stream(stream)>>>(sink, iters, 0.999999, 1e-12);
    DSGB_CHECK_LAUNCH("dsgb_fp64_probe");
    *flops = 2LL * PROBE_CHAINS * (int64_t)iters * blocks * PROBE_THREADS;
    return DSGB_OK;
}
