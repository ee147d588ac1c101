// Host check of csrc/aa_scan.cuh: the scanline span ends from the float32
// intercept equal max(0, min(ceil / floor(x), hi)) of the float64 intercept,
// over random rectangle edges at pixel-coordinate magnitudes, edges whose
// intercept is placed within 1e-15 ... 1e-3 of an integer, near-horizontal
// and near-vertical edges and large coordinates.  Prints "ok" with the share
// of calls that fell back to float64, or the first mismatch, and exits 1 on
// a mismatch.  Then the float32 pixel classification against the float64
// tests over random and axis-aligned segments (along exactly 0 on integer
// endpoints), every pixel of their bounding boxes.  Compiled with g++
// -ffp-contract=off by tests/test_f64cmp.py.
#define __host__
#define __device__
#define __forceinline__ inline
#include "aa_scan.cuh"

#include <cstdio>
#include <random>

using namespace dsgb;

static long long ref(double x, long long hi, bool up) {
    const double c = up ? std::ceil(x) : std::floor(x);
    long long k;
    if (std::isnan(c)) k = 0;
    else if (c >= 9223372036854775808.0) k = 9223372036854775807ll;
    else if (c < -9223372036854775808.0) k = -9223372036854775807ll - 1;
    else k = (long long)c;
    k = k < hi ? k : hi;
    return k > 0 ? k : 0;
}

static long long n_calls = 0, n_fast = 0;

static int check(unsigned y, double cx0, double cy0, double cx1, double cy1, long long hi) {
    const double yd = (double)y;
    const double x = aa_x_intercept(yd, cx0, cy0, cx1, cy1);
    float xf;
    n_calls += 1;
    if (!f64_eq(cy0, cy1) && aa_x_intercept_f32(y, cx0, cy0, cx1, cy1, xf)) n_fast += 1;
    const long long c = aa_scan_bound<true>(y, yd, cx0, cy0, cx1, cy1, hi);
    const long long f = aa_scan_bound<false>(y, yd, cx0, cy0, cx1, cy1, hi);
    if (c != ref(x, hi, true) || f != ref(x, hi, false)) {
        std::printf("mismatch y=%u cx0=%a cy0=%a cx1=%a cy1=%a x=%.17g ceil %lld/%lld floor %lld/%lld\n", y, cx0, cy0,
                    cx1, cy1, x, c, ref(x, hi, true), f, ref(x, hi, false));
        return 1;
    }
    return 0;
}

int main() {
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> pos(-50.0, 1100.0), ang(0.0, 6.283185307179586), unit(0.0, 1.0);
    const long long his[] = {1023, 511, 4095, 0, -1};
    // random edges of 0.01 .. 20 pixels, every scanline they span (and one beyond each end)
    for (int i = 0; i < 400000; ++i) {
        const double cx0 = pos(rng), cy0 = pos(rng), len = 0.01 * std::pow(2000.0, unit(rng)), a = ang(rng);
        const double cx1 = cx0 + len * std::cos(a), cy1 = cy0 + len * std::sin(a);
        const long long hi = his[i % 5];
        const double lo = std::fmin(cy0, cy1), up = std::fmax(cy0, cy1);
        for (long long y = (long long)std::floor(lo) - 1; y <= (long long)std::ceil(up) + 1; ++y)
            if (y >= 0 && check((unsigned)y, cx0, cy0, cx1, cy1, hi)) return 1;
    }
    // intercepts placed next to an integer
    const double deltas[] = {0.0, 1e-15, -1e-15, 1e-12, -1e-12, 1e-9, -1e-9, 1e-7, -1e-7, 1e-5, -1e-5, 1e-3, -1e-3};
    for (int i = 0; i < 200000; ++i) {
        const unsigned y = (unsigned)(rng() % 1000) + 1;
        const double cy0 = y - 0.5 * unit(rng) - 0.01, cy1 = y + 3.0 * unit(rng) + 0.01;
        const double cx0 = pos(rng);
        const double k = std::floor(pos(rng)), dlt = deltas[i % 13];
        const double f = ((double)y - cy0) / (cy1 - cy0);
        const double cx1 = cx0 + (k + dlt - cx0) / f;
        if (check(y, cx0, cy0, cx1, cy1, 4095)) return 1;
    }
    // near-horizontal, near-vertical, exact integers, large magnitudes
    for (int i = 0; i < 200000; ++i) {
        const unsigned y = (unsigned)(rng() % 5000);
        const double cy0 = y - unit(rng) * std::pow(10.0, -(double)(rng() % 16));
        const double cy1 = cy0 + (rng() % 2 ? 1.0 : -1.0) * std::pow(10.0, -(double)(rng() % 16)) * unit(rng);
        const double scale = std::pow(10.0, (double)(rng() % 9));
        const double cx0 = (unit(rng) - 0.3) * scale, cx1 = cx0 + (unit(rng) - 0.5) * scale * 1e-3;
        if (check(y, cx0, cy0, cx1, cy1, 2147483647ll)) return 1;
        if (check(y, std::floor(cx0), (double)y, std::floor(cx0) + 2.0, (double)y + 1.0, 2147483647ll)) return 1;
    }
    // the pixel classification: every decided case equals the float64 tests' case
    long long n_pix = 0, n_dec = 0;
    for (int i = 0; i < 300000; ++i) {
        const bool axis = i % 7 == 0;                     // axis-aligned, integer endpoints: along hits 0 exactly
        const double x0 = axis ? std::floor(pos(rng)) : pos(rng), y0 = axis ? std::floor(pos(rng)) : pos(rng);
        const double len0 = 0.05 * std::pow(400.0, unit(rng)), a = axis ? 1.5707963267948966 * (rng() % 4) : ang(rng);
        const double dx = axis ? std::round(len0 * std::cos(a)) + (std::cos(a) > 0.5 ? 1 : 0) : len0 * std::cos(a);
        const double dy = axis ? std::round(len0 * std::sin(a)) : len0 * std::sin(a);
        const double x1 = x0 + dx, y1 = y0 + dy;
        double ax = x1 - x0, ay = y1 - y0;
        const double len = std::sqrt(ax * ax + ay * ay);
        if (!(len > 0.0)) continue;
        ax /= len;
        ay /= len;
        const double pa = ang(rng);
        double pax = std::cos(pa), pay = std::sin(pa);
        const double plen = std::sqrt(pax * pax + pay * pay);
        pax /= plen;
        pay /= plen;
        const bool cap_before = rng() % 3 == 0, cap_after = rng() % 3 == 0;
        const AAClassF k{(float)x0, (float)y0, (float)ax, (float)ay, (float)len, (float)pax, (float)pay};
        const long long xa = (long long)std::floor(std::fmin(x0, x1)) - 3, xb = (long long)std::ceil(std::fmax(x0, x1)) + 3;
        const long long ya = (long long)std::floor(std::fmin(y0, y1)) - 3, yb = (long long)std::ceil(std::fmax(y0, y1)) + 3;
        for (long long yy = ya; yy <= yb; ++yy)
            for (long long xx = xa; xx <= xb; ++xx) {
                if (xx < 0 || yy < 0) continue;
                const double xd = (double)xx, yd = (double)yy;
                const double along = (xd - x0) * ax + (yd - y0) * ay;
                int want;
                if (along < 0.0) want = (cap_before || (xd - x0) * pax + (yd - y0) * pay > 0.0) ? AAC_CAP_BEFORE : AAC_NONE;
                else if (along > len) want = cap_after ? AAC_CAP_AFTER : AAC_NONE;
                else want = AAC_SIDE;
                const int got = aa_classify((unsigned)xx, (unsigned)yy, k, cap_before, cap_after);
                n_pix += 1;
                if (got == AAC_EXACT) continue;
                n_dec += 1;
                if (got != want) {
                    std::printf("classify mismatch x=%lld y=%lld x0=%a y0=%a ax=%a ay=%a len=%a got %d want %d\n", xx, yy,
                                x0, y0, ax, ay, len, got, want);
                    return 1;
                }
            }
    }
    std::printf("ok %lld calls, %.4f float32-decided; %lld pixels, %.4f classified in float32\n", n_calls,
                (double)n_fast / (double)n_calls, n_pix, (double)n_dec / (double)n_pix);
    return 0;
}
