// Host check of csrc/f64cmp.cuh: every helper against the IEEE operation it
// replaces, over all pairs of a set of special and random float64 values,
// and f64_from_u32 against the conversion over a sample of uint32 with every
// power of two and its neighbours.  Prints "ok" and exits 0, or prints the
// first mismatch and exits 1.  Compiled with g++ by tests/test_f64cmp.py.
#define __host__
#define __device__
#define __forceinline__ inline
#include "f64cmp.cuh"

#include <cmath>
#include <cstdio>
#include <limits>
#include <random>
#include <vector>

using namespace dsgb;

static double from_bits(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

static int fail(const char *what, double a, double b) {
    std::printf("mismatch %s a=%a (%016llx) b=%a (%016llx)\n", what, a, f64_bits(a), b, f64_bits(b));
    return 1;
}

// max(0, min(cvt(c), hi)) with the device's float64 -> int64 conversion:
// NaN -> 0, out of range saturated.
static long long ref_clamp(double c, long long hi) {
    long long k;
    if (std::isnan(c)) k = 0;
    else if (c >= 9223372036854775808.0) k = std::numeric_limits<long long>::max();
    else if (c < -9223372036854775808.0) k = std::numeric_limits<long long>::min();
    else k = (long long)c;
    k = k < hi ? k : hi;
    return k > 0 ? k : 0;
}

int main() {
    std::vector<double> v;
    const double specials[] = {0.0, 1.0, 2.0, 0.5, 0.25, 1.25, 1.5, 3.0, 1e-300, 1e300,
                               std::numeric_limits<double>::denorm_min(), std::numeric_limits<double>::min(),
                               std::numeric_limits<double>::max(), std::numeric_limits<double>::infinity(),
                               std::nextafter(1.0, 0.0), std::nextafter(1.0, 2.0), std::nextafter(0.0, 1.0)};
    for (double s : specials) {
        v.push_back(s);
        v.push_back(-s);
    }
    // NaNs of both signs, quiet and signalling payloads
    for (unsigned long long b : {0x7FF8000000000000ull, 0x7FF0000000000001ull, 0x7FFFFFFFFFFFFFFFull,
                                 0xFFF8000000000000ull, 0xFFF0000000000001ull, 0xFFFFFFFFFFFFFFFFull})
        v.push_back(from_bits(b));
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u(-4.0, 4.0);
    for (int i = 0; i < 400; ++i) v.push_back(u(rng));
    for (int i = 0; i < 100; ++i) v.push_back(from_bits(rng()));       // any pattern
    for (double k : {1.0, 2.0, 3.0, 511.0, 512.0, 1023.0, 1024.0, 4096.0, 2147483647.0, 2147483648.0, 4294967296.0,
                     9007199254740992.0, 9.3e18}) {
        for (double w : {k, std::nextafter(k, 0.0), std::nextafter(k, 1e300), k + 0.5, k - 0.5}) {
            v.push_back(w);
            v.push_back(-w);
        }
    }
    std::uniform_real_distribution<double> px(-50.0, 3000.0);
    for (int i = 0; i < 300; ++i) v.push_back(px(rng));
    const size_t n = v.size();
    for (size_t i = 0; i < n; ++i) {
        const double a = v[i];
        if (f64_lt0(a) != (a < 0.0)) return fail("lt0", a, 0.0);
        if (f64_gt0(a) != (a > 0.0)) return fail("gt0", a, 0.0);
        {
            const double m = a < 1.0 ? a : 1.0;
            const double c = 0.0 > m ? 0.0 : m;
            const double want = 1.0 - c, got = f64_one_minus_clamp01(a);
            if (f64_bits(want) != f64_bits(got)) return fail("one_minus_clamp01", a, got);
        }
        if (f64_isnan(a) != std::isnan(a)) return fail("isnan", a, 0.0);
        for (long long hi : {-1ll, 0ll, 1ll, 7ll, 1023ll, 2147483647ll}) {
            if (f64_ceil_clamp(a, hi) != ref_clamp(std::ceil(a), hi)) return fail("ceil_clamp", a, (double)hi);
            if (f64_floor_clamp(a, hi) != ref_clamp(std::floor(a), hi)) return fail("floor_clamp", a, (double)hi);
        }
        for (size_t j = 0; j < n; ++j) {
            const double b = v[j];
            if (f64_lt(a, b) != (a < b)) return fail("lt", a, b);
            if (f64_eq(a, b) != (a == b)) return fail("eq", a, b);
            if (f64_abs_lt(a, b) != (std::fabs(a) < std::fabs(b))) return fail("abs_lt", a, b);
            if (!std::signbit(a) && !std::isnan(a) && f64_nonneg_gt(a, b) != (a > b)) return fail("nonneg_gt", a, b);
            const bool b_nonneg = !(std::signbit(b) && !std::isnan(b));       // b >= +0.0 or NaN
            const bool b_range = !std::signbit(b) && !std::isnan(b);          // b in [+0, +inf]
            if (b_nonneg && f64_gt_nonneg(a, b) != (a > b)) return fail("gt_nonneg", a, b);
            if (b_range && f64_abs_le(a, b) != (std::fabs(a) <= b)) return fail("abs_le", a, b);
            if (b_range && f64_in_neg_range(a, b) != (-b <= a && a <= 0.0)) return fail("in_neg_range", a, b);
            if (b_range && !std::signbit(a) && !std::isnan(a) && f64_le_nonneg(a, b) != (a <= b))
                return fail("le_nonneg", a, b);
        }
    }
    // f64_from_u32: every power of two and its neighbours, then a stride through all of uint32
    for (int k = 0; k < 32; ++k)
        for (long long d = -2; d <= 2; ++d) {
            const long long x = (1ll << k) + d;
            if (x < 0 || x > 0xFFFFFFFFll) continue;
            if (f64_bits(f64_from_u32((unsigned)x)) != f64_bits((double)x))
                return fail("from_u32", (double)x, f64_from_u32((unsigned)x));
        }
    for (unsigned long long x = 0; x <= 0xFFFFFFFFull; x += 997) {
        if (f64_bits(f64_from_u32((unsigned)x)) != f64_bits((double)x))
            return fail("from_u32", (double)x, f64_from_u32((unsigned)x));
    }
    if (f64_bits(f64_from_u32(0xFFFFFFFFu)) != f64_bits(4294967295.0)) return fail("from_u32", 4294967295.0, 0);
    std::printf("ok %zu values\n", n);
    return 0;
}
