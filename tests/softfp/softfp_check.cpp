// Host check of softfp.cuh: every function against the host's IEEE-754 operations, bit for bit,
// on edge cases and random inputs.  Prints one line per function: name, cases, mismatches, and
// the first mismatch.  Built and run by tests/test_softfp_cpu.py.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

// every estimate of ral_sf_rcp_estimate can be moved by a number of ulps (0 except in the
// division-under-perturbed-reciprocal check below)
#define RAL_SF_TEST_RCP_ULPS 1
int ral_sf_test_rcp_ulps = 0;
#include "softfp.cuh"

static uint64_t bits(double d) { uint64_t b; std::memcpy(&b, &d, 8); return b; }
static double dbl(uint64_t b) { double d; std::memcpy(&d, &b, 8); return d; }
static uint32_t fbits(float f) { uint32_t b; std::memcpy(&b, &f, 4); return b; }
static float flt(uint32_t b) { float f; std::memcpy(&f, &b, 4); return f; }

// distance in units in the last place (finite doubles)
static long long ulps(double a, double b) {
    auto ord = [](double d) { long long v; std::memcpy(&v, &d, 8); return v < 0 ? -(v & 0x7fffffffffffffffll) : v; };
    const long long d = ord(a) - ord(b);
    return d < 0 ? -d : d;
}

// same value, or both NaN
static bool same_d(double a, double b) { return (std::isnan(a) && std::isnan(b)) || bits(a) == bits(b); }
static bool same_f(float a, float b) { return (std::isnan(a) && std::isnan(b)) || fbits(a) == fbits(b); }

// the host's comparisons, kept out of line so that they are evaluated as written
__attribute__((noinline)) static unsigned host_compare(double a, double b) {
    return (unsigned)(a < b) | (unsigned)(a <= b) << 1 | (unsigned)(a > b) << 2 | (unsigned)(a >= b) << 3 |
           (unsigned)(a == b) << 4 | (unsigned)(a != b) << 5;
}

struct Counter {
    const char* name;
    long long n = 0, bad = 0;
    char first[256] = "";
    void report() { std::printf("%s %lld %lld %s\n", name, n, bad, first); }
};

static std::vector<double> special_doubles() {
    std::vector<double> v = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 1.5, -1.5, 2.0, 3.0, -3.0, 0.1, -0.1, 1e308, -1e308,
                             1e-308, -1e-308, 4.9e-324, -4.9e-324, 2.2250738585072014e-308,
                             std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                             std::numeric_limits<double>::quiet_NaN(), 9007199254740992.0, 9007199254740993.0,
                             -9007199254740992.0, 4503599627370496.5, 4503599627370495.5, 9.2233720368547758e18,
                             -9.2233720368547758e18, 9.2233720368547748e18, 0.49999999999999994, -0.49999999999999994,
                             1.7976931348623157e308, 3.4028234663852886e38, 3.4028235677973366e38, 1.401298464324817e-45,
                             7.006492321624085e-46, 7.006492321624087e-46, 1.1754943508222875e-38,
                             1.1754942807573643e-38, 1.1754943157898259e-38};
    return v;
}

int main(int argc, char** argv) {
    const long long N = argc > 1 ? atoll(argv[1]) : 2000000;
    std::mt19937_64 rng(12345);
    auto rand_double = [&]() -> double {
        switch (rng() % 6) {
        case 0: return dbl(rng());                                       // any bit pattern
        case 1: return (double)(int64_t)(rng() >> (rng() % 64));          // integers of all sizes
        case 2: return std::ldexp((double)(rng() >> 11), (int)(rng() % 120) - 60);  // moderate range
        case 3: return (double)(int32_t)rng() / (double)(1 + (rng() % 1000));
        case 4: return std::ldexp(1.0, (int)(rng() % 2100) - 1075) * (rng() & 1 ? -1 : 1);
        default: return (double)(float)dbl(rng());
        }
    };
    std::vector<double> sp = special_doubles();

    Counter cdiv64{"div64"};
    auto check_div64 = [&](long long a, long long b) {
        if (b == 0 || b == -1) return;
        cdiv64.n++;
        if ((a / b != ral_sf_div64(a, b) || a % b != ral_sf_mod64(a, b)) && cdiv64.bad++ == 0)
            std::snprintf(cdiv64.first, sizeof cdiv64.first, "%lld / %lld: want %lld %lld got %lld %lld", a, b, a / b,
                          a % b, ral_sf_div64(a, b), ral_sf_mod64(a, b));
    };
    Counter cd16{"div64_16"};
    auto check_d16 = [&](long long a, long long b) {  // 1 <= |b| < 2^16
        cd16.n++;
        if ((a / b != ral_sf_div64_16(a, b) || a % b != ral_sf_mod64_16(a, b)) && cd16.bad++ == 0)
            std::snprintf(cd16.first, sizeof cd16.first, "%lld / %lld: want %lld %lld got %lld %lld", a, b, a / b,
                          a % b, ral_sf_div64_16(a, b), ral_sf_mod64_16(a, b));
    };
    Counter cdc{"divc"};
    auto check_divc = [&](long long a, long long b) {  // by a precomputed divider (every b)
        const RalDivider v = ral_sf_make_divider(b);
        long long wq, wr;
        if (b == 0) wq = wr = 0;
        else if (b == -1) wq = (long long)(0ull - (unsigned long long)a), wr = 0;
        else wq = a / b, wr = a % b;
        cdc.n++;
        const long long gq = ral_sf_divc(a, b, v.mult, v.shift_mode), gr = ral_sf_modc(a, b, v.mult, v.shift_mode);
        if ((gq != wq || gr != wr) && cdc.bad++ == 0)
            std::snprintf(cdc.first, sizeof cdc.first, "%lld / %lld: want %lld %lld got %lld %lld", a, b, wq, wr, gq, gr);
    };
    Counter cd32{"div64_32"};
    auto check_d32 = [&](unsigned long long n, unsigned int d) {
        if (d == 0) return;
        cd32.n++;
        unsigned long long q, r;
        ral_sf_udivmod64_32(n, d, &q, &r);
        if ((q != n / d || r != n % d) && cd32.bad++ == 0)
            std::snprintf(cd32.first, sizeof cd32.first, "%llu / %u: want %llu %llu got %llu %llu", n, d, n / d, n % d, q, r);
    };
    // sin / cos: within one ulp of the host's libm (which is within one ulp of the exact value)
    Counter csin{"sincos"};
    auto check_trig = [&](double x) {
        csin.n++;
        const long long a = ulps(std::sin(x), ral_sf_sin(x)), b = ulps(std::cos(x), ral_sf_cos(x));
        const bool nan_ok = std::isnan(x) ? (std::isnan(ral_sf_sin(x)) && std::isnan(ral_sf_cos(x))) : true;
        if ((!nan_ok || (!std::isnan(x) && !std::isinf(x) && (a > 1 || b > 1))) && csin.bad++ == 0)
            std::snprintf(csin.first, sizeof csin.first, "%a: sin %lld ulp, cos %lld ulp", x, a, b);
    };
    Counter cdiv{"div"}, cfloor{"floor"}, cceil{"ceil"}, cabs{"fabs"}, ccmp{"compare"}, ci2d{"i2d"}, cd2i{"d2i"},
        cf2d{"f2d"}, cd2f{"d2f"}, czero{"is_zero"};
    auto check_div = [&](double a, double b) {
        cdiv.n++;
        const double w = a / b, g = ral_sf_div(a, b);
        if (!same_d(w, g) && cdiv.bad++ == 0)
            std::snprintf(cdiv.first, sizeof cdiv.first, "%a/%a want %a got %a", a, b, w, g);
    };
    auto check_unary = [&](double x) {
        cfloor.n++; cceil.n++; cabs.n++; czero.n++; cd2f.n++;
        if (!same_d(std::floor(x), ral_sf_floor(x)) && cfloor.bad++ == 0)
            std::snprintf(cfloor.first, sizeof cfloor.first, "%a want %a got %a", x, std::floor(x), ral_sf_floor(x));
        if (!same_d(std::ceil(x), ral_sf_ceil(x)) && cceil.bad++ == 0)
            std::snprintf(cceil.first, sizeof cceil.first, "%a want %a got %a", x, std::ceil(x), ral_sf_ceil(x));
        if (!same_d(std::fabs(x), ral_sf_fabs(x)) && cabs.bad++ == 0)
            std::snprintf(cabs.first, sizeof cabs.first, "%a", x);
        if ((x == 0.0) != ral_sf_is_zero(x) && czero.bad++ == 0)
            std::snprintf(czero.first, sizeof czero.first, "%a", x);
        if (!same_f((float)x, ral_sf_d2f(x)) && cd2f.bad++ == 0)
            std::snprintf(cd2f.first, sizeof cd2f.first, "%a want %a got %a", x, (double)(float)x, (double)ral_sf_d2f(x));
        // double -> int64 as cvt.rzi.s64.f64 on the GPU: NaN -> INT64_MIN, saturating
        cd2i.n++;
        long long w;
        if (std::isnan(x)) w = INT64_MIN;
        else if (x >= 9223372036854775808.0) w = INT64_MAX;
        else if (x <= -9223372036854775808.0) w = INT64_MIN;
        else w = (long long)x;
        if (w != ral_sf_d2i(x) && cd2i.bad++ == 0)
            std::snprintf(cd2i.first, sizeof cd2i.first, "%a want %lld got %lld", x, w, ral_sf_d2i(x));
    };
    auto check_cmp = [&](double a, double b) {
        ccmp.n++;
        const unsigned want = host_compare(a, b);
        const unsigned got = (unsigned)ral_sf_lt(a, b) | (unsigned)ral_sf_le(a, b) << 1 | (unsigned)ral_sf_gt(a, b) << 2 |
                             (unsigned)ral_sf_ge(a, b) << 3 | (unsigned)ral_sf_eq(a, b) << 4 |
                             (unsigned)ral_sf_ne(a, b) << 5;
        if (want != got && ccmp.bad++ == 0)
            std::snprintf(ccmp.first, sizeof ccmp.first, "%a vs %a (%llx %llx): want %x got %x", a, b,
                          (unsigned long long)bits(a), (unsigned long long)bits(b), want, got);
    };
    for (double a : sp) {
        check_unary(a);
        for (double b : sp) {
            check_div(a, b);
            check_cmp(a, b);
        }
    }
    for (long long k = 0; k < N; k++) {
        const double a = rand_double(), b = rand_double();
        check_div(a, b);
        check_cmp(a, b);
        check_cmp(a, a);
        check_unary(a);
        // quotients near 1 and exact quotients exercise the rounding boundaries
        check_div(a, a * (1.0 + std::ldexp((double)(rng() % 64) - 32, -52)));
        const double q = std::ldexp((double)(rng() >> 11), -(int)(rng() % 40));
        check_div(q * b, b);
        // int64 -> double
        ci2d.n++;
        const long long x = (long long)(rng() >> (rng() % 64)) * ((rng() & 1) ? -1 : 1);
        if (!same_d((double)x, ral_sf_i2d(x)) && ci2d.bad++ == 0)
            std::snprintf(ci2d.first, sizeof ci2d.first, "%lld want %a got %a", x, (double)x, ral_sf_i2d(x));
        // 64-bit integer division: operands of every magnitude, divisors near powers of two
        const long long xa = (long long)(rng() >> (rng() % 64)) * ((rng() & 1) ? -1 : 1);
        long long xb = (long long)(rng() >> (rng() % 64)) * ((rng() & 1) ? -1 : 1);
        check_div64(xa, xb);
        check_div64(xa, (long long)(1 + rng() % 1000));
        xb = (long long)(1ull << (rng() % 63)) + (long long)(rng() % 3) - 1;
        check_div64(xa, xb);
        check_div64(INT64_MIN, xb);
        check_trig(a);
        check_trig(std::ldexp((double)(rng() >> 11), -53) * 2e6 * ((rng() & 1) ? -1 : 1));
        check_trig(std::ldexp(1.0 + (double)(rng() >> 11) * 0x1p-53, (int)(rng() % 50) - 28));
        // next to multiples of pi/2, where the reduced argument is smallest
        const double kpi2 = (double)(long long)(rng() % 600000) * 1.5707963267948966;
        check_trig(std::nextafter(kpi2, 0.0));
        check_trig(kpi2);
        check_trig(std::nextafter(kpi2, 1e300));
        check_d32(rng() >> (rng() % 64), (unsigned)(rng() >> (32 + rng() % 32)));
        check_d32(rng(), (unsigned)(1 + rng() % 1000));
        check_d32(rng(), 0xffffffffu - (unsigned)(rng() % 3));
        check_d32(rng(), (1u << (rng() % 32)) + (unsigned)(rng() % 3) - 1u);
        check_div64(INT64_MAX, xb);
        // division by a precomputed divider: divisors of every size and sign, powers of two and
        // their neighbours, the extremes; dividends likewise
        {
            const long long pb = (long long)(1ull << (rng() % 63)) + (long long)(rng() % 3) - 1;
            const long long dvs[] = {xb, (long long)(0ull - (unsigned long long)xb), (long long)(1 + rng() % 1000), -(long long)(1 + rng() % 1000), pb, -pb,
                                     0, 1, -1, 2, -2, 3, 7, -7, INT64_MAX, INT64_MIN, INT64_MIN + 1,
                                     (long long)(rng() >> 1), (long long)(1ull << 62), -(long long)(1ull << 62)};
            for (long long dd : dvs) {
                check_divc(xa, dd);
                check_divc(INT64_MIN, dd);
                check_divc(INT64_MAX, dd);
                check_divc((long long)rng(), dd);
                check_divc(dd, dd);
                check_divc((long long)((unsigned long long)dd - 1ull), dd);
            }
        }
        // divisors below 2^16: every size, powers of two and their neighbours, the extremes
        const long long d16 = (long long)(1 + (rng() >> (48 + rng() % 16)) % 65535) * ((rng() & 1) ? -1 : 1);
        const long long p16 = (long long)(1ull << (rng() % 16)) + (long long)(rng() % 3) - 1;
        for (long long dd : {d16, p16 > 0 ? p16 : 1ll, 65535ll, -65535ll, 1ll, 2ll, -2ll}) {
            if (dd == -1) continue;
            check_d16(xa, dd);
            check_d16(INT64_MIN, dd);
            check_d16(INT64_MAX, dd);
            check_d16((long long)rng(), dd);
        }
        // float -> double
        cf2d.n++;
        const float f = flt((uint32_t)rng());
        if (!same_d((double)f, ral_sf_f2d(f)) && cf2d.bad++ == 0)
            std::snprintf(cf2d.first, sizeof cf2d.first, "%a", (double)f);
    }
    // division with the reciprocal estimate moved by -4 .. +4 ulps (the GPU's rcp.approx is within
    // one), on divisors whose top 32 bits sit at the ends of their range and dividends at the ends of
    // the quotient range [1, 2)
    Counter cdivr{"div_rcp"};
    for (int pert = -4; pert <= 4; ++pert) {
        ral_sf_test_rcp_ulps = pert;
        const long long per = std::max(1ll, N / 8);
        for (long long k = 0; k < per; k++) {
            unsigned long long dh;
            switch (rng() % 4) {
            case 0: dh = (1ull << 31) + rng() % 8; break;
            case 1: dh = (1ull << 32) - 1 - rng() % 8; break;
            case 2: dh = (1ull << 31) | (1ull << (rng() % 31)); break;
            default: dh = (1ull << 31) | (rng() >> 33); break;
            }
            const unsigned long long dl = (rng() % 3 == 0) ? 0 : ((rng() % 2) ? (1ull << 21) - 1 : rng() >> 43);
            const unsigned long long mb = (dh << 21) | dl;
            unsigned long long ma;
            switch (rng() % 5) {
            case 0: ma = mb; break;
            case 1: ma = mb - 1 - rng() % 4; break;                     // just below: doubled
            case 2: ma = (mb + 1 + rng() % 4) & ((1ull << 53) - 1); break;
            case 3: ma = (1ull << 53) - 1 - rng() % 4; break;
            default: ma = rng() >> 11; break;
            }
            ma |= 1ull << 52;
            const int ea = 900 + (int)(rng() % 200), eb = 900 + (int)(rng() % 200);
            const double a = dbl(((unsigned long long)ea << 52) | (ma & ((1ull << 52) - 1)) | ((rng() & 1) << 63));
            const double b = dbl(((unsigned long long)eb << 52) | (mb & ((1ull << 52) - 1)));
            cdivr.n++;
            const double w = a / b, g = ral_sf_div(a, b);
            if (!same_d(w, g) && cdivr.bad++ == 0)
                std::snprintf(cdivr.first, sizeof cdivr.first, "%a/%a (rcp %+d ulp) want %a got %a", a, b, pert, w, g);
        }
    }
    ral_sf_test_rcp_ulps = 0;
    cdivr.report();
    for (long long x : std::vector<long long>{0ll, 1ll, -1ll, (long long)INT64_MAX, (long long)INT64_MIN, (1ll << 53) + 1, -(1ll << 53) - 1, (1ll << 62) + 3}) {
        ci2d.n++;
        if (!same_d((double)x, ral_sf_i2d(x)) && ci2d.bad++ == 0)
            std::snprintf(ci2d.first, sizeof ci2d.first, "%lld", x);
    }
    for (double v : sp) check_trig(v);
    for (double v : {0.7853981633974483, 0.7853981633974482, 0.7853981633974484, 0x1p-26, 0x1p-27, 0x1p20,
                     0x1.fffffffffffffp19, 3.141592653589793, 1.5707963267948966, 1e6, -1e6})
        check_trig(v);
    for (Counter* c : {&csin, &cdc, &cd16, &cd32, &cdiv64, &cdiv, &cfloor, &cceil, &cabs, &ccmp, &ci2d, &cd2i, &cf2d, &cd2f, &czero}) c->report();
    return 0;
}
