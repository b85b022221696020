// textscan.cuh — fields of delimited text rows parsed into column values (the scan side of a
// scan -> filter fusion).
//
// A table scan over a delimited text file (the reference's csv_parser, src/io/data_parser/
// CSVParser.cpp, which hands the bytes to cudf's CSV reader with '|' as the default delimiter, no
// header and blank lines skipped) turns each field into a value of the schema's dtype.  The rules
// here, shared by the GPU scan kernel and the host tests:
//
// * a field is the bytes between two delimiters (or a row's ends); spaces around it are ignored;
//   an empty field, or one that does not read as the dtype, is null;
// * integers: an optional sign and decimal digits, accumulated modulo 2^64 and narrowed to the
//   column's width by two's complement truncation;
// * floating point: an optional sign, digits with an optional decimal point, an optional exponent
//   (e or E, optional sign, up to five digits); the value is the decimal number rounded to the
//   nearest double (ties to even), then to float for FLOAT32 columns.  It is computed exactly
//   when the significand has at most 19 digits and either fits in 53 bits with a power of ten
//   |e| <= 22 (one correctly rounded multiply or divide of two exact doubles, Clinger's fast
//   path) or is small enough to absorb the excess power of ten; other values are refused (the
//   scan reports an error rather than round them differently);
// * dates: YYYY-MM-DD, years 0001-9999 (DATE32: days since 1970-01-01; DATE64: milliseconds),
//   and for DATE64 optionally a time HH:MM:SS after a space or 'T'; proleptic Gregorian, UTC.
//
// The file compiles as CUDA device code (the NVRTC prelude) and as plain C++ on the host, where
// the tests compare every function with the host's own conversions.
#ifndef RAL_TEXTSCAN_CUH_
#define RAL_TEXTSCAN_CUH_

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define RAL_TX __host__ __device__ __forceinline__
#else
#define RAL_TX static inline
#endif

// field validity: a value, a null, or a value this scan refuses to round
#define RAL_TX_NULL 0
#define RAL_TX_OK 1
#define RAL_TX_REFUSED 2

RAL_TX bool ral_tx_digit(unsigned char c) { return c >= '0' && c <= '9'; }

// [p, e) without the spaces at either end
RAL_TX void ral_tx_trim(const char* s, long long& p, long long& e) {
    while (p < e && s[p] == ' ') ++p;
    while (e > p && s[e - 1] == ' ') --e;
}

RAL_TX int ral_tx_parse_int(const char* s, long long p, long long e, long long* out) {
    ral_tx_trim(s, p, e);
    if (p >= e) return RAL_TX_NULL;
    bool neg = false;
    if (s[p] == '+' || s[p] == '-') {
        neg = s[p] == '-';
        ++p;
    }
    if (p >= e) return RAL_TX_NULL;
    unsigned long long v = 0;
    for (; p < e; ++p) {
        const unsigned char c = (unsigned char)s[p];
        if (!ral_tx_digit(c)) return RAL_TX_NULL;
        v = v * 10ull + (unsigned long long)(c - '0');
    }
    *out = (long long)(neg ? 0ull - v : v);
    return RAL_TX_OK;
}

// 10^k for k <= 22: every one is an exact double
RAL_TX double ral_tx_pow10(int k) {
    double r = 1.0;
    double b = 10.0;
    while (k) {  // exact: every partial product is a power of ten below 2^53 * 2^k
        if (k & 1) r *= b;
        b *= b;
        k >>= 1;
    }
    return r;
}

RAL_TX double ral_tx_mul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
RAL_TX double ral_tx_div(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

RAL_TX int ral_tx_parse_double(const char* s, long long p, long long e, double* out) {
    ral_tx_trim(s, p, e);
    if (p >= e) return RAL_TX_NULL;
    bool neg = false;
    if (s[p] == '+' || s[p] == '-') {
        neg = s[p] == '-';
        ++p;
    }
    unsigned long long m = 0;
    int sig = 0;         // significant digits taken into m
    int e10 = 0;         // decimal exponent of m
    int digits = 0;      // digits seen in the significand
    bool dot = false;
    for (; p < e; ++p) {
        const unsigned char c = (unsigned char)s[p];
        if (c == '.') {
            if (dot) return RAL_TX_NULL;
            dot = true;
            continue;
        }
        if (!ral_tx_digit(c)) break;
        ++digits;
        if (m == 0 && c == '0') {  // a leading zero: only moves the exponent after the point
            if (dot) --e10;
            continue;
        }
        if (sig == 19) {  // a 20th significant digit: beyond the exact range unless it is zero
            if (c != '0') return RAL_TX_REFUSED;
            if (!dot) ++e10;
            continue;
        }
        m = m * 10ull + (unsigned long long)(c - '0');
        ++sig;
        if (dot) --e10;
    }
    if (digits == 0) return RAL_TX_NULL;
    if (p < e) {
        const unsigned char c = (unsigned char)s[p];
        if (c != 'e' && c != 'E') return RAL_TX_NULL;
        ++p;
        bool eneg = false;
        if (p < e && (s[p] == '+' || s[p] == '-')) {
            eneg = s[p] == '-';
            ++p;
        }
        if (p >= e) return RAL_TX_NULL;
        int x = 0, nd = 0;
        for (; p < e; ++p) {
            const unsigned char d = (unsigned char)s[p];
            if (!ral_tx_digit(d)) return RAL_TX_NULL;
            if (++nd > 5) return RAL_TX_REFUSED;
            x = x * 10 + (d - '0');
        }
        e10 += eneg ? -x : x;
    }
    double v;
    if (m == 0) {
        v = 0.0;
    } else {
        const unsigned long long two53 = 1ull << 53;
        if (e10 > 22 && m <= two53) {
            // absorb the excess power of ten into the significand while it stays exact
            while (e10 > 22 && m <= two53 / 10ull) {
                m *= 10ull;
                --e10;
            }
        }
        if (m > two53 || e10 > 22 || e10 < -22) return RAL_TX_REFUSED;
        const double dm = (double)m;  // exact: m <= 2^53
        v = e10 >= 0 ? ral_tx_mul(dm, ral_tx_pow10(e10)) : ral_tx_div(dm, ral_tx_pow10(-e10));
    }
    *out = neg ? -v : v;
    return RAL_TX_OK;
}

// Days from 1970-01-01 of a proleptic Gregorian date (the public days-from-civil algorithm: a
// year starting in March, 400-year eras of 146097 days).
RAL_TX long long ral_tx_days_from_civil(long long y, unsigned m, unsigned d) {
    y -= m <= 2 ? 1 : 0;
    const long long era = (y >= 0 ? y : y - 399) / 400;
    const unsigned yoe = (unsigned)(y - era * 400);
    const unsigned doy = (153u * (m + (m > 2 ? -3 : 9)) + 2u) / 5u + d - 1u;
    const unsigned doe = yoe * 365u + yoe / 4u - yoe / 100u + doy;
    return era * 146097ll + (long long)doe - 719468ll;
}

RAL_TX bool ral_tx_num(const char* s, long long p, int n, unsigned* out) {
    unsigned v = 0;
    for (int i = 0; i < n; ++i) {
        const unsigned char c = (unsigned char)s[p + i];
        if (!ral_tx_digit(c)) return false;
        v = v * 10u + (unsigned)(c - '0');
    }
    *out = v;
    return true;
}

// YYYY-MM-DD, and for with_time HH:MM:SS after ' ' or 'T'; *out = days, or milliseconds when
// with_time is set (the time optional).
RAL_TX int ral_tx_parse_date(const char* s, long long p, long long e, bool with_time, long long* out) {
    ral_tx_trim(s, p, e);
    if (p >= e) return RAL_TX_NULL;
    const long long n = e - p;
    if (n < 10 || s[p + 4] != '-' || s[p + 7] != '-') return RAL_TX_NULL;
    unsigned y, mo, d;
    if (!ral_tx_num(s, p, 4, &y) || !ral_tx_num(s, p + 5, 2, &mo) || !ral_tx_num(s, p + 8, 2, &d)) return RAL_TX_NULL;
    if (y < 1 || mo < 1 || mo > 12 || d < 1) return RAL_TX_NULL;  // years 0001-9999
    const bool leap = (y % 4u == 0u && y % 100u != 0u) || y % 400u == 0u;
    const unsigned mdays = mo == 2 ? (leap ? 29u : 28u) : ((mo == 4 || mo == 6 || mo == 9 || mo == 11) ? 30u : 31u);
    if (d > mdays) return RAL_TX_NULL;
    const long long days = ral_tx_days_from_civil((long long)y, mo, d);
    if (!with_time) {
        if (n != 10) return RAL_TX_NULL;
        *out = days;
        return RAL_TX_OK;
    }
    long long secs = 0;
    if (n != 10) {
        if (n != 19 || (s[p + 10] != ' ' && s[p + 10] != 'T') || s[p + 13] != ':' || s[p + 16] != ':')
            return RAL_TX_NULL;
        unsigned h, mi, se;
        if (!ral_tx_num(s, p + 11, 2, &h) || !ral_tx_num(s, p + 14, 2, &mi) || !ral_tx_num(s, p + 17, 2, &se))
            return RAL_TX_NULL;
        if (h > 23 || mi > 59 || se > 59) return RAL_TX_NULL;
        secs = (long long)h * 3600 + (long long)mi * 60 + (long long)se;
    }
    *out = (days * 86400ll + secs) * 1000ll;
    return RAL_TX_OK;
}

#endif  // RAL_TEXTSCAN_CUH_
