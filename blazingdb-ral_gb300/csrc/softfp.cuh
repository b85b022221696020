// softfp.cuh — exactly rounded IEEE-754 binary64 operations on the integer pipes.
//
// GB300 issues about two FP64 instructions per clock per SM against 64+ integer instructions,
// and an IEEE double division alone is a sequence of about nine FP64-pipe instructions.  The
// expression kernels are FP64-bound long before they are HBM-bound, so the operations below
// compute the same bits as the hardware instructions (division, floor / ceil, comparisons and
// the int64 / float32 <-> double conversions) with integer arithmetic instead, leaving the FP64
// pipe to add, subtract and multiply.
//
// Every function returns exactly what the IEEE operation (round to nearest even) returns for
// every input, including -0, infinities and NaN (NaN results are the default quiet NaN or the
// input NaN, as the hardware produces them; callers compare NaNs as NaN).  Inputs outside a
// function's fast path (zero, subnormal, infinite or NaN operands, subnormal or overflowing
// quotients) fall back to the hardware instruction.
//
// Methods: division by a Newton-Raphson reciprocal (one step in 32-bit, one in 64-bit fixed
// point) seeded from a single-precision reciprocal estimate, then an exact remainder correction of
// the quotient and round-to-nearest-even from the remainder (the schoolbook method of e.g. Muller et al.,
// "Handbook of Floating-Point Arithmetic", ch. 9); comparisons on the sign-magnitude keys of the
// bit patterns; conversions by normalising shifts with explicit round-to-nearest-even.
//
// The file compiles as CUDA device code (NVRTC prelude, nvcc) and as plain C++ on the host,
// where the tests check it bit for bit against the host's own IEEE operations.
#ifndef RAL_SOFTFP_CUH_
#define RAL_SOFTFP_CUH_

#if defined(__CUDACC__)
#define RAL_SF __host__ __device__ __forceinline__
#else
#define RAL_SF static inline
#endif

#define RAL_SF_SIGN 0x8000000000000000ull
#define RAL_SF_EXP 0x7ff0000000000000ull
#define RAL_SF_FRAC 0x000fffffffffffffull
#define RAL_SF_IMPL 0x0010000000000000ull

RAL_SF unsigned long long ral_sf_bits(double d) {
#if defined(__CUDA_ARCH__)
    return (unsigned long long)__double_as_longlong(d);
#else
    unsigned long long b;
    __builtin_memcpy(&b, &d, 8);
    return b;
#endif
}

// The bits of a double through an opaque move, for the functions whose tests on the bits the
// compiler would otherwise turn back into floating-point operations on the FP64 pipe (a zero test
// into an FP64 compare, a sign mask into an FP64 absolute value, an exponent test into a NaN
// compare).  Elsewhere the plain bits keep register pressure lower.
RAL_SF unsigned long long ral_sf_obits(double d) {
#if defined(__CUDA_ARCH__)
    unsigned long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(d));
    return b;
#else
    return ral_sf_bits(d);
#endif
}

RAL_SF double ral_sf_double(unsigned long long b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double d;
    __builtin_memcpy(&d, &b, 8);
    return d;
#endif
}

RAL_SF unsigned int ral_sf_fbits(float f) {
#if defined(__CUDA_ARCH__)
    return (unsigned int)__float_as_uint(f);
#else
    unsigned int b;
    __builtin_memcpy(&b, &f, 4);
    return b;
#endif
}

RAL_SF float ral_sf_float(unsigned int b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    __builtin_memcpy(&f, &b, 4);
    return f;
#endif
}

RAL_SF unsigned long long ral_sf_umulh(unsigned long long a, unsigned long long b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}

RAL_SF int ral_sf_clz64(unsigned long long x) {  // x != 0
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

// 1/x to about 22 bits (rcp.approx on the GPU: at most one ulp from 1/x).  On the host the tests
// can move the estimate by RAL_SF_TEST_RCP_ULPS ulps to show that every caller's refinement and
// correction steps hold for an estimate several ulps off.
#if !defined(__CUDA_ARCH__) && defined(RAL_SF_TEST_RCP_ULPS)
extern int ral_sf_test_rcp_ulps;
#endif
RAL_SF float ral_sf_rcp_estimate(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#elif defined(RAL_SF_TEST_RCP_ULPS)
    const float r = 1.0f / x;
    unsigned b;
    __builtin_memcpy(&b, &r, 4);
    b = (unsigned)((int)b + ral_sf_test_rcp_ulps);
    float o;
    __builtin_memcpy(&o, &b, 4);
    return o;
#else
    return 1.0f / x;
#endif
}

// ---- hardware fallbacks for the inputs outside the fast paths -----------------------------

RAL_SF double ral_sf_hw_div(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

// ---- division --------------------------------------------------------------------------------

RAL_SF unsigned int ral_sf_umulhi32(unsigned int a, unsigned int b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (unsigned int)(((unsigned long long)a * b) >> 32);
#endif
}

// a / b rounded to nearest even.
//
// With both operands normal, the significands ma, mb in [2^52, 2^53) (ma doubled when below mb,
// so ma / mb is in [1, 2)) give the quotient Q = floor(ma * 2^53 / mb) in [2^53, 2^54) and the
// remainder R = ma * 2^53 - Q * mb, from which the result rounds.  Q comes from schoolbook long
// division in two digits with a 32-bit reciprocal v ~ 2^63 / dh of the divisor's top 32 bits
// dh = mb >> 21 (Muller et al., "Handbook of Floating-Point Arithmetic", ch. 9):
//   * v: the float reciprocal of mb's top 24 bits (assembled from the float's fields, no
//     conversion instruction), then one Newton step in integer arithmetic: |v - 2^63 / dh| < 2;
//   * digit 1: q1 = umulhi(ma >> 22, v) estimates T1 = ma * 2^30 / mb within [-4, +3] units (the
//     reciprocal's error, the truncated dividend and divisor, the floor); taken 4 low, its
//     remainder R1 = ma * 2^30 - q1 * mb lies in [mb, 8 mb] < 2^56 and is exact in 64 bits;
//   * digit 2: umulhi(R1 >> 25, v) / 16 estimates T2 = R1 * 2^23 / mb (below 2^26) within
//     [-0.094, +0.063] units (the reciprocal is within 1.002 units of 2^63 / dh for every dh, the
//     dividend and divisor are truncated); taken 2/16 low and floored, q2 is floor(T2) or one less,
//     so R = R1 * 2^23 - q2 * mb (exact modulo 2^64) lies in [0, 2 mb) and needs one test.
// Only 32 x 32-bit products and 64-bit adds and shifts: no 64 x 64-bit multiply.
RAL_SF double ral_sf_div(double a, double b) {
    const unsigned long long A = ral_sf_bits(a), B = ral_sf_bits(b);
    const unsigned ea = (unsigned)(A >> 52) & 0x7ffu, eb = (unsigned)(B >> 52) & 0x7ffu;
    // fast path: both operands normal and finite
    if (ea - 1u >= 2046u || eb - 1u >= 2046u) return ral_sf_hw_div(a, b);
    unsigned long long ma = (A & RAL_SF_FRAC) | RAL_SF_IMPL;
    const unsigned long long mb = (B & RAL_SF_FRAC) | RAL_SF_IMPL;
    int e = (int)ea - (int)eb + 1023;
    if (ma < mb) {  // quotient of the significands in [1, 2)
        ma <<= 1;
        e -= 1;
    }
    const unsigned dh = (unsigned)(mb >> 21);  // in [2^31, 2^32)
    unsigned v;
    {
        // r ~ 2^31 / dh from the float 1.f of mb's top 24 bits; v0 = r * 2^32 from r's fields
        const float r = ral_sf_rcp_estimate(ral_sf_float(0x3f800000u | ((unsigned)(mb >> 29) & 0x7fffffu)));
        // r is within a few ulps of 1 / [1, 2): biased exponent 125 or 126 below 1 (the 24-bit
        // significand shifted left by 7 or 8 stays below 2^32), 127 at or above 1 (saturated)
        const unsigned rb = ral_sf_fbits(r);
        const unsigned re = (rb >> 23) & 0xffu;
        const unsigned v0 = re >= 127u ? 0xffffffffu : (((rb & 0x7fffffu) | 0x800000u) << (re - 118u));
        // Newton: v1 = v0 + v0 * (2^63 - dh * v0) / 2^63, the error term (|err| < 2^43) scaled down
        // to 22 bits so that its product with v0 is one 32 x 32-bit multiply
        const long long err = (long long)((1ull << 63) - (unsigned long long)dh * v0);
        const unsigned mag = (unsigned)((err < 0 ? 0ull - (unsigned long long)err : (unsigned long long)err) >> 21);
        const unsigned long long corr = ((unsigned long long)mag * v0) >> 42;
        long long v1 = err < 0 ? (long long)v0 - (long long)corr : (long long)v0 + (long long)corr;
        if (v1 > 0xffffffffll) v1 = 0xffffffffll;
        v = (unsigned)v1;
    }
    const unsigned q1 = ral_sf_umulhi32((unsigned)(ma >> 22), v) - 4u;
    const unsigned long long r1 = (ma << 30) - (unsigned long long)q1 * mb;          // in [mb, 8 mb]
    // the digit estimate, 2/16 low: never above floor(R1 * 2^23 / mb), at most one below it
    const unsigned q2 = (ral_sf_umulhi32((unsigned)(r1 >> 25), v) - 2u) >> 4;
    unsigned long long q = ((unsigned long long)q1 << 23) + q2;
    unsigned long long r = (r1 << 23) - (unsigned long long)q2 * mb;  // in [0, 2 mb)
    if (r >= mb) {
        q += 1;
        r -= mb;
    }
    // q in [2^53, 2^54): 53 significand bits, one rounding bit, sticky = r != 0
    unsigned long long m = q >> 1;
    m += (q & 1ull) & ((r != 0ull ? 1ull : 0ull) | (m & 1ull));
    // m in [2^52, 2^53]: added to (e - 1) << 52 it carries a rounded-up 2^53 into the exponent
    if (e <= 0 || e + (int)(m >> 53) >= 2047) return ral_sf_hw_div(a, b);  // subnormal or overflowing quotient
    return ral_sf_double(((A ^ B) & RAL_SF_SIGN) + ((unsigned long long)(e - 1) << 52) + m);
}

// An integer the compiler cannot see through.  A double chosen between two constants (0.0, 1.0,
// -1.0) by a truth value is otherwise turned into an integer -> double conversion, which runs on
// the FP64 pipe; the callers instead AND a constant's bits with an opaque mask.
RAL_SF unsigned long long ral_sf_opaque(unsigned long long x) {
#if defined(__CUDA_ARCH__)
    asm("mov.b64 %0, %1;" : "=l"(x) : "l"(x));
#endif
    return x;
}

// ---- rounding to an integer ------------------------------------------------------------------

// floor and ceil by masking the fraction bits.  With e the biased exponent: e >= 1075 is already
// integral (or infinite / NaN); below 1023 (|x| < 1) the mask covers every bit but the sign, and
// the result is the signed zero or -1 / +1; otherwise the mask covers the fraction bits below the
// binary point.  Rounding away from zero adds one unit at the binary point to the truncated bits
// (the carry may move into the exponent).
RAL_SF double ral_sf_floor(double x) {
    const unsigned long long A = ral_sf_obits(x);
    const unsigned e = (unsigned)(A >> 52) & 0x7ffu;
    if (e >= 1075u) return x;  // integral, infinite or NaN
    const bool small = e < 1023u;
    const unsigned long long mask = small ? ~RAL_SF_SIGN : (RAL_SF_FRAC >> (e - 1023u));
    if ((A & mask) == 0) return x;  // integral, or a zero
    const unsigned long long t = A & ~mask;  // truncated toward zero (a signed zero when small)
    if (!(A >> 63)) return ral_sf_double(t);
    // negative with a fraction: one unit more in magnitude (-1.0 when small)
    return ral_sf_double(small ? 0xbff0000000000000ull : t + ((mask + 1) & ~RAL_SF_SIGN));
}

RAL_SF double ral_sf_ceil(double x) {
    const unsigned long long A = ral_sf_obits(x);
    const unsigned e = (unsigned)(A >> 52) & 0x7ffu;
    if (e >= 1075u) return x;
    const bool small = e < 1023u;
    const unsigned long long mask = small ? ~RAL_SF_SIGN : (RAL_SF_FRAC >> (e - 1023u));
    if ((A & mask) == 0) return x;
    const unsigned long long t = A & ~mask;
    if (A >> 63) return ral_sf_double(t);  // negative: truncation (-0.0 when small)
    return ral_sf_double(small ? 0x3ff0000000000000ull : t + ((mask + 1) & ~RAL_SF_SIGN));
}

RAL_SF double ral_sf_fabs(double x) { return ral_sf_double(ral_sf_obits(x) & ~RAL_SF_SIGN); }

// ---- comparisons -------------------------------------------------------------------------------

RAL_SF bool ral_sf_isnan_bits(unsigned long long A) { return (A & ~RAL_SF_SIGN) > RAL_SF_EXP; }

// Order-preserving signed key of a non-NaN double; -0 and +0 share the key 0.
RAL_SF long long ral_sf_key(unsigned long long A) {
    if ((A << 1) == 0) return 0;
    return (long long)((A >> 63) ? (A ^ 0x7fffffffffffffffull) : A);
}

RAL_SF bool ral_sf_lt(double a, double b) {
    const unsigned long long A = ral_sf_obits(a), B = ral_sf_obits(b);
    return !ral_sf_isnan_bits(A) && !ral_sf_isnan_bits(B) && ral_sf_key(A) < ral_sf_key(B);
}
RAL_SF bool ral_sf_le(double a, double b) {
    const unsigned long long A = ral_sf_obits(a), B = ral_sf_obits(b);
    return !ral_sf_isnan_bits(A) && !ral_sf_isnan_bits(B) && ral_sf_key(A) <= ral_sf_key(B);
}
RAL_SF bool ral_sf_gt(double a, double b) { return ral_sf_lt(b, a); }
RAL_SF bool ral_sf_ge(double a, double b) { return ral_sf_le(b, a); }
RAL_SF bool ral_sf_eq(double a, double b) {
    const unsigned long long A = ral_sf_obits(a), B = ral_sf_obits(b);
    return !ral_sf_isnan_bits(A) && !ral_sf_isnan_bits(B) && ral_sf_key(A) == ral_sf_key(B);
}
RAL_SF bool ral_sf_ne(double a, double b) { return !ral_sf_eq(a, b); }
// x == 0.0 (either zero; NaN is not zero)
RAL_SF bool ral_sf_is_zero(double x) { return (ral_sf_obits(x) << 1) == 0; }

// ---- conversions -----------------------------------------------------------------------------

// int64 -> double, rounded to nearest even
RAL_SF double ral_sf_i2d(long long x) {
    if (x == 0) return 0.0;
    const unsigned long long s = x < 0 ? RAL_SF_SIGN : 0ull;
    const unsigned long long u = x < 0 ? 0ull - (unsigned long long)x : (unsigned long long)x;
    const int lz = ral_sf_clz64(u);
    const unsigned long long n = u << lz;  // top bit set
    unsigned long long m = n >> 11;        // 53 bits
    const unsigned long long rest = n & 0x7ffull;
    int e = 1086 - lz;
    if (rest > 0x400ull || (rest == 0x400ull && (m & 1u))) {
        m += 1;
        if (m == (1ull << 53)) {
            m >>= 1;
            e += 1;
        }
    }
    return ral_sf_double(s | ((unsigned long long)e << 52) | (m & RAL_SF_FRAC));
}

// double -> int64 as cvt.rzi.s64.f64 does it on the GPU: truncating, out of range saturates,
// NaN -> INT64_MIN
RAL_SF long long ral_sf_d2i(double d) {
    const unsigned long long A = ral_sf_obits(d);
    const int e = (int)((A >> 52) & 0x7ff);
    if (ral_sf_isnan_bits(A)) return (long long)RAL_SF_SIGN;
    if (e < 1023) return 0;
    const bool neg = (A >> 63) != 0;
    if (e >= 1023 + 63) return neg ? (long long)RAL_SF_SIGN : 0x7fffffffffffffffll;
    const unsigned long long m = (A & RAL_SF_FRAC) | RAL_SF_IMPL;
    const int sh = e - 1075;
    const unsigned long long v = sh >= 0 ? (m << sh) : (m >> (-sh));
    return neg ? (long long)(0ull - v) : (long long)v;
}

// float -> double (exact)
RAL_SF double ral_sf_f2d(float f) {
    const unsigned int F = ral_sf_fbits(f);
    const unsigned long long s = (unsigned long long)(F >> 31) << 63;
    const unsigned int e = (F >> 23) & 0xffu;
    unsigned long long m = F & 0x7fffffu;
    if (e == 0xffu) {
        // infinity, or NaN made quiet with its payload kept in the top fraction bits
        return ral_sf_double(s | RAL_SF_EXP | (m << 29) | (m ? (1ull << 51) : 0ull));
    }
    if (e == 0) {
        if (m == 0) return ral_sf_double(s);
        // subnormal float: m * 2^-149 with the leading one at bit p
        const int p = 63 - ral_sf_clz64(m);
        const unsigned long long frac = (m << (52 - p)) & RAL_SF_FRAC;
        return ral_sf_double(s | ((unsigned long long)(p - 149 + 1023) << 52) | frac);
    }
    return ral_sf_double(s | ((unsigned long long)(e + 896) << 52) | (m << 29));
}

// v >> sh rounded to nearest even (sh in 1..63)
RAL_SF unsigned long long ral_sf_shift_rne(unsigned long long v, int sh) {
    const unsigned long long q = v >> sh;
    const unsigned long long rest = v & ((1ull << sh) - 1);
    const unsigned long long half = 1ull << (sh - 1);
    return q + ((rest > half || (rest == half && (q & 1u))) ? 1u : 0u);
}

// double -> float, rounded to nearest even (overflow to infinity, subnormal results)
RAL_SF float ral_sf_d2f(double d) {
    const unsigned long long A = ral_sf_obits(d);
    const unsigned int s = (unsigned int)(A >> 63) << 31;
    const int e = (int)((A >> 52) & 0x7ff);
    const unsigned long long frac = A & RAL_SF_FRAC;
    if (e == 0x7ff) {
        // infinity, or quiet NaN with the top payload bits
        return ral_sf_float(s | 0x7f800000u | (frac ? (0x400000u | (unsigned int)(frac >> 29)) : 0u));
    }
    if (e == 0) return ral_sf_float(s);  // zero or a double subnormal (far below the float range)
    const unsigned long long m = frac | RAL_SF_IMPL;  // 53 bits
    const int ef = e - 1023 + 127;
    if (ef >= 255) return ral_sf_float(s | 0x7f800000u);
    if (ef >= 1) {
        const unsigned long long r = ral_sf_shift_rne(m, 29);  // 24 bits, or 2^24 after a carry
        // a carry out of the significand bumps the exponent through the add; 255 means infinity
        const unsigned long long bits = ((unsigned long long)ef << 23) + (r - (1ull << 23));
        return ral_sf_float(s | (bits >= 0x7f800000ull ? 0x7f800000u : (unsigned int)bits));
    }
    // subnormal float result: value = m * 2^(e - 1075), float subnormal unit 2^-149
    const int sh = 29 + (1 - ef);
    if (sh > 63) return ral_sf_float(s);
    const unsigned long long r = ral_sf_shift_rne(m, sh);  // may round up to the smallest normal
    return ral_sf_float(s | (unsigned int)r);
}

// ---- 64-bit integer division ------------------------------------------------------------------

// n / d and n % d for 1 <= d < 2^32: two 2-by-1 word divisions with a 32-bit reciprocal of the
// normalised divisor (Moller and Granlund, "Improved division by invariant integers", IEEE Trans.
// Computers 60(2), 2011, algorithm 4); the reciprocal floor((2^64 - 1) / d) - 2^32 comes from a float
// estimate and an exact integer correction.
RAL_SF unsigned int ral_sf_clz32(unsigned int x) {  // x != 0
#if defined(__CUDA_ARCH__)
    return (unsigned int)__clz((int)x);
#else
    return (unsigned int)__builtin_clz(x);
#endif
}

RAL_SF void ral_sf_div_2by1(unsigned int u1, unsigned int u0, unsigned int d, unsigned int v, unsigned int* q,
                            unsigned int* r) {
    const unsigned long long p = (unsigned long long)v * u1 + (((unsigned long long)u1 << 32) | u0);
    unsigned int q1 = (unsigned int)(p >> 32) + 1u;
    const unsigned int q0 = (unsigned int)p;
    unsigned int rr = u0 - q1 * d;
    if (rr > q0) {
        q1 -= 1u;
        rr += d;
    }
    if (rr >= d) {
        q1 += 1u;
        rr -= d;
    }
    *q = q1;
    *r = rr;
}

RAL_SF void ral_sf_udivmod64_32(unsigned long long n, unsigned int d, unsigned long long* q_out,
                                unsigned long long* r_out) {
    const unsigned int s = ral_sf_clz32(d);
    const unsigned int dn = d << s;  // top bit set
    // v0 ~ 2^64 / dn - 2^32 from a float reciprocal, assembled from its fields
    const float f = ral_sf_rcp_estimate((float)dn);                 // ~ 1 / dn, in (2^-32, 2^-31]
    const unsigned fb = ral_sf_fbits(f);
    const int sh = (int)((fb >> 23) & 0xffu) - 86;                  // f * 2^64 = (2^23 + M) << sh
    const unsigned long long big = (unsigned long long)((fb & 0x7fffffu) | 0x800000u) << (sh > 0 ? sh : 0);
    unsigned long long v0 = big > 0x1ffffffffull ? 0xffffffffull : (big < 0x100000000ull ? 0ull : big - 0x100000000ull);
    // exact: v = floor((2^64 - 1) / dn) - 2^32, i.e. e = 2^64 - 1 - (2^32 + v) dn in [0, dn)
    const unsigned long long A = ~((unsigned long long)dn << 32);
    long long e = (long long)(A - v0 * dn);
    const int adj = (int)((float)e * f);                            // ~ e / dn, |adj| < 2^13
    v0 = (unsigned long long)((long long)v0 + adj);
    e = (long long)(A - v0 * dn);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (e < 0) {
            v0 -= 1;
            e += dn;
        }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (e >= (long long)dn) {
            v0 += 1;
            e -= dn;
        }
    }
    const unsigned int v = (unsigned int)v0;
    // numerator n << s as three words; the top word is below dn
    const unsigned long long ns = n << s;
    const unsigned int w2 = s ? (unsigned int)(n >> (64 - s)) : 0u;
    unsigned int q1, q0, r;
    ral_sf_div_2by1(w2, (unsigned int)(ns >> 32), dn, v, &q1, &r);
    ral_sf_div_2by1(r, (unsigned int)ns, dn, v, &q0, &r);
    *q_out = ((unsigned long long)q1 << 32) | q0;
    *r_out = r >> s;
}


// n / d and n % d for 1 <= d < 2^16 with 32-bit operations only.  m = floor((2^32 - 1) / d) lies
// in [2^32 / d - 1, 2^32 / d], so for any 32-bit x the high word of x * m is floor(x / d) or one
// less (x * m / 2^32 > x / d - x / 2^32 > x / d - 1), and one remainder test corrects it.  The
// dividend is taken as 32 + 16 + 16 bits (32 + 16 below 2^48), most significant first (long
// division in base 2^16 after the first word): each partial remainder is below d < 2^16, so the
// next partial dividend (remainder << 16 | next 16 bits) stays below 2^32.
RAL_SF unsigned int ral_sf_divstep16(unsigned int x, unsigned int d, unsigned int m, unsigned int* r) {
    unsigned int q = ral_sf_umulhi32(x, m);
    unsigned int rr = x - q * d;  // in [0, 2d)
    if (rr >= d) {
        q += 1u;
        rr -= d;
    }
    *r = rr;
    return q;
}

// The same with m = floor((2^32 - 1) / d) given (a table of them spares the division).
RAL_SF void ral_sf_udivmod64_16m(unsigned long long n, unsigned int d, unsigned int m, unsigned long long* q_out,
                                 unsigned long long* r_out) {
    unsigned int r;
    if ((n >> 48) == 0) {  // a dividend below 2^48 (the common case) as 32 + 16 bits: two steps
        const unsigned int q1 = ral_sf_divstep16((unsigned int)(n >> 16), d, m, &r);
        const unsigned int q0 = ral_sf_divstep16((r << 16) | ((unsigned int)n & 0xffffu), d, m, &r);
        *q_out = ((unsigned long long)q1 << 16) | q0;
        *r_out = r;
        return;
    }
    const unsigned int q2 = ral_sf_divstep16((unsigned int)(n >> 32), d, m, &r);
    const unsigned int lo = (unsigned int)n;
    const unsigned int q1 = ral_sf_divstep16((r << 16) | (lo >> 16), d, m, &r);
    const unsigned int q0 = ral_sf_divstep16((r << 16) | (lo & 0xffffu), d, m, &r);
    *q_out = ((unsigned long long)q2 << 32) | ((unsigned long long)q1 << 16) | q0;
    *r_out = r;
}

RAL_SF void ral_sf_udivmod64_16(unsigned long long n, unsigned int d, unsigned long long* q_out,
                                unsigned long long* r_out) {
    ral_sf_udivmod64_16m(n, d, 0xffffffffu / d, q_out, r_out);
}

// Signed quotient and remainder (C semantics) for 1 <= |b| < 2^16; b == -1 is left to the caller.
RAL_SF long long ral_sf_div64_16(long long a, long long b) {
    const unsigned long long ua = a < 0 ? 0ull - (unsigned long long)a : (unsigned long long)a;
    const unsigned int ub = (unsigned int)(b < 0 ? 0ll - b : b);
    unsigned long long q, r;
    ral_sf_udivmod64_16(ua, ub, &q, &r);
    return ((a < 0) != (b < 0)) ? (long long)(0ull - q) : (long long)q;
}
RAL_SF long long ral_sf_mod64_16(long long a, long long b) {
    const unsigned long long ua = a < 0 ? 0ull - (unsigned long long)a : (unsigned long long)a;
    const unsigned int ub = (unsigned int)(b < 0 ? 0ll - b : b);
    unsigned long long q, r;
    ral_sf_udivmod64_16(ua, ub, &q, &r);
    return a < 0 ? (long long)(0ull - r) : (long long)r;
}

// n / d and n % d for d >= 1, exactly, by the same reciprocal method: a float seed for
// 2^127 / (d normalised), two Newton steps in 64-bit fixed point, a quotient estimate within a
// few units and an exact correction from the remainder.
RAL_SF void ral_sf_udivmod64(unsigned long long n, unsigned long long d, unsigned long long* q_out,
                             unsigned long long* r_out) {
    if (d > n) {
        *q_out = 0;
        *r_out = n;
        return;
    }
    if ((n >> 32) == 0) {  // both fit in 32 bits: the 32-bit division
        const unsigned q32 = (unsigned)n / (unsigned)d;
        *q_out = q32;
        *r_out = n - (unsigned long long)q32 * d;
        return;
    }
    if ((d >> 32) == 0) {  // 32-bit divisor: two word divisions
        ral_sf_udivmod64_32(n, (unsigned int)d, q_out, r_out);
        return;
    }
    if (d >> 63) {  // d >= 2^63 and d <= n: the quotient is 1
        *q_out = 1;
        *r_out = n - d;
        return;
    }
    const int s = ral_sf_clz64(d);  // >= 1
    const unsigned long long dn = d << s;
    const float seed = ral_sf_rcp_estimate((float)(unsigned)(dn >> 40));  // ~ 2^40 / dn
    const unsigned sb = ral_sf_fbits(seed);
    const int sh = (int)((sb >> 23) & 0xffu) - 63;
    const unsigned long long sm = (unsigned long long)((sb & 0x7fffffu) | 0x800000u);
    unsigned long long y = sh >= 41 ? 0xffffffffffffffffull : (sh <= 0 ? sm : sm << sh);  // ~ 2^127 / dn
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const unsigned long long plo = dn * y, phi = ral_sf_umulh(dn, y);
        const unsigned long long p63 = (phi << 1) | (plo >> 63);  // (dn * y) >> 63, mod 2^64
        const long long err = (long long)(0ull - p63);            // (2^127 - dn * y) >> 63
        const unsigned long long mag = err < 0 ? (0ull - (unsigned long long)err) : (unsigned long long)err;
        const unsigned long long corr = ral_sf_umulh(y, mag);
        y = err < 0 ? y - corr : y + corr;
    }
    // n / d = n * 2^s / dn ~ (n * y) >> (127 - s)
    unsigned long long q = ral_sf_umulh(n, y) >> (63 - s);
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // too large: q * d > n
        if (ral_sf_umulh(q, d) != 0 || q * d > n) q -= 1;
    }
    unsigned long long r = n - q * d;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (r >= d) {
            q += 1;
            r -= d;
        }
    }
    *q_out = q;
    *r_out = r;
}

// Signed quotient and remainder with C semantics (truncation; the remainder takes the
// dividend's sign); d == 0 and d == -1 are left to the caller.
RAL_SF long long ral_sf_div64(long long a, long long b) {
    const unsigned long long ua = a < 0 ? 0ull - (unsigned long long)a : (unsigned long long)a;
    const unsigned long long ub = b < 0 ? 0ull - (unsigned long long)b : (unsigned long long)b;
    unsigned long long q, r;
    ral_sf_udivmod64(ua, ub, &q, &r);
    return ((a < 0) != (b < 0)) ? (long long)(0ull - q) : (long long)q;
}
RAL_SF long long ral_sf_mod64(long long a, long long b) {
    const unsigned long long ua = a < 0 ? 0ull - (unsigned long long)a : (unsigned long long)a;
    const unsigned long long ub = b < 0 ? 0ull - (unsigned long long)b : (unsigned long long)b;
    unsigned long long q, r;
    ral_sf_udivmod64(ua, ub, &q, &r);
    return a < 0 ? (long long)(0ull - r) : (long long)r;
}

// ---- 64-bit integer division by an invariant divisor -------------------------------------------
//
// n / d and n % d (C semantics: truncation, the remainder takes the dividend's sign) for a divisor
// known before the kernel runs, a literal of the program.  The host finds a multiplier M and a shift
// s once; then trunc(n / d) = (high word of M * n, plus n when d > 0 > M, minus n when d < 0 < M)
// shifted right arithmetically by s, plus one when that is negative (Granlund and Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994; the signed multiplier search
// of Warren, "Hacker's Delight", 2nd ed., section 10-4, carried to 64 bits).  Divisors without a
// multiplier (0, 1, -1, INT64_MIN) are marked by a mode in the shift word and handled directly, with
// this library's values for the undefined cases: x / 0 = x % 0 = 0, INT64_MIN / -1 = INT64_MIN.
struct RalDivider {
    long long mult;
    long long shift_mode;  // bits 0-7: s; bits 8+: 0 multiplier, 1 d = 0, 2 d = 1, 3 d = -1, 4 d = INT64_MIN
};

RAL_SF RalDivider ral_sf_make_divider(long long d) {
    RalDivider v{0, 0};
    if (d == 0 || d == 1 || d == -1 || d == (long long)RAL_SF_SIGN) {
        v.shift_mode = (long long)(d == 0 ? 1 : d == 1 ? 2 : d == -1 ? 3 : 4) << 8;
        return v;
    }
    const unsigned long long two63 = RAL_SF_SIGN;
    const unsigned long long ad = d < 0 ? 0ull - (unsigned long long)d : (unsigned long long)d;
    const unsigned long long t = two63 + ((unsigned long long)d >> 63);
    const unsigned long long anc = t - 1 - t % ad;  // |nc|: the largest dividend with nc % ad == ad - 1
    int p = 63;
    unsigned long long q1 = two63 / anc, r1 = two63 - q1 * anc;  // 2^p / |nc|
    unsigned long long q2 = two63 / ad, r2 = two63 - q2 * ad;    // 2^p / |d|
    unsigned long long delta;
    do {
        p += 1;
        q1 <<= 1;
        r1 <<= 1;
        if (r1 >= anc) {
            q1 += 1;
            r1 -= anc;
        }
        q2 <<= 1;
        r2 <<= 1;
        if (r2 >= ad) {
            q2 += 1;
            r2 -= ad;
        }
        delta = ad - r2;
    } while (q1 < delta || (q1 == delta && r1 == 0));
    const unsigned long long m = q2 + 1;
    v.mult = (long long)(d < 0 ? 0ull - m : m);
    v.shift_mode = p - 64;
    return v;
}

RAL_SF long long ral_sf_mulhs(long long a, long long b) {
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    return (long long)(((__int128)a * b) >> 64);
#endif
}

RAL_SF long long ral_sf_divc(long long n, long long d, long long mult, long long shift_mode) {
    const int mode = (int)(shift_mode >> 8);
    if (mode != 0) {
        if (mode == 1) return 0;
        if (mode == 2) return n;
        if (mode == 3) return (long long)(0ull - (unsigned long long)n);
        return n == (long long)RAL_SF_SIGN ? 1 : 0;
    }
    unsigned long long q = (unsigned long long)ral_sf_mulhs(mult, n);
    if (d > 0 && mult < 0) q += (unsigned long long)n;
    else if (d < 0 && mult > 0) q -= (unsigned long long)n;
    long long qs = (long long)q >> (int)(shift_mode & 0xff);
    return qs + (long long)((unsigned long long)qs >> 63);
}

RAL_SF long long ral_sf_modc(long long n, long long d, long long mult, long long shift_mode) {
    if ((shift_mode >> 8) == 1) return 0;  // d == 0
    const long long q = ral_sf_divc(n, d, mult, shift_mode);
    return (long long)((unsigned long long)n - (unsigned long long)q * (unsigned long long)d);
}

// ---- sine and cosine ---------------------------------------------------------------------------

// 64-bit value V (a leading one anywhere) times 2^E, rounded to nearest even as a double (normal
// results only; the callers' values lie in [2^-30, 2])
RAL_SF double ral_sf_pack(unsigned long long V, int E, unsigned long long sign) {
    const int lz = ral_sf_clz64(V);
    V <<= lz;
    E -= lz;
    unsigned long long m = V >> 11;
    const unsigned long long rest = V & 0x7ffull;
    if (rest > 0x400ull || (rest == 0x400ull && (m & 1u))) m += 1;
    int be = E + 63 + 1023;
    if (m == (1ull << 53)) {
        m >>= 1;
        be += 1;
    }
    return ral_sf_double(sign | ((unsigned long long)be << 52) | (m & RAL_SF_FRAC));
}

// Fixed-point constants, each the nearest (or, for 2/pi and pi/2, the truncated) value:
// 2/pi * 2^192 in three words, pi/2 * 2^127 in two words, and 2^63 / n! for the Taylor series
// sin(r)/r = sum (-1)^n r^(2n) / (2n+1)!  and  cos(r) = sum (-1)^n r^(2n) / (2n)!.
#define RAL_SF_2PI_W2 0xa2f9836e4e441529ull
#define RAL_SF_2PI_W1 0xfc2757d1f534ddc0ull
#define RAL_SF_2PI_W0 0xdb6295993c439041ull
#define RAL_SF_PI2_HI 0xc90fdaa22168c234ull
#define RAL_SF_PI2_LO 0xc4c6628b80dc1cd1ull

// sin(|r|) (want_cos false) or cos(|r|) for r = rm * 2^-(64 + sr), rm normalised, |r| <= pi/4
RAL_SF double ral_sf_sincos_poly(unsigned long long rm, int sr, bool want_cos, unsigned long long sign) {
    const unsigned long long zz = ral_sf_umulh(rm, rm);  // r^2 * 2^(64 + 2 sr)
    const unsigned long long z = 2 * sr >= 64 ? 0ull : (zz >> (2 * sr));  // r^2 in Q0.64
    if (want_cos) {
        // 2^63 / (2n)!, n = 10 .. 0
        const unsigned long long c[11] = {0x8000000000000000ull, 0x4000000000000000ull, 0x0555555555555555ull,
                                          0x002d82d82d82d82eull, 0x0000d00d00d00d01ull, 0x0000024fc9f6ef14ull,
                                          0x000000047bb63bfeull, 0x00000000064e5d2aull, 0x000000000006b9fdull,
                                          0x00000000000005a1ull, 0x0000000000000004ull};
        unsigned long long p = c[10];
#pragma unroll
        for (int n = 9; n >= 0; --n) p = c[n] - ral_sf_umulh(p, z);
        return ral_sf_pack(p, -63, sign);
    }
    // 2^63 / (2n+1)!, n = 9 .. 0
    const unsigned long long c[10] = {0x8000000000000000ull, 0x1555555555555555ull, 0x0111111111111111ull,
                                      0x0006806806806807ull, 0x0000171de3a556c7ull, 0x00000035cc8acfebull,
                                      0x000000005849184full, 0x00000000006b9fd0ull, 0x000000000000654bull,
                                      0x000000000000004cull};
    unsigned long long p = c[9];
#pragma unroll
    for (int n = 8; n >= 0; --n) p = c[n] - ral_sf_umulh(p, z);
    // sin(r) = r * p: value = umulh(rm, p) * 2^(-63 - sr)
    return ral_sf_pack(ral_sf_umulh(rm, p), -63 - sr, sign);
}

RAL_SF double ral_sf_hw_sin(double x) {
#if defined(__CUDA_ARCH__)
    return sin(x);
#else
    return __builtin_sin(x);
#endif
}
RAL_SF double ral_sf_hw_cos(double x) {
#if defined(__CUDA_ARCH__)
    return cos(x);
#else
    return __builtin_cos(x);
#endif
}

// sin(x) (want_cos false) or cos(x) within one ulp, for 2^-26 <= |x| < 2^20; other inputs use
// the library functions.  Method: Payne-Hanek-style reduction x * 2/pi = k + f with a 192-bit
// fixed-point 2/pi (exact product with the 53-bit significand), r = f * pi/2 to 128 bits, then
// the Taylor series of sin(r)/r or cos(r) in 64-bit fixed point by Horner's rule.
RAL_SF double ral_sf_sincos(double x, bool want_cos) {
    const unsigned long long X = ral_sf_obits(x);
    const int ex = (int)((X >> 52) & 0x7ff);
    const unsigned long long xsign = X & RAL_SF_SIGN;
    if (ex < 1023 - 26 || ex >= 1023 + 20) return want_cos ? ral_sf_hw_cos(x) : ral_sf_hw_sin(x);
    const unsigned long long m = (X & RAL_SF_FRAC) | RAL_SF_IMPL;
    const int e2 = ex - 1075;  // x = m * 2^e2
    unsigned long long rm;
    int sr;
    unsigned q;
    bool rneg = false;
    if ((X & ~RAL_SF_SIGN) < 0x3fe921fb54442d18ull) {  // |x| < pi/4: r = x exactly
        rm = m << 11;
        sr = -53 - e2;
        q = 0;
    } else {
        // P = m * (2/pi * 2^192), four words
        const unsigned long long t0 = m * RAL_SF_2PI_W0, h0 = ral_sf_umulh(m, RAL_SF_2PI_W0);
        const unsigned long long t1 = m * RAL_SF_2PI_W1, h1 = ral_sf_umulh(m, RAL_SF_2PI_W1);
        const unsigned long long t2 = m * RAL_SF_2PI_W2, h2 = ral_sf_umulh(m, RAL_SF_2PI_W2);
        (void)t0;
        const unsigned long long p1 = h0 + t1;
        const unsigned long long a1 = p1 < h0 ? 1ull : 0ull;
        const unsigned long long s2 = h1 + t2;
        const unsigned long long a2a = s2 < h1 ? 1ull : 0ull;
        const unsigned long long p2 = s2 + a1;
        const unsigned long long a2 = a2a + (p2 < s2 ? 1ull : 0ull);
        const unsigned long long p3 = h2 + a2;
        // x * 2/pi = P * 2^(e2 - 192): sh = 192 - e2 fraction bits, v = sh - 192 in [33, 53]
        const int v = -e2;
        unsigned long long k = p3 >> v;
        unsigned long long fhi = (p2 >> v) | (p3 << (64 - v));
        unsigned long long flo = (p1 >> v) | (p2 << (64 - v));
        if (fhi >> 63) {  // f >= 1/2: the nearer quadrant is k + 1, and r = (f - 1) pi/2 < 0
            k += 1;
            flo = 0ull - flo;
            fhi = ~fhi + (flo == 0 ? 1ull : 0ull);
            rneg = true;
        }
        q = (unsigned)(k & 3u);
        // r = f * pi/2 in Q0.128: (f * pi2) >> 127, from the three high partial products
        const unsigned long long ac_lo = fhi * RAL_SF_PI2_HI, ac_hi = ral_sf_umulh(fhi, RAL_SF_PI2_HI);
        const unsigned long long ad = ral_sf_umulh(fhi, RAL_SF_PI2_LO), bc = ral_sf_umulh(flo, RAL_SF_PI2_HI);
        unsigned long long lo = ac_lo + ad;
        unsigned long long hi = ac_hi + (lo < ac_lo ? 1ull : 0ull);
        const unsigned long long lo2 = lo + bc;
        hi += lo2 < lo ? 1ull : 0ull;
        lo = lo2;
        const unsigned long long rhi = (hi << 1) | (lo >> 63), rlo = lo << 1;
        if (rhi != 0) {
            const int lz = ral_sf_clz64(rhi);
            rm = lz ? ((rhi << lz) | (rlo >> (64 - lz))) : rhi;
            sr = lz;
        } else {
            if (rlo == 0) return want_cos ? ral_sf_hw_cos(x) : ral_sf_hw_sin(x);
            const int lz = ral_sf_clz64(rlo);
            rm = rlo << lz;
            sr = 64 + lz;
        }
    }
    // quadrant: sin(x) = [s, c, -s, -c][q], cos(x) = [c, -s, -c, s][q] with s = sin r, c = cos r
    const bool use_cos = want_cos ? (q & 1u) == 0 : (q & 1u) == 1;
    bool neg;
    if (want_cos) neg = (q == 1 || q == 2);
    else neg = (q >= 2);
    if (!use_cos && rneg) neg = !neg;               // sin(-|r|) = -sin|r|
    if (!want_cos && xsign) neg = !neg;             // sin(-x) = -sin x; cos is even
    return ral_sf_sincos_poly(rm, sr, use_cos, neg ? RAL_SF_SIGN : 0ull);
}

RAL_SF double ral_sf_sin(double x) { return ral_sf_sincos(x, false); }
RAL_SF double ral_sf_cos(double x) { return ral_sf_sincos(x, true); }

#endif  // RAL_SOFTFP_CUH_
