// device_rt.cuh — device-side building blocks of the generated expression kernels.
//
// This file is compiled twice: by NVRTC as the prelude of every generated
// kernel (embedded into the library as a string at build time, after
// softfp.cuh), and by nvcc as part of the ahead-of-time kernels.  Under NVRTC
// it includes nothing, so that NVRTC needs no include path.
//
// Arithmetic follows the reference interpreter's C++ semantics on {int64,
// double} registers (src/Interpreter/interpreter_ops.cuh:574-838): explicit
// _rn intrinsics keep every double operation separately rounded (never
// contracted into an FMA), integer add/sub/mul wrap, double->int64 truncates
// and saturates with NaN -> INT64_MIN (cvt.rzi.s64.f64 on the GPU).
#ifndef RAL_DEVICE_RT_CUH_
#define RAL_DEVICE_RT_CUH_

typedef long long ral_i64;
typedef unsigned long long ral_u64;
typedef unsigned int ral_u32;

#define RAL_FI __device__ __forceinline__

// ---- double operations that have integer-pipe versions -----------------------------------
// RAL_SOFT_FP 1 (the default): division, floor / ceil / fabs, comparisons and the conversions
// run as the exact integer-arithmetic versions of softfp.cuh, which leave the FP64 pipe to add,
// subtract and multiply; 0: the hardware instructions.  Both give the same bits.
#ifndef RAL_SOFT_FP
#define RAL_SOFT_FP 1
#endif
#ifndef RAL_SOFTFP_CUH_
#include "softfp.cuh"
#endif
#if RAL_SOFT_FP
RAL_FI ral_i64 ral_d2i(double d) { return ral_sf_d2i(d); }
RAL_FI double ral_i2d(ral_i64 x) { return ral_sf_i2d(x); }
RAL_FI double ral_ddiv(double a, double b) { return ral_sf_div(a, b); }
// RAL_SOFT_ROUND 0: floor / ceil by the FP64 pipe's rounding instruction (one FP64 instruction
// against ~28 integer ones; same bits), the other operations staying on the integer pipes
#ifndef RAL_SOFT_ROUND
#define RAL_SOFT_ROUND 1
#endif
#if RAL_SOFT_ROUND
RAL_FI double ral_dfloor(double x) { return ral_sf_floor(x); }
RAL_FI double ral_dceil(double x) { return ral_sf_ceil(x); }
#else
RAL_FI double ral_dfloor(double x) { return floor(x); }
RAL_FI double ral_dceil(double x) { return ceil(x); }
#endif
RAL_FI bool ral_dlt(double a, double b) { return ral_sf_lt(a, b); }
RAL_FI bool ral_dle(double a, double b) { return ral_sf_le(a, b); }
RAL_FI bool ral_dgt(double a, double b) { return ral_sf_gt(a, b); }
RAL_FI bool ral_dge(double a, double b) { return ral_sf_ge(a, b); }
RAL_FI bool ral_deq(double a, double b) { return ral_sf_eq(a, b); }
RAL_FI bool ral_dne(double a, double b) { return ral_sf_ne(a, b); }
RAL_FI double ral_f2d(float f) { return ral_sf_f2d(f); }
RAL_FI float ral_d2f(double d) { return ral_sf_d2f(d); }
#else
RAL_FI ral_i64 ral_d2i(double d) { return __double2ll_rz(d); }
RAL_FI double ral_i2d(ral_i64 x) { return __ll2double_rn(x); }
RAL_FI double ral_ddiv(double a, double b) { return __ddiv_rn(a, b); }
RAL_FI double ral_dfloor(double x) { return floor(x); }
RAL_FI double ral_dceil(double x) { return ceil(x); }
RAL_FI bool ral_dlt(double a, double b) { return a < b; }
RAL_FI bool ral_dle(double a, double b) { return a <= b; }
RAL_FI bool ral_dgt(double a, double b) { return a > b; }
RAL_FI bool ral_dge(double a, double b) { return a >= b; }
RAL_FI bool ral_deq(double a, double b) { return a == b; }
RAL_FI bool ral_dne(double a, double b) { return a != b; }
RAL_FI double ral_f2d(float f) { return (double)f; }
RAL_FI float ral_d2f(double d) { return __double2float_rn(d); }
#endif
// sin / cos: RAL_SOFT_TRIG 0 (the default) uses the library functions, 1 the integer-pipe
// versions of softfp.cuh (within one ulp).  Unlike the exact operations above the two differ in
// the last bit, so the choice is the same for every kernel of a process.  Measured on GB300 the
// library functions are faster: the 256-program mix ran 138 ms batched / 158 ms as plain calls
// with them and 155 / 172 ms with the integer-pipe versions (whose two polynomial paths diverge
// within a warp by quadrant).
#ifndef RAL_SOFT_TRIG
#define RAL_SOFT_TRIG 0
#endif
#if RAL_SOFT_TRIG
RAL_FI double ral_dsin(double x) { return ral_sf_sin(x); }
RAL_FI double ral_dcos(double x) { return ral_sf_cos(x); }
#else
RAL_FI double ral_dsin(double x) { return sin(x); }
RAL_FI double ral_dcos(double x) { return cos(x); }
#endif
RAL_FI double ral_dfabs(double x) { return ral_sf_fabs(x); }
RAL_FI bool ral_dzero(double x) { return ral_sf_is_zero(x); }
RAL_FI double ral_bits_d(ral_i64 b) { return __longlong_as_double(b); }
RAL_FI ral_i64 ral_d_bits(double d) { return __double_as_longlong(d); }
// a truth value as 1.0 / 0.0 from the bits of 1.0 and an opaque mask (a select between the two
// constants is turned into an integer -> double conversion on the FP64 pipe)
RAL_FI double ral_b2d(bool b) {
    return __longlong_as_double((long long)(ral_sf_opaque(0ull - (ral_u64)b) & 0x3ff0000000000000ull));
}
// (one ? 1.0 : 0.0) * x, the same bits as the multiply: a finite x times 1.0 is x and times 0.0
// is a zero with x's sign; an infinite or NaN x takes the FP64 instruction (NaN, or inf * 1.0).
// The 0/1 operand comes from a comparison or a logical operator of the program.  The rare case is
// a call, so that the compiler does not issue its multiply, predicated off, for every row.
static __device__ __noinline__ double ral_dmul_rare(double a, double b) { return __dmul_rn(a, b); }
RAL_FI double ral_dmul01(bool one, double x) {
    const ral_u64 b = ral_sf_bits(x);
    if ((b & 0x7ff0000000000000ull) == 0x7ff0000000000000ull) return ral_dmul_rare(ral_b2d(one), x);
    return one ? x : __longlong_as_double((long long)(b & 0x8000000000000000ull));
}

// ---- integer ops (two's complement wrap, as the GPU executes them) -------------------------
RAL_FI ral_i64 ral_addi(ral_i64 a, ral_i64 b) { return (ral_i64)((ral_u64)a + (ral_u64)b); }
RAL_FI ral_i64 ral_subi(ral_i64 a, ral_i64 b) { return (ral_i64)((ral_u64)a - (ral_u64)b); }
RAL_FI ral_i64 ral_muli(ral_i64 a, ral_i64 b) { return (ral_i64)((ral_u64)a * (ral_u64)b); }
// Integer division by zero, and INT64_MIN / -1, are undefined in the reference (plain C++ `/`
// and `%` in device code).  Here they are defined, identically in every kernel: x / 0 = 0,
// x % 0 = 0, INT64_MIN / -1 = INT64_MIN (wrap), x % -1 = 0.  Without the guards the result
// would depend on how the compiler happened to treat the undefined case.
// The quotient and remainder themselves: RAL_SOFT_INT_DIV 3 (the default) divides by divisors
// below 2^16 with three 32-bit word steps (ral_sf_udivmod64_16) and by larger ones with the
// compiler's 64-bit division, whose reciprocal step runs on the FP64 pipe; 0 uses the compiler's
// for every divisor; 2 uses the 2-by-1 word division of softfp.cuh for divisors that fit in 32
// bits; 1 uses the integer-only division for every divisor.  All are exact.  Measured on the
// 12-op projection (200M rows, divisors in [1, 1000]): 3 = 3.32 ms, 0 = 3.78 ms, 2 = 3.97 ms,
// 1 = 4.6 ms -- the 2-by-1 and Newton versions free the FP64 pipe but cost more integer work
// than they save there; the word steps cost little of either.
#ifndef RAL_SOFT_INT_DIV
#define RAL_SOFT_INT_DIV 3
#endif
RAL_FI bool ral_small_divisor(ral_i64 b) {
    const ral_u64 m = b < 0 ? 0ull - (ral_u64)b : (ral_u64)b;
    return m <= 0xffffffffull;
}
RAL_FI bool ral_tiny_divisor(ral_i64 b) {
    const ral_u64 m = b < 0 ? 0ull - (ral_u64)b : (ral_u64)b;
    return m < 0x10000ull;
}
RAL_FI ral_i64 ral_divi(ral_i64 a, ral_i64 b) {
    if (b == 0) return 0;
    if (b == -1) return (ral_i64)(0ull - (ral_u64)a);
#if RAL_SOFT_INT_DIV == 1
    return ral_sf_div64(a, b);
#elif RAL_SOFT_INT_DIV == 2
    return ral_small_divisor(b) ? ral_sf_div64(a, b) : a / b;
#elif RAL_SOFT_INT_DIV == 3
    return ral_tiny_divisor(b) ? ral_sf_div64_16(a, b) : a / b;
#else
    return a / b;
#endif
}
RAL_FI ral_i64 ral_modi(ral_i64 a, ral_i64 b) {
    if (b == 0 || b == -1) return 0;
#if RAL_SOFT_INT_DIV == 1
    return ral_sf_mod64(a, b);
#elif RAL_SOFT_INT_DIV == 2
    return ral_small_divisor(b) ? ral_sf_mod64(a, b) : a % b;
#elif RAL_SOFT_INT_DIV == 3
    return ral_tiny_divisor(b) ? ral_sf_mod64_16(a, b) : a % b;
#else
    return a % b;
#endif
}
// ral_divi / ral_modi for kernels that keep the reciprocals m(d) = floor((2^32 - 1) / d) of the
// divisors below RAL_RCP_TAB in a shared-memory table (the eval kernel of a program that divides
// by a column): m is the table's entry for |b|, or 0 when |b| is not below RAL_RCP_TAB (then the
// compiler's division).  Same results as ral_divi / ral_modi.
#define RAL_RCP_TAB 4096
// the rare divisors outside the table, out of line: they do not add to the caller's registers
static __device__ __noinline__ ral_i64 ral_div_wide(ral_i64 a, ral_i64 b) { return a / b; }
static __device__ __noinline__ ral_i64 ral_mod_wide(ral_i64 a, ral_i64 b) { return a % b; }
RAL_FI ral_i64 ral_divi_m(ral_i64 a, ral_i64 b, unsigned m) {
    if (b == 0) return 0;
    if (b == -1) return (ral_i64)(0ull - (ral_u64)a);
    if (m == 0u) return ral_div_wide(a, b);
    const ral_u64 ua = a < 0 ? 0ull - (ral_u64)a : (ral_u64)a;
    const unsigned ub = (unsigned)(b < 0 ? 0ll - b : b);
    unsigned long long q, r;
    ral_sf_udivmod64_16m(ua, ub, m, &q, &r);
    return ((a < 0) != (b < 0)) ? (ral_i64)(0ull - q) : (ral_i64)q;
}
RAL_FI ral_i64 ral_modi_m(ral_i64 a, ral_i64 b, unsigned m) {
    if (b == 0 || b == -1) return 0;
    if (m == 0u) return ral_mod_wide(a, b);
    const ral_u64 ua = a < 0 ? 0ull - (ral_u64)a : (ral_u64)a;
    const unsigned ub = (unsigned)(b < 0 ? 0ll - b : b);
    unsigned long long q, r;
    ral_sf_udivmod64_16m(ua, ub, m, &q, &r);
    return a < 0 ? (ral_i64)(0ull - r) : (ral_i64)r;
}
// Integer POWER: the reference multiplies `base` into 1, `e` times (e <= 0 -> 1);
// square-and-multiply gives the same value modulo 2^64.
RAL_FI ral_i64 ral_powi(ral_i64 base, ral_i64 e) {
    ral_u64 acc = 1, b = (ral_u64)base;
    if (e <= 0) return 1;
    ral_u64 ue = (ral_u64)e;
    while (ue) {
        if (ue & 1ull) acc *= b;
        b *= b;
        ue >>= 1;
    }
    return (ral_i64)acc;
}

// ---- calendar extraction (interpreter_ops.cuh:61-153) --------------------------------------
// Days-from-civil inverse on 32-bit int / unsigned arithmetic as written there.
// Every signed add/sub/mul that can overflow for out-of-range inputs is done in
// unsigned arithmetic, i.e. it wraps the way the GPU's integer instructions do.
struct RalCivil { ral_i64 y, m, d; };
RAL_FI int ral_wadd(int a, int b) { return (int)((unsigned)a + (unsigned)b); }
RAL_FI int ral_wmul(int a, int b) { return (int)((unsigned)a * (unsigned)b); }
RAL_FI RalCivil ral_civil(int z) {
    const int era = (z >= 0 ? z : ral_wadd(z, -146096)) / 146097;
    const unsigned doe = (unsigned)ral_wadd(z, -ral_wmul(era, 146097));
    const unsigned yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
    const int y = ral_wadd((int)yoe, ral_wmul(era, 400));
    const unsigned doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
    const unsigned mp = (5 * doy + 2) / 153;
    const unsigned m = mp + (mp < 10 ? 3u : (unsigned)-9);
    RalCivil c;
    c.y = (m <= 2) ? (ral_i64)y + 1 : (ral_i64)y;
    c.m = (ral_i64)m;
    c.d = (ral_i64)(doy - (153 * mp + 2) / 5 + 1);
    return c;
}
#define RAL_MS_DAY 86400000ll
#define RAL_MS_HOUR 3600000ll
#define RAL_MS_MINUTE 60000ll
#define RAL_MS_SECOND 1000ll
RAL_FI int ral_z_days(ral_i64 d) { return (int)(unsigned)((ral_u64)d + 719468ull); }
RAL_FI int ral_z_ms(ral_i64 t) {
    const ral_i64 a = t >= 0 ? t : (ral_i64)((ral_u64)t - (ral_u64)(RAL_MS_DAY - 1));
    return (int)(unsigned)((ral_u64)(a / RAL_MS_DAY) + 719468ull);
}
RAL_FI ral_i64 ral_year32(ral_i64 d) { return ral_civil(ral_z_days(d)).y; }
RAL_FI ral_i64 ral_month32(ral_i64 d) { return ral_civil(ral_z_days(d)).m; }
RAL_FI ral_i64 ral_day32(ral_i64 d) { return ral_civil(ral_z_days(d)).d; }
RAL_FI ral_i64 ral_year64(ral_i64 t) { return ral_civil(ral_z_ms(t)).y; }
RAL_FI ral_i64 ral_month64(ral_i64 t) { return ral_civil(ral_z_ms(t)).m; }
RAL_FI ral_i64 ral_day64(ral_i64 t) { return ral_civil(ral_z_ms(t)).d; }
RAL_FI ral_i64 ral_hour64(ral_i64 t) {
    return t >= 0 ? ((t % RAL_MS_DAY) / RAL_MS_HOUR) : ((RAL_MS_DAY + (t % RAL_MS_DAY)) / RAL_MS_HOUR);
}
RAL_FI ral_i64 ral_minute64(ral_i64 t) {
    return t >= 0 ? ((t % RAL_MS_HOUR) / RAL_MS_MINUTE) : ((RAL_MS_HOUR + (t % RAL_MS_HOUR)) / RAL_MS_MINUTE);
}
RAL_FI ral_i64 ral_second64(ral_i64 t) {
    return t >= 0 ? ((t % RAL_MS_MINUTE) / RAL_MS_SECOND) : ((RAL_MS_MINUTE + (t % RAL_MS_MINUTE)) / RAL_MS_SECOND);
}

// ---- L2 prefetch of a contiguous range (one bulk request; 16-byte aligned start, size a
// multiple of 16, within the allocation) -----------------------------------------------------
RAL_FI void ral_prefetch_l2(const void* p, unsigned bytes) {
    if (bytes < 16u) return;
    unsigned long long g;
    asm("cvta.to.global.u64 %0, %1;" : "=l"(g) : "l"(p));
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(g), "r"(bytes) : "memory");
}

// ---- vector loads / stores of G consecutive elements ---------------------------------------
template <int BYTES> struct RalVecT;
template <> struct RalVecT<16> { typedef uint4 T; };
template <> struct RalVecT<8> { typedef uint2 T; };
template <> struct RalVecT<4> { typedef unsigned int T; };
template <> struct RalVecT<2> { typedef unsigned short T; };
template <> struct RalVecT<1> { typedef unsigned char T; };

// Streaming load of G elements starting at p[row]; p + row must be aligned to G*sizeof(E).
template <typename E, int G>
RAL_FI void ral_ldg(const E* __restrict__ p, ral_i64 row, E (&v)[G]) {
    typedef typename RalVecT<sizeof(E) * G>::T V;
    union { V vec; E e[G]; } u;
    u.vec = __ldcs(reinterpret_cast<const V*>(p + row));
#pragma unroll
    for (int g = 0; g < G; ++g) v[g] = u.e[g];
}
// Same, through the read-only cache with normal eviction: for data read again soon.
template <typename E, int G>
RAL_FI void ral_ldg_keep(const E* __restrict__ p, ral_i64 row, E (&v)[G]) {
    typedef typename RalVecT<sizeof(E) * G>::T V;
    union { V vec; E e[G]; } u;
    u.vec = __ldg(reinterpret_cast<const V*>(p + row));
#pragma unroll
    for (int g = 0; g < G; ++g) v[g] = u.e[g];
}
template <typename E, int G>
RAL_FI void ral_stg(E* __restrict__ p, ral_i64 row, const E (&v)[G]) {
    typedef typename RalVecT<sizeof(E) * G>::T V;
    union { V vec; E e[G]; } u;
#pragma unroll
    for (int g = 0; g < G; ++g) u.e[g] = v[g];
    __stcs(reinterpret_cast<V*>(p + row), u.vec);
}

// ---- bulk copies into shared memory (TMA) completing on an mbarrier ---------------------------
// A warp's stage of a staged kernel is filled by one lane: arrive.expect_tx announces the bytes,
// then one cp.async.bulk per contiguous range (16-byte aligned addresses, size a multiple of 16)
// completes them; the warp waits on the barrier's phase parity.  Waits are bounded: after
// RAL_STAGE_SPIN_LIMIT polls the wait gives up and reports it.
#define RAL_STAGE_SPIN_LIMIT (1l << 20)
RAL_FI unsigned ral_smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
RAL_FI void ral_mbar_init(ral_u64* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(ral_smem_u32(bar)), "r"(count) : "memory");
}
RAL_FI void ral_mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
RAL_FI void ral_mbar_expect_tx(ral_u64* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ral_smem_u32(bar)), "r"(bytes)
                 : "memory");
}
RAL_FI void ral_bulk_g2s(void* dst, const void* src, unsigned bytes, ral_u64* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(ral_smem_u32(dst)), "l"(src), "r"(bytes), "r"(ral_smem_u32(bar))
                 : "memory");
}
RAL_FI bool ral_mbar_test(ral_u64* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(ral_smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// true when the phase completed; false after the spin limit
RAL_FI bool ral_mbar_wait(ral_u64* bar, unsigned parity) {
    for (long spins = 0; spins < RAL_STAGE_SPIN_LIMIT; ++spins)
        if (ral_mbar_test(bar, parity)) return true;
    return false;
}
// Vector load of G consecutive elements from shared memory (the staged copy of a column).
template <typename E, int G>
RAL_FI void ral_lds(const E* p, int row, E (&v)[G]) {
    typedef typename RalVecT<sizeof(E) * G>::T V;
    union { V vec; E e[G]; } u;
    u.vec = *reinterpret_cast<const V*>(p + row);
#pragma unroll
    for (int g = 0; g < G; ++g) v[g] = u.e[g];
}

// ---- status-word access for the single-pass scan --------------------------------------------
// A tile's status word carries its own value, and nothing else is published through it, so
// relaxed gpu-scope accesses suffice: a store needs no fence (which would wait for the
// tile's outstanding data stores) and a load reads the coherent copy in L2.
RAL_FI ral_u64 ral_ld_status(const ral_u64* p) {
    ral_u64 v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
RAL_FI void ral_st_status(ral_u64* p, ral_u64 v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
RAL_FI ral_u32 ral_lanemask_lt() {
    ral_u32 m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---- decoupled look-back (single-pass prefix over tiles) -----------------------------------
// Status word of a tile: top two bits = state (1 aggregate known, 2 inclusive prefix known),
// low 62 bits = the value.  Called by all 32 lanes of one warp of the tile's block; returns
// the tile's exclusive prefix.  Tiles must be numbered in the order blocks took them (a ticket
// counter), so every predecessor is already running and the wait ends; it is still bounded:
// after RAL_LOOKBACK_SPIN_LIMIT polls the error word is set and the tile publishes what it has.
#define RAL_FLAG_AGGREGATE (1ull << 62)
#define RAL_FLAG_INCLUSIVE (2ull << 62)
#define RAL_VALUE_MASK ((1ull << 62) - 1)
#define RAL_LOOKBACK_SPIN_LIMIT (1l << 22)
// The two halves of a look-back: a tile's count is published as soon as it is known (tile 0's is
// its inclusive prefix), and the exclusive prefix is looked up later -- a warp that holds two
// tiles publishes the second before it looks back for the first.  A tile's status stays empty
// only while its own warp evaluates it, which waits on nothing, so every wait ends.
__device__ __forceinline__ void ral_lookback_publish(ral_u64* status, ral_i64 tile, ral_u64 aggregate) {
    if ((threadIdx.x & 31) == 0)
        ral_st_status(status + tile, (tile == 0 ? RAL_FLAG_INCLUSIVE : RAL_FLAG_AGGREGATE) | aggregate);
}
__device__ __forceinline__ ral_u64 ral_lookback_published(ral_u64* status, ral_i64 tile, ral_u64 aggregate,
                                                          ral_u64* error_word) {
    const int lane = threadIdx.x & 31;
    if (tile == 0) return 0;
    // The nearest predecessor is usually still in its own pass 1 when a tile gets here: lane 0
    // alone polls it until it has published, with a growing pause, so that a waiting warp costs
    // one load per round instead of 32; then the warp reads 32 predecessors per round.  (Reading
    // 4 or 8 predecessors per lane and round -- fewer rounds for long walks -- measured slower:
    // the status words are written by other SMs, and most walks end within 64 tiles.)
    long spins = 0;
    {
        unsigned pause = 32;
        for (;;) {
            ral_u64 s0 = 0;
            if (lane == 0) s0 = ral_ld_status(status + tile - 1);
            s0 = __shfl_sync(0xffffffffu, s0, 0);
            if (s0 & ~RAL_VALUE_MASK) break;
            if (++spins > RAL_LOOKBACK_SPIN_LIMIT) {
                if (lane == 0) atomicExch((unsigned long long*)error_word, 1ull);
                break;
            }
            __nanosleep(pause);
            if (pause < 256) pause <<= 1;
        }
    }
    ral_u64 excl = 0;
    ral_i64 j = tile - 1 - lane;
    for (;;) {
        const ral_u64 s = j >= 0 ? ral_ld_status(status + j) : RAL_FLAG_INCLUSIVE;
        const ral_u64 flag = s & ~RAL_VALUE_MASK;
        const ral_u32 incl = __ballot_sync(0xffffffffu, flag == RAL_FLAG_INCLUSIVE);
        const ral_u32 empty = __ballot_sync(0xffffffffu, flag == 0);
        const int f = incl ? __ffs(incl) - 1 : 32;
        const ral_u32 upto = f >= 31 ? 0xffffffffu : ((2u << f) - 1u);
        if (empty & upto) {
            if (++spins > RAL_LOOKBACK_SPIN_LIMIT) {
                if (lane == 0) atomicExch((unsigned long long*)error_word, 1ull);
                break;
            }
            __nanosleep(64);
            continue;
        }
        ral_u64 v = (lane <= f) ? (s & RAL_VALUE_MASK) : 0;
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        excl += __shfl_sync(0xffffffffu, v, 0);
        if (f < 32) break;
        j -= 32;
    }
    if (lane == 0) ral_st_status(status + tile, RAL_FLAG_INCLUSIVE | ((excl + aggregate) & RAL_VALUE_MASK));
    return excl;
}
__device__ __forceinline__ ral_u64 ral_lookback(ral_u64* status, ral_i64 tile, ral_u64 aggregate, ral_u64* error_word) {
    ral_lookback_publish(status, tile, aggregate);
    return ral_lookback_published(status, tile, aggregate, error_word);
}

// ---- grid-wide barrier of a cooperative launch ----------------------------------------------
// Called by one thread per block after a block barrier.  The counter is never reset: the host
// passes its value before the launch, and the barrier is reached when every block has added one
// (target = that value + gridDim.x).  The release fence before the add makes the block's earlier
// writes (ordered before this thread by the block barrier) visible to every block that sees the
// counter reach its target; the acquire load orders the block's later reads after theirs.
// Bounded: past RAL_GRID_SPIN_LIMIT polls the thread adds one to *error_word (a count the host
// compares with its value before the launch) and returns.
#define RAL_GRID_SPIN_LIMIT (1l << 22)
RAL_FI void ral_grid_barrier(ral_u64* counter, ral_u64 target, ral_u64* error_word) {
    __threadfence();
    atomicAdd((unsigned long long*)counter, 1ull);
    long spins = 0;
    unsigned pause = 32;
    for (;;) {
        ral_u64 v;
        asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(counter) : "memory");
        if (v >= target) break;
        if (++spins > RAL_GRID_SPIN_LIMIT) {
            atomicAdd((unsigned long long*)error_word, 1ull);
            break;
        }
        __nanosleep(pause);
        if (pause < 256) pause <<= 1;
    }
    __threadfence();
}

#endif  // RAL_DEVICE_RT_CUH_
