// selftest.cpp — on-device check that the integer-pipe double operations (softfp.cuh) give the
// same bits as the GPU's own FP64 instructions, over random and edge-case inputs.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "engine.h"
#include "jit.h"

namespace ral {

namespace {

const char* kSelftestSource = R"RALSRC(
RAL_FI ral_u64 st_mix(ral_u64 x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}
RAL_FI double st_double(ral_u64 r, ral_u64 r2) {
    switch (r2 % 6) {
    case 0: return __longlong_as_double((long long)r);
    case 1: return (double)(long long)(r >> (r2 % 64));
    case 2: return ldexp((double)(r >> 11), (int)((r2 >> 8) % 120) - 60);
    case 3: return (double)(int)r / (double)(1 + ((r2 >> 8) % 1000));
    case 4: return ldexp((r2 & 256) ? -1.0 : 1.0, (int)((r >> 3) % 2100) - 1075);
    default: return (double)__uint_as_float((unsigned)r);
    }
}
RAL_FI long long st_ulps(double a, double b) {
    long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    x = x < 0 ? -(x & 0x7fffffffffffffffll) : x;
    y = y < 0 ? -(y & 0x7fffffffffffffffll) : y;
    return x > y ? x - y : y - x;
}
RAL_FI bool st_same(double a, double b) {
    return (a != a && b != b) || __double_as_longlong(a) == __double_as_longlong(b);
}
RAL_FI void st_bad(unsigned long long* out, int k, double a, double b) {
    if (atomicAdd(out + 2 * 16 + k, 1ull) == 0) {
        out[k * 2] = (unsigned long long)__double_as_longlong(a);
        out[k * 2 + 1] = (unsigned long long)__double_as_longlong(b);
    }
}
// out: 16 pairs of first-mismatch operands, then 16 mismatch counters
extern "C" __global__ void ral_softfp_selftest(unsigned long long* out, long long n, unsigned long long seed) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const ral_u64 r0 = st_mix(seed + 4 * i), r1 = st_mix(seed + 4 * i + 1), r2 = st_mix(seed + 4 * i + 2),
                      r3 = st_mix(seed + 4 * i + 3);
        const double a = st_double(r0, r2), b0 = st_double(r1, r3);
        // every fourth divisor makes a quotient near one or an exact quotient
        const double b = (r3 & 3) == 0 ? a * (1.0 + ldexp((double)((int)(r2 % 64) - 32), -52))
                       : (r3 & 3) == 1 ? b0 : b0;
        const double num = (r3 & 3) == 1 ? ldexp((double)(r2 >> 11), -(int)(r1 % 40)) * b : a;
        if (!st_same(ral_sf_div(num, b), __ddiv_rn(num, b))) st_bad(out, 0, num, b);
        if (!st_same(ral_sf_floor(a), floor(a))) st_bad(out, 1, a, 0.0);
        if (!st_same(ral_sf_ceil(a), ceil(a))) st_bad(out, 2, a, 0.0);
        const unsigned hw = (unsigned)(a < b0) | (unsigned)(a <= b0) << 1 | (unsigned)(a > b0) << 2 |
                            (unsigned)(a >= b0) << 3 | (unsigned)(a == b0) << 4 | (unsigned)(a != b0) << 5;
        const unsigned sw = (unsigned)ral_sf_lt(a, b0) | (unsigned)ral_sf_le(a, b0) << 1 |
                            (unsigned)ral_sf_gt(a, b0) << 2 | (unsigned)ral_sf_ge(a, b0) << 3 |
                            (unsigned)ral_sf_eq(a, b0) << 4 | (unsigned)ral_sf_ne(a, b0) << 5;
        if (hw != sw) st_bad(out, 3, a, b0);
        const long long x = (long long)(r1 >> (r0 % 64)) * ((r0 & 64) ? -1 : 1);
        if (!st_same(ral_sf_i2d(x), __ll2double_rn(x))) st_bad(out, 4, __longlong_as_double(x), 0.0);
        if (ral_sf_d2i(a) != __double2ll_rz(a)) st_bad(out, 5, a, __longlong_as_double(__double2ll_rz(a)));
        const float f = __uint_as_float((unsigned)r3);
        if (!st_same(ral_sf_f2d(f), (double)f)) st_bad(out, 6, (double)f, 0.0);
        const float g1 = ral_sf_d2f(a), g2 = __double2float_rn(a);
        if (!((g1 != g1 && g2 != g2) || __float_as_uint(g1) == __float_as_uint(g2))) st_bad(out, 7, a, 0.0);
        if (ral_sf_is_zero(a) != (a == 0.0)) st_bad(out, 8, a, 0.0);
        if (!st_same(ral_sf_fabs(a), fabs(a))) st_bad(out, 9, a, 0.0);
        const long long ia = (long long)(r0 >> (r1 % 64)) * ((r1 & 128) ? -1 : 1);
        long long ib = (r2 & 1) ? (long long)(r3 >> (r2 % 64)) * ((r3 & 128) ? -1 : 1) : (long long)(1 + r3 % 1000);
        if (ib == 0 || ib == -1) ib = 7;
        if (ral_sf_div64(ia, ib) != ia / ib || ral_sf_mod64(ia, ib) != ia % ib)
            st_bad(out, 10, __longlong_as_double(ia), __longlong_as_double(ib));
        const long long ic = (long long)(1 + (r2 >> 40) % 65535) * ((r2 & 2) ? -1 : 1);
        if (ral_sf_div64_16(ia, ic) != ia / ic || ral_sf_mod64_16(ia, ic) != ia % ic)
            st_bad(out, 10, __longlong_as_double(ia), __longlong_as_double(ic));
        // sin / cos: approximations on both sides, so within 2 ulp of the library's
        const double t = (r3 & 1) ? a : ldexp((double)(r0 >> 11), -53) * 2e6 * ((r1 & 1) ? -1.0 : 1.0);
        if (t == t && t - t == 0.0) {
            if (st_ulps(ral_sf_sin(t), sin(t)) > 2 || st_ulps(ral_sf_cos(t), cos(t)) > 2) st_bad(out, 11, t, 0.0);
        }
    }
}
)RALSRC";

}  // namespace

int softfp_selftest(long long n, unsigned long long seed, long long* counts, unsigned long long* first_operands) {
    GeneratedKernel gk;
    gk.name = "ral_softfp_selftest";
    gk.source = kSelftestSource;
    std::string err;
    const CompiledKernel* k = jit_get(gk, err);
    if (!k) return set_error(kJitError, err);
    unsigned long long* d = nullptr;
    if (int e = check_cuda(cudaMalloc(&d, 48 * 8), "cudaMalloc")) return e;
    cudaMemset(d, 0, 48 * 8);
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* args[] = {&d, &n, &seed};
    int rc = check_cuda(cudaLaunchKernel((const void*)k->kernel, dim3(sms * 8), dim3(256), args, 0, 0),
                        "launch of the soft-FP self-test");
    unsigned long long h[48] = {};
    if (!rc) rc = check_cuda(cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost), "soft-FP self-test");
    cudaFree(d);
    if (rc) return rc;
    for (int i = 0; i < 16; i++) {
        counts[i] = (long long)h[32 + i];
        first_operands[2 * i] = h[2 * i];
        first_operands[2 * i + 1] = h[2 * i + 1];
    }
    return kSuccess;
}

}  // namespace ral
