// Float64 division, reciprocal and square root from the hardware's
// approximate reciprocal and reciprocal square root, for kernels bound by
// GB300's float64 pipe (2 lanes per SM and cycle).
//
// rcp.approx.ftz.f64 and rsqrt.approx.ftz.f64 give about 20 correct bits;
// the first terms of the series of the exact correction finish the job:
// with e = 1 - b*r0, 1/b = r0/(1 - e) = r0*(1 + e + e^2 + ...); with
// s0 = x*y and r = 1 - s0*y, sqrt(x) = s0*(1 - r)^(-1/2) = s0*(1 + r/2 +
// 3r^2/8 + ...) and 1/sqrt(x) = y*(1 + r/2 + 3r^2/8 + ...) (Newton-Raphson
// taken to second order in series form, P. Markstein, IBM J. Res. Dev. 34
// (1990) 111).  Three to five float64 instructions, no slow path; a warp
// whose operands leave a safe exponent range takes IEEE division or square
// root instead.  Zero tests run on the integer pipe.
#pragma once
#include <cuda_runtime.h>

namespace veris {

__device__ __forceinline__ double rcp_seed(double b) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(b));
    return r;
}

__device__ __forceinline__ double rsqrt_seed(double x) {
    double r;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    return r;
}

// positive, normal, and at least 2^64 away from both ends of the exponent
// range (so neither the seed nor its square flushes or overflows)
__device__ __forceinline__ bool seed_range(double b) {
    const int hi = __double2hiint(b);
    return hi >= (64 << 20) && hi < (1984 << 20);
}

// the bits of x through a move the compiler cannot fold back into a float
// comparison (which would run on the float64 pipe)
__device__ __forceinline__ unsigned long long bits_of(double x) {
    unsigned long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return b;
}

__device__ __forceinline__ bool is_zero(double x) { return (bits_of(x) << 1) == 0; }

// a / b for b in seed_range: r0 ~ 1/b, e = 1 - b*r0, 1/b = r0*(1 + e + e^2 + O(e^3))
__device__ __forceinline__ double div_series(double a, double b) {
    const double r0 = rcp_seed(b);
    const double e = fma(-b, r0, 1.0);
    return a * fma(r0, fma(e, e, e), r0);
}

// sqrt(x) for x in seed_range: y ~ x^(-1/2), s0 = x*y, r = 1 - s0*y,
// sqrt(x) = s0*(1 - r)^(-1/2) = s0*(1 + r/2 + 3r^2/8 + O(r^3))
__device__ __forceinline__ double sqrt_series(double x) {
    const double y = rsqrt_seed(x);
    const double s0 = x * y;
    const double r = fma(-s0, y, 1.0);
    return fma(s0, r * fma(0.375, r, 0.5), s0);
}

// a / b on the lanes of `m` (all of which call it); IEEE division for the
// whole warp when any b leaves the seed range (zero, denormal, negative,
// huge, NaN)
__device__ __forceinline__ double div64(double a, double b, unsigned m) {
    if (__all_sync(m, seed_range(b))) return div_series(a, b);
    return a / b;
}

// sqrt(x), x >= 0 or -0, on the lanes of `m`
__device__ __forceinline__ double sqrt64(double x, unsigned m) {
    const bool z = is_zero(x);
    if (__all_sync(m, z || seed_range(x))) {
        const double s = sqrt_series(z ? 1.0 : x);
        return z ? 0.0 : s;
    }
    return sqrt(x);
}

// x > y for x, y >= 0 (or -0); false when x is NaN, as the float comparison
__device__ __forceinline__ bool gt_nonneg(double x, double y) {
    const long long a = (long long)bits_of(x), b = (long long)bits_of(y);
    return a > b && a <= 0x7ff0000000000000LL;
}

// 1/b for b in seed_range
__device__ __forceinline__ double rcp_series(double b) {
    const double r0 = rcp_seed(b);
    const double e = fma(-b, r0, 1.0);
    return fma(r0, fma(e, e, e), r0);
}

// 1/sqrt(x) for x in seed_range: y ~ x^(-1/2), r = 1 - x*y^2,
// x^(-1/2) = y*(1 - r)^(-1/2) = y*(1 + r/2 + 3r^2/8 + O(r^3))
__device__ __forceinline__ double rsqrt_series(double x) {
    const double y = rsqrt_seed(x);
    const double r = fma(-(x * y), y, 1.0);
    return fma(y, r * fma(0.375, r, 0.5), y);
}

// 1/b on the lanes of `m`; IEEE division for the whole warp when any b
// leaves the seed range
__device__ __forceinline__ double rcp64(double b, unsigned m) {
    if (__all_sync(m, seed_range(b))) return rcp_series(b);
    return 1.0 / b;
}

// 1/sqrt(x), x > 0, on the lanes of `m`
__device__ __forceinline__ double rsqrt64(double x, unsigned m) {
    if (__all_sync(m, seed_range(x))) return rsqrt_series(x);
    return 1.0 / sqrt(x);
}

// The same per lane, for code where the lanes that reach the call are not
// known (data-dependent branches): the series where the operand is in the
// seed range, IEEE otherwise (a warp whose lanes disagree runs both).
__device__ __forceinline__ double div_lane(double a, double b) {
    return seed_range(b) ? div_series(a, b) : a / b;
}
__device__ __forceinline__ double rcp_lane(double b) { return seed_range(b) ? rcp_series(b) : 1.0 / b; }
__device__ __forceinline__ double sqrt_lane(double x) {
    if (is_zero(x)) return x;
    return seed_range(x) ? sqrt_series(x) : sqrt(x);
}
__device__ __forceinline__ double rsqrt_lane(double x) { return seed_range(x) ? rsqrt_series(x) : 1.0 / sqrt(x); }

}  // namespace veris
