// Forward-mode dual numbers for the adjoint kernels.
//
// Dual<N> carries a float64 value and its derivatives with respect to N
// chosen inputs.  The pointwise parts of the sea-ice step (growth and its
// surface-temperature Newton solve, the post-advection clean-up) and the
// local stencil of each advective flux are evaluated once with Dual inputs,
// which yields their exact local Jacobian (branches follow the values, as in
// the forward code); the adjoint kernels then apply its transpose.
#pragma once

#include <cuda_runtime.h>

namespace veris {

template <int N>
struct Dual {
    double v;
    double d[N];
    __host__ __device__ Dual() : v(0.0) {
        for (int k = 0; k < N; ++k) d[k] = 0.0;
    }
    __host__ __device__ Dual(double x) : v(x) {
        for (int k = 0; k < N; ++k) d[k] = 0.0;
    }
    __host__ __device__ static Dual var(double x, int k) {
        Dual r(x);
        r.d[k] = 1.0;
        return r;
    }
};

template <class S>
__host__ __device__ inline double val(const S &x) { return x.v; }
__host__ __device__ inline double val(double x) { return x; }

#define DUAL_BIN(OP, EXPR_D)                                                                          \
    template <int N>                                                                                  \
    __host__ __device__ inline Dual<N> operator OP(const Dual<N> &a, const Dual<N> &b) {              \
        Dual<N> r;                                                                                    \
        r.v = a.v OP b.v;                                                                             \
        for (int k = 0; k < N; ++k) r.d[k] = EXPR_D;                                                  \
        return r;                                                                                     \
    }
DUAL_BIN(+, a.d[k] + b.d[k])
DUAL_BIN(-, a.d[k] - b.d[k])
DUAL_BIN(*, a.d[k] * b.v + a.v * b.d[k])
#undef DUAL_BIN

template <int N>
__host__ __device__ inline Dual<N> operator/(const Dual<N> &a, const Dual<N> &b) {
    Dual<N> r;
    r.v = a.v / b.v;
    const double ib = 1.0 / b.v;
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N> &a) {
    Dual<N> r;
    r.v = -a.v;
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
// mixed operands
#define DUAL_MIX(OP)                                                                                        \
    template <int N>                                                                                        \
    __host__ __device__ inline Dual<N> operator OP(const Dual<N> &a, double b) { return a OP Dual<N>(b); } \
    template <int N>                                                                                        \
    __host__ __device__ inline Dual<N> operator OP(double a, const Dual<N> &b) { return Dual<N>(a) OP b; }
DUAL_MIX(+)
DUAL_MIX(-)
DUAL_MIX(*)
DUAL_MIX(/)
#undef DUAL_MIX

#define DUAL_CMP(OP)                                                                                          \
    template <int N>                                                                                          \
    __host__ __device__ inline bool operator OP(const Dual<N> &a, const Dual<N> &b) { return a.v OP b.v; } \
    template <int N>                                                                                          \
    __host__ __device__ inline bool operator OP(const Dual<N> &a, double b) { return a.v OP b; }           \
    template <int N>                                                                                          \
    __host__ __device__ inline bool operator OP(double a, const Dual<N> &b) { return a OP b.v; }
DUAL_CMP(<)
DUAL_CMP(>)
DUAL_CMP(<=)
DUAL_CMP(>=)
DUAL_CMP(==)
DUAL_CMP(!=)
#undef DUAL_CMP

template <int N>
__device__ inline Dual<N> vsqrt(const Dual<N> &a) {
    Dual<N> r;
    r.v = ::sqrt(a.v);
    const double g = r.v > 0.0 ? 0.5 / r.v : 0.0;   // subgradient 0 at 0
    for (int k = 0; k < N; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <int N>
__device__ inline Dual<N> vrsqrt(const Dual<N> &a) {
    Dual<N> r;
    r.v = ::rsqrt(a.v);
    const double g = -0.5 * r.v * r.v * r.v;   // d x^(-1/2) / dx
    for (int k = 0; k < N; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <int N>
__device__ inline Dual<N> vexp(const Dual<N> &a) {
    Dual<N> r;
    r.v = ::exp(a.v);
    for (int k = 0; k < N; ++k) r.d[k] = r.v * a.d[k];
    return r;
}
template <int N>
__device__ inline Dual<N> vexp10(const Dual<N> &a) {
    Dual<N> r;
    r.v = ::exp10(a.v);
    const double g = r.v * 2.302585092994045684;   // d/dx 10^x = 10^x ln 10
    for (int k = 0; k < N; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <int N>
__device__ inline Dual<N> vexp2(const Dual<N> &a) {
    Dual<N> r;
    r.v = ::exp2(a.v);
    const double g = r.v * 0.6931471805599453094;   // d/dx 2^x = 2^x ln 2
    for (int k = 0; k < N; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <int N>
__device__ inline Dual<N> vlog(const Dual<N> &a) {
    Dual<N> r;
    r.v = ::log(a.v);
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] / a.v;
    return r;
}
template <int N>
__device__ inline Dual<N> vfabs(const Dual<N> &a) {
    return a.v < 0.0 ? -a : a;   // subgradient +1 at 0
}

// the same names for plain float64, so templated code calls one spelling
__device__ inline double vsqrt(double x) { return ::sqrt(x); }
__device__ inline double vrsqrt(double x) { return ::rsqrt(x); }
__device__ inline double vexp(double x) { return ::exp(x); }
__device__ inline double vexp10(double x) { return ::exp10(x); }
__device__ inline double vexp2(double x) { return ::exp2(x); }
__device__ inline double vlog(double x) { return ::log(x); }
__device__ inline double vfabs(double x) { return ::fabs(x); }
__device__ inline float vfabs(float x) { return ::fabsf(x); }

// select-type min/max: the chosen operand's derivatives (first one on ties)
template <class S>
__device__ inline S smax(const S &a, const S &b) { return a > b ? a : b; }
template <class S>
__device__ inline S smin(const S &a, const S &b) { return a < b ? a : b; }

}  // namespace veris
