// Self-check of the float64 division, reciprocal and square roots of
// f64math.cuh (the float64 EVP subcycle, its adjoint, the free drift and the
// bulk formula use them in place of IEEE division and square root): each
// form evaluated elementwise, so that a caller can measure them against
// correctly rounded results and IEEE special values.
#include "common.cuh"
#include "f64math.cuh"

namespace veris {

namespace {

constexpr int CHECK_THREADS = 256;

// out (planar, n each): div64(a, b), div_lane(a, b), rcp64(b), rcp_lane(b),
// sqrt64(b), sqrt_lane(b), rsqrt64(b), rsqrt_lane(b); the warp forms decide
// per warp, so a warp that mixes in- and out-of-range operands takes IEEE
__global__ void __launch_bounds__(CHECK_THREADS) f64math_check_kernel(const double *a, const double *b, int64_t n,
                                                                     double *out) {
    const int64_t i = (int64_t)blockIdx.x * CHECK_THREADS + threadIdx.x;
    const bool act = i < n;
    const unsigned m = __ballot_sync(0xffffffffu, act);
    if (!act) return;
    const double x = a[i], y = b[i];
    out[i] = div64(x, y, m);
    out[n + i] = div_lane(x, y);
    out[2 * n + i] = rcp64(y, m);
    out[3 * n + i] = rcp_lane(y);
    out[4 * n + i] = sqrt64(y, m);
    out[5 * n + i] = sqrt_lane(y);
    out[6 * n + i] = rsqrt64(y, m);
    out[7 * n + i] = rsqrt_lane(y);
}

}  // namespace

}  // namespace veris

extern "C" int veris_f64_math_check(const double *a, const double *b, int64_t n, double *out, veris_stream_t s) {
    VERIS_REQUIRE(n >= 0, VERIS_ERR_ARG);
    if (n == 0) return VERIS_OK;
    VERIS_REQUIRE(a && b && out, VERIS_ERR_ARG);
    const int64_t blocks = (n + veris::CHECK_THREADS - 1) / veris::CHECK_THREADS;
    VERIS_REQUIRE(blocks <= 0x7fffffff, VERIS_ERR_ARG);
    veris::f64math_check_kernel<<<(unsigned)blocks, veris::CHECK_THREADS, 0, (cudaStream_t)s>>>(a, b, n, out);
    return veris::launch_status();
}
