// The routines on either side of the dynamics: the free-drift ice velocities
// (veris/freedrift_solver.py:5-62) and the bulk-formula fluxes over open
// ocean that produce the atmospheric forcing (veris/heat_flux_MITgcm.py:5-123).
//
// Free drift.  The reference solves a 2x2 problem at every C point and
// averages the C-point velocities onto the U and V faces.  Here one warp owns
// a strip of 31 output columns (lane 0 solves the column to the strip's south
// for its neighbour) and walks down a few rows: the U average needs the row
// above, which the lane still holds from its previous step, and the V average
// needs the column to the south, one shuffle away; the east and north
// neighbours of the C-point averages (WindForcingX, uOcean at i+1) are the
// next row's own loads, carried in registers.  Every C point is solved about
// 1.1 times (float64, 16-row walks) or 1.3 times (float32, 4-row walks).
//
// The angle of the solution enters the reference only through
// cos(rhsA - atan2(t3, t2)) and sin(rhsA - atan2(t3, t2)), with rhsA =
// atan2(rhsY, rhsX).  Both are ratios of the operands already at hand
// (cos(a - b) = cos a cos b + sin a sin b and cos(atan2(y, x)) = x / |(x, y)|),
// so the walk evaluates them with one square root and one division instead of
// two arctangents, a sine and a cosine: GB300's float64 pipe does two fused
// multiply-adds per SM and cycle, and the trigonometric forms would cost
// several times the memory time of the routine.  The results differ from the
// reference's by rounding only.
//
// Bulk formula.  Pointwise; the five fixed psi-function iterations run in
// registers.  On a stable layer (huol > 0) the reference's unstable terms
// are multiplied by exactly zero, so they are skipped there.  A NULL output
// pointer skips that output's store (the reference's own caller discards the
// last three, seaice_global_4deg.py:761).
//
// Both routines are bound by GB300's float64 pipe in float64 (2 lanes per SM
// and cycle): their divisions, reciprocals and square roots take the
// series-refined hardware approximations of f64math.cuh (per lane, IEEE
// where an operand leaves the safe range).  In float32 the bulk formula is
// bound by instruction issue: its divisions, logarithms, exponential and the
// square roots of the psi functions use the hardware approximations
// (__fdividef, __logf, __expf, rsqrtf: a few units in
// the last place, inside the float32 forms' 1e-4 bound against the
// reference); the free drift keeps IEEE-rounded float32 arithmetic.
#include <cmath>

#include "common.cuh"
#include "f64math.cuh"

namespace veris {

// division, reciprocal and square roots of each precision
template <class T>
struct Fm;
template <>
struct Fm<double> {
    static __device__ __forceinline__ double log(double x) { return ::log(x); }
    static __device__ __forceinline__ double exp(double x) { return ::exp(x); }
    static __device__ __forceinline__ double fdiv(double a, double b) { return div_lane(a, b); }
    static __device__ __forceinline__ double root(double x) { return sqrt_lane(x); }
    static __device__ __forceinline__ double root_ge1(double x) { return sqrt_lane(x); }
    static __device__ __forceinline__ double rcp(double x) { return rcp_lane(x); }
    static __device__ __forceinline__ double div(double a, double b) { return div_lane(a, b); }
    // 1 / (a sqrt(x)) for a > 0, x > 0
    static __device__ __forceinline__ double rnorm(double a, double x) { return rcp_lane(a) * rsqrt_lane(x); }
};
template <>
struct Fm<float> {
    static __device__ __forceinline__ float log(float x) { return __logf(x); }
    static __device__ __forceinline__ float exp(float x) { return __expf(x); }
    static __device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ float root(float x) { return sqrtf(x); }
    // x >= 1: the approximate reciprocal square root times x (a few ulps)
    static __device__ __forceinline__ float root_ge1(float x) { return x * rsqrtf(x); }
    static __device__ __forceinline__ float rcp(float x) { return 1.f / x; }
    static __device__ __forceinline__ float div(float a, float b) { return a / b; }
    static __device__ __forceinline__ float rnorm(float a, float x) { return 1.f / (a * sqrtf(x)); }
};

// rows per walk: float64 is bound by its arithmetic and walks long (fewer
// C points solved twice); float32 is bound by memory latency and walks short,
// unrolled, so that all its rows' loads are in flight together
constexpr int FD_LANES = 31, FD_WARPS = 8;
template <class T>
struct FdRows { static constexpr int value = sizeof(T) == 8 ? 16 : 4; };

template <class T>
struct FdArgs {
    const T *wfx, *wfy, *uo, *vo, *h, *fc, *mu, *mv;
    T *u, *v;
    T rhoIce, t1n, t1s, t1n_inv, t1s_inv;   // 1 / (Cd rhoSea) and its reciprocal, per hemisphere
};

// veris/freedrift_solver.py:13-53 at one C point, given the C-point averages
template <class T>
__device__ __forceinline__ void fd_center(const FdArgs<T> &a, T tauX, T tauY, T uOc, T vOc, T h, T f,
                                          T &uC, T &vC) {
    const T mIceCor = a.rhoIce * h * f;
    const T rhsX = -tauX - mIceCor * vOc;
    const T rhsY = -tauY + mIceCor * uOc;
    const T n2 = rhsX * rhsX + rhsY * rhsY;
    const T rhsN = n2 > T(0) ? Fm<T>::root(n2) : T(0);
    const bool south = f < T(0);
    const T t1 = south ? a.t1s : a.t1n;
    const T t1sq = t1 * t1;
    const T t2 = t1sq * (mIceCor * mIceCor);
    const T t3 = t1sq * (rhsN * rhsN);
    const T t4 = t2 * t2 + T(4) * t3;
    const T solN = t3 > T(0) ? Fm<T>::root(T(0.5) * (Fm<T>::root(t4) - t2)) : T(0);
    uC = uOc;
    vC = vOc;
    if (solN > T(0)) {
        // solN > 0 implies rhsN > 0 and p2 > 0: both angles are defined
        const T p2 = (south ? a.t1s_inv : a.t1n_inv) * (solN * solN);
        const T p3 = mIceCor * solN;
        const T r = Fm<T>::rnorm(rhsN, p2 * p2 + p3 * p3);
        const T cosA = (rhsX * p2 + rhsY * p3) * r;
        const T sinA = (rhsY * p2 - rhsX * p3) * r;
        uC = uOc - solN * cosA;
        vC = vOc - solN * sinA;
    }
}

template <class T>
__global__ void __launch_bounds__(FD_WARPS * 32)
freedrift_kernel(Dims d, FdArgs<T> a, int n_strips) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * FD_WARPS + (threadIdx.x >> 5);
    const int strip = w % n_strips, band = w / n_strips;
    constexpr int ROWS = FdRows<T>::value;
    const int i_first = band * ROWS;
    if (i_first >= d.NX) return;
    const int i_end = min(i_first + ROWS, d.NX);
    const int jc = strip * FD_LANES + lane - 1;            // lane 0: the column to the south
    const bool live = jc < d.NY;                           // columns past the edge feed nothing
    const int j = d.wy(live ? jc : d.NY - 1);
    const int jn = d.wy(j + 1);
    const bool store = live && lane > 0;

    // the row above the band, then the band itself
    int i = d.wx(i_first - 1);
    int64_t o = (int64_t)i * d.ld;
    T wfx = __ldg(a.wfx + o + j), uo = __ldg(a.uo + o + j);
    T uPrev = T(0);
#pragma unroll
    for (int q = 0; q <= ROWS; ++q) {
        const int r = i_first - 1 + q;
        if (r >= i_end) break;
        const int in = d.wx(i + 1);
        const int64_t on = (int64_t)in * d.ld;
        const T wfxN = __ldg(a.wfx + on + j), uoN = __ldg(a.uo + on + j);
        const T tauX = T(0.5) * (wfx + wfxN);
        const T tauY = T(0.5) * (__ldg(a.wfy + o + j) + __ldg(a.wfy + o + jn));
        const T uOc = T(0.5) * (uo + uoN);
        const T vOc = T(0.5) * (__ldg(a.vo + o + j) + __ldg(a.vo + o + jn));
        T uC, vC;
        fd_center(a, tauX, tauY, uOc, vOc, __ldg(a.h + o + j), __ldg(a.fc + o + j), uC, vC);
        const T vS = __shfl_up_sync(0xffffffffu, vC, 1);
        if (r >= i_first && store) {
            a.u[o + j] = T(0.5) * (uPrev + uC) * __ldg(a.mu + o + j);
            a.v[o + j] = T(0.5) * (vS + vC) * __ldg(a.mv + o + j);
        }
        uPrev = uC;
        wfx = wfxN;
        uo = uoN;
        i = in;
        o = on;
    }
}

template <class T>
__device__ __forceinline__ T bk_sign(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : x); }

template <class T>
struct BulkArgs {
    const T *uw, *vw, *ta, *qa, *tsf;
    T *flwupa, *flha, *fsha, *df0dT, *ust, *vst, *evp, *ssq, *dEvdT;
    int64_t n;
    T zvir, cpdair, karman, latvap, emis, gamma_blk, rhoAir, stefBoltz, czol, aln, rdn;
    T g, rlatvap, rzvir;   // rdn / karman, 1 / latvap, 1 / zvir
};

template <class T>
__global__ void __launch_bounds__(256) bulkf_kernel(BulkArgs<T> a) {
    const T ht = T(2.0), pi = T(3.14159265358979323846);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const T uw = __ldg(a.uw + k), vw = __ldg(a.vw + k);
        const T ta = __ldg(a.ta + k), qa = __ldg(a.qa + k), tsf = __ldg(a.tsf + k);
        const T lath = a.latvap;
        const T us = Fm<T>::root(uw * uw + vw * vw);
        const T usm = us > T(1) ? us : T(1);
        const T t0 = ta * (T(1) + a.zvir * qa);
        const T rtsf = Fm<T>::fdiv(T(1), tsf);
        const T ssq = T(3.797915) * Fm<T>::exp(lath * (T(7.93252e-6) - T(2.166847e-3) * rtsf)) * T(1.0 / 1013.0);
        const T deltap = ta - tsf + a.gamma_blk * ht;
        const T delq = qa - ssq;
        const T qden = a.rzvir + qa;
        // With rd = rdn / Dm and rh = re = rdn / Dh (Dm = Dh = 1 before the
        // first iteration), ustar = rd usm, tstar = rh deltap, qstar = rh delq:
        //   huol = czol / ustar^2 (tstar / t0 + qstar / qden) = K Dm^2 / Dh,
        //   K = czol (deltap qden + delq t0) / (t0 qden usm^2 rdn)
        // one division per iteration instead of seven; rounding differs only.
        const T K = Fm<T>::fdiv(a.czol * (deltap * qden + delq * t0), t0 * qden * (usm * usm) * a.rdn);
        T Dm = T(1), Dh = T(1);
        for (int it = 0; it < 5; ++it) {
            T huol = it == 0 ? K : Fm<T>::fdiv(K * (Dm * Dm), Dh);
            const T ah = fabs(huol);
            huol = (ah < T(10) ? ah : T(10)) * bk_sign(huol);
            T psimh, psixh;
            if (huol > T(0)) {
                psimh = psixh = T(-5) * huol;       // stable: the unstable terms carry a factor 0
            } else {
                const T stable = T(0.5) + T(0.5) * bk_sign(huol);
                const T sq = Fm<T>::root_ge1(fabs(T(1) - T(16) * huol));   // huol <= 0: at least 1
                const T xsq = sq > T(1) ? sq : T(1);
                const T x = Fm<T>::root_ge1(xsq);
                const T l2 = T(2) * Fm<T>::log(T(0.5) * (T(1) + xsq));
                psimh = T(-5) * huol * stable +
                        (T(1) - stable) * (T(2) * Fm<T>::log(T(0.5) * (T(1) + x)) + l2 - T(2) * atan(x) + pi * T(0.5));
                psixh = T(-5) * huol * stable + (T(1) - stable) * l2;
            }
            Dm = T(1) + a.g * (a.aln - psimh);
            Dh = T(1) + a.g * (a.aln - psixh);
        }
        const T rhrd = Fm<T>::fdiv(a.rdn * a.rdn, Dm * Dh);   // rh rd (= re rd)
        const T csha = a.rhoAir * a.cpdair * us * rhrd;
        const T clha = a.rhoAir * lath * us * rhrd;
        const T flha = clha * delq;
        if (a.fsha) a.fsha[k] = csha * deltap;
        if (a.flha) a.flha[k] = flha;
        if (a.evp) a.evp[k] = -flha * a.rlatvap;
        const T t2 = tsf * tsf, t3 = t2 * tsf;
        if (a.flwupa) a.flwupa[k] = a.emis * a.stefBoltz * (t2 * t2);
        const T devdt = clha * ssq * T(2.166847e-3) * (rtsf * rtsf);
        if (a.df0dT) a.df0dT[k] = -(T(4) * a.emis * a.stefBoltz * t3) + (-csha) + (-lath * devdt);
        if (a.dEvdT) a.dEvdT[k] = devdt;
        if (a.ssq) a.ssq[k] = ssq;
        const T cdn = Fm<T>::fdiv(T(2.7e-3), usm) + T(0.142e-3) + T(0.0764e-3) * usm;
        const T ws = a.rhoAir * cdn * us;
        if (a.ust) a.ust[k] = ws * uw;
        if (a.vst) a.vst[k] = ws * vw;
    }
}

template <class T>
static int freedrift(const VerisGrid *g, const VerisParams *p, const Fields<T> *vs, T *u, T *v,
                     veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && u && v, VERIS_ERR_ARG);
    FdArgs<T> a;
    a.wfx = vs->WindForcingX;
    a.wfy = vs->WindForcingY;
    a.uo = vs->uOcean;
    a.vo = vs->vOcean;
    a.h = vs->hIceMean;
    a.fc = vs->fCori;
    a.mu = vs->iceMaskU;
    a.mv = vs->iceMaskV;
    a.u = u;
    a.v = v;
    // veris/freedrift_solver.py:35-46: tmp1 = 1 / (drag rhoSea), later 1 / tmp1
    const double t1n = 1.0 / (p->waterIceDrag * p->rhoSea), t1s = 1.0 / (p->waterIceDrag_south * p->rhoSea);
    a.rhoIce = T(p->rhoIce);
    a.t1n = T(t1n);
    a.t1s = T(t1s);
    a.t1n_inv = T(1.0 / t1n);
    a.t1s_inv = T(1.0 / t1s);
    const int n_strips = (d.NY + FD_LANES - 1) / FD_LANES;
    const int n_bands = (d.NX + FdRows<T>::value - 1) / FdRows<T>::value;
    const int warps = n_strips * n_bands;
    freedrift_kernel<T><<<(warps + FD_WARPS - 1) / FD_WARPS, FD_WARPS * 32, 0, (cudaStream_t)s>>>(d, a, n_strips);
    return launch_status();
}

template <class T>
static int bulkf(const VerisParams *p, int64_t n, const T *uw, const T *vw, const T *ta, const T *qa,
                 const T *tsf, T *flwupa, T *flha, T *fsha, T *df0dT, T *ust, T *vst, T *evp, T *ssq,
                 T *dEvdT, veris_stream_t s) {
    VERIS_REQUIRE(p && n >= 0, VERIS_ERR_ARG);
    if (n == 0) return VERIS_OK;
    VERIS_REQUIRE(uw && vw && ta && qa && tsf, VERIS_ERR_ARG);
    BulkArgs<T> a{uw, vw, ta, qa, tsf, flwupa, flha, fsha, df0dT, ust, vst, evp, ssq, dEvdT, n};
    // veris/heat_flux_MITgcm.py:45-50, 62-64: the constants of the scheme
    a.zvir = T(p->zvir);
    a.cpdair = T(p->cpdair);
    a.karman = T(p->karman);
    a.latvap = T(p->latvap);
    a.emis = T(p->ocean_emissivity);
    a.gamma_blk = T(p->gamma_blk);
    a.rhoAir = T(p->rhoAir);
    a.stefBoltz = T(p->stefBoltz);
    a.czol = T(10.0 * p->karman * p->grav);
    a.aln = T(std::log(2.0 / 10.0));
    a.rdn = T(p->karman / std::log(10.0 / 0.0005));
    a.g = T(p->karman / std::log(10.0 / 0.0005) / p->karman);
    a.rlatvap = T(1.0 / p->latvap);
    a.rzvir = T(1) / a.zvir;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n + 255) / 256;
    const int64_t cap = (int64_t)(sms > 0 ? sms : 148) * 8;
    const int blocks = (int)(want < cap ? want : cap);
    bulkf_kernel<T><<<blocks, 256, 0, (cudaStream_t)s>>>(a);
    return launch_status();
}

}  // namespace veris

using namespace veris;

extern "C" {

int veris_freedrift_solver_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                               double *uIce, double *vIce, veris_stream_t s) {
    return freedrift<double>(g, p, reinterpret_cast<const Fields<double> *>(vs), uIce, vIce, s);
}

int veris_freedrift_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF32 *vs,
                               float *uIce, float *vIce, veris_stream_t s) {
    return freedrift<float>(g, p, reinterpret_cast<const Fields<float> *>(vs), uIce, vIce, s);
}

int veris_bulkf_formula_lanl_f64(const VerisParams *p, int64_t n, const double *uw, const double *vw,
                                 const double *ta, const double *qa, const double *tsf,
                                 const double *ocn_mask, double *flwupa, double *flha, double *fsha,
                                 double *df0dT, double *ust, double *vst, double *evp, double *ssq,
                                 double *dEvdT, veris_stream_t s) {
    (void)ocn_mask;   // the reference takes only its shape (lath = ones_like(ocn_mask) * latvap)
    return bulkf<double>(p, n, uw, vw, ta, qa, tsf, flwupa, flha, fsha, df0dT, ust, vst, evp, ssq, dEvdT, s);
}

int veris_bulkf_formula_lanl_f32(const VerisParams *p, int64_t n, const float *uw, const float *vw,
                                 const float *ta, const float *qa, const float *tsf, const float *ocn_mask,
                                 float *flwupa, float *flha, float *fsha, float *df0dT, float *ust,
                                 float *vst, float *evp, float *ssq, float *dEvdT, veris_stream_t s) {
    (void)ocn_mask;
    return bulkf<float>(p, n, uw, vw, ta, qa, tsf, flwupa, flha, fsha, df0dT, ust, vst, evp, ssq, dEvdT, s);
}

}  // extern "C"
