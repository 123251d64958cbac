// Flux-limited advection of hIceMean, hSnowMean and Area
// (veris/advection.py:15-175) and the post-advection clean-up
// (veris/clean_up.py:5-47).
//
// Dimensionally split: zonal fluxes, zonal update, meridional fluxes (of the
// zonally updated field), meridional update.  Each phase is one launch over
// all advected fields (blockIdx.z = field).  The fluxes are stored with the
// halo fill the reference applies to them fused into the store.
#include "stencil.cuh"

namespace veris {

constexpr int ABX = 32, ABY = 8;
constexpr int MAX_ADV_FIELDS = 3;

template <class T>
struct AdvIO {
    const T *field[MAX_ADV_FIELDS];  // field before advection
    T *F[MAX_ADV_FIELDS];            // zonal flux
    T *f1[MAX_ADV_FIELDS];           // after the zonal update
    T *G[MAX_ADV_FIELDS];            // meridional flux
    T *out[MAX_ADV_FIELDS];          // after the meridional update, masked
};

// veris/advection.py:170-175
template <class T>
__device__ __forceinline__ T superbee(T cr) {
    const T a = T(2) * cr < T(1) ? T(2) * cr : T(1);
    const T b = cr < T(2) ? cr : T(2);
    const T m = a > b ? a : b;
    return m > T(0) ? m : T(0);
}

// limited flux through one face given the three slopes, the transport and
// the Courant number (veris/advection.py:107-126)
template <class T>
__device__ __forceinline__ T limited_flux(T fm, T f0, T Rjm, T Rj, T Rjp, T trans, T cfl, T CrMax) {
    T cr = trans > T(0) ? Rjm : Rjp;
    cr = fabs(Rj) * CrMax > fabs(cr) ? cr / Rj : sgn(cr) * CrMax * sgn(Rj);
    cr = superbee(cr);
    return trans * (f0 + fm) * T(0.5) - fabs(trans) * ((T(1) - cr) + cfl * cr) * Rj * T(0.5);
}

template <class T>
__device__ __forceinline__ T zonal_flux_at(const Ctx<T> &c, const T *fld, const T *uT, int i, int j) {
    if (i < 2 || i > c.d.NX - 2) return T(0);
    const Fields<T> &f = c.f;
    const int64_t o = c.d.raw(i, j);
    const int64_t L = c.d.ld;
    auto m = [&](int64_t q) { return __ldg(f.iceMaskU + q) * __ldg(f.maskInU + q); };
    const T fmm = __ldg(fld + o - 2 * L), fm = __ldg(fld + o - L), f0 = __ldg(fld + o), fp = __ldg(fld + o + L);
    const T Rjp = (fp - f0) * m(o + L);
    const T Rj = (f0 - fm) * m(o);
    const T Rjm = (fm - fmm) * m(o - L);
    const T cfl = fabs(__ldg(f.uIce + o) * T(c.p.deltatTherm) * __ldg(f.recip_dxC + o));
    return limited_flux(fm, f0, Rjm, Rj, Rjp, __ldg(uT + o), cfl, T(c.p.CrMax));
}

template <class T>
__device__ __forceinline__ T meridional_flux_at(const Ctx<T> &c, const T *fld, const T *vT, int i, int j) {
    if (j < 2 || j > c.d.NY - 2) return T(0);
    const Fields<T> &f = c.f;
    const int64_t o = c.d.raw(i, j);
    auto m = [&](int64_t q) { return __ldg(f.iceMaskV + q) * __ldg(f.maskInV + q); };
    const T fmm = __ldg(fld + o - 2), fm = __ldg(fld + o - 1), f0 = __ldg(fld + o), fp = __ldg(fld + o + 1);
    const T Rjp = (fp - f0) * m(o + 1);
    const T Rj = (f0 - fm) * m(o);
    const T Rjm = (fm - fmm) * m(o - 1);
    const T cfl = fabs(__ldg(f.vIce + o) * T(c.p.deltatTherm) * __ldg(f.recip_dyC + o));
    return limited_flux(fm, f0, Rjm, Rj, Rjp, __ldg(vT + o), cfl, T(c.p.CrMax));
}

template <class T>
__device__ __forceinline__ T utrans_at(const Ctx<T> &c, int64_t o) {
    return __ldg(c.f.uIce + o) * (__ldg(c.f.dyG + o) * __ldg(c.f.iceMaskU + o));
}
template <class T>
__device__ __forceinline__ T vtrans_at(const Ctx<T> &c, int64_t o) {
    return __ldg(c.f.vIce + o) * (__ldg(c.f.dxG + o) * __ldg(c.f.iceMaskV + o));
}

// transports (written once, shared by all fields)
template <class T>
__global__ void transport_kernel(Ctx<T> c, T *uT, T *vT) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y;
    if (i >= c.d.NX || j >= c.d.NY) return;
    const int64_t o = c.d.raw(i, j);
    uT[o] = utrans_at(c, o);
    vT[o] = vtrans_at(c, o);
}

template <class T>
__global__ void zonal_flux_kernel(Ctx<T> c, HaloFill h, AdvIO<T> io, const T *uT) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y, q = blockIdx.z;
    if (i >= c.d.NX || j >= c.d.NY) return;
    store_filled(io.F[q], c.d, h, i, j, zonal_flux_at(c, io.field[q], uT, i, j));
}

template <class T>
__global__ void zonal_update_kernel(Ctx<T> c, AdvIO<T> io) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y, q = blockIdx.z;
    if (i >= c.d.NX || j >= c.d.NY) return;
    const int64_t o = c.d.raw(i, j);
    const T *F = io.F[q];
    io.f1[q][o] = __ldg(io.field[q] + o) - T(c.p.deltatTherm) * __ldg(c.f.maskInC + o) * __ldg(c.f.recip_rA + o) *
                                               (c.ld(F, i + 1, j) - __ldg(F + o));
}

template <class T>
__global__ void meridional_flux_kernel(Ctx<T> c, HaloFill h, AdvIO<T> io, const T *vT) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y, q = blockIdx.z;
    if (i >= c.d.NX || j >= c.d.NY) return;
    store_filled(io.G[q], c.d, h, i, j, meridional_flux_at(c, io.f1[q], vT, i, j));
}

template <class T>
__global__ void meridional_update_kernel(Ctx<T> c, AdvIO<T> io) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y, q = blockIdx.z;
    if (i >= c.d.NX || j >= c.d.NY) return;
    const int64_t o = c.d.raw(i, j);
    const T *G = io.G[q];
    const T f = __ldg(io.f1[q] + o) - T(c.p.deltatTherm) * __ldg(c.f.maskInC + o) * __ldg(c.f.recip_rA + o) *
                                          (c.ld(G, i, j + 1) - __ldg(G + o));
    io.out[q][o] = f * __ldg(c.f.iceMask + o);
}

// standalone flux routines (the reference's calc_ZonalFlux/calc_MeridionalFlux
// take the transport as an argument)
template <class T>
__global__ void zonal_flux_only_kernel(Ctx<T> c, HaloFill h, const T *fld, const T *uT, T *F) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y;
    if (i >= c.d.NX || j >= c.d.NY) return;
    store_filled(F, c.d, h, i, j, zonal_flux_at(c, fld, uT, i, j));
}
template <class T>
__global__ void meridional_flux_only_kernel(Ctx<T> c, HaloFill h, const T *fld, const T *vT, T *G) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y;
    if (i >= c.d.NX || j >= c.d.NY) return;
    store_filled(G, c.d, h, i, j, meridional_flux_at(c, fld, vT, i, j));
}

template <class T>
__global__ void limiter_kernel(const T *cr, T *phi, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        phi[k] = superbee(cr[k]);
}

// veris/clean_up.py:5-47, clean-up and ridging in one pass
template <class T>
__global__ void clean_up_kernel(Ctx<T> c, T *h_o, T *hs_o, T *A_o, T *TS_o, T *osh_o, T *oshs_o, int ridge) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y;
    if (i >= c.d.NX || j >= c.d.NY) return;
    const int64_t o = c.d.raw(i, j);
    const T h0 = __ldg(c.f.hIceMean + o), hs0 = __ldg(c.f.hSnowMean + o), A0 = __ldg(c.f.Area + o);
    const T osh = -h0 > T(0) ? -h0 : T(0);
    const T oshs = -hs0 > T(0) ? -hs0 : T(0);
    T h = h0 > T(0) ? h0 : T(0);
    T hs = hs0 > T(0) ? hs0 : T(0);
    T A = A0 > T(0) ? A0 : T(0);
    const bool thin = h <= T(c.p.hIce_min);
    if (thin) {
        h = h * T(0);
        hs = hs * T(0);
    }
    const T TS = thin ? T(c.p.celsius2K) : __ldg(c.f.TSurf + o);
    if (h == T(0) && hs == T(0)) A = T(0);
    if (h > T(0) || hs > T(0)) A = A > T(c.p.Area_min) ? A : T(c.p.Area_min);
    if (h_o) h_o[o] = h;
    if (hs_o) hs_o[o] = hs;
    if (A_o) A_o[o] = ridge ? (A < T(1) ? A : T(1)) : A;
    if (TS_o) TS_o[o] = TS;
    if (osh_o) osh_o[o] = osh;
    if (oshs_o) oshs_o[o] = oshs;
}

template <class T>
__global__ void ridging_kernel(Ctx<T> c, T *A_o) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y;
    if (i >= c.d.NX || j >= c.d.NY) return;
    const int64_t o = c.d.raw(i, j);
    const T A = __ldg(c.f.Area + o);
    A_o[o] = A < T(1) ? A : T(1);
}

static size_t round_up_a(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <class T>
static int advect(const VerisGrid *g, const VerisParams *p, const Fields<T> *vs, int nf, const T *const *in,
                  T *const *out, void *ws, size_t ws_bytes, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs, VERIS_ERR_ARG);
    VERIS_REQUIRE(p->extensiveFld, VERIS_ERR_UNSUPPORTED);
    const size_t fb = round_up_a((size_t)d.NX * d.ld * sizeof(T), 256);
    VERIS_REQUIRE(ws && ws_bytes >= (size_t)(2 + 3 * MAX_ADV_FIELDS) * fb, VERIS_ERR_WORKSPACE);
    for (int q = 0; q < nf; ++q) VERIS_REQUIRE(in[q] && out[q], VERIS_ERR_ARG);
    Ctx<T> c;
    c.f = *vs;
    c.d = d;
    c.p = *p;
    const HaloFill h = halo_fill_of(*p);
    char *w = static_cast<char *>(ws);
    T *uT = reinterpret_cast<T *>(w);
    T *vT = reinterpret_cast<T *>(w + fb);
    AdvIO<T> io;
    for (int q = 0; q < MAX_ADV_FIELDS; ++q) {
        io.field[q] = q < nf ? in[q] : nullptr;
        io.out[q] = q < nf ? out[q] : nullptr;
        io.F[q] = reinterpret_cast<T *>(w + (2 + q) * fb);
        io.f1[q] = reinterpret_cast<T *>(w + (2 + MAX_ADV_FIELDS + q) * fb);
        io.G[q] = reinterpret_cast<T *>(w + (2 + 2 * MAX_ADV_FIELDS + q) * fb);
    }
    cudaStream_t st = (cudaStream_t)s;
    dim3 bl(ABX, ABY);
    dim3 g2((d.NY + ABX - 1) / ABX, (d.NX + ABY - 1) / ABY);
    dim3 g3(g2.x, g2.y, nf);
    // every flux point is stored: zero outside the reference's slice, the
    // periodic image inside a refreshed halo
    transport_kernel<T><<<g2, bl, 0, st>>>(c, uT, vT);
    zonal_flux_kernel<T><<<g3, bl, 0, st>>>(c, h, io, uT);
    zonal_update_kernel<T><<<g3, bl, 0, st>>>(c, io);
    meridional_flux_kernel<T><<<g3, bl, 0, st>>>(c, h, io, vT);
    meridional_update_kernel<T><<<g3, bl, 0, st>>>(c, io);
    return launch_status();
}

}  // namespace veris

using namespace veris;

#define ADV_CTX(T)                                                               \
    Dims d;                                                                      \
    VERIS_CHECK_GRID(g, d);                                                      \
    VERIS_REQUIRE(p && vs, VERIS_ERR_ARG);                                       \
    Ctx<T> c;                                                                    \
    c.f = *reinterpret_cast<const Fields<T> *>(vs);                              \
    c.d = d;                                                                     \
    c.p = *p;                                                                    \
    cudaStream_t st = (cudaStream_t)s;                                           \
    dim3 bl(ABX, ABY), g2((d.NY + ABX - 1) / ABX, (d.NX + ABY - 1) / ABY);

extern "C" {

size_t veris_advection_workspace_bytes(const VerisGrid *g, int32_t elem_size) {
    Dims d;
    if (check_grid(g, &d) != VERIS_OK || (elem_size != 4 && elem_size != 8)) return 0;
    return (size_t)(2 + 3 * MAX_ADV_FIELDS) * round_up_a((size_t)d.NX * d.ld * elem_size, 256);
}

int veris_limiter_f64(const double *cr, double *phi, int64_t n, veris_stream_t s) {
    VERIS_REQUIRE(n >= 0, VERIS_ERR_ARG);
    if (n == 0) return VERIS_OK;
    VERIS_REQUIRE(cr && phi, VERIS_ERR_ARG);
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    limiter_kernel<double><<<blocks, 256, 0, (cudaStream_t)s>>>(cr, phi, n);
    return launch_status();
}

int veris_calc_zonal_flux_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                              const double *field, const double *uT, double *F, veris_stream_t s) {
    ADV_CTX(double)
    VERIS_REQUIRE(field && uT && F, VERIS_ERR_ARG);
    zonal_flux_only_kernel<double><<<g2, bl, 0, st>>>(c, halo_fill_of(*p), field, uT, F);
    return launch_status();
}

int veris_calc_meridional_flux_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                   const double *field, const double *vT, double *G, veris_stream_t s) {
    ADV_CTX(double)
    VERIS_REQUIRE(field && vT && G, VERIS_ERR_ARG);
    meridional_flux_only_kernel<double><<<g2, bl, 0, st>>>(c, halo_fill_of(*p), field, vT, G);
    return launch_status();
}

int veris_calc_advection_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                             const double *field, double *out, void *ws, size_t ws_bytes, veris_stream_t s) {
    const double *in[1] = {field};
    double *o[1] = {out};
    return advect<double>(g, p, reinterpret_cast<const Fields<double> *>(vs), 1, in, o, ws, ws_bytes, s);
}

int veris_advection_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, double *h,
                        double *hs, double *A, void *ws, size_t ws_bytes, veris_stream_t s) {
    VERIS_REQUIRE(vs, VERIS_ERR_ARG);
    const double *in[3] = {vs->hIceMean, vs->hSnowMean, vs->Area};
    double *o[3] = {h, hs, A};
    return advect<double>(g, p, reinterpret_cast<const Fields<double> *>(vs), 3, in, o, ws, ws_bytes, s);
}

int veris_advection_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF32 *vs, float *h,
                        float *hs, float *A, void *ws, size_t ws_bytes, veris_stream_t s) {
    VERIS_REQUIRE(vs, VERIS_ERR_ARG);
    const float *in[3] = {vs->hIceMean, vs->hSnowMean, vs->Area};
    float *o[3] = {h, hs, A};
    return advect<float>(g, p, reinterpret_cast<const Fields<float> *>(vs), 3, in, o, ws, ws_bytes, s);
}

int veris_clean_up_advection_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                 double *h, double *hs, double *A, double *TS, double *osh, double *oshs,
                                 veris_stream_t s) {
    ADV_CTX(double)
    VERIS_REQUIRE(h && hs && A && TS && osh && oshs, VERIS_ERR_ARG);
    clean_up_kernel<double><<<g2, bl, 0, st>>>(c, h, hs, A, TS, osh, oshs, 0);
    return launch_status();
}

int veris_ridging_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, double *A,
                      veris_stream_t s) {
    ADV_CTX(double)
    VERIS_REQUIRE(A, VERIS_ERR_ARG);
    ridging_kernel<double><<<g2, bl, 0, st>>>(c, A);
    return launch_status();
}

}  // extern "C"
