// Flux-limited advection of hIceMean, hSnowMean and Area
// (veris/advection.py:15-175) and the post-advection clean-up
// (veris/clean_up.py:5-47).
//
// Dimensionally split: zonal fluxes, zonal update, meridional fluxes (of the
// zonally updated field), meridional update.  Each phase is one launch over
// all advected fields (blockIdx.z = field).  The fluxes are stored with the
// halo fill the reference applies to them fused into the store.
#include "stencil.cuh"
#include "dual.cuh"

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

// limited flux through one face (veris/advection.py:107-126) from the four
// field values around the face, their slope masks, the transport and the
// Courant number.  S is the arithmetic type, or a dual number when the
// adjoint needs the local Jacobian; the branches follow the values.
template <class S>
__device__ __forceinline__ S superbee_t(const S &cr) {
    const S a = S(2) * cr < S(1) ? S(2) * cr : S(1);
    const S b = cr < S(2) ? cr : S(2);
    const S m = a > b ? a : b;
    return m > S(0) ? m : S(0);
}

template <class S>
__device__ __forceinline__ S limited_flux_t(const S &fmm, const S &fm, const S &f0, const S &fp, double mm,
                                            double m0, double mp, const S &trans, const S &cfl, double CrMax) {
    const S Rjp = (fp - f0) * mp;
    const S Rj = (f0 - fm) * m0;
    const S Rjm = (fm - fmm) * mm;
    S cr = trans > 0 ? Rjm : Rjp;
    if (vfabs(Rj) * CrMax > vfabs(cr)) cr = cr / Rj;
    else cr = S(double(sgn(val(cr))) * CrMax * double(sgn(val(Rj))));
    cr = superbee_t(cr);
    return trans * (f0 + fm) * 0.5 - vfabs(trans) * ((1 - cr) + cfl * cr) * Rj * 0.5;
}

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

// ------------------------------------------------------------- adjoint
// Adjoint of the advection of up to three fields (veris/advection.py:28-91)
// in float64.  With c = deltatTherm * maskInC / rA, the forward is
//   f1 = f - c (F(i+1) - F(i)),  f2 = f1 - c (G(j+1) - G(j)),  out = f2 * iceMask
// where F reads f(i-2..i+1) and u(i), G reads f1(j-2..j+1) and v(j), and both
// are stored with the halo images of their fill.

struct AdvAdjIO {
    const double *field[MAX_ADV_FIELDS];   // f before advection
    const double *f1[MAX_ADV_FIELDS];      // f after the zonal update (forward recompute)
    const double *lout[MAX_ADV_FIELDS];    // adjoint of out
    double *l2[MAX_ADV_FIELDS];            // adjoint of f2 (= iceMask * lout), scratch
    double *l1[MAX_ADV_FIELDS];            // adjoint of f1, scratch
    double *lin[MAX_ADV_FIELDS];           // adjoint of f, accumulated
    double *lu, *lv;                       // adjoints of u, v, accumulated
};

__global__ void adv_adj_init_kernel(Ctx<double> c, AdvAdjIO io) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y, q = blockIdx.z;
    if (i >= c.d.NX || j >= c.d.NY) return;
    const int64_t o = c.d.raw(i, j);
    const double l = __ldg(c.f.iceMask + o) * io.lout[q][o];
    io.l2[q][o] = l;
    io.l1[q][o] = l;
}

__global__ void adv_adj_copy_kernel(Ctx<double> c, AdvAdjIO io) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y, q = blockIdx.z;
    if (i >= c.d.NX || j >= c.d.NY) return;
    const int64_t o = c.d.raw(i, j);
    io.lin[q][o] += io.l1[q][o];
}

// adjoint of the update through the flux at face (i, j) of axis AXIS: the
// flux adjoint lF(x) = c(x) ln(x) - c(x-1) ln(x-1), folded from its halo
// images onto the source face, then pushed through the flux's local Jacobian
template <int AXIS>
__global__ void flux_adjoint_kernel(Ctx<double> c, HaloFill h, AdvAdjIO io) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y, q = blockIdx.z;
    const Dims &d = c.d;
    if (i >= d.NX || j >= d.NY) return;
    const bool hx = h.x_fill && in_xhalo(d, h.olx, i);
    const bool hy = h.y_fill && in_yhalo(d, h.oly, j);
    if (hx || hy) return;   // an image: its adjoint is handled by the source face
    const int along = AXIS == 0 ? i : j;
    const int nalong = AXIS == 0 ? d.NX : d.NY;
    if (along < 2 || along > nalong - 2) return;   // flux is the constant zero there
    const double *ln = AXIS == 0 ? io.l1[q] : io.l2[q];
    auto cf = [&](int a, int b) {
        const int64_t o = d.at(a, b);
        return c.p.deltatTherm * __ldg(c.f.maskInC + o) * __ldg(c.f.recip_rA + o);
    };
    auto lF = [&](int a, int b) {
        const int ap = AXIS == 0 ? a - 1 : a, bp = AXIS == 0 ? b : b - 1;
        return cf(a, b) * ln[d.at(a, b)] - cf(ap, bp) * ln[d.at(ap, bp)];
    };
    double lam = lF(i, j);
    {   // images of this face in the refreshed halos
        int ix[2] = {i, -1}, jy[2] = {j, -1};
        if (h.x_fill) {
            if (i + d.nx < d.NX && in_xhalo(d, h.olx, i + d.nx)) ix[1] = i + d.nx;
            else if (i - d.nx >= 0 && in_xhalo(d, h.olx, i - d.nx)) ix[1] = i - d.nx;
        }
        if (h.y_fill) {
            if (j + d.ny < d.NY && in_yhalo(d, h.oly, j + d.ny)) jy[1] = j + d.ny;
            else if (j - d.ny >= 0 && in_yhalo(d, h.oly, j - d.ny)) jy[1] = j - d.ny;
        }
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                if (!(a == 0 && b == 0) && ix[a] >= 0 && jy[b] >= 0) lam += lF(ix[a], jy[b]);
    }
    if (lam == 0.0) return;
    const double *fld = AXIS == 0 ? io.field[q] : io.f1[q];
    const int64_t s = AXIS == 0 ? d.ld : 1;   // stride along the axis
    const int64_t o = d.raw(i, j);
    using D = Dual<5>;
    const D fmm = D::var(fld[o - 2 * s], 0), fm = D::var(fld[o - s], 1), f0 = D::var(fld[o], 2),
            fp = D::var(fld[o + s], 3);
    const double *vel = AXIS == 0 ? c.f.uIce : c.f.vIce;
    const D w = D::var(vel[o], 4);
    const double *mA = AXIS == 0 ? c.f.iceMaskU : c.f.iceMaskV;
    const double *mB = AXIS == 0 ? c.f.maskInU : c.f.maskInV;
    auto m = [&](int64_t k) { return mA[k] * mB[k]; };
    const double area = AXIS == 0 ? c.f.dyG[o] * c.f.iceMaskU[o] : c.f.dxG[o] * c.f.iceMaskV[o];
    const double rd = AXIS == 0 ? c.f.recip_dxC[o] : c.f.recip_dyC[o];
    const D trans = w * area;
    const D cfl = vfabs(w * c.p.deltatTherm * rd);
    const D F = limited_flux_t(fmm, fm, f0, fp, m(o - s), m(o), m(o + s), trans, cfl, c.p.CrMax);
    double *lf = AXIS == 0 ? io.lin[q] : io.l1[q];
    atomicAdd(lf + o - 2 * s, lam * F.d[0]);
    atomicAdd(lf + o - s, lam * F.d[1]);
    atomicAdd(lf + o, lam * F.d[2]);
    atomicAdd(lf + o + s, lam * F.d[3]);
    atomicAdd((AXIS == 0 ? io.lu : io.lv) + o, lam * F.d[4]);
}

// veris/clean_up.py:5-47 followed by ridging, for the ice state of one point
template <class S>
__device__ void cleanup_point(const VerisParams &p, S &h, S &hs, S &A, S &T) {
    h = h > 0 ? h : S(0.0);
    hs = hs > 0 ? hs : S(0.0);
    A = A > 0 ? A : S(0.0);
    if (h <= p.hIce_min) {
        h = h * 0.0;
        hs = hs * 0.0;
        T = S(p.celsius2K);
    }
    if (h == 0 && hs == 0) A = S(0.0);
    if (h > 0 || hs > 0) A = A > p.Area_min ? A : S(p.Area_min);
    A = A < 1 ? A : S(1.0);
}

// adjoint of clean-up + ridging: l_in = J^T l_out for (h, hs, A, TSurf)
__global__ void cleanup_adjoint_kernel(VerisParams p, Fields<double> f, Dims d, const double *lh, const double *lhs,
                                       const double *lA, const double *lT, double *oh, double *ohs, double *oA,
                                       double *oT) {
    const int j = blockIdx.x * ABX + threadIdx.x, i = blockIdx.y * ABY + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const int64_t o = d.raw(i, j);
    using D = Dual<4>;
    D h = D::var(f.hIceMean[o], 0), hs = D::var(f.hSnowMean[o], 1), A = D::var(f.Area[o], 2),
      T = D::var(f.TSurf[o], 3);
    cleanup_point(p, h, hs, A, T);
    const double l[4] = {lh[o], lhs[o], lA[o], lT[o]};
    const D *out[4] = {&h, &hs, &A, &T};
    double r[4] = {0, 0, 0, 0};
    for (int a = 0; a < 4; ++a)
        for (int k = 0; k < 4; ++k) r[k] += l[a] * out[a]->d[k];
    oh[o] = r[0];
    ohs[o] = r[1];
    oA[o] = r[2];
    oT[o] = r[3];
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

size_t veris_advection_adjoint_workspace_bytes(const VerisGrid *g) {
    const size_t f = veris_advection_workspace_bytes(g, 8);
    return f == 0 ? 0 : f + (f / (2 + 3 * MAX_ADV_FIELDS)) * 2 * MAX_ADV_FIELDS;
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

int veris_advection_adjoint_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                const double *l_h, const double *l_hs, const double *l_A, double *lin_h,
                                double *lin_hs, double *lin_A, double *l_u, double *l_v, void *ws, size_t wsb,
                                veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && l_h && l_hs && l_A && lin_h && lin_hs && lin_A && l_u && l_v, VERIS_ERR_ARG);
    VERIS_REQUIRE(p->extensiveFld, VERIS_ERR_UNSUPPORTED);
    const size_t fb = round_up_a((size_t)d.NX * d.ld * sizeof(double), 256);
    const size_t fwd = (size_t)(2 + 3 * MAX_ADV_FIELDS) * fb;
    VERIS_REQUIRE(ws && wsb >= fwd + 2 * MAX_ADV_FIELDS * fb, VERIS_ERR_WORKSPACE);
    // forward recompute: f1 of each field lives in the forward workspace
    Ctx<double> c;
    c.f = *reinterpret_cast<const Fields<double> *>(vs);
    c.d = d;
    c.p = *p;
    const HaloFill h = halo_fill_of(*p);
    char *w = static_cast<char *>(ws);
    double *uT = reinterpret_cast<double *>(w);
    double *vT = reinterpret_cast<double *>(w + fb);
    AdvIO<double> fio;
    const double *in[3] = {vs->hIceMean, vs->hSnowMean, vs->Area};
    AdvAdjIO aio;
    const double *lo[3] = {l_h, l_hs, l_A};
    double *li[3] = {lin_h, lin_hs, lin_A};
    for (int q = 0; q < MAX_ADV_FIELDS; ++q) {
        fio.field[q] = in[q];
        fio.F[q] = reinterpret_cast<double *>(w + (2 + q) * fb);
        fio.f1[q] = reinterpret_cast<double *>(w + (2 + MAX_ADV_FIELDS + q) * fb);
        fio.G[q] = reinterpret_cast<double *>(w + (2 + 2 * MAX_ADV_FIELDS + q) * fb);
        fio.out[q] = nullptr;
        aio.field[q] = in[q];
        aio.f1[q] = fio.f1[q];
        aio.lout[q] = lo[q];
        aio.l2[q] = reinterpret_cast<double *>(w + fwd + q * fb);
        aio.l1[q] = reinterpret_cast<double *>(w + fwd + (MAX_ADV_FIELDS + q) * fb);
        aio.lin[q] = li[q];
    }
    aio.lu = l_u;
    aio.lv = l_v;
    cudaStream_t st = (cudaStream_t)s;
    dim3 bl(ABX, ABY);
    dim3 g2((d.NY + ABX - 1) / ABX, (d.NX + ABY - 1) / ABY), g3(g2.x, g2.y, 3);
    transport_kernel<double><<<g2, bl, 0, st>>>(c, uT, vT);
    zonal_flux_kernel<double><<<g3, bl, 0, st>>>(c, h, fio, uT);
    zonal_update_kernel<double><<<g3, bl, 0, st>>>(c, fio);
    adv_adj_init_kernel<<<g3, bl, 0, st>>>(c, aio);
    flux_adjoint_kernel<1><<<g3, bl, 0, st>>>(c, h, aio);
    adv_adj_copy_kernel<<<g3, bl, 0, st>>>(c, aio);
    flux_adjoint_kernel<0><<<g3, bl, 0, st>>>(c, h, aio);
    return launch_status();
}

int veris_cleanup_adjoint_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                              const double *lh, const double *lhs, const double *lA, const double *lT, double *oh,
                              double *ohs, double *oA, double *oT, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && lh && lhs && lA && lT && oh && ohs && oA && oT, VERIS_ERR_ARG);
    dim3 bl(ABX, ABY), g2((d.NY + ABX - 1) / ABX, (d.NX + ABY - 1) / ABY);
    cleanup_adjoint_kernel<<<g2, bl, 0, (cudaStream_t)s>>>(*p, *reinterpret_cast<const Fields<double> *>(vs), d, lh,
                                                           lhs, lA, lT, oh, ohs, oA, oT);
    return launch_status();
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
