// Once-per-step routines of the sea-ice dynamics and the inner EVP routines
// as standalone kernels: dynamics preparation, strain rates, viscosities,
// drag coefficients, stress divergence, ocean stress and the halo fill.
//
// One thread per padded point; threadIdx.x runs along y (the contiguous
// axis) so that a warp touches 32 consecutive elements of a row.
#include "stencil.cuh"

namespace veris {

constexpr int BX = 32, BY = 8;

inline dim3 grid2d(const Dims &d) { return dim3((d.NY + BX - 1) / BX, (d.NX + BY - 1) / BY); }

#define POINT_IJ                                      \
    const int j = blockIdx.x * BX + threadIdx.x;      \
    const int i = blockIdx.y * BY + threadIdx.y;      \
    if (i >= c.d.NX || j >= c.d.NY) return;           \
    const int64_t k = c.d.raw(i, j);

template <class T>
static Ctx<T> make_ctx(const Dims &d, const VerisParams &p, const Fields<T> &f) {
    Ctx<T> c;
    c.f = f;
    c.d = d;
    c.p = p;
    return c;
}

// --------------------------------------------------------------- halo fill
// veris/fill_overlap.py:6-18; sources of every filled halo point are interior
// points, so the fill is safe in place.
template <class T>
__global__ void fill_kernel(T *A, Dims d, HaloFill h) {
    const int j = blockIdx.x * BX + threadIdx.x;
    const int i = blockIdx.y * BY + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const bool hx = h.x_fill && in_xhalo(d, h.olx, i);
    const bool hy = h.y_fill && in_yhalo(d, h.oly, j);
    if (!hx && !hy) return;
    int si = i, sj = j;
    if (hx) si = i < h.olx ? i + d.nx : i - d.nx;
    if (hy) sj = j < h.oly ? j + d.ny : j - d.ny;
    A[d.raw(i, j)] = A[d.raw(si, sj)];
}

template <class T>
static int fill_overlap(const VerisGrid *g, const VerisParams *p, T *A, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && A, VERIS_ERR_ARG);
    HaloFill h = halo_fill_of(*p);
    if (!h.x_fill && !h.y_fill) return VERIS_OK;
    fill_kernel<T><<<grid2d(d), dim3(BX, BY), 0, (cudaStream_t)s>>>(A, d, h);
    return launch_status();
}

// transpose of the halo fill, out of place: the adjoint held by each halo
// image moves onto its interior source and the image's own becomes zero
__global__ void fill_adjoint_kernel(const double *lin, double *lout, Dims d, HaloFill h) {
    const int j = blockIdx.x * BX + threadIdx.x;
    const int i = blockIdx.y * BY + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const int64_t o = d.raw(i, j);
    if ((h.x_fill && in_xhalo(d, h.olx, i)) || (h.y_fill && in_yhalo(d, h.oly, j))) {
        lout[o] = 0.0;
        return;
    }
    int ix = -1, jy = -1;
    if (h.x_fill) {
        if (i + d.nx < d.NX && in_xhalo(d, h.olx, i + d.nx)) ix = i + d.nx;
        else if (i - d.nx >= 0 && in_xhalo(d, h.olx, i - d.nx)) ix = i - d.nx;
    }
    if (h.y_fill) {
        if (j + d.ny < d.NY && in_yhalo(d, h.oly, j + d.ny)) jy = j + d.ny;
        else if (j - d.ny >= 0 && in_yhalo(d, h.oly, j - d.ny)) jy = j - d.ny;
    }
    double acc = lin[o];
    if (ix >= 0) acc += lin[d.raw(ix, j)];
    if (jy >= 0) acc += lin[d.raw(i, jy)];
    if (ix >= 0 && jy >= 0) acc += lin[d.raw(ix, jy)];
    lout[o] = acc;
}

// ------------------------------------------------------- step preparation
template <class T>
__global__ void sea_ice_mass_kernel(Ctx<T> c, T *mC, T *mU, T *mV) {
    POINT_IJ
    auto mass = [&](int a, int b) {
        return T(c.p.rhoIce) * c.ld(c.f.hIceMean, a, b) + T(c.p.rhoSnow) * c.ld(c.f.hSnowMean, a, b);
    };
    const T m0 = mass(i, j);
    mC[k] = m0;
    mU[k] = T(0.5) * (m0 + mass(i - 1, j));
    mV[k] = T(0.5) * (m0 + mass(i, j - 1));
}

template <class T>
__global__ void area_ws_kernel(Ctx<T> c, T *AW, T *AS) {
    POINT_IJ
    const T a = c.ld(c.f.Area, i, j);
    AW[k] = T(0.5) * (a + c.ld(c.f.Area, i - 1, j));
    AS[k] = T(0.5) * (a + c.ld(c.f.Area, i, j - 1));
}

template <class T>
__global__ void strength_kernel(Ctx<T> c, T *P) {
    POINT_IJ
    P[k] = T(c.p.pStar) * c.ld(c.f.hIceMean, i, j) * exp(-T(c.p.cStar) * (T(1) - c.ld(c.f.Area, i, j))) *
           c.ld(c.f.iceMask, i, j);
}

// veris/dynsolver.py:44-68: air-ice stress components at the C point
template <class T>
__device__ __forceinline__ void tau_c(const Ctx<T> &c, int i, int j, T &tx, T &ty) {
    T urel, vrel;
    if (c.p.useRelativeWind) {
        urel = c.ld(c.f.uWind, i, j) - T(0.5) * (c.ld(c.f.uIce, i, j) + c.ld(c.f.uIce, i + 1, j));
        vrel = c.ld(c.f.vWind, i, j) - T(0.5) * (c.ld(c.f.vIce, i, j) + c.ld(c.f.vIce, i, j + 1));
    } else {
        urel = c.ld(c.f.uWind, i, j);
        vrel = c.ld(c.f.vWind, i, j);
    }
    const T ws2 = urel * urel + vrel * vrel;
    const T wmin = T(c.p.wSpeedMin);
    const T speed = ws2 < T(c.p.wSpeedMin * c.p.wSpeedMin) ? wmin : sqrt(ws2);
    const T fc = c.ld(c.f.fCori, i, j);
    const T cd = T((double)(fc < T(0) ? c.p.airIceDrag_south : c.p.airIceDrag) * c.p.rhoAir) * speed;
    const T sg = sgn(fc);
    tx = cd * (T(c.p.cosWin) * urel - sg * T(c.p.sinWin) * vrel);
    ty = cd * (T(c.p.cosWin) * vrel + sg * T(c.p.sinWin) * urel);
}

template <class T>
__device__ __forceinline__ void tau_uv(const Ctx<T> &c, int i, int j, T &tauX, T &tauY) {
    T tx0, ty0, txw, tyw, txs, tys;
    tau_c(c, i, j, tx0, ty0);
    tau_c(c, i - 1, j, txw, tyw);
    tau_c(c, i, j - 1, txs, tys);
    tauX = T(0.5) * (tx0 + txw) * c.ld(c.f.iceMaskU, i, j);
    tauY = T(0.5) * (ty0 + tys) * c.ld(c.f.iceMaskV, i, j);
}

// The U/V averages of the once-per-step C-point quantities (air stress,
// ocean drag) take the C point of the output and its west or south
// neighbour: a block first evaluates them at the (BY+1) x (BX+1) C points its
// outputs touch (one evaluation, with its float64 square root, per point
// instead of three), then averages from shared memory.  The evaluations are
// the same calls with the same (wrapped) indices, so the results are
// unchanged.
template <class T, class F>
__device__ __forceinline__ void tile_c_points(const Ctx<T> &c, T (*a)[BX + 1], T (*b)[BX + 1], F eval) {
    const int i0 = blockIdx.y * BY - 1, j0 = blockIdx.x * BX - 1;
    for (int e = threadIdx.y * BX + threadIdx.x; e < (BY + 1) * (BX + 1); e += BX * BY) {
        const int r = e / (BX + 1), q = e - r * (BX + 1);
        const int i = i0 + r, j = j0 + q;   // -1 at the first tiles: wrapped by the loads
        T x = T(0), y = T(0);
        if (i < c.d.NX && j < c.d.NY) eval(i, j, x, y);
        a[r][q] = x;
        if (b) b[r][q] = y;
    }
    __syncthreads();
}

// tau_uv from a block's tile of C-point stresses
template <class T>
__device__ __forceinline__ void tau_uv_tile(const Ctx<T> &c, const T (*stx)[BX + 1], const T (*sty)[BX + 1], int i,
                                            int j, T &tauX, T &tauY) {
    const int r = threadIdx.y + 1, q = threadIdx.x + 1;
    tauX = T(0.5) * (stx[r][q] + stx[r - 1][q]) * c.ld(c.f.iceMaskU, i, j);
    tauY = T(0.5) * (sty[r][q] + sty[r][q - 1]) * c.ld(c.f.iceMaskV, i, j);
}

template <class T>
__global__ void __launch_bounds__(BX * BY) tau_xy_kernel(Ctx<T> c, T *tauX, T *tauY) {
    __shared__ T stx[BY + 1][BX + 1], sty[BY + 1][BX + 1];
    tile_c_points(c, stx, sty, [&](int i, int j, T &x, T &y) { tau_c(c, i, j, x, y); });
    POINT_IJ
    T tX, tY;
    tau_uv_tile(c, stx, sty, i, j, tX, tY);
    tauX[k] = tX;
    tauY[k] = tY;
}

// veris/dynsolver.py:91-101: geopotential of the sea surface
template <class T>
__device__ __forceinline__ T phi_surf(const Ctx<T> &c, int i, int j) {
    T phi = T(c.p.gravity) * c.ld(c.f.ssh_an, i, j);
    if (c.p.useRealFreshWaterFlux)
        phi = phi + (c.ld(c.f.surfPress, i, j) +
                     c.ld(c.f.SeaIceLoad, i, j) * T(c.p.gravity) * T(c.p.seaIceLoadFac)) *
                        T(c.p.recip_rhoSea);
    else
        phi = phi + c.ld(c.f.surfPress, i, j) * T(c.p.recip_rhoSea);
    return phi;
}

template <class T>
__global__ void __launch_bounds__(BX * BY) wind_forcing_kernel(Ctx<T> c, T *fxo, T *fyo) {
    __shared__ T stx[BY + 1][BX + 1], sty[BY + 1][BX + 1];
    tile_c_points(c, stx, sty, [&](int i, int j, T &x, T &y) { tau_c(c, i, j, x, y); });
    POINT_IJ
    T tX, tY;
    tau_uv_tile(c, stx, sty, i, j, tX, tY);
    T fx = tX * c.ld(c.f.AreaW, i, j);
    T fy = tY * c.ld(c.f.AreaS, i, j);
    const T phi = phi_surf(c, i, j);
    fx = fx - c.ld(c.f.SeaIceMassU, i, j) * c.ld(c.f.recip_dxC, i, j) * (phi - phi_surf(c, i - 1, j));
    fy = fy - c.ld(c.f.SeaIceMassV, i, j) * c.ld(c.f.recip_dyC, i, j) * (phi - phi_surf(c, i, j - 1));
    fxo[k] = fx;
    fyo[k] = fy;
}

// ------------------------------------------------------ EVP inner routines
template <class T>
__global__ void strainrates_kernel(Ctx<T> c, const T *u, const T *v, T *e11, T *e22, T *e12) {
    POINT_IJ
    T a, b;
    strain_c(c, u, v, i, j, a, b);
    e11[k] = a;
    e22[k] = b;
    e12[k] = strain_z(c, u, v, i, j);
}

template <class T>
__global__ void viscosities_kernel(Ctx<T> c, const T *e11, const T *e22, const T *e12, T *zeta,
                                   T *eta, T *press) {
    POINT_IJ
    auto z = [&](int a, int b) { return c.ld(c.f.rAz, a, b) * sq(c.ld(e12, a, b)); };
    T zt, et, pr, dl;
    viscosity_c(c, i, j, c.ld(e11, i, j), c.ld(e22, i, j), z(i, j), z(i + 1, j), z(i, j + 1),
                z(i + 1, j + 1), zt, et, pr, dl);
    zeta[k] = zt;
    eta[k] = et;
    press[k] = pr;
}

template <class T>
__global__ void c2z_kernel(Ctx<T> c, const T *C, int noSlip, T *Z) {
    POINT_IJ
    const T zs = C[c.d.at(i, j)] + C[c.d.at(i - 1, j)];
    const T zss = C[c.d.at(i, j - 1)] + C[c.d.at(i - 1, j - 1)];
    Z[k] = c2z_norm(c, i, j, noSlip != 0) * (zs + zss);
}

template <class T>
__global__ void ocean_drag_kernel(Ctx<T> c, const T *u, const T *v, T *cd) {
    POINT_IJ
    cd[k] = ocean_drag_c(c, u, v, i, j);
}

template <class T>
__global__ void basal_drag_kernel(Ctx<T> c, const T *u, const T *v, T *cb) {
    POINT_IJ
    cb[k] = basal_drag_c(c, u, v, i, j);
}

template <class T>
__global__ void side_drag_kernel(Ctx<T> c, const T *u, const T *v, T *sU, T *sV) {
    POINT_IJ
    const T sp0 = ice_speed_c(c, u, v, i, j);
    sU[k] = side_drag_u(c, i, j, sp0, ice_speed_c(c, u, v, i - 1, j));
    sV[k] = side_drag_v(c, i, j, sp0, ice_speed_c(c, u, v, i, j - 1));
}

template <class T>
__global__ void stressdiv_kernel(Ctx<T> c, const T *s11, const T *s22, const T *s12, T *dX,
                                 T *dY) {
    POINT_IJ
    const Fields<T> &f = c.f;
    const T a0 = c.ld(s11, i, j) * c.ld(f.dyV, i, j);
    const T aw = c.ld(s11, i - 1, j) * c.ld(f.dyV, i - 1, j);
    const T b0 = c.ld(s12, i, j) * c.ld(f.dxV, i, j);
    const T bn = c.ld(s12, i, j + 1) * c.ld(f.dxV, i, j + 1);
    dX[k] = (a0 - aw - b0 + bn) * c.ld(f.recip_rAu, i, j);
    const T a1 = c.ld(s22, i, j) * c.ld(f.dxU, i, j);
    const T as = c.ld(s22, i, j - 1) * c.ld(f.dxU, i, j - 1);
    const T b1 = c.ld(s12, i, j) * c.ld(f.dyU, i, j);
    const T be = c.ld(s12, i + 1, j) * c.ld(f.dyU, i + 1, j);
    dY[k] = (a1 - as - b1 + be) * c.ld(f.recip_rAv, i, j);
}

// veris/ocean_stress.py:19-37 with the halo fill of :39 fused into the store
template <class T>
__global__ void __launch_bounds__(BX * BY) ocean_stress_kernel(Ctx<T> c, HaloFill h, T *su, T *sv) {
    __shared__ T scd[BY + 1][BX + 1];
    const Fields<T> &f = c.f;
    const T *u = f.uIce, *v = f.vIce;
    tile_c_points(c, scd, (T(*)[BX + 1]) nullptr,
                  [&](int i, int j, T &x, T &) { x = ocean_drag_c(c, u, v, i, j); });
    POINT_IJ
    (void)k;
    const int r = threadIdx.y + 1, q = threadIdx.x + 1;
    const T cd0 = scd[r][q], cdw = scd[r - 1][q], cds = scd[r][q - 1];
    auto du = [&](int a, int b) { return c.ld(u, a, b) - c.ld(f.uOcean, a, b); };
    auto dv = [&](int a, int b) { return c.ld(v, a, b) - c.ld(f.vOcean, a, b); };
    const T sg = sgn(c.ld(f.fCori, i, j));
    const T sinW = T(c.p.sinWatOcn), cosW = T(c.p.cosWatOcn);
    // cDrag * dvAtC at C(i,j) and C(i,j-1); cDrag * duAtC at C(i,j) and C(i-1,j)
    const T a0 = cd0 * (T(0.5) * (dv(i, j) + dv(i, j + 1)));
    const T as = cds * (T(0.5) * (dv(i, j - 1) + dv(i, j)));
    const T b0 = cd0 * (T(0.5) * (du(i, j) + du(i + 1, j)));
    const T bw = cdw * (T(0.5) * (du(i - 1, j) + du(i, j)));
    const T ou = T(0.5) * (cd0 + cdw) * cosW * du(i, j) - sg * sinW * T(0.5) * (a0 + as);
    const T ov = T(0.5) * (cd0 + cds) * cosW * dv(i, j) + sg * sinW * T(0.5) * (b0 + bw);
    store_filled(su, c.d, h, i, j, ou);
    store_filled(sv, c.d, h, i, j, ov);
}

// ------------------------------------------------ dynamics-preparation adjoint
// Reverse of SeaIceMass, AreaWS, WindForcingXY (with tauXY) and SeaIceStrength
// (veris/area_mass.py:5-28, veris/dynsolver.py:7-84,
// veris/dynamics_routines.py:5-18), in float64, as three gather passes.
struct PrepAdj {
    // adjoints of the preparation's outputs (inputs of this pass)
    const double *lP, *lmC, *lmU, *lmV, *lAW, *lAS, *lWX, *lWY;
    // scratch: totals at U/V points and the wind-stress adjoints at C points
    double *ltX, *ltY, *lAWt, *lASt, *lmUt, *lmVt, *lur, *lvr;
    // accumulated adjoints of the ice state
    double *lh, *lhs, *lA, *lu, *lv;
    double *scal;   // [0] P*, [1] airIceDrag, [2] airIceDrag_south
};

__global__ void prep_adj_uv_kernel(Ctx<double> c, PrepAdj a) {
    POINT_IJ
    double tX, tY;
    tau_uv(c, i, j, tX, tY);
    const double phi = phi_surf(c, i, j);
    const double lwx = a.lWX[k], lwy = a.lWY[k];
    // AreaW/AreaS of this state (the table's may be another step's)
    const double A0 = c.ld(c.f.Area, i, j);
    a.ltX[k] = 0.5 * (A0 + c.ld(c.f.Area, i - 1, j)) * lwx;
    a.ltY[k] = 0.5 * (A0 + c.ld(c.f.Area, i, j - 1)) * lwy;
    a.lAWt[k] = a.lAW[k] + tX * lwx;
    a.lASt[k] = a.lAS[k] + tY * lwy;
    a.lmUt[k] = a.lmU[k] - c.ld(c.f.recip_dxC, i, j) * (phi - phi_surf(c, i - 1, j)) * lwx;
    a.lmVt[k] = a.lmV[k] - c.ld(c.f.recip_dyC, i, j) * (phi - phi_surf(c, i, j - 1)) * lwy;
}

__global__ void prep_adj_c_kernel(Ctx<double> c, PrepAdj a) {
    const int j = blockIdx.x * BX + threadIdx.x;
    const int i = blockIdx.y * BY + threadIdx.y;
    double sP = 0.0, sN = 0.0, sS = 0.0;
    if (i < c.d.NX && j < c.d.NY) {
        const int64_t k = c.d.raw(i, j);
        const Fields<double> &f = c.f;
        // wind stress at C: tauX(U i) = 0.5 (tx(i) + tx(i-1)) mskU(i)
        const double ltx = 0.5 * (c.ld(f.iceMaskU, i, j) * a.ltX[k] + c.ld(f.iceMaskU, i + 1, j) * a.ltX[c.d.at(i + 1, j)]);
        const double lty = 0.5 * (c.ld(f.iceMaskV, i, j) * a.ltY[k] + c.ld(f.iceMaskV, i, j + 1) * a.ltY[c.d.at(i, j + 1)]);
        double urel, vrel;
        if (c.p.useRelativeWind) {
            urel = c.ld(f.uWind, i, j) - 0.5 * (c.ld(f.uIce, i, j) + c.ld(f.uIce, i + 1, j));
            vrel = c.ld(f.vWind, i, j) - 0.5 * (c.ld(f.vIce, i, j) + c.ld(f.vIce, i, j + 1));
        } else {
            urel = c.ld(f.uWind, i, j);
            vrel = c.ld(f.vWind, i, j);
        }
        const double ws2 = urel * urel + vrel * vrel;
        const bool floored = ws2 < c.p.wSpeedMin * c.p.wSpeedMin;
        const double speed = floored ? c.p.wSpeedMin : sqrt(ws2);
        const double fc = c.ld(f.fCori, i, j);
        const bool south = fc < 0;
        const double D = (south ? c.p.airIceDrag_south : c.p.airIceDrag) * c.p.rhoAir;
        const double sg = sgn(fc), cw = c.p.cosWin, sw = c.p.sinWin;
        const double ax = cw * urel - sg * sw * vrel, ay = cw * vrel + sg * sw * urel;
        const double su = floored ? 0.0 : urel / speed, sv = floored ? 0.0 : vrel / speed;
        // tx = D speed ax, ty = D speed ay
        a.lur[k] = D * (ltx * (su * ax + speed * cw) + lty * (su * ay + speed * sg * sw));
        a.lvr[k] = D * (ltx * (sv * ax - speed * sg * sw) + lty * (sv * ay + speed * cw));
        const double lD = c.p.rhoAir * speed * (ltx * ax + lty * ay);
        if (south) sS = lD; else sN = lD;
        // ice strength P = P* h exp(-C* (1 - A)) mask
        const double h = c.ld(f.hIceMean, i, j), A = c.ld(f.Area, i, j), m = c.ld(f.iceMask, i, j);
        const double e = exp(-c.p.cStar * (1.0 - A));
        const double lP = a.lP[k];
        sP = lP * h * e * m;
        double lh = lP * c.p.pStar * e * m, lA = lP * c.p.pStar * h * e * c.p.cStar * m;
        // masses: mU(i) = (mC(i) + mC(i-1))/2, mV(j) = (mC(j) + mC(j-1))/2
        const double lmC = a.lmC[k] + 0.5 * (a.lmUt[k] + a.lmUt[c.d.at(i + 1, j)]) +
                           0.5 * (a.lmVt[k] + a.lmVt[c.d.at(i, j + 1)]);
        lh += c.p.rhoIce * lmC;
        a.lhs[k] += c.p.rhoSnow * lmC;
        // areas: AW(i) = (A(i) + A(i-1))/2, AS(j) = (A(j) + A(j-1))/2
        lA += 0.5 * (a.lAWt[k] + a.lAWt[c.d.at(i + 1, j)]) + 0.5 * (a.lASt[k] + a.lASt[c.d.at(i, j + 1)]);
        a.lh[k] += lh;
        a.lA[k] += lA;
    }
    // scalar sums: warp shuffles, one atomic per warp
    for (int off = 16; off > 0; off >>= 1) {
        sP += __shfl_down_sync(0xffffffffu, sP, off);
        sN += __shfl_down_sync(0xffffffffu, sN, off);
        sS += __shfl_down_sync(0xffffffffu, sS, off);
    }
    if (threadIdx.x == 0) {
        if (sP != 0.0) atomicAdd(a.scal + 0, sP);
        if (sN != 0.0) atomicAdd(a.scal + 1, sN);
        if (sS != 0.0) atomicAdd(a.scal + 2, sS);
    }
}

__global__ void prep_adj_vel_kernel(Ctx<double> c, PrepAdj a) {
    POINT_IJ
    if (!c.p.useRelativeWind) return;
    // urel(C i) = uWind - (u(i) + u(i+1))/2: u(i) enters C(i) and C(i-1)
    a.lu[k] += -0.5 * (a.lur[k] + a.lur[c.d.at(i - 1, j)]);
    a.lv[k] += -0.5 * (a.lvr[k] + a.lvr[c.d.at(i, j - 1)]);
}

}  // namespace veris

using namespace veris;

#define PREP_BEGIN(T, FT)                              \
    Dims d;                                            \
    VERIS_CHECK_GRID(g, d);                            \
    VERIS_REQUIRE(p && vs, VERIS_ERR_ARG);             \
    Ctx<T> c = make_ctx<T>(d, *p, *reinterpret_cast<const Fields<T> *>(vs)); \
    cudaStream_t st = (cudaStream_t)s;                 \
    dim3 gr = grid2d(d), bl(BX, BY);

extern "C" {

int veris_fill_overlap_f64(const VerisGrid *g, const VerisParams *p, double *A, veris_stream_t s) {
    return fill_overlap<double>(g, p, A, s);
}
int veris_fill_overlap_adjoint_f64(const VerisGrid *g, const VerisParams *p, const double *lam_in,
                                   double *lam_out, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && lam_in && lam_out && lam_in != lam_out, VERIS_ERR_ARG);
    fill_adjoint_kernel<<<grid2d(d), dim3(BX, BY), 0, (cudaStream_t)s>>>(lam_in, lam_out, d, halo_fill_of(*p));
    return launch_status();
}
int veris_fill_overlap_f32(const VerisGrid *g, const VerisParams *p, float *A, veris_stream_t s) {
    return fill_overlap<float>(g, p, A, s);
}

int veris_sea_ice_mass_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                           double *mC, double *mU, double *mV, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(mC && mU && mV, VERIS_ERR_ARG);
    sea_ice_mass_kernel<double><<<gr, bl, 0, st>>>(c, mC, mU, mV);
    return launch_status();
}

int veris_area_ws_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                      double *AW, double *AS, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(AW && AS, VERIS_ERR_ARG);
    area_ws_kernel<double><<<gr, bl, 0, st>>>(c, AW, AS);
    return launch_status();
}

int veris_tau_xy_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                     double *tX, double *tY, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(tX && tY, VERIS_ERR_ARG);
    tau_xy_kernel<double><<<gr, bl, 0, st>>>(c, tX, tY);
    return launch_status();
}

int veris_wind_forcing_xy_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                              double *fx, double *fy, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(fx && fy, VERIS_ERR_ARG);
    wind_forcing_kernel<double><<<gr, bl, 0, st>>>(c, fx, fy);
    return launch_status();
}

int veris_sea_ice_strength_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                               double *P, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(P, VERIS_ERR_ARG);
    strength_kernel<double><<<gr, bl, 0, st>>>(c, P);
    return launch_status();
}

int veris_strainrates_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                          const double *u, const double *v, double *e11, double *e22, double *e12,
                          veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(u && v && e11 && e22 && e12, VERIS_ERR_ARG);
    strainrates_kernel<double><<<gr, bl, 0, st>>>(c, u, v, e11, e22, e12);
    return launch_status();
}

int veris_viscosities_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                          const double *e11, const double *e22, const double *e12, double *zeta,
                          double *eta, double *press, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(e11 && e22 && e12 && zeta && eta && press, VERIS_ERR_ARG);
    viscosities_kernel<double><<<gr, bl, 0, st>>>(c, e11, e22, e12, zeta, eta, press);
    return launch_status();
}

int veris_c_point_to_z_point_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                 const double *C, int32_t noSlip, double *Z, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(C && Z, VERIS_ERR_ARG);
    c2z_kernel<double><<<gr, bl, 0, st>>>(c, C, noSlip, Z);
    return launch_status();
}

int veris_ocean_drag_coeffs_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                const double *u, const double *v, double *cd, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(u && v && cd, VERIS_ERR_ARG);
    ocean_drag_kernel<double><<<gr, bl, 0, st>>>(c, u, v, cd);
    return launch_status();
}

int veris_basal_drag_coeffs_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                const double *u, const double *v, double *cb, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(u && v && cb, VERIS_ERR_ARG);
    basal_drag_kernel<double><<<gr, bl, 0, st>>>(c, u, v, cb);
    return launch_status();
}

int veris_side_drag_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                        const double *u, const double *v, double *sU, double *sV, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(u && v && sU && sV, VERIS_ERR_ARG);
    side_drag_kernel<double><<<gr, bl, 0, st>>>(c, u, v, sU, sV);
    return launch_status();
}

int veris_stressdiv_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                        const double *s11, const double *s22, const double *s12, double *dX,
                        double *dY, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(s11 && s22 && s12 && dX && dY, VERIS_ERR_ARG);
    stressdiv_kernel<double><<<gr, bl, 0, st>>>(c, s11, s22, s12, dX, dY);
    return launch_status();
}

size_t veris_prep_adjoint_workspace_bytes(const VerisGrid *g) {
    Dims d;
    if (check_grid(g, &d) != VERIS_OK) return 0;
    return 8 * (((size_t)d.NX * d.ld * sizeof(double) + 255) / 256 * 256);
}

int veris_prep_adjoint_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                           const VerisFieldsF64 *lprep, double *lh, double *lhs, double *lA, double *lu, double *lv,
                           double *scalars, void *ws, size_t wsb, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(lprep && lh && lhs && lA && lu && lv && scalars, VERIS_ERR_ARG);
    VERIS_REQUIRE(!p->useRealFreshWaterFlux, VERIS_ERR_UNSUPPORTED);
    const size_t fb = ((size_t)d.NX * d.ld * sizeof(double) + 255) / 256 * 256;
    VERIS_REQUIRE(ws && wsb >= 8 * fb, VERIS_ERR_WORKSPACE);
    const VerisFieldsF64 &L = *lprep;
    VERIS_REQUIRE(L.SeaIceStrength && L.SeaIceMassC && L.SeaIceMassU && L.SeaIceMassV && L.AreaW && L.AreaS &&
                      L.WindForcingX && L.WindForcingY,
                  VERIS_ERR_ARG);
    PrepAdj a;
    a.lP = L.SeaIceStrength;
    a.lmC = L.SeaIceMassC;
    a.lmU = L.SeaIceMassU;
    a.lmV = L.SeaIceMassV;
    a.lAW = L.AreaW;
    a.lAS = L.AreaS;
    a.lWX = L.WindForcingX;
    a.lWY = L.WindForcingY;
    double **scr[8] = {&a.ltX, &a.ltY, &a.lAWt, &a.lASt, &a.lmUt, &a.lmVt, &a.lur, &a.lvr};
    for (int q = 0; q < 8; ++q) *scr[q] = reinterpret_cast<double *>(static_cast<char *>(ws) + q * fb);
    a.lh = lh;
    a.lhs = lhs;
    a.lA = lA;
    a.lu = lu;
    a.lv = lv;
    a.scal = scalars;
    prep_adj_uv_kernel<<<gr, bl, 0, st>>>(c, a);
    prep_adj_c_kernel<<<gr, bl, 0, st>>>(c, a);
    prep_adj_vel_kernel<<<gr, bl, 0, st>>>(c, a);
    return launch_status();
}

int veris_ocean_stress_uv_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                              double *su, double *sv, veris_stream_t s) {
    PREP_BEGIN(double, VerisFieldsF64)
    VERIS_REQUIRE(su && sv, VERIS_ERR_ARG);
    ocean_stress_kernel<double><<<gr, bl, 0, st>>>(c, halo_fill_of(*p), su, sv);
    return launch_status();
}

}  // extern "C"
