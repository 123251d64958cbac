// Point formulas of the C-grid stencils, shared by the standalone routine
// kernels and the tiled EVP subcycle.
//
// Every function evaluates one output at padded point (i, j); neighbours are
// read with periodic wrap over the padded array (the reference's roll).  The
// arithmetic follows the reference's order of operations so that float64
// results agree with the NumPy reference to rounding.
#pragma once

#include "common.cuh"

namespace veris {

template <class T>
struct Ctx {
    Fields<T> f;
    Dims d;
    VerisParams p;
    __device__ __forceinline__ T ld(const T *a, int i, int j) const { return __ldg(a + d.at(i, j)); }
};

// veris/dynamics_routines.py:151-158: e11, e22 at the C point
template <class T>
__device__ __forceinline__ void strain_c(const Ctx<T> &c, const T *u, const T *v, int i, int j,
                                         T &e11, T &e22) {
    const T u0 = c.ld(u, i, j), ue = c.ld(u, i + 1, j);
    const T v0 = c.ld(v, i, j), vn = c.ld(v, i, j + 1);
    const T dudx = (ue - u0) * c.ld(c.f.recip_dxU, i, j);
    const T uave = (ue + u0) * T(0.5);
    const T dvdy = (vn - v0) * c.ld(c.f.recip_dyV, i, j);
    const T vave = (vn + v0) * T(0.5);
    const T mC = c.ld(c.f.maskInC, i, j);
    e11 = (dudx + vave * c.ld(c.f.k2AtC, i, j)) * mC;
    e22 = (dvdy + uave * c.ld(c.f.k1AtC, i, j)) * mC;
}

// veris/dynamics_routines.py:161-215: e12 at the Z point
template <class T>
__device__ __forceinline__ T strain_z(const Ctx<T> &c, const T *u, const T *v, int i, int j) {
    const T u0 = c.ld(u, i, j), us = c.ld(u, i, j - 1);
    const T v0 = c.ld(v, i, j), vw = c.ld(v, i - 1, j);
    const T rdyU = c.ld(c.f.recip_dyU, i, j);
    const T rdxV = c.ld(c.f.recip_dxV, i, j);
    const T dudy = (u0 - us) * rdyU;
    const T uave = (u0 + us) * T(0.5);
    const T dvdx = (v0 - vw) * rdxV;
    const T vave = (v0 + vw) * T(0.5);
    const T *m = c.f.iceMask;
    T mz = c.ld(m, i, j) * c.ld(m, i - 1, j);
    mz = mz * (c.ld(m, i, j - 1) * c.ld(m, i - 1, j - 1));
    T e12 = T(0.5) * (dudy + dvdx - c.ld(c.f.k1AtZ, i, j) * vave - c.ld(c.f.k2AtZ, i, j) * uave) * mz;
    if (c.p.noSlip) {
        const T *mU = c.f.iceMaskU, *mV = c.f.iceMaskV;
        const T hU = c.ld(mU, i, j) - c.ld(mU, i, j - 1);
        const T hV = c.ld(mV, i, j) - c.ld(mV, i - 1, j);
        e12 = e12 + (T(2.0) * uave * rdyU * hU + T(2.0) * vave * rdxV * hV);
        if (c.p.secondOrderBC) {
            const T mU0 = c.ld(mU, i, j), mUw = c.ld(mU, i - 1, j);
            const T mV0 = c.ld(mV, i, j), mVs = c.ld(mV, i, j - 1);
            T h2U = (mU0 - mUw) / T(3.0);
            T h2V = (mV0 - mVs) / T(3.0);
            h2U = h2U * (c.ld(mU, i - 2, j) * mUw + c.ld(mU, i + 1, j) * mU0);
            h2V = h2V * (c.ld(mV, i, j - 2) * mVs + c.ld(mV, i, j + 1) * mV0);
            e12 = e12 + T(0.5) * (rdyU * (T(6.0) * uave - c.ld(u, i - 2, j) * mUw - c.ld(u, i + 1, j) * mU0) * h2U +
                                  rdxV * (T(6.0) * vave - c.ld(v, i, j - 2) * mVs - c.ld(v, i, j + 1) * mV0) * h2V);
        }
    }
    return e12;
}

// veris/dynamics_routines.py:233-266 from e11, e22 at C and the four rAz*e12^2
// Z-point products around it (z00 = Z(i,j), z10 = Z(i+1,j), z01 = Z(i,j+1), ...)
template <class T>
__device__ __forceinline__ void viscosity_c(const Ctx<T> &c, int i, int j, T e11, T e22, T z00,
                                            T z10, T z01, T z11, T &zeta, T &eta, T &press,
                                            T &delta) {
    const T rsq = T(1.0 / (c.p.PlasDefCoeff * c.p.PlasDefCoeff));
    const T e12Csq = T(0.25) * c.ld(c.f.recip_rA, i, j) * ((z00 + z10) + (z01 + z11));
    const T dsq = sq(e11 + e22) + rsq * (sq(e11 - e22) + T(4.0) * e12Csq);
    delta = sqrt(dsq);
    const T P = c.ld(c.f.SeaIceStrength, i, j);
    const T tsf = T(c.p.tensileStrFac), prf = T(c.p.pressReplFac);
    zeta = T(0.5) * (P * (T(1) + tsf)) / (delta + T(c.p.deltaMin));
    eta = zeta * rsq;
    press = (P * (T(1) - prf) + T(2.0) * zeta * delta * prf / (T(1) + tsf)) * (T(1) - tsf);
}

// veris/averaging.py:11-16: the normalisation of the C->Z mean
template <class T>
__device__ __forceinline__ T c2z_norm(const Ctx<T> &c, int i, int j, bool noSlip) {
    const T *m = c.f.iceMask;
    T n = c.ld(m, i, j) + c.ld(m, i - 1, j);
    n = n + (c.ld(m, i, j - 1) + c.ld(m, i - 1, j - 1));
    if (noSlip) return n > T(0) ? T(1.0) / n : T(0.0);
    return n == T(4.0) ? T(0.25) : T(0.0);
}

// veris/dynamics_routines.py:31-50: linear ocean drag at the C point
template <class T>
__device__ __forceinline__ T ocean_drag_c(const Ctx<T> &c, const T *u, const T *v, int i, int j) {
    const T fc = c.ld(c.f.fCori, i, j);
    const T dc = T((double)(fc < T(0) ? c.p.waterIceDrag_south : c.p.waterIceDrag) * c.p.rhoSea);
    const T du = (c.ld(u, i, j) - c.ld(c.f.uOcean, i, j)) * c.ld(c.f.maskInU, i, j);
    const T due = (c.ld(u, i + 1, j) - c.ld(c.f.uOcean, i + 1, j)) * c.ld(c.f.maskInU, i + 1, j);
    const T dv = (c.ld(v, i, j) - c.ld(c.f.vOcean, i, j)) * c.ld(c.f.maskInV, i, j);
    const T dvn = (c.ld(v, i, j + 1) - c.ld(c.f.vOcean, i, j + 1)) * c.ld(c.f.maskInV, i, j + 1);
    const T t = T(0.25) * (sq(du + due) + sq(dv + dvn));
    const T cmin = T(c.p.cDragMin);
    const T cd = (dc * dc * t > T(c.p.cDragMin * c.p.cDragMin)) ? dc * sqrt(t) : cmin;
    return cd * c.ld(c.f.iceMask, i, j);
}

// veris/dynamics_routines.py:65-94: basal drag at the C point
template <class T>
__device__ __forceinline__ T basal_drag_c(const Ctx<T> &c, const T *u, const T *v, int i, int j) {
    const T A = c.ld(c.f.Area, i, j);
    if (!(A > T(0.01))) return T(0.0);
    const T um = c.ld(u, i, j) * c.ld(c.f.maskInU, i, j);
    const T ume = c.ld(u, i + 1, j) * c.ld(c.f.maskInU, i + 1, j);
    const T vm = c.ld(v, i, j) * c.ld(c.f.maskInV, i, j);
    const T vmn = c.ld(v, i, j + 1) * c.ld(c.f.maskInV, i, j + 1);
    T t = T(0.25) * (um * um + ume * ume + vm * vm + vmn * vmn);
    t = T(c.p.basalDragK2) / sqrt(t + T(c.p.basalDragU0 * c.p.basalDragU0));
    const T hcrit = fabs(c.ld(c.f.R_low, i, j)) * A / T(c.p.basalDragK1);
    const T fac = T(10.0);
    return t * log(exp(fac * (c.ld(c.f.hIceMean, i, j) - hcrit)) + T(1.0)) * (T(1.0) / fac) *
           exp(-T(c.p.cBasalStar) * (T(1.0) - A));
}

// veris/dynamics_routines.py:110-112: ice speed at the C point (side drag)
template <class T>
__device__ __forceinline__ T ice_speed_c(const Ctx<T> &c, const T *u, const T *v, int i, int j) {
    return T(0.5) * sqrt(sq(c.ld(u, i, j) + c.ld(u, i + 1, j)) + sq(c.ld(v, i, j) + c.ld(v, i, j + 1)));
}

// veris/dynamics_routines.py:115-138 from the speeds at C(i,j) and its west
// (U) or south (V) neighbour
template <class T>
__device__ __forceinline__ T side_drag_u(const Ctx<T> &c, int i, int j, T sp0, T spw) {
    const T spU = c.ld(c.f.AreaW, i, j) > T(0) ? T(0.5) * (sp0 + spw) : T(0);
    T m;
    if (c.p.use_coastline) m = c.ld(c.f.Fu, i, j);
    else {
        const T *mU = c.f.iceMaskU;
        m = (T(2) - c.ld(mU, i - 1, j) - c.ld(mU, i + 1, j)) * c.ld(mU, i, j);
    }
    return c.ld(c.f.SeaIceMassU, i, j) * T(c.p.sideDragCoeff) * m / (spU + T(c.p.sideDragU0));
}
template <class T>
__device__ __forceinline__ T side_drag_v(const Ctx<T> &c, int i, int j, T sp0, T sps) {
    const T spV = c.ld(c.f.AreaS, i, j) > T(0) ? T(0.5) * (sp0 + sps) : T(0);
    T m;
    if (c.p.use_coastline) m = c.ld(c.f.Fv, i, j);
    else {
        const T *mV = c.f.iceMaskV;
        m = (T(2) - c.ld(mV, i, j - 1) - c.ld(mV, i, j + 1)) * c.ld(mV, i, j);
    }
    return c.ld(c.f.SeaIceMassV, i, j) * T(c.p.sideDragCoeff) * m / (spV + T(c.p.sideDragU0));
}

}  // namespace veris
