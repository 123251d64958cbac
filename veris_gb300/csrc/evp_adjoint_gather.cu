// Adjoint of one mEVP subcycle (veris/evp_solver.py:21-254) in four gather
// passes, arranged for GB300's float64 pipe (float64) and for its memory
// system (float32).
//
// The subcycle maps (u, v, sigma1, sigma2, sigma12) to the next state
// through C-point viscosities, stresses and drag, Z-point sigma12 and the
// U/V momentum update (the fast form of evp_fast.cuh: step constants
// folded once per step).  Its adjoint is a sum over the stencil of every
// output; here each pass computes, for every point of one grid position
// (U/V, Z or C), the adjoint terms that position contributes, and the next
// pass gathers them from its neighbours:
//
//   P1  U and V points: the momentum update's adjoint (one reciprocal of its
//       denominator per point), the terms its C and Z neighbours gather
//       (drag-coefficient, Coriolis, stress-divergence and basal shares) and
//       the adjoints of the point's own constants;
//   P2  Z points: sigma12's adjoint, its share in the neighbouring
//       viscosities and in e12;
//   P3  C points: sigma1/sigma2 adjoints, viscosity, Delta, strain-rate,
//       Coriolis, ocean and basal drag adjoints;
//   P4  U and V points: the gathered velocity and ocean-velocity adjoints.
//
// In float32 without a turning angle, P4 of each subcycle and P1 of the
// subcycle before it run as one pass (uv_link_kernel): what P4 gathers at a
// point is what that P1 reads there.  On grids of more CTAs than the GPU
// holds at once, the float32 P3 and the fused pass are bounded to 32
// registers (eight CTAs per SM): latency-bound, they gain more from the
// resident warps than they lose to spills.
//
// Every point is computed once, nothing is recomputed on rings and nothing
// is accumulated with atomics (each input adjoint is written by the pass
// that owns its position).  In float64 the forward's Delta, zeta and drag
// coefficient come from the tape the float64 forward writes (evp_fast.cu),
// so the adjoint takes no square root of the forward's; its reciprocals and
// the basal drag's reciprocal square root use the series-refined hardware
// approximations of f64math.cuh, masks are selects and zero tests run on the
// integer pipe.  A float32 tape (the register walk's) holds the walk's own
// Delta, zeta and drag coefficient beside its state; a float32 segment
// recomputed from a checkpoint does not, and two first passes recompute e12,
// then Delta, zeta and the drag coefficient, with IEEE-rounded float32 square
// roots and reciprocals.
//
// Non-differentiable points take the subgradients of the shared-memory
// form (evp_adjoint.cu): 0 at Delta = 0 and on the drag floor's constant
// branch, and nothing through the "denominator = 0 -> 1" guard.
#include <cstring>

#include "evp_adjoint.cuh"
#include "f64math.cuh"

namespace veris {

namespace adj {

namespace {

constexpr unsigned ALL = 0xffffffffu;
constexpr int BX = 32, BY = 8;   // 32 points along j (contiguous) x 8 rows per 256-thread block

// the step's scalars, products folded once on the host
template <class T>
struct KT {
    T bU, bU1;                 // beta/dt, (beta + 1)/dt
    T hc, sinH;                // 0.5 cos(turning angle), 0.5 sin(turning angle)
    T am1, ra2, rah;      // (alpha - 1)/alpha, 2/alpha, 0.5/alpha
    T hkp, rsq, dmin;     // half the press factor, 1/e^2, Delta_min
    T nh1, nh2, nh3, nh4;    // 0.5/alpha/n: sigma12's average over n wet C points
    T dcq2N, dcq2S, cmin2, cmin;   // the drag test (as the float64 forward takes it) and floor
    T kXN, kXS;                // (rhoSea drag)^2 / 4: 2 d cDrag/dX = kX / cDrag
    double wN, wS;             // rhoSea / (rhoSea drag): d cDrag / d drag = cDrag * w
    T U02;                     // basal U0^2
};

template <class T>
KT<T> kt(const FastScalars<T> &k, double rhoSea) {
    KT<T> s;
    s.bU = k.bU;
    s.bU1 = k.bU1;
    s.hc = k.halfCos;
    s.sinH = 0.5 * k.sinW;
    s.am1 = k.alpha_m1 * k.ralpha;
    s.ra2 = 2.0 * k.ralpha;
    s.rah = 0.5 * k.ralpha;
    s.hkp = 0.5 * k.kp;
    s.rsq = k.rsq;
    s.dmin = k.deltaMin;
    s.nh1 = 0.5 * k.ralpha;
    s.nh2 = 0.5 * k.ralpha * 0.5;
    s.nh3 = 0.5 * k.ralpha * (1.0 / 3.0);
    s.nh4 = 0.5 * k.ralpha * 0.25;
    s.dcq2N = 0.25 * k.dN2;
    s.dcq2S = 0.25 * k.dS2;
    s.cmin2 = k.cmin2;
    s.cmin = k.cmin;
    s.kXN = 0.25 * k.dN2;
    s.kXS = 0.25 * k.dS2;
    s.wN = k.dN != T(0) ? rhoSea / (double)k.dN : 0.0;
    s.wS = k.dS != T(0) ? rhoSea / (double)k.dS : 0.0;
    s.U02 = k.U02;
    return s;
}

// the passes' arrays (internal pitch)
template <class T>
struct Scr {
    T *gU, *gV;       // adjoints of the momentum numerators
    T *rU, *rV;       // the same over rA_u, rA_v (stress-divergence shares)
    T *wU0, *wU1;     // a U point's share in dL/dcDrag at C(i, j) and C(i-1, j)
    T *wV0, *wV1;     // a V point's share at C(i, j) and C(i, j-1)
    T *bU, *bV;       // shares in the basal coefficient's adjoint
    T *q0U, *qwU;     // turning-angle shares in d/du of (i, j),(i, j+1) and (i-1, j),(i-1, j+1)
    T *q0V, *qsV;     // the same for v: (i, j),(i+1, j) and (i, j-1),(i+1, j-1)
    T *tZ;            // a Z point's share in the adjoint of each neighbouring zeta
    T *le12;          // e12's adjoint through sigma12
    T *e2;            // rAz e12
    T *uA, *uB;       // a C point's share in d/du of U(i, j) and U(i+1, j)
    T *vA, *vB;       // the same for V(i, j) and V(i, j+1)
    T *ldu, *ldv;     // ocean-drag shares in d/du, d/dv (masked by the U/V point)
    T *wC;            // recip_rA/e^2 dL/dDelta / Delta: twice the adjoint of rAz e12^2
    T *lsb;           // basal shares, times u or v at the U/V point
    T *cb;            // the basal coefficient (recomputed once per subcycle)
    T *e12, *del, *zeta, *cd;   // recomputed forward terms for a tape without them
};
static_assert(sizeof(Scr<float>) == N_SCRATCH * sizeof(float *), "scratch table");

__device__ __forceinline__ int wxp(const Dims &d, int i) { return i < 0 ? i + d.NX : (i >= d.NX ? i - d.NX : i); }
__device__ __forceinline__ int wyp(const Dims &d, int j) { return j < 0 ? j + d.NY : (j >= d.NY ? j - d.NY : j); }

// the four C points around Z(i, j) all wet
__device__ __forceinline__ bool z_wet(uint32_t f0, uint32_t fw, uint32_t fs, uint32_t fws) {
    return (f0 & fw & fs & fws & F_MC) != 0;
}

template <class T>
__device__ __forceinline__ T sel(bool b, T x) { return b ? x : T(0); }

// the arithmetic of each precision: float64 on the series-refined hardware
// approximations (f64math.cuh), float32 IEEE-rounded
template <class T>
struct Fp;
template <>
struct Fp<double> {
    static __device__ __forceinline__ double rcp(double x, unsigned m) { return rcp64(x, m); }
    static __device__ __forceinline__ double rsqrt(double x, unsigned m) { return rsqrt64(x, m); }
    static __device__ __forceinline__ double root(double x, unsigned m) { return sqrt64(x, m); }
    static __device__ __forceinline__ double div(double a, double b, unsigned m) { return div64(a, b, m); }
    static __device__ __forceinline__ bool zero(double x) { return is_zero(x); }
    static __device__ __forceinline__ bool gt(double x, double y) { return gt_nonneg(x, y); }
};
template <>
struct Fp<float> {
    static __device__ __forceinline__ float rcp(float x, unsigned) { return __frcp_rn(x); }
    static __device__ __forceinline__ float rsqrt(float x, unsigned) { return __frsqrt_rn(x); }
    static __device__ __forceinline__ float root(float x, unsigned) { return __fsqrt_rn(x); }
    static __device__ __forceinline__ float div(float a, float b, unsigned) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ bool zero(float x) { return x == 0.f; }
    static __device__ __forceinline__ bool gt(float x, float y) { return x > y; }
};

// products the float64 preparation folds once per step (evp_fast.cu); the
// float32 workspace does not hold them, so float32 forms them here
template <class T>
struct Fold {
    const FastConsts<T> &c;
    const KT<T> &k;
    __device__ __forceinline__ T hAW(int64_t o) const {
        if constexpr (sizeof(T) == 8) return c.hAW[o]; else return k.hc * c.AW[o];
    }
    __device__ __forceinline__ T hAS(int64_t o) const {
        if constexpr (sizeof(T) == 8) return c.hAS[o]; else return k.hc * c.AS[o];
    }
    __device__ __forceinline__ T mUb1(int64_t o) const {
        if constexpr (sizeof(T) == 8) return c.mUb1[o]; else return c.mU[o] * k.bU1;
    }
    __device__ __forceinline__ T mVb1(int64_t o) const {
        if constexpr (sizeof(T) == 8) return c.mVb1[o]; else return c.mV[o] * k.bU1;
    }
    __device__ __forceinline__ T mUb(int64_t o) const {
        if constexpr (sizeof(T) == 8) return c.mUb[o]; else return c.mU[o] * k.bU;
    }
    __device__ __forceinline__ T mVb(int64_t o) const {
        if constexpr (sizeof(T) == 8) return c.mVb[o]; else return c.mV[o] * k.bU;
    }
    __device__ __forceinline__ T rdyUh(int j) const {   // 0.5 recip_dyU
        if constexpr (sizeof(T) == 8) return c.rdyUh_y[j]; else return T(0.5) * c.rdyU_y[j];
    }
    __device__ __forceinline__ T rdxVh(int i) const {   // 0.5 recip_dxV
        if constexpr (sizeof(T) == 8) return c.rdxVh_x[i]; else return T(0.5) * c.rdxV_x[i];
    }
    __device__ __forceinline__ T dyVh(int j) const {
        if constexpr (sizeof(T) == 8) return c.dyVh_y[j]; else return T(0.5) * c.dyV_y[j];
    }
    __device__ __forceinline__ T dxUh(int i) const {
        if constexpr (sizeof(T) == 8) return c.dxUh_x[i]; else return T(0.5) * c.dxU_x[i];
    }
    __device__ __forceinline__ T rsqrA(int64_t o) const {   // recip_rA / e^2 = 4 rsq (0.25 / rA)
        if constexpr (sizeof(T) == 8) return c.rsqrA[o]; else return T(4) * k.rsq * c.qrA[o];
    }
    __device__ __forceinline__ T mf4(int64_t o) const {   // mfC / 2
        if constexpr (sizeof(T) == 8) return c.mf4[o]; else return T(0.5) * c.mfC[o];
    }
};

// ------------------------------------------------------------------ P0
// the basal drag coefficient at every C point, as the forward computes it
// (veris/dynamics_routines.py:55-96 with the step factor folded)
template <class T>
__global__ void __launch_bounds__(BX * BY) basal_kernel(Dims d, int64_t lp, FastConsts<T> c, TapeG<T> t, KT<T> k,
                                                         Scr<T> s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    const int64_t o = (int64_t)i * lp + j;
    const int64_t oe = (int64_t)wxp(d, i + 1) * lp + j, on = (int64_t)i * lp + wyp(d, j + 1);
    const uint32_t f0 = c.flags[o], fe = c.flags[oe], fn = c.flags[on];
    const T a_ = sel<T>(f0 & F_INU, t.U(o)), b_ = sel<T>(fe & F_INU, t.U(oe));
    const T c_ = sel<T>(f0 & F_INV, t.V(o)), e_ = sel<T>(fn & F_INV, t.V(on));
    const T q = T(0.25) * (a_ * a_ + b_ * b_ + c_ * c_ + e_ * e_);
    s.cb[o] = Fp<T>::div(c.bfac[o], Fp<T>::root(q + k.U02, m), m);
}

// e12 at Z(i, j) (veris/dynamics_routines.py:160-175), as the float64
// forward computes it: 0.5 rdyU, 0.5 rdxV folded, the no-slip boundary
// terms only in warps that have one
template <class T>
__device__ __forceinline__ T e12_at(const Fold<T> &F, const TapeG<T> &t, unsigned m, int i, int j, int64_t o,
                                    int64_t ow, int64_t os, uint32_t f0, uint32_t fw, uint32_t fs, uint32_t fws) {
    const bool mz = z_wet(f0, fw, fs, fws);
    const int hU = (int)((f0 & F_MU) != 0) - (int)((fs & F_MU) != 0);
    const int hV = (int)((f0 & F_MV) != 0) - (int)((fw & F_MV) != 0);
    const T u0 = t.U(o), us = t.U(os), v0 = t.V(o), vw = t.V(ow);
    const T ry = F.rdyUh(j), rx = F.rdxVh(i);
    if (__any_sync(m, (hU | hV) != 0)) {
        const T hu2 = hU == 0 ? T(0) : (hU > 0 ? T(2) : T(-2));
        const T hv2 = hV == 0 ? T(0) : (hV > 0 ? T(2) : T(-2));
        const T tu = fma(hu2, u0 + us, mz ? u0 - us : T(0));
        const T tv = fma(hv2, v0 + vw, mz ? v0 - vw : T(0));
        return fma(ry, tu, rx * tv);
    }
    return mz ? fma(ry, u0 - us, rx * (v0 - vw)) : T(0);
}

// P0 for a tape without the forward's terms: e12 at every Z point, then
// Delta, zeta and cDrag at every C point (veris/dynamics_routines.py:21-52,
// 220-268), as the fast forward computes them
template <class T>
__global__ void __launch_bounds__(BX * BY) e12_kernel(Dims d, int64_t lp, FastConsts<T> c, TapeG<T> t, KT<T> k,
                                                       Scr<T> s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    const int iw = wxp(d, i - 1), js = wyp(d, j - 1);
    const int64_t o = (int64_t)i * lp + j, ow = (int64_t)iw * lp + j, os = (int64_t)i * lp + js,
                  ows = (int64_t)iw * lp + js;
    const Fold<T> F{c, k};
    s.e12[o] = e12_at(F, t, m, i, j, o, ow, os, c.flags[o], c.flags[ow], c.flags[os], c.flags[ows]);
}

template <class T>
__global__ void __launch_bounds__(BX * BY) viscosity_kernel(Dims d, int64_t lp, FastConsts<T> c, TapeG<T> t,
                                                             KT<T> k, Scr<T> s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    const int ie = wxp(d, i + 1), jn = wyp(d, j + 1);
    const int64_t o = (int64_t)i * lp + j, oe = (int64_t)ie * lp + j, on = (int64_t)i * lp + jn,
                  oen = (int64_t)ie * lp + jn;
    const Fold<T> F{c, k};
    const uint32_t f0 = c.flags[o], fe = c.flags[oe], fn = c.flags[on];
    const bool inC = f0 & F_INC, mC = f0 & F_MC;
    const T u0 = t.U(o), ue = t.U(oe), v0 = t.V(o), vn = t.V(on);
    const T e11 = inC ? (ue - u0) * c.rdxU_x[i] : T(0);
    const T e22 = inC ? (vn - v0) * c.rdyV_y[j] : T(0);
    const T ep = e11 + e22, em = e11 - e22;
    auto zq = [&](int64_t z) { const T e = s.e12[z]; return c.rAz[z] * (e * e); };
    const T zs = (zq(o) + zq(oe)) + (zq(on) + zq(oen));
    const T d2 = fma(F.rsqrA(o), zs, fma(k.rsq * em, em, ep * ep));
    const T del = Fp<T>::root(d2, m);
    s.del[o] = del;
    s.zeta[o] = Fp<T>::div(c.Ph[o], del + k.dmin, m);
    const T du0 = (f0 & F_INU) ? u0 - c.uOc[o] : T(0);
    const T du1 = (fe & F_INU) ? ue - c.uOc[oe] : T(0);
    const T dv0 = (f0 & F_INV) ? v0 - c.vOc[o] : T(0);
    const T dv1 = (fn & F_INV) ? vn - c.vOc[on] : T(0);
    const T A = du0 + du1, B = dv0 + dv1;
    const T X = fma(B, B, A * A);
    const bool south = f0 & F_SOUTH;
    const bool fast = Fp<T>::gt((south ? k.dcq2S : k.dcq2N) * X, k.cmin2);
    // cDrag = 0.5 rhoSea drag sqrt(X) = sqrt((rhoSea drag)^2/4 X) above the floor
    s.cd[o] = mC ? (fast ? Fp<T>::root((south ? k.dcq2S : k.dcq2N) * X, m) : k.cmin) : T(0);
}

// the adjoint of a U or V point's new velocity, with the adjoints of its
// images in a filled halo added (the transpose of the fill); 0 at image
// points, whose values the forward copies rather than computes
template <class T>
__device__ __forceinline__ void own_adjoints(const Dims &d, const HaloFill &h, const LamG<T> &l, int i, int j,
                                             T &LU, T &LV) {
    LU = LV = T(0);
    const bool hx = h.x_fill && in_xhalo(d, h.olx, i);
    const bool hy = h.y_fill && in_yhalo(d, h.oly, j);
    if (hx || hy) return;
    LU = l.lu[(int64_t)i * l.ldl + j];
    LV = l.lv[(int64_t)i * l.ldl + j];
    int ix[2] = {i, -1}, jy[2] = {j, -1};
    if (h.x_fill) {
        if (i + d.nx < d.NX && in_xhalo(d, h.olx, i + d.nx)) ix[1] = i + d.nx;
        else if (i - d.nx >= 0 && in_xhalo(d, h.olx, i - d.nx)) ix[1] = i - d.nx;
    }
    if (h.y_fill) {
        if (j + d.ny < d.NY && in_yhalo(d, h.oly, j + d.ny)) jy[1] = j + d.ny;
        else if (j - d.ny >= 0 && in_yhalo(d, h.oly, j - d.ny)) jy[1] = j - d.ny;
    }
    if (ix[1] < 0 && jy[1] < 0) return;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            if ((a == 0 && b == 0) || ix[a] < 0 || jy[b] < 0) continue;
            LU += l.lu[(int64_t)ix[a] * l.ldl + jy[b]];
            LV += l.lv[(int64_t)ix[a] * l.ldl + jy[b]];
        }
}

// ------------------------------------------------------------------ P1
// U(i, j):  u' = wet ? num / den : 0 with
//   den = mU (beta+1)/dt + kU [+ AW (cb + cb_w)/2],  kU = cos/2 AW (cd + cd_w),
//   num = mU beta/dt u + cU + kU uOc + (Fv + Fv_w)/2 [+ turning] + rrAu (dyV (s11 - s11_w) + dxV (s12'_n - s12'))
// (veris/evp_solver.py:113-187); V(i, j) the same with the j neighbours.
// P1 at U(i, j), V(i, j) given the adjoints LU, LV of its new velocities;
// luo, lvo: ocean-velocity adjoint shares of the subcycle after it (its P4
// run in the same kernel), added to a.uOc, a.vOc before this subcycle's
// (the order of the separate passes); MERGE: there are such shares
template <class T, bool BASAL, bool TURN, bool MERGE>
__device__ __forceinline__ void p1_point(const Dims &d, int64_t lp, const FastConsts<T> &c, const TapeG<T> &t,
                                         const LamG<T> &l, const Adj<T> &a, const KT<T> &k, const Scr<T> &s,
                                         unsigned m, int i, int j, T LU, T LV, T luo, T lvo) {
    const Fold<T> F{c, k};
    const int iw = wxp(d, i - 1), js = wyp(d, j - 1);
    const int64_t o = (int64_t)i * lp + j, ow = (int64_t)iw * lp + j, os = (int64_t)i * lp + js;
    const uint32_t f0 = c.flags[o];
    const T cd0 = t.cd[o], cdw = t.cd[ow], cds = t.cd[os];
    T cb0 = T(0), cbw = T(0), cbs = T(0);
    if (BASAL) {
        cb0 = s.cb[o];
        cbw = s.cb[ow];
        cbs = s.cb[os];
    }
    T sg = T(0);
    if (TURN) sg = (f0 & F_SPOS) ? T(1) : ((f0 & F_SNEG) ? T(-1) : T(0));
    if (!__any_sync(m, f0 & F_MU)) {   // a warp of dry U points: no momentum adjoint, nothing to add
        if (MERGE) a.uOc[o] += luo;
        l.ou[o] = T(0);
        s.gU[o] = T(0);
        s.rU[o] = T(0);
        s.wU0[o] = T(0);
        if (TURN) s.wU1[o] = s.q0U[o] = s.qwU[o] = T(0);
        if (BASAL) s.bU[o] = T(0);
    } else {   // U point (hAW = cos/2 AW, mUb = mU beta/dt, mUb1 = mU (beta+1)/dt)
        const T hA = F.hAW(o), uo = c.uOc[o], u0 = t.U(o);
        const T S = cd0 + cdw, kU = hA * S;
        T den = F.mUb1(o) + kU;
        if (BASAL) den = fma(T(0.5) * c.AW[o], cb0 + cbw, den);
        const bool guard = Fp<T>::zero(den);
        const T r = Fp<T>::rcp(guard ? T(1) : den, m);
        const T g = sel<T>(f0 & F_MU, LU * r);
        const T lden = guard ? T(0) : -t.UN(o) * g;
        const T Y = fma(uo, g, lden);   // d/dkU
        const T W = hA * Y;
        l.ou[o] = F.mUb(o) * g;
        a.mU[o] = fma(k.bU * u0, g, fma(k.bU1, lden, a.mU[o]));
        a.cU[o] += g;
        T lAW = fma(k.hc * S, Y, a.AW[o]);
        if (BASAL) {
            lAW = fma(T(0.5) * (cb0 + cbw), lden, lAW);
            s.bU[o] = T(0.5) * c.AW[o] * lden;
        }
        a.uOc[o] = fma(kU, g, MERGE ? a.uOc[o] + luo : a.uOc[o]);
        s.gU[o] = g;
        s.rU[o] = c.rrAu[o] * g;
        if (TURN) {
            // num -= sg sin/2 AW (cd (du + du_n)/2 + cd_w (du_w + du_wn)/2) where SeaIceMassU != 0, du = uOc - u
            const int jn = wyp(d, j + 1);
            const int64_t on = (int64_t)i * lp + jn, own_ = (int64_t)iw * lp + jn;
            const T tu = sel<T>(f0 & F_LMU, -sg * k.sinH);
            const T pn = T(0.5) * ((uo - u0) + (c.uOc[on] - t.U(on)));
            const T pw = T(0.5) * ((c.uOc[ow] - t.U(ow)) + (c.uOc[own_] - t.U(own_)));
            lAW = fma(tu * fma(cd0, pn, cdw * pw), g, lAW);
            const T tg = tu * c.AW[o] * g;
            s.wU0[o] = fma(tg, pn, W);
            s.wU1[o] = fma(tg, pw, W);
            s.q0U[o] = T(0.5) * tg * cd0;
            s.qwU[o] = T(0.5) * tg * cdw;
        } else {
            s.wU0[o] = W;
        }
        a.AW[o] = lAW;
    }
    if (!__any_sync(m, f0 & F_MV)) {
        if (MERGE) a.vOc[o] += lvo;
        l.ov[o] = T(0);
        s.gV[o] = T(0);
        s.rV[o] = T(0);
        s.wV0[o] = T(0);
        if (TURN) s.wV1[o] = s.q0V[o] = s.qsV[o] = T(0);
        if (BASAL) s.bV[o] = T(0);
    } else {   // V point
        const T hA = F.hAS(o), vo = c.vOc[o], v0 = t.V(o);
        const T S = cd0 + cds, kV = hA * S;
        T den = F.mVb1(o) + kV;
        if (BASAL) den = fma(T(0.5) * c.AS[o], cb0 + cbs, den);
        const bool guard = Fp<T>::zero(den);
        const T r = Fp<T>::rcp(guard ? T(1) : den, m);
        const T g = sel<T>(f0 & F_MV, LV * r);
        const T lden = guard ? T(0) : -t.VN(o) * g;
        const T Y = fma(vo, g, lden);
        const T W = hA * Y;
        l.ov[o] = F.mVb(o) * g;
        a.mV[o] = fma(k.bU * v0, g, fma(k.bU1, lden, a.mV[o]));
        a.cV[o] += g;
        T lAS = fma(k.hc * S, Y, a.AS[o]);
        if (BASAL) {
            lAS = fma(T(0.5) * (cb0 + cbs), lden, lAS);
            s.bV[o] = T(0.5) * c.AS[o] * lden;
        }
        a.vOc[o] = fma(kV, g, MERGE ? a.vOc[o] + lvo : a.vOc[o]);
        s.gV[o] = g;
        s.rV[o] = c.rrAv[o] * g;
        if (TURN) {
            // num += sg sin/2 AS (cd (dv + dv_e)/2 + cd_s (dv_s + dv_se)/2) where SeaIceMassV != 0, dv = vOc - v
            const int ie = wxp(d, i + 1);
            const int64_t oe = (int64_t)ie * lp + j, ose = (int64_t)ie * lp + js;
            const T tv = sel<T>(f0 & F_LMV, sg * k.sinH);
            const T pe = T(0.5) * ((vo - v0) + (c.vOc[oe] - t.V(oe)));
            const T ps = T(0.5) * ((c.vOc[os] - t.V(os)) + (c.vOc[ose] - t.V(ose)));
            lAS = fma(tv * fma(cd0, pe, cds * ps), g, lAS);
            const T tg = tv * c.AS[o] * g;
            s.wV0[o] = fma(tg, pe, W);
            s.wV1[o] = fma(tg, ps, W);
            s.q0V[o] = T(0.5) * tg * cd0;
            s.qsV[o] = T(0.5) * tg * cds;
        } else {
            s.wV0[o] = W;
        }
        a.AS[o] = lAS;
    }
}

template <class T, bool BASAL, bool TURN>
__global__ void __launch_bounds__(BX * BY) uv_reverse_kernel(Dims d, int64_t lp, HaloFill h, FastConsts<T> c,
                                                              TapeG<T> t, LamG<T> l, Adj<T> a, KT<T> k, Scr<T> s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    T LU, LV;
    own_adjoints(d, h, l, i, j, LU, LV);
    p1_point<T, BASAL, TURN, false>(d, lp, c, t, l, a, k, s, m, i, j, LU, LV, T(0), T(0));
}

// ------------------------------------------------------------------ P2
// Z(i, j): sigma12' = (alpha-1)/alpha sigma12 + 0.5/alpha/n e12 * (sum of
// the four zeta) (veris/evp_solver.py:101-103, veris/averaging.py:4-19)
template <class T>
__global__ void __launch_bounds__(BX * BY) z_reverse_kernel(Dims d, int64_t lp, FastConsts<T> c, TapeG<T> t,
                                                             LamG<T> l, KT<T> k, Scr<T> s, bool e12_ready) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    const Fold<T> F{c, k};
    const int iw = wxp(d, i - 1), js = wyp(d, j - 1);
    const int64_t o = (int64_t)i * lp + j, ow = (int64_t)iw * lp + j, os = (int64_t)i * lp + js,
                  ows = (int64_t)iw * lp + js;
    // sigma12' at Z(i, j) enters sdx of U(i, j) (-) and U(i, j-1) (+), sdy of V(i, j) (-) and V(i-1, j) (+)
    const T L = fma(c.dxV_x[i], s.rU[os] - s.rU[o], fma(c.dyU_y[j], s.rV[ow] - s.rV[o], l.ls12[(int64_t)i * l.ldl + j]));
    l.os12[o] = k.am1 * L;
    const uint32_t f0 = c.flags[o], fw = c.flags[ow], fs = c.flags[os], fws = c.flags[ows];
    const uint32_t n = (f0 & F_MC) + (fw & F_MC) + (fs & F_MC) + (fws & F_MC);
    const T nh = n == 4 ? k.nh4 : (n == 3 ? k.nh3 : (n == 2 ? k.nh2 : (n == 1 ? k.nh1 : T(0))));
    const T e = e12_ready ? s.e12[o] : e12_at(F, t, m, i, j, o, ow, os, f0, fw, fs, fws);
    const T zs = (t.zeta[o] + t.zeta[ow]) + (t.zeta[os] + t.zeta[ows]);
    const T cz = nh * L;
    s.tZ[o] = cz * e;
    s.le12[o] = cz * zs;
    s.e2[o] = c.rAz[o] * e;
}

// ------------------------------------------------------------------ P3
// C(i, j): strain rates, Delta, zeta and the stress update
// (veris/dynamics_routines.py:143-268, veris/evp_solver.py:80-100), ocean
// drag (veris/dynamics_routines.py:21-52), basal drag (:55-96) and the
// Coriolis terms (veris/evp_solver.py:124-131)
template <class T, bool BASAL, bool TURN>
__device__ __forceinline__ void c_reverse_body(const Dims &d, int64_t lp, const FastConsts<T> &c, const TapeG<T> &t,
                                               const LamG<T> &l, const Adj<T> &a, const KT<T> &k,
                                               const Scr<T> &s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    T dragN = T(0), dragS = T(0);   // float32: this warp's water-drag terms
    if (act) {
        const Fold<T> F{c, k};
        const int ie = wxp(d, i + 1), jn = wyp(d, j + 1);
        const int64_t o = (int64_t)i * lp + j, oe = (int64_t)ie * lp + j, on = (int64_t)i * lp + jn,
                      oen = (int64_t)ie * lp + jn;
        const uint32_t f0 = c.flags[o], fe = c.flags[oe], fn = c.flags[on];
        const bool mC = f0 & F_MC, inC = f0 & F_INC;
        // shares gathered from U(i, j), U(i+1, j), V(i, j), V(i, j+1)
        const T sU = s.gU[o] + s.gU[oe], sV = s.gV[o] + s.gV[on];
        const T lcd = (s.wU0[o] + (TURN ? s.wU1[oe] : s.wU0[oe])) + (s.wV0[o] + (TURN ? s.wV1[on] : s.wV0[on]));
        // sig11 = (sigma1' + sigma2')/2 enters U(i, j) (+) and U(i+1, j) (-) as rrAu dyV,
        // sig22 = (sigma1' - sigma2')/2 V(i, j) (+) and V(i, j+1) (-) as rrAv dxU
        const T h11 = F.dyVh(j) * (s.rU[o] - s.rU[oe]);
        const T h22 = F.dxUh(i) * (s.rV[o] - s.rV[on]);
        const T L1 = l.ls1[(int64_t)i * l.ldl + j] + (h11 + h22);
        const T L2 = l.ls2[(int64_t)i * l.ldl + j] + (h11 - h22);
        l.os1[o] = sel<T>(mC, k.am1 * L1);
        l.os2[o] = sel<T>(mC, k.am1 * L2);
        // sigma1' = mC ((alpha-1)/alpha sigma1 + zeta (2 ep - kp Delta)/alpha),
        // sigma2' = mC ((alpha-1)/alpha sigma2 + zeta em/(2 alpha)): h1 = 2 d/dsigma1'/alpha, h2 = d/dsigma2'/(2 alpha)
        const T h1 = sel<T>(mC, k.ra2 * L1), h2 = sel<T>(mC, k.rah * L2);
        // strain rates (recomputed from the tape's velocities)
        const T u0 = t.U(o), ue = t.U(oe), v0 = t.V(o), vn = t.V(on);
        const T rdx = c.rdxU_x[i], rdy = c.rdyV_y[j];
        const T e11 = inC ? (ue - u0) * rdx : T(0);
        const T e22 = inC ? (vn - v0) * rdy : T(0);
        const T ep = e11 + e22, em = e11 - e22;
        const T del = t.del[o], zeta = t.zeta[o];
        const T tz = (s.tZ[o] + s.tZ[oe]) + (s.tZ[on] + s.tZ[oen]);
        const T lz = fma(fma(-k.hkp, del, ep), h1, fma(em, h2, tz));
        // zeta = Ph/(Delta + Delta_min)
        const T rz = Fp<T>::rcp(del + k.dmin, m);
        a.Ph[o] = fma(lz, rz, a.Ph[o]);
        // where the ice strength is 0, zeta = 0 and nothing flows back through Delta
        T q = T(0), le11 = T(0), le22 = T(0);
        if (__any_sync(m, !Fp<T>::zero(zeta))) {
            T lep = zeta * h1, lem = zeta * h2;
            const T ldel = fma(-zeta * rz, lz, -k.hkp * lep);
            // Delta = sqrt(ep^2 + rsq em^2 + (recip_rA/e^2) sum rAz e12^2); 0 at Delta = 0.  q = 2 dL/dDelta^2
            const bool dz = Fp<T>::zero(del);
            const T rdel = Fp<T>::rcp(dz ? T(1) : del, m);
            q = dz ? T(0) : ldel * rdel;
            lep = fma(ep, q, lep);
            lem = fma(k.rsq * em, q, lem);
            le11 = inC ? (lep + lem) * rdx : T(0);
            le22 = inC ? (lep - lem) * rdy : T(0);
        }
        s.wC[o] = F.rsqrA(o) * q;
        // Coriolis: Fv = mfC (v + v_n) enters U(i, j), U(i+1, j) with 1/2, Fu = mfC (u + u_e)
        // V(i, j), V(i, j+1) with -1/2 (mf4 = mfC/2)
        const T mf = F.mf4(o);
        a.mfC[o] = fma(T(0.5), fma(v0 + vn, sU, -((u0 + ue) * sV)), a.mfC[o]);
        const T fv = mf * sU, fu = -mf * sV;
        s.uA[o] = fu - le11;
        s.uB[o] = fu + le11;
        s.vA[o] = fv - le22;
        s.vB[o] = fv + le22;
        // ocean drag: cd = 0.5 rhoSea drag sqrt(X), X = (du + du_e)^2 + (dv + dv_n)^2, above its floor
        // (the branch taken exactly as the forward takes it)
        const T du0 = (f0 & F_INU) ? u0 - c.uOc[o] : T(0);
        const T du1 = (fe & F_INU) ? ue - c.uOc[oe] : T(0);
        const T dv0 = (f0 & F_INV) ? v0 - c.vOc[o] : T(0);
        const T dv1 = (fn & F_INV) ? vn - c.vOc[on] : T(0);
        const T A = du0 + du1, B = dv0 + dv1;
        const T X = fma(B, B, A * A);
        const bool south = f0 & F_SOUTH;
        const bool fast = mC && Fp<T>::gt((south ? k.dcq2S : k.dcq2N) * X, k.cmin2);
        T lX2 = T(0);   // 2 dL/dX
        if (__any_sync(m, fast)) {
            const T cd = t.cd[o];
            const T rc = Fp<T>::rcp(fast ? cd : T(1), m);
            if (fast) {
                lX2 = lcd * (south ? k.kXS : k.kXN) * rc;
                if constexpr (sizeof(T) == 8) a.dragC[o] = fma(lcd, cd, a.dragC[o]);   // reduced once, after the sweep
                else if (south) dragS = lcd * cd;
                else dragN = lcd * cd;
            }
        }
        s.ldu[o] = A * lX2;
        s.ldv[o] = B * lX2;
        if (BASAL) {
            // cb = bfac / sqrt(0.25 (a^2 + b^2 + c^2 + e^2) + U0^2), a = inU u, b = inU_e u_e, c = inV v, e = inV_n v_n
            const T lcb = (s.bU[o] + s.bU[oe]) + (s.bV[o] + s.bV[on]);
            const T a_ = sel<T>(f0 & F_INU, u0), b_ = sel<T>(fe & F_INU, ue);
            const T c_ = sel<T>(f0 & F_INV, v0), e_ = sel<T>(fn & F_INV, vn);
            const T qb = T(0.25) * (a_ * a_ + b_ * b_ + c_ * c_ + e_ * e_) + k.U02;
            const T rs = Fp<T>::rsqrt(qb, m);
            const T bf = c.bfac[o];
            a.bfac[o] += lcb * rs;
            s.lsb[o] = T(-0.25) * bf * rs * rs * rs * lcb;
        }
    }
    // float32: the water-drag gradients as float32 warp sums, one float64 atomic per warp
    // (d cDrag / d drag = cDrag rhoSea / (rhoSea drag))
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            dragN += __shfl_down_sync(ALL, dragN, off);
            dragS += __shfl_down_sync(ALL, dragS, off);
        }
        if ((threadIdx.x & 31) == 0) {
            if (dragN != 0.f) atomicAdd(a.dragN, (double)dragN * k.wN);
            if (dragS != 0.f) atomicAdd(a.dragS, (double)dragS * k.wS);
        }
    }
}

template <class T, bool BASAL, bool TURN>
__global__ void __launch_bounds__(BX * BY) c_reverse_kernel(Dims d, int64_t lp, FastConsts<T> c, TapeG<T> t,
                                                             LamG<T> l, Adj<T> a, KT<T> k, Scr<T> s) {
    c_reverse_body<T, BASAL, TURN>(d, lp, c, t, l, a, k, s);
}

// On a float32 grid of more CTAs than the GPU holds at once, eight CTAs per
// SM (32 registers, 20-24 bytes spilled): the latency-bound pass gains more
// from the resident warps than it loses to the spills (a 0.1-degree reverse
// step 383.7 -> 375.1 ms); on a grid the GPU holds at once the spills would
// only cost.
template <class T, bool BASAL, bool TURN>
__global__ void __launch_bounds__(BX * BY, 8) c_reverse_occ_kernel(Dims d, int64_t lp, FastConsts<T> c, TapeG<T> t,
                                                                   LamG<T> l, Adj<T> a, KT<T> k, Scr<T> s) {
    c_reverse_body<T, BASAL, TURN>(d, lp, c, t, l, a, k, s);
}

// e12's full adjoint at Z(i, j): its share through sigma12 plus
// rAz e12 times the e12^2 shares gathered from C(i, j), C(i-1, j),
// C(i, j-1), C(i-1, j-1)
template <class T>
__device__ __forceinline__ T le12_at(const Scr<T> &s, int64_t o, int64_t ow, int64_t os, int64_t ows) {
    return fma(s.e2[o], (s.wC[o] + s.wC[ow]) + (s.wC[os] + s.wC[ows]), s.le12[o]);
}

// d e12(Z) / d u (or v) in units of 0.5 rdyU (0.5 rdxV): 2 h + sign mz at
// the Z point's own U (V) point (sign +1) and at its southern (western) one
// (sign -1), h = iceMaskU - its southern neighbour (iceMaskV - its western
// one); a small integer, selected rather than converted
template <class T>
__device__ __forceinline__ T e12_coef(bool mz, int h, int sign) {
    const int v = 2 * h + (mz ? sign : 0);
    return v == 0 ? T(0) : v == 1 ? T(1) : v == -1 ? T(-1) : v == 2 ? T(2) : v == -2 ? T(-2) : v == 3 ? T(3) : T(-3);
}

// ------------------------------------------------------------------ P4
// U(i, j), V(i, j): the velocity and ocean-velocity adjoints gathered from
// the C points (strain rates, drag, basal drag, Coriolis), the Z points
// (e12) and the turning-angle terms of the neighbouring U, V points
// P4 at U(i, j), V(i, j): the velocity adjoints gathered from the C and Z
// points (lu, lv: to be added to the momentum share P1 left in l.ou, l.ov)
// and the ocean-velocity shares (luo, lvo); `m` the lanes that call it.
// VOTE false: no warp vote (for lanes that call it alone; the no-slip terms'
// general form then runs everywhere, with the same values)
template <class T, bool BASAL, bool TURN, bool VOTE = true>
__device__ __forceinline__ void p4_point(const Dims &d, int64_t lp, const FastConsts<T> &c, const TapeG<T> &t,
                                         const KT<T> &k, const Scr<T> &s, unsigned m, int i, int j, T &lu_out,
                                         T &lv_out, T &luo_out, T &lvo_out) {
    const Fold<T> F{c, k};
    const int iw = wxp(d, i - 1), ie = wxp(d, i + 1), js = wyp(d, j - 1), jn = wyp(d, j + 1);
    const int64_t o = (int64_t)i * lp + j, ow = (int64_t)iw * lp + j, oe = (int64_t)ie * lp + j,
                  os = (int64_t)i * lp + js, on = (int64_t)i * lp + jn, ows = (int64_t)iw * lp + js,
                  own_ = (int64_t)iw * lp + jn, oes = (int64_t)ie * lp + js;
    const uint32_t f0 = c.flags[o], fw = c.flags[ow], fe = c.flags[oe], fs = c.flags[os], fn = c.flags[on],
                   fws = c.flags[ows], fwn = c.flags[own_], fes = c.flags[oes];
    // e12 adjoints at Z(i, j), Z(i, j+1), Z(i+1, j)
    const T z0 = le12_at(s, o, ow, os, ows);
    const T zn = le12_at(s, on, own_, o, ow);
    const T ze = le12_at(s, oe, o, oes, os);
    // e12(Z) = 0.5 rdyU (2 hU (u + u_s) + mz (u - u_s)) + 0.5 rdxV (2 hV (v + v_w) + mz (v - v_w))
    const int hU0 = (int)((f0 & F_MU) != 0) - (int)((fs & F_MU) != 0);
    const int hUn = (int)((fn & F_MU) != 0) - (int)((f0 & F_MU) != 0);
    const int hV0 = (int)((f0 & F_MV) != 0) - (int)((fw & F_MV) != 0);
    const int hVe = (int)((fe & F_MV) != 0) - (int)((f0 & F_MV) != 0);
    const bool mz0 = z_wet(f0, fw, fs, fws), mzn = z_wet(fn, fwn, f0, fw), mze = z_wet(fe, f0, fes, fs);
    const T ru0 = z0 * F.rdyUh(j), run = zn * F.rdyUh(jn);
    const T rv0 = z0 * F.rdxVh(i), rve = ze * F.rdxVh(ie);
    T lu, lv;
    if (!VOTE || __any_sync(m, (hU0 | hUn | hV0 | hVe) != 0)) {   // no-slip boundary terms in this warp
        lu = fma(ru0, e12_coef<T>(mz0, hU0, 1), run * e12_coef<T>(mzn, hUn, -1));
        lv = fma(rv0, e12_coef<T>(mz0, hV0, 1), rve * e12_coef<T>(mze, hVe, -1));
    } else {
        lu = sel<T>(mz0, ru0) - sel<T>(mzn, run);
        lv = sel<T>(mz0, rv0) - sel<T>(mze, rve);
    }
    // strain rates and Coriolis (C(i, j) and C(i-1, j) for u; C(i, j), C(i, j-1) for v)
    lu += s.uA[o] + s.uB[ow];
    lv += s.vA[o] + s.vB[os];
    // ocean drag: du = inU (u - uOc) at C(i, j) and C(i-1, j)
    const bool inU = f0 & F_INU, inV = f0 & F_INV;
    const T du = sel<T>(inU, s.ldu[o] + s.ldu[ow]);
    const T dv = sel<T>(inV, s.ldv[o] + s.ldv[os]);
    lu += du;
    lv += dv;
    T luo = -du, lvo = -dv;
    if (BASAL) {
        lu = fma(sel<T>(inU, t.U(o)), s.lsb[o] + s.lsb[ow], lu);
        lv = fma(sel<T>(inV, t.V(o)), s.lsb[o] + s.lsb[os], lv);
    }
    if (TURN) {
        // du = uOc - u of U(i, j) enters U(i, j), U(i, j-1) (q0) and U(i+1, j), U(i+1, j-1) (qw)
        const T qu = (s.q0U[o] + s.q0U[os]) + (s.qwU[oe] + s.qwU[oes]);
        // dv = vOc - v of V(i, j) enters V(i, j), V(i-1, j) (q0) and V(i, j+1), V(i-1, j+1) (qs)
        const T qv = (s.q0V[o] + s.q0V[ow]) + (s.qsV[on] + s.qsV[own_]);
        lu -= qu;
        lv -= qv;
        luo += qu;
        lvo += qv;
    }
    lu_out = lu;
    lv_out = lv;
    luo_out = luo;
    lvo_out = lvo;
}

template <class T, bool BASAL, bool TURN>
__global__ void __launch_bounds__(BX * BY) uv_gather_kernel(Dims d, int64_t lp, FastConsts<T> c, TapeG<T> t,
                                                             LamG<T> l, Adj<T> a, KT<T> k, Scr<T> s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    T lu, lv, luo, lvo;
    p4_point<T, BASAL, TURN>(d, lp, c, t, k, s, m, i, j, lu, lv, luo, lvo);
    const int64_t o = (int64_t)i * lp + j;
    l.ou[o] += lu;
    l.ov[o] += lv;
    a.uOc[o] += luo;
    a.vOc[o] += lvo;
}

// P4 of subcycle k and P1 of subcycle k - 1 in one pass (no turning angle).
// The velocity adjoints P4 gathers at a point, added to its momentum share
// (which P1 of subcycle k left in l4.ou, l4.ov) and to those of the point's
// images in a filled halo (their P4 terms evaluated here as well), are what
// P1 of subcycle k - 1 reads there: they stay in registers, and the
// ocean-velocity adjoints take one read-modify-write for both subcycles, in
// the separate passes' order of additions.  t4, l4: subcycle k; t1, l1:
// subcycle k - 1.
template <class T, bool BASAL>
__device__ __forceinline__ void uv_link_body(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c,
                                             const TapeG<T> &t4, const TapeG<T> &t1, const LamG<T> &l4,
                                             const LamG<T> &l1, const Adj<T> &a, const KT<T> &k, const Scr<T> &s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    T lu, lv, luo, lvo;
    p4_point<T, BASAL, false>(d, lp, c, t4, k, s, m, i, j, lu, lv, luo, lvo);
    // own_adjoints of the separate passes, on subcycle k's completed adjoints
    T LU = T(0), LV = T(0);
    const bool hx = h.x_fill && in_xhalo(d, h.olx, i);
    const bool hy = h.y_fill && in_yhalo(d, h.oly, j);
    if (!(hx || hy)) {
        const int64_t o = (int64_t)i * lp + j;
        LU = l4.ou[o] + lu;
        LV = l4.ov[o] + lv;
        int ix[2] = {i, -1}, jy[2] = {j, -1};
        if (h.x_fill) {
            if (i + d.nx < d.NX && in_xhalo(d, h.olx, i + d.nx)) ix[1] = i + d.nx;
            else if (i - d.nx >= 0 && in_xhalo(d, h.olx, i - d.nx)) ix[1] = i - d.nx;
        }
        if (h.y_fill) {
            if (j + d.ny < d.NY && in_yhalo(d, h.oly, j + d.ny)) jy[1] = j + d.ny;
            else if (j - d.ny >= 0 && in_yhalo(d, h.oly, j - d.ny)) jy[1] = j - d.ny;
        }
        if (ix[1] >= 0 || jy[1] >= 0) {   // a point whose images lie in a filled halo (the edges)
#pragma unroll 1
            for (int q3 = 1; q3 < 4; ++q3) {   // images (i, j'), (i', j), (i', j') in the separate passes' order
                const int x = q3 >> 1, y = q3 & 1;
                if (ix[x] < 0 || jy[y] < 0) continue;
                T qu, qv, qo, qp;
                p4_point<T, BASAL, false, false>(d, lp, c, t4, k, s, 0u, ix[x], jy[y], qu, qv, qo, qp);
                const int64_t q = (int64_t)ix[x] * lp + jy[y];
                LU += l4.ou[q] + qu;
                LV += l4.ov[q] + qv;
            }
        }
    }
    p1_point<T, BASAL, false, true>(d, lp, c, t1, l1, a, k, s, m, i, j, LU, LV, luo, lvo);
}

template <class T, bool BASAL>
__global__ void __launch_bounds__(BX * BY) uv_link_kernel(Dims d, int64_t lp, HaloFill h, FastConsts<T> c,
                                                           TapeG<T> t4, TapeG<T> t1, LamG<T> l4, LamG<T> l1,
                                                           Adj<T> a, KT<T> k, Scr<T> s) {
    uv_link_body<T, BASAL>(d, lp, h, c, t4, t1, l4, l1, a, k, s);
}

// On a grid of more CTAs than the GPU holds at once, eight CTAs per SM (32
// registers, spilling).  On 3600 x 1800 a reverse step took 400.0 ms with
// the passes separate, 428.6 / 401.2 / 389.5 ms with the fused one at four
// / five / six CTAs per SM, and with P3 at eight CTAs 375.1 ms at six,
// 364.7 ms at eight.
template <class T, bool BASAL>
__global__ void __launch_bounds__(BX * BY, 8) uv_link_occ_kernel(Dims d, int64_t lp, HaloFill h, FastConsts<T> c,
                                                                 TapeG<T> t4, TapeG<T> t1, LamG<T> l4, LamG<T> l1,
                                                                 Adj<T> a, KT<T> k, Scr<T> s) {
    uv_link_body<T, BASAL>(d, lp, h, c, t4, t1, l4, l1, a, k, s);
}

}  // namespace

// padded cells from which the float32 passes P3 and P4+P1 run at eight CTAs
// per SM (the *_occ_kernel forms; 2^19: 3600 x 1800 faster so; 360 x 180,
// whose passes fit the GPU at once, slower: 1-degree trajectory 3.75x
// against 3.53-3.60x)
constexpr int64_t OCCUPY_CELLS = 1 << 19;

// The passes of one subcycle in phases: head (the recomputed terms of a
// tape without them, the basal coefficient, P1), body (P2, P3), tail (P4),
// or, chaining the sweep, the link (the next subcycle's recomputed terms and
// basal coefficient, then P4 fused with its P1).
template <class T>
static TapeG<T> with_terms(TapeG<T> t, const Scr<T> &s) {
    if (t.del == nullptr) {   // a tape without the forward's terms (float32 segment)
        t.del = s.del;
        t.zeta = s.zeta;
        t.cd = s.cd;
    }
    return t;
}

template <class T, bool B>
static void pre_p1(const Dims &d, int64_t lp, const FastConsts<T> &c, const KT<T> &k, const TapeG<T> &t,
                   const Scr<T> &s, dim3 grd, dim3 blk, cudaStream_t st) {
    if (t.del == nullptr) {
        e12_kernel<T><<<grd, blk, 0, st>>>(d, lp, c, t, k, s);
        viscosity_kernel<T><<<grd, blk, 0, st>>>(d, lp, c, t, k, s);
    }
    if (B) basal_kernel<T><<<grd, blk, 0, st>>>(d, lp, c, with_terms(t, s), k, s);
}

template <class T, bool B, bool R>
static int run_phases(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c, const KT<T> &k,
                      const TapeG<T> &t, const LamG<T> &l, const Adj<T> &a, const Scr<T> &s, bool head,
                      const TapeG<T> *tp, const LamG<T> *lpv, cudaStream_t st) {
    const dim3 blk(BX, BY), grd((d.NY + BX - 1) / BX, (d.NX + BY - 1) / BY);
    const TapeG<T> tt = with_terms(t, s);
    if (head) {
        pre_p1<T, B>(d, lp, c, k, t, s, grd, blk, st);
        uv_reverse_kernel<T, B, R><<<grd, blk, 0, st>>>(d, lp, h, c, tt, l, a, k, s);
    }
    z_reverse_kernel<T><<<grd, blk, 0, st>>>(d, lp, c, tt, l, k, s, t.del == nullptr);
    // float32 on a grid of more CTAs than the GPU holds: P3 and the fused pass at eight CTAs per SM
    const bool occupy = sizeof(T) == 4 && (int64_t)d.NX * d.NY >= OCCUPY_CELLS;
    if constexpr (sizeof(T) == 4) {
        if (occupy) c_reverse_occ_kernel<T, B, R><<<grd, blk, 0, st>>>(d, lp, c, tt, l, a, k, s);
        else c_reverse_kernel<T, B, R><<<grd, blk, 0, st>>>(d, lp, c, tt, l, a, k, s);
    } else {
        c_reverse_kernel<T, B, R><<<grd, blk, 0, st>>>(d, lp, c, tt, l, a, k, s);
    }
    if (tp) {
        if constexpr (!R && sizeof(T) == 4) {
            pre_p1<T, B>(d, lp, c, k, *tp, s, grd, blk, st);
            const TapeG<T> t1 = with_terms(*tp, s);
            if (occupy) uv_link_occ_kernel<T, B><<<grd, blk, 0, st>>>(d, lp, h, c, tt, t1, l, *lpv, a, k, s);
            else uv_link_kernel<T, B><<<grd, blk, 0, st>>>(d, lp, h, c, tt, t1, l, *lpv, a, k, s);
        }
    } else {
        uv_gather_kernel<T, B, R><<<grd, blk, 0, st>>>(d, lp, c, tt, l, a, k, s);
    }
    return launch_status();
}

template <class T>
static int phases(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c, const FastScalars<T> &k,
                  double rhoSea, const TapeG<T> &t, const LamG<T> &l, const Adj<T> &a, T *const scratch[N_SCRATCH],
                  bool basal, bool turn, bool head, const TapeG<T> *tp, const LamG<T> *lpv, cudaStream_t st) {
    if (tp && turn) return VERIS_ERR_ARG;   // the link keeps no turning-angle shares
    Scr<T> s;
    std::memcpy(&s, scratch, sizeof s);
    const KT<T> kk = kt<T>(k, rhoSea);
    if (basal)
        return turn ? run_phases<T, true, true>(d, lp, h, c, kk, t, l, a, s, head, tp, lpv, st)
                    : run_phases<T, true, false>(d, lp, h, c, kk, t, l, a, s, head, tp, lpv, st);
    return turn ? run_phases<T, false, true>(d, lp, h, c, kk, t, l, a, s, head, tp, lpv, st)
                : run_phases<T, false, false>(d, lp, h, c, kk, t, l, a, s, head, tp, lpv, st);
}

template <class T>
int adjoint_gather_subcycle(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c,
                            const FastScalars<T> &k, double rhoSea, const TapeG<T> &t, const LamG<T> &l,
                            const Adj<T> &a, T *const scratch[N_SCRATCH], bool basal, bool turn, cudaStream_t st) {
    return phases<T>(d, lp, h, c, k, rhoSea, t, l, a, scratch, basal, turn, true, nullptr, nullptr, st);
}

template <class T>
int adjoint_gather_chain(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c,
                         const FastScalars<T> &k, double rhoSea, const TapeG<T> &t, const LamG<T> &l,
                         const Adj<T> &a, T *const scratch[N_SCRATCH], bool basal, bool head,
                         const TapeG<T> *t_prev, const LamG<T> *l_prev, cudaStream_t st) {
    if ((t_prev == nullptr) != (l_prev == nullptr)) return VERIS_ERR_ARG;
    return phases<T>(d, lp, h, c, k, rhoSea, t, l, a, scratch, basal, false, head, t_prev, l_prev, st);
}

// the per-cell water-drag sums of the whole sweep, by hemisphere: block sums in float64 (fixed
// trees), one atomic per block and hemisphere
__global__ void __launch_bounds__(256) reduce_drag_kernel(Dims d, int64_t lp, const uint32_t *flags,
                                                          const double *dragC, double wN, double wS, double *dragN,
                                                          double *dragS) {
    double n = 0.0, sth = 0.0;
    for (int i = blockIdx.x; i < d.NX; i += gridDim.x)
        for (int j = threadIdx.x; j < d.NY; j += blockDim.x) {
            const int64_t o = (int64_t)i * lp + j;
            const double v = dragC[o];
            if (flags[o] & F_SOUTH) sth += v; else n += v;
        }
    __shared__ double part[2][8];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        n += __shfl_down_sync(ALL, n, off);
        sth += __shfl_down_sync(ALL, sth, off);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        part[0][warp] = n;
        part[1][warp] = sth;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < 8; ++q) {
            a += part[0][q];
            b += part[1][q];
        }
        if (a != 0.0) atomicAdd(dragN, a * wN);
        if (b != 0.0) atomicAdd(dragS, b * wS);
    }
}

int reduce_drag(const Dims &d, int64_t lp, const uint32_t *flags, const double *dragC, double wN, double wS,
                double *dragN, double *dragS, cudaStream_t st) {
    const int blocks = d.NX < 1024 ? d.NX : 1024;
    reduce_drag_kernel<<<blocks, 256, 0, st>>>(d, lp, flags, dragC, wN, wS, dragN, dragS);
    return launch_status();
}

template int adjoint_gather_subcycle<double>(const Dims &, int64_t, const HaloFill &, const FastConsts<double> &,
                                             const FastScalars<double> &, double, const TapeG<double> &,
                                             const LamG<double> &, const Adj<double> &, double *const[N_SCRATCH],
                                             bool, bool, cudaStream_t);
template int adjoint_gather_subcycle<float>(const Dims &, int64_t, const HaloFill &, const FastConsts<float> &,
                                            const FastScalars<float> &, double, const TapeG<float> &,
                                            const LamG<float> &, const Adj<float> &, float *const[N_SCRATCH], bool,
                                            bool, cudaStream_t);
template int adjoint_gather_chain<float>(const Dims &, int64_t, const HaloFill &, const FastConsts<float> &,
                                         const FastScalars<float> &, double, const TapeG<float> &,
                                         const LamG<float> &, const Adj<float> &, float *const[N_SCRATCH], bool,
                                         bool, const TapeG<float> *, const LamG<float> *, cudaStream_t);

}  // namespace adj

}  // namespace veris
