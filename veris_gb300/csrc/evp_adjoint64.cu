// Float64 adjoint of one mEVP subcycle (veris/evp_solver.py:21-254) in
// four gather passes, arranged for GB300's float64 pipe.
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
// Every point is computed once, nothing is recomputed on rings and nothing
// is accumulated with atomics (each input adjoint is written by the pass
// that owns its position).  The forward's Delta, zeta and drag coefficient
// come from the tape the float64 forward writes (evp_fast.cu), so the
// adjoint takes no square root of the forward's; its reciprocals and the
// basal drag's reciprocal square root use the series-refined hardware
// approximations of f64math.cuh, masks are selects and zero tests run on the
// integer pipe.
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
struct K64 {
    double bU, bU1;            // beta/dt, (beta + 1)/dt
    double hc, sinH;           // 0.5 cos(turning angle), 0.5 sin(turning angle)
    double am1, ra2, rah;      // (alpha - 1)/alpha, 2/alpha, 0.5/alpha
    double hkp, rsq, dmin;     // half the press factor, 1/e^2, Delta_min
    double nh1, nh2, nh3, nh4; // 0.5/alpha/n: sigma12's average over n wet C points
    double dcq2N, dcq2S, cmin2;   // the drag test (as the float64 forward takes it)
    double kXN, kXS;           // (rhoSea drag)^2 / 4: 2 d cDrag/dX = kX / cDrag
    double wN, wS;             // rhoSea / (rhoSea drag): d cDrag / d drag = cDrag * w
    double U02;                // basal U0^2
};

K64 k64(const FastScalars<double> &k, double rhoSea) {
    K64 s;
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
    s.kXN = 0.25 * k.dN2;
    s.kXS = 0.25 * k.dS2;
    s.wN = k.dN != 0.0 ? rhoSea / k.dN : 0.0;
    s.wS = k.dS != 0.0 ? rhoSea / k.dS : 0.0;
    s.U02 = k.U02;
    return s;
}

// the passes' arrays (internal pitch)
struct Scr {
    double *gU, *gV;       // adjoints of the momentum numerators
    double *rU, *rV;       // the same over rA_u, rA_v (stress-divergence shares)
    double *wU0, *wU1;     // a U point's share in dL/dcDrag at C(i, j) and C(i-1, j)
    double *wV0, *wV1;     // a V point's share at C(i, j) and C(i, j-1)
    double *bU, *bV;       // shares in the basal coefficient's adjoint
    double *q0U, *qwU;     // turning-angle shares in d/du of (i, j),(i, j+1) and (i-1, j),(i-1, j+1)
    double *q0V, *qsV;     // the same for v: (i, j),(i+1, j) and (i, j-1),(i+1, j-1)
    double *tZ;            // a Z point's share in the adjoint of each neighbouring zeta
    double *le12;          // e12's adjoint through sigma12
    double *e2;            // rAz e12
    double *uA, *uB;       // a C point's share in d/du of U(i, j) and U(i+1, j)
    double *vA, *vB;       // the same for V(i, j) and V(i, j+1)
    double *ldu, *ldv;     // ocean-drag shares in d/du, d/dv (masked by the U/V point)
    double *wC;            // recip_rA/e^2 dL/dDelta / Delta: twice the adjoint of rAz e12^2
    double *lsb;           // basal shares, times u or v at the U/V point
    double *cb;            // the basal coefficient (recomputed once per subcycle)
};
static_assert(sizeof(Scr) == N_SCRATCH64 * sizeof(double *), "scratch table");

__device__ __forceinline__ int wxp(const Dims &d, int i) { return i < 0 ? i + d.NX : (i >= d.NX ? i - d.NX : i); }
__device__ __forceinline__ int wyp(const Dims &d, int j) { return j < 0 ? j + d.NY : (j >= d.NY ? j - d.NY : j); }

// 0.5 where the four C points around Z(i, j) are all wet, else 0
__device__ __forceinline__ bool z_wet(uint32_t f0, uint32_t fw, uint32_t fs, uint32_t fws) {
    return (f0 & fw & fs & fws & F_MC) != 0;
}

__device__ __forceinline__ double sel(bool b, double x) { return b ? x : 0.0; }

// ------------------------------------------------------------------ P0
// the basal drag coefficient at every C point, as the forward computes it
// (veris/dynamics_routines.py:55-96 with the step factor folded)
__global__ void __launch_bounds__(BX * BY) basal_kernel(Dims d, int64_t lp, FastConsts<double> c, Tape64 t,
                                                         K64 k, Scr s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    const int64_t o = (int64_t)i * lp + j;
    const int64_t oe = (int64_t)wxp(d, i + 1) * lp + j, on = (int64_t)i * lp + wyp(d, j + 1);
    const uint32_t f0 = c.flags[o], fe = c.flags[oe], fn = c.flags[on];
    const double a_ = sel(f0 & F_INU, t.u[o]), b_ = sel(fe & F_INU, t.u[oe]);
    const double c_ = sel(f0 & F_INV, t.v[o]), e_ = sel(fn & F_INV, t.v[on]);
    const double q = 0.25 * (a_ * a_ + b_ * b_ + c_ * c_ + e_ * e_);
    s.cb[o] = div64(c.bfac[o], sqrt64(q + k.U02, m), m);
}

// the adjoint of a U or V point's new velocity, with the adjoints of its
// images in a filled halo added (the transpose of the fill); 0 at image
// points, whose values the forward copies rather than computes
__device__ __forceinline__ void own_adjoints(const Dims &d, const HaloFill &h, const Lam64 &l, int i, int j,
                                             double &LU, double &LV) {
    LU = LV = 0.0;
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
template <bool BASAL, bool TURN>
__global__ void __launch_bounds__(BX * BY) uv_reverse_kernel(Dims d, int64_t lp, HaloFill h, FastConsts<double> c,
                                                              Tape64 t, Lam64 l, Adj<double> a, K64 k, Scr s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    const int iw = wxp(d, i - 1), js = wyp(d, j - 1);
    const int64_t o = (int64_t)i * lp + j, ow = (int64_t)iw * lp + j, os = (int64_t)i * lp + js;
    const uint32_t f0 = c.flags[o];
    double LU, LV;
    own_adjoints(d, h, l, i, j, LU, LV);
    const double cd0 = t.cd[o], cdw = t.cd[ow], cds = t.cd[os];
    double cb0 = 0.0, cbw = 0.0, cbs = 0.0;
    if (BASAL) {
        cb0 = s.cb[o];
        cbw = s.cb[ow];
        cbs = s.cb[os];
    }
    double sg = 0.0;
    if (TURN) sg = (f0 & F_SPOS) ? 1.0 : ((f0 & F_SNEG) ? -1.0 : 0.0);
    if (!__any_sync(m, f0 & F_MU)) {   // a warp of dry U points: no momentum adjoint, nothing to add
        l.ou[o] = 0.0;
        s.gU[o] = 0.0;
        s.rU[o] = 0.0;
        s.wU0[o] = 0.0;
        if (TURN) s.wU1[o] = s.q0U[o] = s.qwU[o] = 0.0;
        if (BASAL) s.bU[o] = 0.0;
    } else {   // U point (hAW = cos/2 AW, mUb = mU beta/dt, mUb1 = mU (beta+1)/dt folded by the prep)
        const double hA = c.hAW[o], uo = c.uOc[o], u0 = t.u[o];
        const double S = cd0 + cdw, kU = hA * S;
        double den = c.mUb1[o] + kU;
        if (BASAL) den = fma(0.5 * c.AW[o], cb0 + cbw, den);
        const bool guard = is_zero(den);
        const double r = rcp64(guard ? 1.0 : den, m);
        const double g = sel(f0 & F_MU, LU * r);
        const double lden = guard ? 0.0 : -t.un[o] * g;
        const double Y = fma(uo, g, lden);   // d/dkU
        const double W = hA * Y;
        l.ou[o] = c.mUb[o] * g;
        a.mU[o] = fma(k.bU * u0, g, fma(k.bU1, lden, a.mU[o]));
        a.cU[o] += g;
        double lAW = fma(k.hc * S, Y, a.AW[o]);
        if (BASAL) {
            lAW = fma(0.5 * (cb0 + cbw), lden, lAW);
            s.bU[o] = 0.5 * c.AW[o] * lden;
        }
        a.uOc[o] = fma(kU, g, a.uOc[o]);
        s.gU[o] = g;
        s.rU[o] = c.rrAu[o] * g;
        if (TURN) {
            // num -= sg sin/2 AW (cd (du + du_n)/2 + cd_w (du_w + du_wn)/2) where SeaIceMassU != 0, du = uOc - u
            const int jn = wyp(d, j + 1);
            const int64_t on = (int64_t)i * lp + jn, own_ = (int64_t)iw * lp + jn;
            const double tu = sel(f0 & F_LMU, -sg * k.sinH);
            const double pn = 0.5 * ((uo - u0) + (c.uOc[on] - t.u[on]));
            const double pw = 0.5 * ((c.uOc[ow] - t.u[ow]) + (c.uOc[own_] - t.u[own_]));
            lAW = fma(tu * fma(cd0, pn, cdw * pw), g, lAW);
            const double tg = tu * c.AW[o] * g;
            s.wU0[o] = fma(tg, pn, W);
            s.wU1[o] = fma(tg, pw, W);
            s.q0U[o] = 0.5 * tg * cd0;
            s.qwU[o] = 0.5 * tg * cdw;
        } else {
            s.wU0[o] = W;
        }
        a.AW[o] = lAW;
    }
    if (!__any_sync(m, f0 & F_MV)) {
        l.ov[o] = 0.0;
        s.gV[o] = 0.0;
        s.rV[o] = 0.0;
        s.wV0[o] = 0.0;
        if (TURN) s.wV1[o] = s.q0V[o] = s.qsV[o] = 0.0;
        if (BASAL) s.bV[o] = 0.0;
    } else {   // V point
        const double hA = c.hAS[o], vo = c.vOc[o], v0 = t.v[o];
        const double S = cd0 + cds, kV = hA * S;
        double den = c.mVb1[o] + kV;
        if (BASAL) den = fma(0.5 * c.AS[o], cb0 + cbs, den);
        const bool guard = is_zero(den);
        const double r = rcp64(guard ? 1.0 : den, m);
        const double g = sel(f0 & F_MV, LV * r);
        const double lden = guard ? 0.0 : -t.vn[o] * g;
        const double Y = fma(vo, g, lden);
        const double W = hA * Y;
        l.ov[o] = c.mVb[o] * g;
        a.mV[o] = fma(k.bU * v0, g, fma(k.bU1, lden, a.mV[o]));
        a.cV[o] += g;
        double lAS = fma(k.hc * S, Y, a.AS[o]);
        if (BASAL) {
            lAS = fma(0.5 * (cb0 + cbs), lden, lAS);
            s.bV[o] = 0.5 * c.AS[o] * lden;
        }
        a.vOc[o] = fma(kV, g, a.vOc[o]);
        s.gV[o] = g;
        s.rV[o] = c.rrAv[o] * g;
        if (TURN) {
            // num += sg sin/2 AS (cd (dv + dv_e)/2 + cd_s (dv_s + dv_se)/2) where SeaIceMassV != 0, dv = vOc - v
            const int ie = wxp(d, i + 1);
            const int64_t oe = (int64_t)ie * lp + j, ose = (int64_t)ie * lp + js;
            const double tv = sel(f0 & F_LMV, sg * k.sinH);
            const double pe = 0.5 * ((vo - v0) + (c.vOc[oe] - t.v[oe]));
            const double ps = 0.5 * ((c.vOc[os] - t.v[os]) + (c.vOc[ose] - t.v[ose]));
            lAS = fma(tv * fma(cd0, pe, cds * ps), g, lAS);
            const double tg = tv * c.AS[o] * g;
            s.wV0[o] = fma(tg, pe, W);
            s.wV1[o] = fma(tg, ps, W);
            s.q0V[o] = 0.5 * tg * cd0;
            s.qsV[o] = 0.5 * tg * cds;
        } else {
            s.wV0[o] = W;
        }
        a.AS[o] = lAS;
    }
}

// e12 at Z(i, j) (veris/dynamics_routines.py:160-175), as the float64
// forward computes it: 0.5 rdyU, 0.5 rdxV folded, the no-slip boundary
// terms only in warps that have one
__device__ __forceinline__ double e12_at(const FastConsts<double> &c, const Tape64 &t, unsigned m, int i, int j,
                                         int64_t o, int64_t ow, int64_t os, uint32_t f0, uint32_t fw, uint32_t fs,
                                         uint32_t fws) {
    const bool mz = z_wet(f0, fw, fs, fws);
    const int hU = (int)((f0 & F_MU) != 0) - (int)((fs & F_MU) != 0);
    const int hV = (int)((f0 & F_MV) != 0) - (int)((fw & F_MV) != 0);
    const double u0 = t.u[o], us = t.u[os], v0 = t.v[o], vw = t.v[ow];
    const double ry = c.rdyUh_y[j], rx = c.rdxVh_x[i];
    if (__any_sync(m, (hU | hV) != 0)) {
        const double hu2 = hU == 0 ? 0.0 : (hU > 0 ? 2.0 : -2.0);
        const double hv2 = hV == 0 ? 0.0 : (hV > 0 ? 2.0 : -2.0);
        const double tu = fma(hu2, u0 + us, mz ? u0 - us : 0.0);
        const double tv = fma(hv2, v0 + vw, mz ? v0 - vw : 0.0);
        return fma(ry, tu, rx * tv);
    }
    return mz ? fma(ry, u0 - us, rx * (v0 - vw)) : 0.0;
}

// ------------------------------------------------------------------ P2
// Z(i, j): sigma12' = (alpha-1)/alpha sigma12 + 0.5/alpha/n e12 * (sum of
// the four zeta) (veris/evp_solver.py:101-103, veris/averaging.py:4-19)
__global__ void __launch_bounds__(BX * BY) z_reverse_kernel(Dims d, int64_t lp, FastConsts<double> c, Tape64 t,
                                                             Lam64 l, K64 k, Scr s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    const int iw = wxp(d, i - 1), js = wyp(d, j - 1);
    const int64_t o = (int64_t)i * lp + j, ow = (int64_t)iw * lp + j, os = (int64_t)i * lp + js,
                  ows = (int64_t)iw * lp + js;
    // sigma12' at Z(i, j) enters sdx of U(i, j) (-) and U(i, j-1) (+), sdy of V(i, j) (-) and V(i-1, j) (+)
    const double L = fma(c.dxV_x[i], s.rU[os] - s.rU[o],
                         fma(c.dyU_y[j], s.rV[ow] - s.rV[o], l.ls12[(int64_t)i * l.ldl + j]));
    l.os12[o] = k.am1 * L;
    const uint32_t f0 = c.flags[o], fw = c.flags[ow], fs = c.flags[os], fws = c.flags[ows];
    const uint32_t n = (f0 & F_MC) + (fw & F_MC) + (fs & F_MC) + (fws & F_MC);
    const double nh = n == 4 ? k.nh4 : (n == 3 ? k.nh3 : (n == 2 ? k.nh2 : (n == 1 ? k.nh1 : 0.0)));
    const double e = e12_at(c, t, m, i, j, o, ow, os, f0, fw, fs, fws);
    const double zs = (t.zeta[o] + t.zeta[ow]) + (t.zeta[os] + t.zeta[ows]);
    const double cz = nh * L;
    s.tZ[o] = cz * e;
    s.le12[o] = cz * zs;
    s.e2[o] = c.rAz[o] * e;
}

// ------------------------------------------------------------------ P3
// C(i, j): strain rates, Delta, zeta and the stress update
// (veris/dynamics_routines.py:143-268, veris/evp_solver.py:80-100), ocean
// drag (veris/dynamics_routines.py:21-52), basal drag (:55-96) and the
// Coriolis terms (veris/evp_solver.py:124-131)
template <bool BASAL, bool TURN>
__global__ void __launch_bounds__(BX * BY) c_reverse_kernel(Dims d, int64_t lp, FastConsts<double> c, Tape64 t,
                                                             Lam64 l, Adj<double> a, K64 k, Scr s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    double dragN = 0.0, dragS = 0.0;
    if (act) {
        const int ie = wxp(d, i + 1), jn = wyp(d, j + 1);
        const int64_t o = (int64_t)i * lp + j, oe = (int64_t)ie * lp + j, on = (int64_t)i * lp + jn,
                      oen = (int64_t)ie * lp + jn;
        const uint32_t f0 = c.flags[o], fe = c.flags[oe], fn = c.flags[on];
        const bool mC = f0 & F_MC, inC = f0 & F_INC;
        // shares gathered from U(i, j), U(i+1, j), V(i, j), V(i, j+1)
        const double sU = s.gU[o] + s.gU[oe], sV = s.gV[o] + s.gV[on];
        const double lcd = (s.wU0[o] + (TURN ? s.wU1[oe] : s.wU0[oe])) + (s.wV0[o] + (TURN ? s.wV1[on] : s.wV0[on]));
        // sig11 = (sigma1' + sigma2')/2 enters U(i, j) (+) and U(i+1, j) (-) as rrAu dyV,
        // sig22 = (sigma1' - sigma2')/2 V(i, j) (+) and V(i, j+1) (-) as rrAv dxU
        const double h11 = c.dyVh_y[j] * (s.rU[o] - s.rU[oe]);
        const double h22 = c.dxUh_x[i] * (s.rV[o] - s.rV[on]);
        const double L1 = l.ls1[(int64_t)i * l.ldl + j] + (h11 + h22);
        const double L2 = l.ls2[(int64_t)i * l.ldl + j] + (h11 - h22);
        l.os1[o] = sel(mC, k.am1 * L1);
        l.os2[o] = sel(mC, k.am1 * L2);
        // sigma1' = mC ((alpha-1)/alpha sigma1 + zeta (2 ep - kp Delta)/alpha),
        // sigma2' = mC ((alpha-1)/alpha sigma2 + zeta em/(2 alpha)): h1 = 2 d/dsigma1'/alpha, h2 = d/dsigma2'/(2 alpha)
        const double h1 = sel(mC, k.ra2 * L1), h2 = sel(mC, k.rah * L2);
        // strain rates (recomputed from the tape's velocities)
        const double u0 = t.u[o], ue = t.u[oe], v0 = t.v[o], vn = t.v[on];
        const double rdx = c.rdxU_x[i], rdy = c.rdyV_y[j];
        const double e11 = inC ? (ue - u0) * rdx : 0.0;
        const double e22 = inC ? (vn - v0) * rdy : 0.0;
        const double ep = e11 + e22, em = e11 - e22;
        const double del = t.del[o], zeta = t.zeta[o];
        const double tz = (s.tZ[o] + s.tZ[oe]) + (s.tZ[on] + s.tZ[oen]);
        const double lz = fma(fma(-k.hkp, del, ep), h1, fma(em, h2, tz));
        // zeta = Ph/(Delta + Delta_min)
        const double rz = rcp64(del + k.dmin, m);
        a.Ph[o] = fma(lz, rz, a.Ph[o]);
        // where the ice strength is 0, zeta = 0 and nothing flows back through Delta
        double q = 0.0, le11 = 0.0, le22 = 0.0;
        if (__any_sync(m, !is_zero(zeta))) {
            double lep = zeta * h1, lem = zeta * h2;
            const double ldel = fma(-zeta * rz, lz, -k.hkp * lep);
            // Delta = sqrt(ep^2 + rsq em^2 + (recip_rA/e^2) sum rAz e12^2); 0 at Delta = 0.  q = 2 dL/dDelta^2
            const bool dz = is_zero(del);
            const double rdel = rcp64(dz ? 1.0 : del, m);
            q = dz ? 0.0 : ldel * rdel;
            lep = fma(ep, q, lep);
            lem = fma(k.rsq * em, q, lem);
            le11 = inC ? (lep + lem) * rdx : 0.0;
            le22 = inC ? (lep - lem) * rdy : 0.0;
        }
        s.wC[o] = c.rsqrA[o] * q;
        // Coriolis: Fv = mfC (v + v_n) enters U(i, j), U(i+1, j) with 1/2, Fu = mfC (u + u_e)
        // V(i, j), V(i, j+1) with -1/2 (mf4 = mfC/2)
        const double mf = c.mf4[o];
        a.mfC[o] = fma(0.5, fma(v0 + vn, sU, -((u0 + ue) * sV)), a.mfC[o]);
        const double fv = mf * sU, fu = -mf * sV;
        s.uA[o] = fu - le11;
        s.uB[o] = fu + le11;
        s.vA[o] = fv - le22;
        s.vB[o] = fv + le22;
        // ocean drag: cd = 0.5 rhoSea drag sqrt(X), X = (du + du_e)^2 + (dv + dv_n)^2, above its floor
        // (the branch taken exactly as the forward takes it)
        const double du0 = (f0 & F_INU) ? u0 - c.uOc[o] : 0.0;
        const double du1 = (fe & F_INU) ? ue - c.uOc[oe] : 0.0;
        const double dv0 = (f0 & F_INV) ? v0 - c.vOc[o] : 0.0;
        const double dv1 = (fn & F_INV) ? vn - c.vOc[on] : 0.0;
        const double A = du0 + du1, B = dv0 + dv1;
        const double X = fma(B, B, A * A);
        const bool south = f0 & F_SOUTH;
        const bool fast = mC && gt_nonneg((south ? k.dcq2S : k.dcq2N) * X, k.cmin2);
        double lX2 = 0.0;   // 2 dL/dX
        if (__any_sync(m, fast)) {
            const double cd = t.cd[o];
            const double rc = rcp64(fast ? cd : 1.0, m);
            if (fast) {
                lX2 = lcd * (south ? k.kXS : k.kXN) * rc;
                if (south) dragS = lcd * cd; else dragN = lcd * cd;
            }
        }
        s.ldu[o] = A * lX2;
        s.ldv[o] = B * lX2;
        if (BASAL) {
            // cb = bfac / sqrt(0.25 (a^2 + b^2 + c^2 + e^2) + U0^2), a = inU u, b = inU_e u_e, c = inV v, e = inV_n v_n
            const double lcb = (s.bU[o] + s.bU[oe]) + (s.bV[o] + s.bV[on]);
            const double a_ = sel(f0 & F_INU, u0), b_ = sel(fe & F_INU, ue);
            const double c_ = sel(f0 & F_INV, v0), e_ = sel(fn & F_INV, vn);
            const double q = 0.25 * (a_ * a_ + b_ * b_ + c_ * c_ + e_ * e_) + k.U02;
            const double rs = rsqrt64(q, m);
            const double bf = c.bfac[o];
            a.bfac[o] += lcb * rs;
            s.lsb[o] = -0.25 * bf * rs * rs * rs * lcb;
        }
    }
    // the water-drag gradients: warp sums, one atomic per warp
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        dragN += __shfl_down_sync(ALL, dragN, off);
        dragS += __shfl_down_sync(ALL, dragS, off);
    }
    if ((threadIdx.x & 31) == 0) {   // d cDrag / d drag = cDrag rhoSea / (rhoSea drag)
        if (dragN != 0.0) atomicAdd(a.dragN, dragN * k.wN);
        if (dragS != 0.0) atomicAdd(a.dragS, dragS * k.wS);
    }
}

// e12's full adjoint at Z(i, j): its share through sigma12 plus
// 2 rAz e12 times the adjoints of e12^2 gathered from C(i, j), C(i-1, j),
// C(i, j-1), C(i-1, j-1)
__device__ __forceinline__ double le12_at(const Scr &s, int64_t o, int64_t ow, int64_t os, int64_t ows) {
    return fma(s.e2[o], (s.wC[o] + s.wC[ow]) + (s.wC[os] + s.wC[ows]), s.le12[o]);
}

// d e12(Z) / d u (or v) in units of 0.5 rdyU (0.5 rdxV): 2 h + sign mz at
// the Z point's own U (V) point (sign +1) and at its southern (western) one
// (sign -1), h = iceMaskU - its southern neighbour (iceMaskV - its western
// one); a small integer, selected rather than converted
__device__ __forceinline__ double e12_coef(bool mz, int h, int sign) {
    const int v = 2 * h + (mz ? sign : 0);
    return v == 0 ? 0.0 : v == 1 ? 1.0 : v == -1 ? -1.0 : v == 2 ? 2.0 : v == -2 ? -2.0 : v == 3 ? 3.0 : -3.0;
}

// ------------------------------------------------------------------ P4
// U(i, j), V(i, j): the velocity and ocean-velocity adjoints gathered from
// the C points (strain rates, drag, basal drag, Coriolis), the Z points
// (e12) and the turning-angle terms of the neighbouring U, V points
template <bool BASAL, bool TURN>
__global__ void __launch_bounds__(BX * BY) uv_gather_kernel(Dims d, int64_t lp, FastConsts<double> c, Tape64 t,
                                                             Lam64 l, Adj<double> a, Scr s) {
    const int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const bool act = i < d.NX && j < d.NY;
    const unsigned m = __ballot_sync(ALL, act);
    if (!act) return;
    const int iw = wxp(d, i - 1), ie = wxp(d, i + 1), js = wyp(d, j - 1), jn = wyp(d, j + 1);
    const int64_t o = (int64_t)i * lp + j, ow = (int64_t)iw * lp + j, oe = (int64_t)ie * lp + j,
                  os = (int64_t)i * lp + js, on = (int64_t)i * lp + jn, ows = (int64_t)iw * lp + js,
                  own_ = (int64_t)iw * lp + jn, oes = (int64_t)ie * lp + js;
    const uint32_t f0 = c.flags[o], fw = c.flags[ow], fe = c.flags[oe], fs = c.flags[os], fn = c.flags[on],
                   fws = c.flags[ows], fwn = c.flags[own_], fes = c.flags[oes];
    // e12 adjoints at Z(i, j), Z(i, j+1), Z(i+1, j)
    const double z0 = le12_at(s, o, ow, os, ows);
    const double zn = le12_at(s, on, own_, o, ow);
    const double ze = le12_at(s, oe, o, oes, os);
    // e12(Z) = 0.5 rdyU (2 hU (u + u_s) + mz (u - u_s)) + 0.5 rdxV (2 hV (v + v_w) + mz (v - v_w))
    const int hU0 = (int)((f0 & F_MU) != 0) - (int)((fs & F_MU) != 0);
    const int hUn = (int)((fn & F_MU) != 0) - (int)((f0 & F_MU) != 0);
    const int hV0 = (int)((f0 & F_MV) != 0) - (int)((fw & F_MV) != 0);
    const int hVe = (int)((fe & F_MV) != 0) - (int)((f0 & F_MV) != 0);
    const bool mz0 = z_wet(f0, fw, fs, fws), mzn = z_wet(fn, fwn, f0, fw), mze = z_wet(fe, f0, fes, fs);
    const double ru0 = z0 * c.rdyUh_y[j], run = zn * c.rdyUh_y[jn];
    const double rv0 = z0 * c.rdxVh_x[i], rve = ze * c.rdxVh_x[ie];
    double lu, lv;
    if (__any_sync(m, (hU0 | hUn | hV0 | hVe) != 0)) {   // no-slip boundary terms in this warp
        lu = fma(ru0, e12_coef(mz0, hU0, 1), run * e12_coef(mzn, hUn, -1));
        lv = fma(rv0, e12_coef(mz0, hV0, 1), rve * e12_coef(mze, hVe, -1));
    } else {
        lu = sel(mz0, ru0) - sel(mzn, run);
        lv = sel(mz0, rv0) - sel(mze, rve);
    }
    // strain rates and Coriolis (C(i, j) and C(i-1, j) for u; C(i, j), C(i, j-1) for v)
    lu += s.uA[o] + s.uB[ow];
    lv += s.vA[o] + s.vB[os];
    // ocean drag: du = inU (u - uOc) at C(i, j) and C(i-1, j)
    const bool inU = f0 & F_INU, inV = f0 & F_INV;
    const double du = sel(inU, s.ldu[o] + s.ldu[ow]);
    const double dv = sel(inV, s.ldv[o] + s.ldv[os]);
    lu += du;
    lv += dv;
    double luo = -du, lvo = -dv;
    if (BASAL) {
        lu = fma(sel(inU, t.u[o]), s.lsb[o] + s.lsb[ow], lu);
        lv = fma(sel(inV, t.v[o]), s.lsb[o] + s.lsb[os], lv);
    }
    if (TURN) {
        // du = uOc - u of U(i, j) enters U(i, j), U(i, j-1) (q0) and U(i+1, j), U(i+1, j-1) (qw)
        const double qu = (s.q0U[o] + s.q0U[os]) + (s.qwU[oe] + s.qwU[oes]);
        // dv = vOc - v of V(i, j) enters V(i, j), V(i-1, j) (q0) and V(i, j+1), V(i-1, j+1) (qs)
        const double qv = (s.q0V[o] + s.q0V[ow]) + (s.qsV[on] + s.qsV[own_]);
        lu -= qu;
        lv -= qv;
        luo += qu;
        lvo += qv;
    }
    l.ou[o] += lu;
    l.ov[o] += lv;
    a.uOc[o] += luo;
    a.vOc[o] += lvo;
}

}  // namespace

template <bool B, bool R>
static int run_passes(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<double> &c, const K64 &k,
                      const Tape64 &t, const Lam64 &l, const Adj<double> &a, const Scr &s, cudaStream_t st) {
    const dim3 blk(BX, BY), grd((d.NY + BX - 1) / BX, (d.NX + BY - 1) / BY);
    if (B) basal_kernel<<<grd, blk, 0, st>>>(d, lp, c, t, k, s);
    uv_reverse_kernel<B, R><<<grd, blk, 0, st>>>(d, lp, h, c, t, l, a, k, s);
    z_reverse_kernel<<<grd, blk, 0, st>>>(d, lp, c, t, l, k, s);
    c_reverse_kernel<B, R><<<grd, blk, 0, st>>>(d, lp, c, t, l, a, k, s);
    uv_gather_kernel<B, R><<<grd, blk, 0, st>>>(d, lp, c, t, l, a, s);
    return launch_status();
}

int adjoint64_subcycle(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<double> &c,
                       const FastScalars<double> &k, double rhoSea, const Tape64 &t, const Lam64 &l,
                       const Adj<double> &a, double *const scratch[N_SCRATCH64], bool basal, bool turn,
                       cudaStream_t st) {
    Scr s;
    std::memcpy(&s, scratch, sizeof s);
    const K64 kk = k64(k, rhoSea);
    if (basal)
        return turn ? run_passes<true, true>(d, lp, h, c, kk, t, l, a, s, st)
                    : run_passes<true, false>(d, lp, h, c, kk, t, l, a, s, st);
    return turn ? run_passes<false, true>(d, lp, h, c, kk, t, l, a, s, st)
                : run_passes<false, false>(d, lp, h, c, kk, t, l, a, s, st);
}

}  // namespace adj

}  // namespace veris
