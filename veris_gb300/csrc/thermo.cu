// Thermodynamics in float64: the surface-temperature Newton solve
// (veris/solve4temp.py:5-174) and ice growth with the ocean budgets
// (veris/growth.py:8-397).  Both are pointwise; one thread per padded point.
#include <type_traits>

#include "stencil.cuh"
#include "dual.cuh"

namespace veris {

struct S4TIn {
    double hI, hS, Tin, TempFrz;
    double LWdown, ATemp, wSpeed, fCori, SWdown, aqh;
};
struct S4TOut {
    double T, Fio, Fia, pen, fw;
};

__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }

// veris/solve4temp.py:5-174 for one point
__device__ S4TOut solve4temp_point(const VerisParams &p, const S4TIn &x) {
    const double aa1 = 2663.5, aa2 = 12.537, bb1 = 0.622;
    const double Pa = 100000.0;
    const double one_m_bb1 = 1.0 - bb1;
    const double cc1 = p.s4t_cc1, cc2 = p.s4t_cc2, d1 = p.s4t_d1, d1i = p.s4t_d1i;
    const double Tmelt = p.celsius2K;
    const double SurfMeltTemp = Tmelt + p.wetAlbTemp;
    double T = x.Tin;
    const double lwc = dmax(p.minLWdown, x.LWdown);
    const double Ta = dmax(p.celsius2K + p.minTAir, x.ATemp);
    const double ug = dmax(p.wSpeedMin, x.wSpeed);
    const bool ice = x.hI > 0, snow = x.hS > 0;
    const double emiss = snow ? p.snowEmiss : p.iceEmiss;
    const double d3 = emiss * p.stefBoltz;
    const double lw = emiss * lwc;

    double aI = ice ? p.dryIceAlb : 0.0;
    double aS = ice ? p.drySnowAlb : 0.0;
    const bool wet = ice && T >= SurfMeltTemp;
    if (wet) { aI = p.wetIceAlb; aS = p.wetSnowAlb; }
    const bool south = ice && x.fCori < 0;
    if (south) { aI = p.dryIceAlb_south; aS = p.drySnowAlb_south; }
    if (south && T >= SurfMeltTemp) { aI = p.wetIceAlb_south; aS = p.wetSnowAlb_south; }
    double alb = ice ? aI + x.hS / p.hCut * (aS - aI) : 0.0;
    if (x.hS > p.hCut) alb = aS;
    if (x.hS == 0) alb = aI;

    double pen = ice ? p.shortwave * exp(-1.5 * x.hI) : 0.0;
    if (snow) pen = 0.0;
    const double penSW = ice ? -(1 - alb) * pen * x.SWdown : 0.0;
    const double absSW = ice ? (1 - alb) * (1 - pen) * x.SWdown : 0.0;
    const double k = ice ? p.iceConduct * p.snowConduct / (p.snowConduct * x.hI + p.iceConduct * x.hS) : 0.0;

    double Fc, Flh, Fia, dF;
    auto fluxes = [&](double t1) {
        const double t2 = t1 * t1, t3 = t2 * t1, t4 = t2 * t2;
        const double svp = pow(10.0, -aa1 / t1 + aa2);
        const double qs = ice ? bb1 * svp / (Pa - one_m_bb1 * svp) : 0.0;
        const double c3 = pow(10.0, aa1 / t1);
        const double den = cc2 - c3 * Pa;
        const double dqs = ice ? cc1 * c3 / (den * den * t2) : 0.0;
        Fc = ice ? k * (x.TempFrz - t1) : 0.0;
        Flh = ice ? d1i * ug * (qs - x.aqh) : 0.0;
        const double Flw = ice ? t4 * d3 : 0.0;
        const double Fs = ice ? d1 * ug * (t1 - Ta) : 0.0;
        Fia = ice ? (-lw - absSW + Flw + Fs + Flh) : 0.0;
        dF = ice ? 4 * d3 * t3 + d1 * ug + d1i * ug * dqs : 0.0;
    };
    for (int it = 0; it < 6; ++it) {
        fluxes(T);
        T = ice ? T + (Fc - Fia) / (k + dF) : 0.0;
        T = dmin(T, Tmelt);
        T = dmax(T, p.celsius2K + p.minTIce);
    }
    fluxes(T);
    S4TOut o;
    const bool up = Fc > 0;
    o.T = ice ? T : x.Tin;
    o.Fio = up ? Fc : 0.0;
    o.Fia = up ? 0.0 : Fia;
    o.pen = penSW;
    o.fw = ice ? Flh / p.lhSublim : 0.0;
    return o;
}

// veris/solve4temp.py:5-174 for NC thickness categories of one cell at once.
// The categories differ only in their ice and snow thickness; their Newton
// iterations are independent, so they advance in lockstep and the float64
// dependency chains interleave.
// S is double, or a dual number when the adjoint needs the derivatives with
// respect to the ice state (branches follow the values either way).
// 1/x for a float64 x inside the float32 range (a temperature, or the
// saturation denominator c3 Pa - (1-bb1) cc0 ~ 1e15..1e17 here): the
// float32 reciprocal refined by two Newton-Raphson steps r <- r + r (1 - x r),
// relative error ~2^-23 -> ~2^-46 -> float64 rounding
__device__ __forceinline__ double recip_nr(double x) {
    double r = (double)__frcp_rn((float)x);
    r = fma(r, fma(-x, r, 1.0), r);
    r = fma(r, fma(-x, r, 1.0), r);
    return r;
}

template <int NC, class S>
__device__ void solve4temp_multi(const VerisParams &p, const S4TIn &x, const S &Tin, const S *hI, const S *hS,
                                 S *oT, S *oFio, S *oFia, S *oPen) {
    const double aa1 = 2663.5, bb1 = 0.622, Pa = 100000.0;
    const double one_m_bb1 = 1.0 - bb1;
    const double cc0 = p.s4t_cc0, cc1 = p.s4t_cc1, cc2 = p.s4t_cc2, d1 = p.s4t_d1, d1i = p.s4t_d1i;
    const double Tmelt = p.celsius2K, Tmin = p.celsius2K + p.minTIce;
    const double SurfMeltTemp = Tmelt + p.wetAlbTemp;
    const double lwc = dmax(p.minLWdown, x.LWdown);
    const double Ta = dmax(p.celsius2K + p.minTAir, x.ATemp);
    const double ug = dmax(p.wSpeedMin, x.wSpeed);
    const double d1ug = d1 * ug, d1iug = d1i * ug;
    S T[NC], k[NC], lwabs[NC];
    double d3[NC];
    bool ice[NC];
    // penetrating shortwave factor exp(-1.5 hI): the NC = 5 categories of one
    // cell have hI[l] = (2l+1) hI[0], so one exp and its odd powers serve all
    S e1[NC];
    if constexpr (NC == 5) {
        const S E = vexp(-1.5 * hI[0]), E2 = E * E;
        e1[0] = E;
#pragma unroll
        for (int l = 1; l < NC; ++l) e1[l] = e1[l - 1] * E2;
    } else {
#pragma unroll
        for (int l = 0; l < NC; ++l) e1[l] = vexp(-1.5 * hI[l]);
    }
    const double rhCut = 1.0 / p.hCut;
    // the categories scale ice and snow thickness alike (veris/growth.py:62-71):
    // with NC = 5, hI[l] = (2l+1) hI[0] and hS[l] = (2l+1) hS[0], so the
    // effective conductivity is k[0] / (2l+1): one division for the five
    S k0 = S(0.0);
    if constexpr (NC == 5)
        k0 = hI[0] > 0 ? p.iceConduct * p.snowConduct / (p.snowConduct * hI[0] + p.iceConduct * hS[0]) : S(0.0);
#pragma unroll
    for (int l = 0; l < NC; ++l) {
        ice[l] = hI[l] > 0;
        const bool snow = hS[l] > 0;
        const double emiss = snow ? p.snowEmiss : p.iceEmiss;
        d3[l] = emiss * p.stefBoltz;
        const double lw = emiss * lwc;
        double aI = ice[l] ? p.dryIceAlb : 0.0;
        double aS = ice[l] ? p.drySnowAlb : 0.0;
        if (ice[l] && Tin >= SurfMeltTemp) { aI = p.wetIceAlb; aS = p.wetSnowAlb; }
        const bool south = ice[l] && x.fCori < 0;
        if (south) { aI = p.dryIceAlb_south; aS = p.drySnowAlb_south; }
        if (south && Tin >= SurfMeltTemp) { aI = p.wetIceAlb_south; aS = p.wetSnowAlb_south; }
        S alb = ice[l] ? aI + hS[l] * rhCut * (aS - aI) : S(0.0);
        if (hS[l] > p.hCut) alb = S(aS);
        if (hS[l] == 0) alb = S(aI);
        S pen = ice[l] ? p.shortwave * e1[l] : S(0.0);
        if (snow) pen = S(0.0);
        oPen[l] = ice[l] ? -(1 - alb) * pen * x.SWdown : S(0.0);
        const S absSW = ice[l] ? (1 - alb) * (1 - pen) * x.SWdown : S(0.0);
        if constexpr (NC == 5) {
            constexpr double inv_odd[5] = {1.0, 1.0 / 3.0, 1.0 / 5.0, 1.0 / 7.0, 1.0 / 9.0};
            k[l] = ice[l] ? k0 * inv_odd[l] : S(0.0);
        } else {
            k[l] = ice[l] ? p.iceConduct * p.snowConduct / (p.snowConduct * hI[l] + p.iceConduct * hS[l]) : S(0.0);
        }
        lwabs[l] = -lw - absSW;
        T[l] = Tin;
    }
    if constexpr (!std::is_same<S, double>::value) {
        // Derivatives (dual numbers): implicit differentiation at the root.
        // The values come from the float64 solve itself (so every later
        // branch is taken as in the forward); at its root T* of
        // R(T) = Fc(T) - Fia(T), dT* = -R_theta / R_T with R_theta the
        // residual's derivative at fixed T (through the conductivity and
        // the absorbed radiation) and R_T = -(k + dFia/dT), the Newton
        // iteration's own denominator; a root held by the melt or the
        // minimum-temperature clamp has dT* = 0.  The converged Newton
        // iterates have this derivative (the Newton map's derivative in T
        // vanishes at the root), without iterating the dual numbers.
        double hIv[NC], hSv[NC], Tv[NC], Fiov[NC], Fiav[NC], Penv[NC];
#pragma unroll
        for (int l = 0; l < NC; ++l) {
            hIv[l] = val(hI[l]);
            hSv[l] = val(hS[l]);
        }
        solve4temp_multi<NC, double>(p, x, val(Tin), hIv, hSv, Tv, Fiov, Fiav, Penv);
        const double aa1l2 = aa1 * 3.32192809488736234787;
        const double qnum = bb1 * cc0, qsub = one_m_bb1 * cc0;
#pragma unroll
        for (int l = 0; l < NC; ++l) {
            if (!ice[l]) {
                oT[l] = Tin;
                oFio[l] = S(0.0);
                oFia[l] = S(0.0);
                continue;
            }
            const double t = Tv[l], t3 = t * t * t;
            const double rt = 1.0 / t, c3 = ::exp2(aa1l2 * rt);
            const double qs = qnum / (c3 * Pa - qsub), den = cc2 - c3 * Pa;
            const double dqs = cc1 * c3 * (rt * rt) / (den * den);
            const double FiaT = 4 * d3[l] * t3 + d1ug + d1iug * dqs;
            const S Fc = k[l] * (x.TempFrz - t);
            const S Fia = lwabs[l] + (t3 * t * d3[l] + d1ug * (t - Ta) + d1iug * (qs - x.aqh));
            const bool held = t >= Tmelt || t <= Tmin;
            S dT = Fc - Fia;   // its derivative part: R_theta
            const double scale = held ? 0.0 : 1.0 / (val(k[l]) + FiaT);
            S T = Tin, Fo = Fc, Fa = Fia;
            T.v = t;
#pragma unroll
            for (int q = 0; q < (int)(sizeof(S::d) / sizeof(double)); ++q) {
                const double dTq = dT.d[q] * scale;
                T.d[q] = dTq;
                Fo.d[q] = Fc.d[q] - val(k[l]) * dTq;
                Fa.d[q] = Fia.d[q] + FiaT * dTq;
            }
            const bool up = Fiov[l] > 0;
            Fo.v = Fiov[l];
            Fa.v = Fiav[l];
            oT[l] = T;
            oFio[l] = up ? Fo : S(0.0);
            oFia[l] = up ? S(0.0) : Fa;
        }
        return;
    }
    S Fc[NC], Fia[NC];
    bool moving[NC];
#pragma unroll
    for (int l = 0; l < NC; ++l) moving[l] = ice[l];
    // One flux evaluation per category; with `newton` also the Newton update.
    // The residual (Fc - Fia) is evaluated in float64 with two divisions:
    // 10^(aa1/T) = 2^(aa1 log2(10) / T) and, since svp = cc0 / 10^(aa1/T),
    // qs = bb1 svp / (Pa - (1-bb1) svp) = bb1 cc0 / (10^(aa1/T) Pa - (1-bb1) cc0).
    // The Newton derivative only sets the convergence rate, not the root:
    // in float64 arithmetic it and the step use float32 reciprocals (the
    // iteration still converges to the float64 root); dual numbers keep the
    // exact step so that the adjoint differentiates a smooth map.  A
    // category stops once an update moves T by less than 4e-7 T.
    //
    // The final evaluation (float64 only) at a converged category's T, at
    // most 4e-7 T from the last Newton evaluation at t: Fc and the T^4 and
    // sensible terms are evaluated exactly; qs(T) = qs(t) + qs'(t) (T - t),
    // whose error qs'' (T - t)^2 / 2 ~ 3e-11 qs (d ln qs / dT = aa1 ln10 / T^2
    // ~ 0.08 / K) is far inside the parity of the fixed six iterations; this
    // drops the exp2 and the two divisions of that evaluation.
    const double aa1l2 = aa1 * 3.32192809488736234787;   // aa1 log2(10)
    const double qnum = bb1 * cc0, qsub = one_m_bb1 * cc0;
    double qsv[NC], dqsv[NC], tv[NC];
    bool conv[NC];
#pragma unroll
    for (int l = 0; l < NC; ++l) conv[l] = false;
    auto fluxes = [&](bool newton) {
#pragma unroll
        for (int l = 0; l < NC; ++l) {
            if (newton && !moving[l]) continue;
            const S t1 = T[l];
            const S t2 = t1 * t1, t3 = t2 * t1, t4 = t2 * t2;
            if constexpr (std::is_same<S, double>::value) {
                if (!newton && conv[l]) {
                    const double qs = qsv[l] + dqsv[l] * (t1 - tv[l]);
                    Fc[l] = k[l] * (x.TempFrz - t1);
                    Fia[l] = lwabs[l] + t4 * d3[l] + d1ug * (t1 - Ta) + d1iug * (qs - x.aqh);
                    continue;
                }
            }
            S rt, qs, c3;
            if constexpr (std::is_same<S, double>::value) {
                rt = recip_nr(t1);
                c3 = vexp2(aa1l2 * rt);
                qs = qnum * recip_nr(c3 * Pa - qsub);
            } else {
                rt = 1.0 / t1;
                c3 = vexp2(aa1l2 * rt);
                qs = qnum / (c3 * Pa - qsub);
            }
            Fc[l] = ice[l] ? k[l] * (x.TempFrz - t1) : S(0.0);
            const S Flh = ice[l] ? d1iug * (qs - x.aqh) : S(0.0);
            Fia[l] = ice[l] ? (lwabs[l] + t4 * d3[l] + d1ug * (t1 - Ta) + Flh) : S(0.0);
            if (newton) {
                const S den = cc2 - c3 * Pa;
                S Tn;
                if constexpr (std::is_same<S, double>::value) {
                    const float rden = __frcp_rn((float)den);
                    const double dqs = (double)((float)(cc1 * c3) * rden * rden * (float)(rt * rt));
                    const double dF = 4 * d3[l] * t3 + d1ug + d1iug * dqs;
                    Tn = ice[l] ? t1 + (Fc[l] - Fia[l]) * (double)__frcp_rn((float)(k[l] + dF)) : 0.0;
                    qsv[l] = qs;   // and d qs / dT = dqs, for the final evaluation
                    dqsv[l] = dqs;
                    tv[l] = t1;
                } else {
                    const S dqs = cc1 * c3 * (rt * rt) / (den * den);
                    const S dF = ice[l] ? 4 * d3[l] * t3 + d1ug + d1iug * dqs : S(0.0);
                    Tn = ice[l] ? t1 + (Fc[l] - Fia[l]) / (k[l] + dF) : S(0.0);
                }
                Tn = smin(Tn, S(Tmelt));
                Tn = smax(Tn, S(Tmin));
                // |update| <= 4e-7 T (about 1e-4 K): the error left is below
                // 1e-7 of the update (float32 derivative) plus C update^2 with
                // C = F''/2F' ~ 1e-3 / K (at most ~1e-2 / K with the latent
                // heat term), i.e. ~1e-10 K, 4e-13 of T: far inside the
                // float64 parity of the fixed six iterations
                if (vfabs(val(Tn) - val(t1)) <= 4e-7 * val(t1)) {
                    moving[l] = false;
                    conv[l] = ice[l];
                }
                T[l] = Tn;
            }
        }
    };
    if constexpr (std::is_same<S, double>::value) {
        // float32 Newton iterations bring T to ~1e-4 K of the root first; the
        // float64 iterations below then converge in one or two updates
        const float aa1l2f = (float)aa1l2, qnumf = (float)qnum, qsubf = (float)qsub, Paf = (float)Pa;
        const float cc1f = (float)cc1, cc2f = (float)cc2, TFf = (float)x.TempFrz, aqhf = (float)x.aqh;
        const float d1ugf = (float)d1ug, d1iugf = (float)d1iug, Taf = (float)Ta;
        const float Tmeltf = (float)Tmelt, Tminf = (float)Tmin;
#pragma unroll
        for (int l = 0; l < NC; ++l) {
            if (!ice[l]) continue;
            float t = (float)T[l];
            const float kf = (float)k[l], lwf = (float)lwabs[l], d3f = (float)d3[l];
            for (int it = 0; it < 3; ++it) {
                const float rt = __frcp_rn(t);
                const float t2 = t * t;
                const float c3 = exp2f(aa1l2f * rt);
                const float qs = __fdividef(qnumf, c3 * Paf - qsubf);
                const float den = __frcp_rn(cc2f - c3 * Paf);
                const float dqs = (cc1f * c3 * den) * den * (rt * rt);
                const float Fcf = kf * (TFf - t);
                const float Fiaf = lwf + t2 * t2 * d3f + d1ugf * (t - Taf) + d1iugf * (qs - aqhf);
                const float dF = 4.f * d3f * t2 * t + d1ugf + d1iugf * dqs;
                t = fminf(fmaxf(t + (Fcf - Fiaf) * __frcp_rn(kf + dF), Tminf), Tmeltf);
            }
            T[l] = (double)t;
        }
    }
    for (int it = 0; it < 6; ++it) {
        bool any = false;
#pragma unroll
        for (int l = 0; l < NC; ++l) any = any || moving[l];
        if (!any) break;
        fluxes(true);
    }
    fluxes(false);
#pragma unroll
    for (int l = 0; l < NC; ++l) {
        const bool up = Fc[l] > 0;
        oT[l] = ice[l] ? T[l] : Tin;
        oFio[l] = up ? Fc[l] : S(0.0);
        oFia[l] = up ? S(0.0) : Fia[l];
    }
}

template <class S>
struct GrowthOut {
    S h, hs, A, TSurf, EmPmR, forc_salt, Qsw, Qnet, load, pen, rh;
};

// step constants of Growth, formed once on the host (float64 divisions cost
// about ten fused multiply-adds each on GB300's float64 pipe)
struct GrowthK {
    double qi, qs;        // 1 / (rho lhFusion) of ice and snow
    double rqi, rqs;      // rho lhFusion of ice and snow
    double rf2s;          // 1 / rhoFresh2rhoSnow
};

static GrowthK growth_k(const VerisParams &p) {
    GrowthK k;
    k.qi = 1 / (p.rhoIce * p.lhFusion);
    k.qs = 1 / (p.rhoSnow * p.lhFusion);
    k.rqi = p.rhoIce * p.lhFusion;
    k.rqs = p.rhoSnow * p.lhFusion;
    k.rf2s = 1 / p.rhoFresh2rhoSnow;
    return k;
}

// veris/growth.py:8-397 for one point, from the ice state (h, hs, A, TSurf)
// and the forcing of point o
template <class S>
__device__ GrowthOut<S> growth_point(const VerisParams &p, const GrowthK &gk, const Fields<double> &f, int64_t o,
                                     S hIn, S hsIn, S AIn, S TSurfIn) {
    const double qi = gk.qi;
    const double qs = gk.qs;
    const bool noIce = hIn == 0 || AIn == 0;
    const double keep = noIce ? 0.0 : 1.0;
    const S h0 = hIn * keep, hs0 = hsIn * keep, A0 = AIn * keep;
    const bool isIce = h0 > 0;
    const S rregA = vrsqrt(A0 * A0 + p.Area_reg);
    S hIa = isIce ? h0 * rregA : S(0.0);
    const S rhIa = A0 * vrsqrt(h0 * h0 + p.hIce_reg);
    const S hSa = isIce ? hs0 * rregA : S(0.0);
    hIa = smax(hIa, S(0.05));

    const double ocSalt = __ldg(f.ocSalt + o);
    const double TempFrz = p.tempFrz + p.dtempFrz_dS * ocSalt + p.celsius2K;
    S4TIn x;
    x.Tin = val(TSurfIn);
    x.TempFrz = TempFrz;
    x.LWdown = __ldg(f.LWdown + o);
    x.ATemp = __ldg(f.ATemp + o);
    x.wSpeed = __ldg(f.wSpeed + o);
    x.fCori = __ldg(f.fCori + o);
    x.SWdown = __ldg(f.SWdown + o);
    x.aqh = __ldg(f.aqh + o);
    S Tsum = 0, Fio_sum = 0, Fia_sum = 0, pen_sum = 0;
    if (p.nITC == 5) {
        S hIc[5], hSc[5], rT[5], rFio[5], rFia[5], rPen[5];
#pragma unroll
        for (int l = 0; l < 5; ++l) {
            const double pFac = (double)(2 * (l + 1) - 1) * p.recip_nITC;
            hIc[l] = hIa * pFac;
            hSc[l] = hSa * pFac;
        }
        solve4temp_multi<5, S>(p, x, TSurfIn, hIc, hSc, rT, rFio, rFia, rPen);
#pragma unroll
        for (int l = 0; l < 5; ++l) {
            Tsum = Tsum + rT[l];
            Fio_sum = Fio_sum + rFio[l];
            Fia_sum = Fia_sum + rFia[l];
            pen_sum = pen_sum + rPen[l];
        }
    } else {
        for (int l = 0; l < p.nITC; ++l) {
            const double pFac = (double)(2 * (l + 1) - 1) * p.recip_nITC;
            S hIc[1] = {hIa * pFac}, hSc[1] = {hSa * pFac}, rT[1], rFio[1], rFia[1], rPen[1];
            solve4temp_multi<1, S>(p, x, TSurfIn, hIc, hSc, rT, rFio, rFia, rPen);
            Tsum = Tsum + rT[0];
            Fio_sum = Fio_sum + rFio[0];
            Fia_sum = Fia_sum + rFia[0];
            pen_sum = pen_sum + rPen[0];
        }
    }
    GrowthOut<S> g;
    g.TSurf = Tsum * p.recip_nITC;
    const S Fio = Fio_sum * p.recip_nITC * A0;
    S Fia = Fia_sum * p.recip_nITC * A0;
    const S pen = pen_sum * p.recip_nITC * A0;

    const double snowfall = __ldg(f.snowfall + o), precip = __ldg(f.precip + o);
    const bool cold = A0 > 0 && Tsum / (double)p.nITC < p.celsius2K;
    const double snowAcc = (cold ? snowfall + precip : snowfall) * p.rhoFresh2rhoSnow;
    const double rainToSea = cold ? 0.0 : precip;
    const S snowAccOverIce = snowAcc * A0 * p.deltatTherm;

    S gUnder = Fio * qi;
    if (A0 == 0) gUnder = S(0.0);
    const S potMeltRate = -Fia * qs;
    const S potMelt = potMeltRate * p.deltatTherm;
    const bool allMelt = potMelt >= hs0;
    const S meltRate = allMelt ? hs0 * p.recip_deltatTherm : potMeltRate;
    const S toSnow = allMelt ? -hs0 * p.recip_deltatTherm * gk.rqs : Fia;
    Fia = Fia - toSnow;
    const S gSurf = Fia * qi;
    const S gNet = (gUnder + gSurf) * rregA;

    const double t0 = 0.4, t1 = 7 / t0;
    const double t2 = p.stantonNr * p.uStarBase * p.rhoSea * p.cpWater;
    const double sst = dmax(__ldg(f.theta + o), TempFrz);
    const S mltf = 1 + (p.McPheeTaperFac - 1) / (1 + vexp((A0 - t0) * t1));
    const S gML = -t2 * (sst - TempFrz) * mltf * qi;
    const double Qnet_in = __ldg(f.Qnet + o);
    const double gOW = qi * Qnet_in;

    const S dh = gNet * A0 + gOW * (1 - A0) + gML;
    const S dhs = (snowAcc - meltRate) * A0;
    const S half_rh = 0.5 * rhIa;
    S dA_oa = half_rh * gOW * (1 - A0);
    const bool grow = gOW > 0 && (A0 > 0 || dh > 0);
    if (grow) dA_oa = gOW * (1 - A0);
    const double fC = __ldg(f.fCori + o);
    dA_oa = (grow && fC < 0) ? dA_oa * p.recip_h0_south : dA_oa * p.recip_h0;
    const S dA_oi = gML <= 0 ? half_rh * gML : S(0.0);
    const S dA_ia = (gNet <= 0 && h0 > 0) ? half_rh * gNet * A0 : S(0.0);
    const S dA = dA_oa + dA_oi + dA_ia;

    const double mask = __ldg(f.iceMask + o);
    S A = A0 + dA * mask * p.deltatTherm;
    S h = h0 + dh * mask * p.deltatTherm;
    S hs = hs0 + dhs * mask * p.deltatTherm;
    A = smin(smax(A, S(0.0)), S(1.0));
    h = smax(h, S(0.0));
    hs = smax(hs, S(0.0));
    const double alive = (h == 0 || A == 0) ? 0.0 : 1.0;
    A = A * alive;
    hs = hs * alive;
    h = h * alive;
    const S hsub = (hs * p.rhoSnow + h * p.rhoIce) * p.recip_rhoSea;
    const S flood = smax(S(0.0), hsub - h);
    h = h + flood;
    hs = hs - flood * p.rhoIce2rhoSnow;
    g.rh = vrsqrt(h * h + p.hIce_reg);
    g.h = h;
    g.hs = hs;
    g.A = A;

    g.Qsw = pen * A0 + __ldg(f.Qsw + o) * (1 - A0);
    const S dH = h - h0;
    const S melted = hs0 + snowAccOverIce - hs;
    const S E_ice = dH * gk.rqi;
    const S E_out = (A0 * (Fia + Fio + pen) + (1 - A0) * Qnet_in) * p.deltatTherm;
    g.Qnet = (E_out - E_ice) * p.recip_deltatTherm;
    const double sal_fac = (ocSalt > 0 && ocSalt > p.saltIce_ref) ? (1 - p.saltIce_ref / ocSalt) : 1.0;
    const S fw_ice = -dH * p.rhoIce2rhoFresh * sal_fac;
    const double salt_ref = dmin(p.saltIce_ref, ocSalt);
    const double osh = __ldg(f.os_hIceMean + o), oshs = __ldg(f.os_hSnowMean + o);
    const S saltflux = (dH + osh) * salt_ref * mask * p.rhoIce * p.recip_deltatTherm;
    const S fw_snow = melted * gk.rf2s;
    g.EmPmR = mask * ((-__ldg(f.evap + o) - precip) * (1 - A0) - rainToSea * A0 - __ldg(f.runoff + o) -
                      (fw_ice + fw_snow) * p.recip_deltatTherm) * p.rhoFresh +
              mask * (osh * p.rhoIce + oshs * p.rhoSnow) * p.recip_deltatTherm;
    g.forc_salt = g.EmPmR * ocSalt * p.recip_rhoFresh + saltflux;
    g.load = h * p.rhoIce + hs * p.rhoSnow;
    g.pen = pen;
    return g;
}

__global__ void solve4temp_kernel(VerisParams p, Fields<double> f, Dims d, const double *hI, const double *hS,
                                  const double *Tin, const double *TF, double *To, double *Fio, double *Fia,
                                  double *pen, double *fw) {
    const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 8 + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const int64_t o = d.raw(i, j);
    S4TIn x;
    x.hI = hI[o];
    x.hS = hS[o];
    x.Tin = Tin[o];
    x.TempFrz = TF[o];
    x.LWdown = __ldg(f.LWdown + o);
    x.ATemp = __ldg(f.ATemp + o);
    x.wSpeed = __ldg(f.wSpeed + o);
    x.fCori = __ldg(f.fCori + o);
    x.SWdown = __ldg(f.SWdown + o);
    x.aqh = __ldg(f.aqh + o);
    const S4TOut r = solve4temp_point(p, x);
    To[o] = r.T;
    Fio[o] = r.Fio;
    Fia[o] = r.Fia;
    pen[o] = r.pen;
    fw[o] = r.fw;
}

struct GrowthPtrs {
    double *h, *hs, *A, *TSurf, *EmPmR, *forc_salt, *Qsw, *Qnet, *load, *pen, *rh;
};

// rows [i0, i1) of the padded array (Growth is pointwise)
__global__ void __launch_bounds__(128) growth_kernel(VerisParams p, GrowthK gk, Fields<double> f, Dims d,
                                                     GrowthPtrs out, int i0, int i1) {
    const int j = blockIdx.x * 32 + threadIdx.x, i = i0 + blockIdx.y * 4 + threadIdx.y;
    if (i >= i1 || j >= d.NY) return;
    const int64_t o = d.raw(i, j);
    const GrowthOut<double> g = growth_point<double>(p, gk, f, o, __ldg(f.hIceMean + o), __ldg(f.hSnowMean + o),
                                                     __ldg(f.Area + o), __ldg(f.TSurf + o));
    out.h[o] = g.h;
    out.hs[o] = g.hs;
    out.A[o] = g.A;
    out.TSurf[o] = g.TSurf;
    out.EmPmR[o] = g.EmPmR;
    out.forc_salt[o] = g.forc_salt;
    out.Qsw[o] = g.Qsw;
    out.Qnet[o] = g.Qnet;
    out.load[o] = g.load;
    out.pen[o] = g.pen;
    out.rh[o] = g.rh;
}

// adjoint of growth for the ice state: l_in = J^T l_out over (h, hs, A, TSurf)
__global__ void __launch_bounds__(128) growth_adjoint_kernel(VerisParams p, GrowthK gk, Fields<double> f, Dims d,
                                                             const double *lh, const double *lhs, const double *lA,
                                                             const double *lT, double *oh, double *ohs, double *oA,
                                                             double *oT) {
    const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 4 + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const int64_t o = d.raw(i, j);
    using D = Dual<4>;
    const GrowthOut<D> g = growth_point<D>(p, gk, f, o, D::var(f.hIceMean[o], 0), D::var(f.hSnowMean[o], 1),
                                           D::var(f.Area[o], 2), D::var(f.TSurf[o], 3));
    const double l0 = lh[o], l1 = lhs[o], l2 = lA[o], l3 = lT[o];
    double r[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) r[k] = l0 * g.h.d[k] + l1 * g.hs.d[k] + l2 * g.A.d[k] + l3 * g.TSurf.d[k];
    oh[o] = r[0];
    ohs[o] = r[1];
    oA[o] = r[2];
    oT[o] = r[3];
}

}  // namespace veris

using namespace veris;

extern "C" {

int veris_solve4temp_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                         const double *hI, const double *hS, const double *Tin, const double *TF, double *To,
                         double *Fio, double *Fia, double *pen, double *fw, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && hI && hS && Tin && TF && To && Fio && Fia && pen && fw, VERIS_ERR_ARG);
    dim3 gr((d.NY + 31) / 32, (d.NX + 7) / 8);
    solve4temp_kernel<<<gr, dim3(32, 8), 0, (cudaStream_t)s>>>(
        *p, *reinterpret_cast<const Fields<double> *>(vs), d, hI, hS, Tin, TF, To, Fio, Fia, pen, fw);
    return launch_status();
}

int veris_growth_adjoint_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, const double *lh,
                             const double *lhs, const double *lA, const double *lT, double *oh, double *ohs,
                             double *oA, double *oT, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && lh && lhs && lA && lT && oh && ohs && oA && oT, VERIS_ERR_ARG);
    VERIS_REQUIRE(p->nITC >= 1 && p->nITC <= 64, VERIS_ERR_ARG);
    dim3 gr((d.NY + 31) / 32, (d.NX + 3) / 4);
    growth_adjoint_kernel<<<gr, dim3(32, 4), 0, (cudaStream_t)s>>>(*p, growth_k(*p), *reinterpret_cast<const Fields<double> *>(vs),
                                                                   d, lh, lhs, lA, lT, oh, ohs, oA, oT);
    return launch_status();
}

int veris_growth_rows_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, double *h,
                          double *hs, double *A, double *TSurf, double *EmPmR, double *forc_salt, double *Qsw,
                          double *Qnet, double *load, double *pen, double *rh, int32_t row_begin, int32_t row_end,
                          veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && h && hs && A && TSurf && EmPmR && forc_salt && Qsw && Qnet && load && pen && rh,
                  VERIS_ERR_ARG);
    VERIS_REQUIRE(p->nITC >= 1 && p->nITC <= 64, VERIS_ERR_ARG);
    VERIS_REQUIRE(row_begin >= 0 && row_begin < row_end && row_end <= d.NX, VERIS_ERR_ARG);
    GrowthPtrs out{h, hs, A, TSurf, EmPmR, forc_salt, Qsw, Qnet, load, pen, rh};
    dim3 gr((d.NY + 31) / 32, (row_end - row_begin + 3) / 4);
    growth_kernel<<<gr, dim3(32, 4), 0, (cudaStream_t)s>>>(*p, growth_k(*p), *reinterpret_cast<const Fields<double> *>(vs), d,
                                                            out, row_begin, row_end);
    return launch_status();
}

int veris_growth_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, double *h,
                     double *hs, double *A, double *TSurf, double *EmPmR, double *forc_salt, double *Qsw,
                     double *Qnet, double *load, double *pen, double *rh, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    return veris_growth_rows_f64(g, p, vs, h, hs, A, TSurf, EmPmR, forc_salt, Qsw, Qnet, load, pen, rh, 0, d.NX,
                                 s);
}

}  // extern "C"
