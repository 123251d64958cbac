// Register-walking float32 mEVP subcycle, the walk itself
// (veris/evp_solver.py:21-254: the fast form's arithmetic with the TMA
// kernel's approximate square root and division).
//
// One warp owns a strip of 28 output columns (lanes = columns j0-2 .. j0+29,
// i.e. the strip plus a 2-cell ring) and walks down H output rows plus a
// 2-row ring at each end.  At walk step t it has row t's inputs and runs, on
// the rows the stencil chain has completed,
//
//   A  e12 at the Z points of row t            (rows t, t-1)
//   B  viscosities, sigma1/2, drag, Coriolis    at the C points of row t-1
//   C  sigma12 at the Z points of row t-1      (rows t-1, t-2)
//   D  u and v at the U/V points of row t-2     (rows t-1 .. t-3)
//
// Neighbours along a row come from warp shuffles, neighbours across rows from
// the registers of the previous steps: no shared memory and no barrier.  The
// next row's inputs are loaded one step ahead.  Warps are independent; a CTA
// is just a group of them.
//
// The inputs come in 16-byte groups built by the fast form's preparation:
// (uOc, vOc, mfC, Ph) per point, (cU, cV, AW, AS) and the U/V masses per U/V
// point, the four row metrics per row, a 16-bit copy of the flag word, and
// (with PIN) the state itself as (u, v, sigma1, sigma2).  The walk is bound
// by its load/store instruction count and DRAM bytes, which these groups cut;
// shuffles and arithmetic do not bind.
#pragma once

#include "evp_fast.cuh"

namespace veris {
namespace walk {

constexpr int TW = 28;      // output columns per strip

__device__ __forceinline__ float up(float x) { return __shfl_up_sync(0xffffffffu, x, 1); }     // lane - 1
__device__ __forceinline__ float dn(float x) { return __shfl_down_sync(0xffffffffu, x, 1); }   // lane + 1
__device__ __forceinline__ uint32_t upu(uint32_t x) { return __shfl_up_sync(0xffffffffu, x, 1); }
__device__ __forceinline__ uint32_t dnu(uint32_t x) { return __shfl_down_sync(0xffffffffu, x, 1); }

__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// the ring inputs of one staged row (one column per lane)
struct Row {
    float u, v, s1, s2, s12, uo, vo, mf, ph, qr, rz, bf, ac;
    uint32_t f;
    float rdxV, rdxU, dxU, dxV;   // metrics of the row
};

// PIN: the state is the walk's four-value layout, io.u holding (u, v, sigma1, sigma2)
// A1D: the cell areas vary along j only (per-lane constants): qr, rz are not loaded
// COH: the state was written by other warps of the same launch (the
// persistent walk): load it through L2, not the read-only path
template <bool COH, class T>
__device__ __forceinline__ T state_ld(const T *p) {
    if constexpr (COH) return __ldcg(p);
    else return __ldg(p);
}

template <bool BASAL, bool ADAPT = false, bool PIN = false, bool A1D = false, bool COH = false>
__device__ __forceinline__ void load_row(Row &r, const FastConsts<float> &c, const FastIO<float> &io, int64_t lp,
                                         int gi, int gj) {
    const int64_t o = (int64_t)gi * lp + gj;
    if (PIN) {
        const float4 q = state_ld<COH>(reinterpret_cast<const float4 *>(io.u) + o);
        r.u = q.x;
        r.v = q.y;
        r.s1 = q.z;
        r.s2 = q.w;
    } else {
        r.u = state_ld<COH>(io.u + o);
        r.v = state_ld<COH>(io.v + o);
        r.s1 = state_ld<COH>(io.s1 + o);
        r.s2 = state_ld<COH>(io.s2 + o);
    }
    r.s12 = state_ld<COH>(io.s12 + o);
    const float4 om = __ldg(reinterpret_cast<const float4 *>(c.q4O) + o);
    const float2 qz = A1D ? make_float2(0.f, 0.f) : __ldg(reinterpret_cast<const float2 *>(c.pQrRz) + o);
    r.uo = om.x;
    r.vo = om.y;
    r.mf = om.z;
    r.ph = om.w;
    r.qr = qz.x;
    r.rz = qz.y;
    r.bf = BASAL ? __ldg(c.bfac + o) : 0.f;
    r.ac = ADAPT ? __ldg(c.acf + o) : 0.f;
    r.f = __ldg(c.flags16 + o);
    const float4 m = __ldg(reinterpret_cast<const float4 *>(c.xm4) + gi);
    r.rdxV = m.x;
    r.rdxU = m.y;
    r.dxU = m.z;
    r.dxV = m.w;
}

// One walk: the strip of output columns j0 .. j0+27 and output rows
// i0 .. i0+H-1 of one subcycle, by the calling warp (all 32 lanes).
// PRE: load the own-point constants one walk step before stage D uses them.
// ADAPT: adaptive EVP (veris/evp_solver.py:65-73, 97-100, 148-150): alphaC
// from zeta at each C point, alphaZ and the U/V betas averaged from the
// alphaC of the neighbouring C points, carried across rows like zeta.
// PIN / POUT: the input / output state is the walk's own ping-pong layout,
// (u, v, sigma1, sigma2) in 16 bytes per point and sigma12 alone; with POUT
// a row's stresses wait one walk step in registers and are stored with its
// velocities.  A1D: the cell areas (0.25/rA, rAz, 1/rAu, 1/rAv) vary along j
// only and live in registers for the whole walk.  TAPE: Delta, zeta and the
// ocean-drag coefficient of every own C point go to io.tDel, io.tZeta,
// io.tCd (pitch io.ldo): a float32 tape's terms for the adjoint.
template <bool BASAL, bool TURN, int UNROLL, bool PRE = false, bool ADAPT = false, bool PIN = false,
          bool POUT = false, bool A1D = false, bool COH = false, bool TAPE = false>
__device__ __forceinline__ void walk_strip(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<float> &c,
                                           const FastScalars<float> &k, const FastIO<float> &io, int i0, int j0,
                                           int H, int lane) {
    const int jl = j0 - 2 + lane;   // this lane's column (may lie outside [0, NY): wraps)
    const int gj = d.wya(jl);
    const float rdyU = __ldg(c.rdyU_y + gj), rdyV = __ldg(c.rdyV_y + gj);
    const float dyV = __ldg(c.dyV_y + gj), dyU = __ldg(c.dyU_y + gj);
    float qr_j = 0.f, rz_j = 0.f, rrAu_j = 0.f, rrAv_j = 0.f;
    if (A1D) {
        qr_j = __ldg(c.qrA_y + gj);
        rz_j = __ldg(c.rAz_y + gj);
        rrAu_j = __ldg(c.rrAu_y + gj);
        rrAv_j = __ldg(c.rrAv_y + gj);
    }
    const bool own_j = lane >= 2 && lane < 2 + TW && jl < d.NY;
    const bool images = (h.x_fill && (i0 < 4 || i0 + H > d.NX - 4)) || (h.y_fill && (j0 < 4 || j0 + TW > d.NY - 4));
    const int64_t ldo = io.ldo;

    Row Pf, N, A, B, C;   // prefetched (t+1), current (t), and rows t-1, t-2, t-3
    A.f = B.f = C.f = 0u;
    A.u = A.v = A.uo = A.vo = B.u = B.v = B.uo = B.vo = C.u = C.uo = 0.f;
    // per-row results: e12/z2 of row t-1; B- and C-stage outputs of rows t-2 (a) and t-3 (b)
    float e12a = 0.f, z2a = 0.f, zeta_a = 0.f;
    float s11_a = 0.f, s11_b = 0.f, s22_a = 0.f;
    float cd_a = 0.f, cd_b = 0.f, cb_a = 0.f, cb_b = 0.f;
    float fv_a = 0.f, fv_b = 0.f, fu_a = 0.f, s12_a = 0.f;
    float aC_a = 0.f, aC_b = 0.f;   // adaptive alphaC of rows t-2, t-3
    float hs1 = 0.f, hs2 = 0.f;     // POUT: sigma1, sigma2 of the row stage D stores this step
    float o_cU = 0.f, o_cV = 0.f, o_AW = 0.f, o_AS = 0.f, o_mU = 0.f, o_mV = 0.f, o_rrAu = 0.f, o_rrAv = 0.f;
    // row indices advance by one per step: wrapped incrementally (any walk length)
    int gnext = d.wxa(i0 - 2);   // row of the next prefetch
    int gown = d.wxa(i0 - 4);    // row of this step's own-point constants (row t-2)
    load_row<BASAL, ADAPT, PIN, A1D, COH>(Pf, c, io, lp, gnext, gj);
    const int T = H + 4;   // rows i0-2 .. i0+H+1
    // UNROLL = 4 (the rotation period) would rename the row ages instead of
    // copying them; measured slower (register pressure), the kernels use 1
#pragma unroll UNROLL
    for (int t = 0; t < T; ++t) {
        N = Pf;
        gnext = gnext + 1 == d.NX ? 0 : gnext + 1;
        if (t + 1 < T) load_row<BASAL, ADAPT, PIN, A1D, COH>(Pf, c, io, lp, gnext, gj);
        // own-point constants of row t-2 (stage D)
        float cU = 0.f, cV = 0.f, AW = 0.f, AS = 0.f, mU = 0.f, mV = 0.f, rrAu = 0.f, rrAv = 0.f;
        if (PRE) {
            cU = o_cU; cV = o_cV; AW = o_AW; AS = o_AS; mU = o_mU; mV = o_mV; rrAu = o_rrAu; rrAv = o_rrAv;
            if (t >= 3) {   // row t-1, for the next step
                const int gn = gown + 1 == d.NX ? 0 : gown + 1;
                const int64_t on = (int64_t)gn * lp + gj;
                const float4 a = __ldg(reinterpret_cast<const float4 *>(c.q4U) + on);
                o_cU = a.x; o_cV = a.y; o_AW = a.z; o_AS = a.w;
                if (A1D) {
                    const float2 m = __ldg(reinterpret_cast<const float2 *>(c.pMUV) + on);
                    o_mU = m.x; o_mV = m.y; o_rrAu = rrAu_j; o_rrAv = rrAv_j;
                } else {
                    const float4 m = __ldg(reinterpret_cast<const float4 *>(c.q4M) + on);
                    o_mU = m.x; o_mV = m.y; o_rrAu = m.z; o_rrAv = m.w;
                }
            }
        } else if (t >= 4) {
            // the U/V-point constants: two 16-byte loads
            const int64_t ob = (int64_t)gown * lp + gj;
            const float4 a = __ldg(reinterpret_cast<const float4 *>(c.q4U) + ob);
            cU = a.x; cV = a.y; AW = a.z; AS = a.w;
            if (A1D) {
                const float2 m = __ldg(reinterpret_cast<const float2 *>(c.pMUV) + ob);
                mU = m.x; mV = m.y; rrAu = rrAu_j; rrAv = rrAv_j;
            } else {
                const float4 m = __ldg(reinterpret_cast<const float4 *>(c.q4M) + ob);
                mU = m.x; mV = m.y; rrAu = m.z; rrAv = m.w;
            }
        }

        // ---- A: e12 at Z points of row t
        const uint32_t fs = upu(N.f), fws = upu(A.f);
        const float mzh = (N.f & A.f & fs & fws & F_MC) ? 0.5f : 0.f;
        const float hU = one_if<float>(N.f, F_MU) - one_if<float>(fs, F_MU);
        const float hV = one_if<float>(N.f, F_MV) - one_if<float>(A.f, F_MV);
        const float us = up(N.u);
        const float e12n = rdyU * (mzh * (N.u - us) + hU * (N.u + us)) + N.rdxV * (mzh * (N.v - A.v) + hV * (N.v + A.v));
        const float z2n = (A1D ? rz_j : N.rz) * (e12n * e12n);

        float zeta_new = 0.f, s11_new = 0.f, s22_new = 0.f, cd_new = 0.f, cb_new = 0.f, fv_new = 0.f, fu_new = 0.f;
        float s12_new = 0.f, aC_new = 0.f, ns1 = 0.f, ns2 = 0.f;
        if (t >= 2) {
            // ---- B: C points of row t-1 (A holds its inputs, N the next row)
            const float mInC = one_if<float>(A.f, F_INC);
            const float vn = dn(A.v);
            const float e11 = (N.u - A.u) * A.rdxU * mInC;
            const float e22 = (vn - A.v) * rdyV * mInC;
            const float e12c = (A1D ? qr_j : A.qr) * ((z2a + z2n) + (dn(z2a) + dn(z2n)));
            const float ep = e11 + e22, em = e11 - e22;
            const float delta = sqrt_approx(ep * ep + k.rsq * (em * em + 4.f * e12c));
            const float zeta = __fdividef(A.ph, delta + k.deltaMin);
            zeta_new = zeta;
            const float mC = one_if<float>(A.f, F_MC);
            float am1 = k.alpha_m1, ral = k.ralpha;
            if (ADAPT) {
                const float aC = fmaxf(sqrt_approx(zeta * A.ac) * mC, k.aMin);
                aC_new = aC;
                am1 = aC - 1.f;
                ral = __fdividef(1.f, aC);
            }
            const float press = k.kp * zeta * delta;
            const float s1 = (A.s1 * am1 + (2.f * zeta * ep - press)) * ral * mC;
            const float s2 = (A.s2 * am1 + 0.5f * zeta * em) * ral * mC;
            ns1 = s1;
            ns2 = s2;
            s11_new = 0.5f * (s1 + s2) * dyV;
            s22_new = 0.5f * (s1 - s2) * A.dxU;
            const int oi = i0 + t - 3;
            if (own_j && t >= 3 && t <= H + 2 && oi < d.NX) {
                const int64_t wo = (int64_t)oi * ldo + jl;
                if (!POUT) {
                    io.s1o[wo] = s1;
                    io.s2o[wo] = s2;
                }
            }
            const uint32_t fe = N.f, fn = dnu(A.f);
            const float du0 = (A.u - A.uo) * one_if<float>(A.f, F_INU);
            const float du1 = (N.u - N.uo) * one_if<float>(fe, F_INU);
            const float dv0 = (A.v - A.vo) * one_if<float>(A.f, F_INV);
            const float dv1 = (vn - dn(A.vo)) * one_if<float>(fn, F_INV);
            const float tt = 0.25f * ((du0 + du1) * (du0 + du1) + (dv0 + dv1) * (dv0 + dv1));
            const bool south = A.f & F_SOUTH;
            const float dc = south ? k.dS : k.dN, dc2 = south ? k.dS2 : k.dN2;
            cd_new = ((dc2 * tt > k.cmin2) ? dc * sqrt_approx(tt) : k.cmin) * mC;
            if (TAPE && own_j && t >= 3 && t <= H + 2 && i0 + t - 3 < d.NX) {
                const int64_t wo = (int64_t)(i0 + t - 3) * ldo + jl;
                io.tDel[wo] = delta;
                io.tZeta[wo] = zeta;
                io.tCd[wo] = cd_new;
            }
            if (BASAL) {
                const float a = A.u * one_if<float>(A.f, F_INU), b = N.u * one_if<float>(fe, F_INU);
                const float cc = A.v * one_if<float>(A.f, F_INV), e = vn * one_if<float>(fn, F_INV);
                const float sq2 = 0.25f * (a * a + b * b + cc * cc + e * e);
                cb_new = __fdividef(A.bf, sqrt_approx(sq2 + k.U02));
            }
            fv_new = A.mf * (A.v + vn);
            fu_new = A.mf * (A.u + N.u);
        }
        if (t >= 3) {
            // ---- C: sigma12 at Z points of row t-1
            const uint32_t fa = A.f, fb = B.f, fas = upu(A.f), fbs = upu(B.f);
            const int n = ((fa & F_MC) ? 1 : 0) + ((fb & F_MC) ? 1 : 0) + ((fas & F_MC) ? 1 : 0) + ((fbs & F_MC) ? 1 : 0);
            const float norm = n == 0 ? 0.f : (n == 1 ? 1.f : (n == 2 ? 0.5f : (n == 3 ? 1.f / 3.f : 0.25f)));
            const float zz = norm * ((zeta_new + zeta_a) + (up(zeta_new) + up(zeta_a)));
            float am1 = k.alpha_m1, ral = k.ralpha;
            if (ADAPT) {
                const float aZ = 0.5f * (0.5f * (aC_new + up(aC_new)) + 0.5f * (aC_a + up(aC_a)));
                am1 = aZ - 1.f;
                ral = __fdividef(1.f, aZ);
            }
            s12_new = (A.s12 * am1 + 0.5f * zz * e12a) * ral;
            const int oi = i0 + t - 3;
            if (own_j && t <= H + 2 && oi < d.NX) io.s12o[(int64_t)oi * ldo + jl] = s12_new;
        }
        if (t >= 4) {
            // ---- D: u, v at the U/V points of row t-2 (B holds its inputs)
            const int oi = i0 + t - 4;
            const uint32_t f0 = B.f;
            float un, vnew;
            // beta/dt and (beta+1)/dt at the U and V points
            float bU = k.bU, bU1 = k.bU1, bV = k.bU, bV1 = k.bU1;
            if (ADAPT) {
                bU = 0.5f * (aC_a + aC_b) * k.rdt;
                bU1 = bU + k.rdt;
                bV = 0.5f * (aC_a + up(aC_a)) * k.rdt;
                bV1 = bV + k.rdt;
            }
            {   // U point
                const float kU = k.halfCos * AW * (cd_a + cd_b);
                float fx = cU + kU * B.uo + 0.5f * (fv_a + fv_b);
                if (TURN) {
                    const float sg = (f0 & F_SPOS) ? 1.f : ((f0 & F_SNEG) ? -1.f : 0.f);
                    const float du0 = B.uo - B.u, dun = dn(B.uo - B.u);
                    const float duw = C.uo - C.u, duwn = dn(C.uo - C.u);
                    fx -= sg * k.sinW * 0.5f * (cd_a * 0.5f * (du0 + dun) + cd_b * 0.5f * (duw + duwn)) *
                          one_if<float>(f0, F_LMU) * AW;
                }
                const float sdx = rrAu * ((s11_a - s11_b) + B.dxV * (dn(s12_a) - s12_a));
                float den = mU * bU1 + kU;
                if (BASAL) den += 0.5f * AW * (cb_a + cb_b);
                den = den == 0.f ? 1.f : den;
                un = one_if<float>(f0, F_MU) * __fdividef(bU * mU * B.u + fx + sdx, den);
            }
            {   // V point
                const float cds = up(cd_a);
                const float kV = k.halfCos * AS * (cd_a + cds);
                float fy = cV + kV * B.vo - 0.5f * (fu_a + up(fu_a));
                if (TURN) {
                    const float sg = (f0 & F_SPOS) ? 1.f : ((f0 & F_SNEG) ? -1.f : 0.f);
                    const float dv0 = B.vo - B.v, dve = A.vo - A.v;
                    const float dvs = up(B.vo - B.v), dvse = up(A.vo - A.v);
                    fy += sg * k.sinW * 0.5f * (cd_a * 0.5f * (dv0 + dve) + cds * 0.5f * (dvs + dvse)) *
                          one_if<float>(f0, F_LMV) * AS;
                }
                const float sdy = rrAv * ((s22_a - up(s22_a)) + dyU * (s12_new - s12_a));
                float den = mV * bV1 + kV;
                if (BASAL) den += 0.5f * AS * (cb_a + up(cb_a));
                den = den == 0.f ? 1.f : den;
                vnew = one_if<float>(f0, F_MV) * __fdividef(bV * mV * B.v + fy + sdy, den);
            }
            if (own_j && oi < d.NX) {
                if (images) {
                    if (POUT) {
                        store_filled_quad(reinterpret_cast<float4 *>(io.uo), ldo, d, h, oi, jl,
                                          make_float4(un, vnew, hs1, hs2));
                    } else {
                        store_filled_ld(io.uo, ldo, d, h, oi, jl, un);
                        store_filled_ld(io.vo, ldo, d, h, oi, jl, vnew);
                    }
                } else {
                    if (POUT) {
                        reinterpret_cast<float4 *>(io.uo)[(int64_t)oi * ldo + jl] = make_float4(un, vnew, hs1, hs2);
                    } else {
                        io.uo[(int64_t)oi * ldo + jl] = un;
                        io.vo[(int64_t)oi * ldo + jl] = vnew;
                    }
                }
            }
        }
        // ---- rotate: rows move one age back
        C = B;
        B = A;
        A = N;
        e12a = e12n;
        z2a = z2n;
        zeta_a = zeta_new;
        s11_b = s11_a;
        s11_a = s11_new;
        s22_a = s22_new;
        cd_b = cd_a;
        cd_a = cd_new;
        cb_b = cb_a;
        cb_a = cb_new;
        fv_b = fv_a;
        fv_a = fv_new;
        fu_a = fu_new;
        s12_a = s12_new;
        aC_b = aC_a;
        aC_a = aC_new;
        if (POUT) {
            hs1 = ns1;
            hs2 = ns2;
        }
        gown = gown + 1 == d.NX ? 0 : gown + 1;
    }
}

}  // namespace walk
}  // namespace veris
