// One tile of one fast-form float32/float64 mEVP subcycle
// (veris/evp_solver.py:21-254) run from shared memory by one CTA: the tile's
// inputs plus a 2-cell ring are staged, then strain rates -> viscosities ->
// stresses -> drag -> velocities pass through shared memory with a barrier
// between stages.  Used by the single-domain shared-memory kernel and by the
// batched-ensemble kernel, so both compute bit-identical values.
#pragma once

#include "evp_fast.cuh"

namespace veris {

constexpr int FAST_THREADS = 256;

template <class T, int TI_, int TJ_>
struct TileSmem {
    static constexpr int TI = TI_, TJ = TJ_;
    static constexpr int WS = TJ + 4, HS = TI + 4, NS = WS * HS;   // staged inputs, origin -2
    static constexpr int WZ = TJ + 3, HZ = TI + 3, NZ = WZ * HZ;   // e12, origin -1
    static constexpr int WB = TJ + 2, HB = TI + 2, NB = WB * HB;   // zeta, origin -1
    static constexpr int WC = TJ + 1, HC = TI + 1, NC = WC * HC;   // C ring (origin -1) and Z (origin 0)
    static constexpr size_t bytes() {
        return sizeof(T) * (size_t)(4 * NS + 2 * NZ + NB + 6 * NC) + sizeof(uint32_t) * NS;
    }
};

// d: the domain's grid (wrap extents); internal arrays use pitch lp; the
// tile's origin is (i0, j0); every thread of the CTA (FAST_THREADS) calls it
template <class T, int TI, int TJ, bool BASAL, bool TURN>
__device__ __forceinline__ void fast_tile(unsigned char *smem_raw, const Dims &d, int64_t lp, const HaloFill &h,
                                          const FastConsts<T> &c, const FastScalars<T> &k, const FastIO<T> &io,
                                          int i0, int j0) {
    using S = TileSmem<T, TI, TJ>;
    T *sU = reinterpret_cast<T *>(smem_raw);
    T *sV = sU + S::NS;
    T *sUo = sV + S::NS;
    T *sVo = sUo + S::NS;
    T *sE12 = sVo + S::NS;
    T *sZq = sE12 + S::NZ;       // stage A/B only; reused for sigma12 in C/D
    T *sZeta = sZq + S::NZ;
    T *sS11 = sZeta + S::NB;
    T *sS22 = sS11 + S::NC;
    T *sCd = sS22 + S::NC;
    T *sCb = sCd + S::NC;
    T *sFv = sCb + S::NC;
    T *sFu = sFv + S::NC;
    uint32_t *sF = reinterpret_cast<uint32_t *>(sFu + S::NC);
    T *sS12 = sZq;

    const int tid = threadIdx.x;
#define IS(li, lj) (((li) + 2) * S::WS + ((lj) + 2))
#define IZ(li, lj) (((li) + 1) * S::WZ + ((lj) + 1))
#define IB(li, lj) (((li) + 1) * S::WB + ((lj) + 1))
#define IC(li, lj) (((li) + 1) * S::WC + ((lj) + 1))
#define IZZ(li, lj) ((li) * S::WC + (lj))

    // ---- stage inputs (tile + 2-cell ring, periodic wrap over the padded array)
    for (int idx = tid; idx < S::NS; idx += FAST_THREADS) {
        const int li = idx / S::WS - 2, lj = idx % S::WS - 2;
        const int64_t o = (int64_t)d.wxt(i0 + li) * lp + d.wyt(j0 + lj);
        sU[idx] = __ldg(io.u + o);
        sV[idx] = __ldg(io.v + o);
        sUo[idx] = __ldg(c.uOc + o);
        sVo[idx] = __ldg(c.vOc + o);
        sF[idx] = __ldg(c.flags + o);
    }
    __syncthreads();

    // ---- A: e12 at Z points [-1, TI+1] x [-1, TJ+1]
    for (int idx = tid; idx < S::NZ; idx += FAST_THREADS) {
        const int li = idx / S::WZ - 1, lj = idx % S::WZ - 1;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const uint32_t f0 = sF[IS(li, lj)], fw = sF[IS(li - 1, lj)], fs = sF[IS(li, lj - 1)],
                       fws = sF[IS(li - 1, lj - 1)];
        const T mzh = (f0 & fw & fs & fws & F_MC) ? T(0.5) : T(0);
        const T hU = one_if<T>(f0, F_MU) - one_if<T>(fs, F_MU);
        const T hV = one_if<T>(f0, F_MV) - one_if<T>(fw, F_MV);
        const T u0 = sU[IS(li, lj)], us = sU[IS(li, lj - 1)];
        const T v0 = sV[IS(li, lj)], vw = sV[IS(li - 1, lj)];
        const T e = __ldg(c.rdyU_y + gj) * (mzh * (u0 - us) + hU * (u0 + us)) +
                    __ldg(c.rdxV_x + gi) * (mzh * (v0 - vw) + hV * (v0 + vw));
        sE12[idx] = e;
        sZq[idx] = __ldg(c.rAz + (int64_t)gi * lp + gj) * (e * e);
    }
    __syncthreads();

    // ---- B: viscosities at C [-1, TI] x [-1, TJ]; stresses, drag, Coriolis on [-1, TI) x [-1, TJ)
    for (int idx = tid; idx < S::NB; idx += FAST_THREADS) {
        const int li = idx / S::WB - 1, lj = idx % S::WB - 1;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const int64_t o = (int64_t)gi * lp + gj;
        const uint32_t f0 = sF[IS(li, lj)];
        const T mInC = one_if<T>(f0, F_INC);
        const T u0 = sU[IS(li, lj)], ue = sU[IS(li + 1, lj)];
        const T v0 = sV[IS(li, lj)], vn = sV[IS(li, lj + 1)];
        const T e11 = (ue - u0) * __ldg(c.rdxU_x + gi) * mInC;
        const T e22 = (vn - v0) * __ldg(c.rdyV_y + gj) * mInC;
        const T e12c = __ldg(c.qrA + o) *
                       ((sZq[IZ(li, lj)] + sZq[IZ(li + 1, lj)]) + (sZq[IZ(li, lj + 1)] + sZq[IZ(li + 1, lj + 1)]));
        const T ep = e11 + e22, em = e11 - e22;
        const T delta = sqrt(ep * ep + k.rsq * (em * em + T(4) * e12c));
        const T zeta = __ldg(c.Ph + o) / (delta + k.deltaMin);
        sZeta[idx] = zeta;
        if (li < TI && lj < TJ) {
            const int q = IC(li, lj);
            const T mC = one_if<T>(f0, F_MC);
            const T press = k.kp * zeta * delta;
            const T s1 = (__ldg(io.s1 + o) * k.alpha_m1 + (T(2) * zeta * ep - press)) * k.ralpha * mC;
            const T s2 = (__ldg(io.s2 + o) * k.alpha_m1 + T(0.5) * zeta * em) * k.ralpha * mC;
            sS11[q] = T(0.5) * (s1 + s2) * __ldg(c.dyV_y + gj);
            sS22[q] = T(0.5) * (s1 - s2) * __ldg(c.dxU_x + gi);
            if (li >= 0 && lj >= 0 && i0 + li < d.NX && j0 + lj < d.NY) {
                const int64_t w = (int64_t)gi * io.ldo + gj;
                io.s1o[w] = s1;
                io.s2o[w] = s2;
            }
            // ocean drag at C
            const uint32_t fe = sF[IS(li + 1, lj)], fn = sF[IS(li, lj + 1)];
            const T du0 = (u0 - sUo[IS(li, lj)]) * one_if<T>(f0, F_INU);
            const T du1 = (ue - sUo[IS(li + 1, lj)]) * one_if<T>(fe, F_INU);
            const T dv0 = (v0 - sVo[IS(li, lj)]) * one_if<T>(f0, F_INV);
            const T dv1 = (vn - sVo[IS(li, lj + 1)]) * one_if<T>(fn, F_INV);
            const T t = T(0.25) * ((du0 + du1) * (du0 + du1) + (dv0 + dv1) * (dv0 + dv1));
            const bool south = f0 & F_SOUTH;
            const T dc = south ? k.dS : k.dN, dc2 = south ? k.dS2 : k.dN2;
            sCd[q] = ((dc2 * t > k.cmin2) ? dc * sqrt(t) : k.cmin) * mC;
            if (BASAL) {
                const T a = u0 * one_if<T>(f0, F_INU), b = ue * one_if<T>(fe, F_INU);
                const T cc = v0 * one_if<T>(f0, F_INV), e = vn * one_if<T>(fn, F_INV);
                const T s = T(0.25) * (a * a + b * b + cc * cc + e * e);
                sCb[q] = __ldg(c.bfac + o) / sqrt(s + k.U02);
            }
            const T mf = __ldg(c.mfC + o);
            sFv[q] = mf * (v0 + vn);
            sFu[q] = mf * (u0 + ue);
        }
    }
    __syncthreads();

    // ---- C: sigma12 at Z [0, TI] x [0, TJ] (sZq is dead: reuse it)
    for (int idx = tid; idx < S::NC; idx += FAST_THREADS) {
        const int li = idx / S::WC, lj = idx % S::WC;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const int n = ((sF[IS(li, lj)] & F_MC) ? 1 : 0) + ((sF[IS(li - 1, lj)] & F_MC) ? 1 : 0) +
                      ((sF[IS(li, lj - 1)] & F_MC) ? 1 : 0) + ((sF[IS(li - 1, lj - 1)] & F_MC) ? 1 : 0);
        const T norm = n == 0 ? T(0) : (n == 1 ? T(1) : (n == 2 ? T(0.5) : (n == 3 ? T(1) / T(3) : T(0.25))));
        const T zz = norm * ((sZeta[IB(li, lj)] + sZeta[IB(li - 1, lj)]) +
                             (sZeta[IB(li, lj - 1)] + sZeta[IB(li - 1, lj - 1)]));
        const T s12 = (__ldg(io.s12 + (int64_t)gi * lp + gj) * k.alpha_m1 + T(0.5) * zz * sE12[IZ(li, lj)]) * k.ralpha;
        sS12[idx] = s12;
        if (li < TI && lj < TJ && i0 + li < d.NX && j0 + lj < d.NY) io.s12o[(int64_t)gi * io.ldo + gj] = s12;
    }
    __syncthreads();

    // ---- D: u, v at the tile's U and V points
    for (int idx = tid; idx < TI * TJ; idx += FAST_THREADS) {
        const int li = idx / TJ, lj = idx % TJ;
        const int gi = i0 + li, gj = j0 + lj;
        if (gi >= d.NX || gj >= d.NY) continue;
        const int64_t o = (int64_t)gi * lp + gj;
        const uint32_t f0 = sF[IS(li, lj)];
        const T u0 = sU[IS(li, lj)], v0 = sV[IS(li, lj)];
        const T cd0 = sCd[IC(li, lj)], cdw = sCd[IC(li - 1, lj)], cds = sCd[IC(li, lj - 1)];
        const T sdxv = __ldg(c.dxV_x + gi), sdyu = __ldg(c.dyU_y + gj);
        {   // U point
            const T AW = __ldg(c.AW + o), mU = __ldg(c.mU + o);
            const T kU = k.halfCos * AW * (cd0 + cdw);
            T fx = __ldg(c.cU + o) + kU * sUo[IS(li, lj)] + T(0.5) * (sFv[IC(li, lj)] + sFv[IC(li - 1, lj)]);
            if (TURN) {
                const T sg = (f0 & F_SPOS) ? T(1) : ((f0 & F_SNEG) ? T(-1) : T(0));
                const T du0 = sUo[IS(li, lj)] - u0, dun = sUo[IS(li, lj + 1)] - sU[IS(li, lj + 1)];
                const T duw = sUo[IS(li - 1, lj)] - sU[IS(li - 1, lj)];
                const T duwn = sUo[IS(li - 1, lj + 1)] - sU[IS(li - 1, lj + 1)];
                fx -= sg * k.sinW * T(0.5) * (cd0 * T(0.5) * (du0 + dun) + cdw * T(0.5) * (duw + duwn)) *
                      one_if<T>(f0, F_LMU) * AW;
            }
            const T sdx = __ldg(c.rrAu + o) *
                          ((sS11[IC(li, lj)] - sS11[IC(li - 1, lj)]) + sdxv * (sS12[IZZ(li, lj + 1)] - sS12[IZZ(li, lj)]));
            T den = mU * k.bU1 + kU;
            if (BASAL) den += T(0.5) * AW * (sCb[IC(li, lj)] + sCb[IC(li - 1, lj)]);
            den = den == T(0) ? T(1) : den;
            const T un = one_if<T>(f0, F_MU) * (k.bU * mU * u0 + fx + sdx) / den;
            store_filled_ld(io.uo, io.ldo, d, h, gi, gj, un);
        }
        {   // V point
            const T AS = __ldg(c.AS + o), mV = __ldg(c.mV + o);
            const T kV = k.halfCos * AS * (cd0 + cds);
            T fy = __ldg(c.cV + o) + kV * sVo[IS(li, lj)] - T(0.5) * (sFu[IC(li, lj)] + sFu[IC(li, lj - 1)]);
            if (TURN) {
                const T sg = (f0 & F_SPOS) ? T(1) : ((f0 & F_SNEG) ? T(-1) : T(0));
                const T dv0 = sVo[IS(li, lj)] - v0, dve = sVo[IS(li + 1, lj)] - sV[IS(li + 1, lj)];
                const T dvs = sVo[IS(li, lj - 1)] - sV[IS(li, lj - 1)];
                const T dvse = sVo[IS(li + 1, lj - 1)] - sV[IS(li + 1, lj - 1)];
                fy += sg * k.sinW * T(0.5) * (cd0 * T(0.5) * (dv0 + dve) + cds * T(0.5) * (dvs + dvse)) *
                      one_if<T>(f0, F_LMV) * AS;
            }
            const T sdy = __ldg(c.rrAv + o) *
                          ((sS22[IC(li, lj)] - sS22[IC(li, lj - 1)]) + sdyu * (sS12[IZZ(li + 1, lj)] - sS12[IZZ(li, lj)]));
            T den = mV * k.bU1 + kV;
            if (BASAL) den += T(0.5) * AS * (sCb[IC(li, lj)] + sCb[IC(li, lj - 1)]);
            den = den == T(0) ? T(1) : den;
            const T vn = one_if<T>(f0, F_MV) * (k.bU * mV * v0 + fy + sdy) / den;
            store_filled_ld(io.vo, io.ldo, d, h, gi, gj, vn);
        }
    }
#undef IS
#undef IZ
#undef IB
#undef IC
#undef IZZ
}

}  // namespace veris
