// Adjoint of the mEVP subcycle loop (veris/evp_solver.py:21-319), fast form.
//
// Reverse-mode derivative of one subcycle
//   (u, v, sigma1, sigma2, sigma12) -> (u', v', sigma1', sigma2', sigma12')
// with the step constants folded as in the fast forward (evp_fast.cuh): given
// the adjoints of the outputs it adds the adjoints of the inputs, of the
// folded constants (ice-strength factor, Coriolis factor, masses, areas,
// u/dt + wind forcing, ocean velocities, basal factor) and of the two water
// drag coefficients.
//
// This file holds the driver of the sweep (checkpoints, segment recompute,
// tapes, the reverse loop, the fold back onto the fields) and the float32
// tile kernel below, which the sweep uses on float32 grids under 2^19
// padded cells; float64 and larger float32 grids take the gather passes of
// evp_adjoint_gather.cu.
//
// The tile kernel: one CTA per TI x TJ tile.  The CTA recomputes the forward intermediates it
// needs on the tile plus its ring (strain rates, e12, Delta, zeta, drag
// coefficients) from the subcycle's input state; it takes the output u', v'
// from the next state of the sweep.  It then propagates the adjoints of its
// own output points backwards stage by stage.  Every forward map is linear
// in its adjoint, so a tile may propagate the share of an intermediate's
// adjoint that its own outputs produce: shares of different tiles add up.
// Contributions to neighbouring points go to shared-memory accumulators
// (shared atomics), which are added to global memory with atomics at the end.
//
// Non-differentiable points take these subgradients: sqrt at Delta = 0 and at
// a drag argument of 0 give 0; the ocean-drag floor (cDragMin) and the
// "denominator = 0 -> 1" guard contribute nothing on their constant branch.
#include <atomic>

#include "evp_adjoint.cuh"

namespace veris {

namespace adj {

constexpr int TJ = 32, THREADS = 256;   // tile columns and threads; rows TI per instantiation

template <class T>
struct Io {
    const T *u, *v, *s1, *s2, *s12;     // state at the start of the subcycle (pitch lp)
    const T *un, *vn;                   // u', v' (pitch ldn)
    const T *lu, *lv, *ls1, *ls2, *ls12; // adjoints of the outputs (pitch ldl)
    T *ou, *ov, *os1, *os2, *os12;       // adjoints of the inputs, accumulated (pitch lp)
    int64_t ldn, ldl;
    int64_t sst = 1;   // element stride of u, v, un, vn: 1 planar, 4 in the register walk's (u, v, sigma1, sigma2) layout
};

// shared-memory regions (local coordinates, origin and size)
template <int R0, int C0, int H_, int W_>
struct Region {
    static constexpr int r0 = R0, c0 = C0, H = H_, W = W_;
    __host__ __device__ static constexpr int n() { return H * W; }
    __device__ static __forceinline__ int at(int li, int lj) { return (li - r0) * W + (lj - c0); }
};
// a TI x TJ tile's regions
template <int TI>
struct Geo {
    using RS = Region<-2, -2, TI + 4, TJ + 4>;   // staged inputs and the u/v adjoint accumulators
    using RZ = Region<-1, -1, TI + 3, TJ + 3>;   // e12 and its adjoint
    using RB = Region<-1, -1, TI + 2, TJ + 2>;   // zeta, Delta and the zeta adjoint
    using RC = Region<-1, -1, TI + 1, TJ + 1>;   // drag coefficients, C-point adjoints
    using RZ2 = Region<0, 0, TI + 1, TJ + 1>;    // sigma12' adjoint
};

template <class T, int TI>
struct Smem {
    using G = Geo<TI>;
    static constexpr int NT = 8 * G::RS::n() + 2 * G::RZ::n() + 3 * G::RB::n() + 8 * G::RC::n() + G::RZ2::n();
    static constexpr size_t bytes() { return sizeof(T) * (size_t)NT + sizeof(uint32_t) * G::RS::n(); }
};

__device__ __forceinline__ double atomic_add(double *a, double v) { return atomicAdd(a, v); }
__device__ __forceinline__ float atomic_add(float *a, float v) { return atomicAdd(a, v); }

template <class T, bool BASAL, bool TURN, int TI>
__global__ void __launch_bounds__(THREADS)
evp_adjoint_kernel(Dims d, int64_t lp, HaloFill h, FastConsts<T> c, FastScalars<T> k, Io<T> io, Adj<T> a,
                   T rhoSea) {
    using RS = typename Geo<TI>::RS;
    using RZ = typename Geo<TI>::RZ;
    using RB = typename Geo<TI>::RB;
    using RC = typename Geo<TI>::RC;
    using RZ2 = typename Geo<TI>::RZ2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *p = reinterpret_cast<T *>(smem_raw);
    T *sU = p; p += RS::n();
    T *sV = p; p += RS::n();
    T *sUo = p; p += RS::n();
    T *sVo = p; p += RS::n();
    T *lU = p; p += RS::n();     // adjoint accumulators of u, v, uOcean, vOcean
    T *lV = p; p += RS::n();
    T *lUo = p; p += RS::n();
    T *lVo = p; p += RS::n();
    T *sE12 = p; p += RZ::n();
    T *lE12 = p; p += RZ::n();
    T *sZeta = p; p += RB::n();
    T *sDel = p; p += RB::n();
    T *lZeta = p; p += RB::n();
    T *sCd = p; p += RC::n();
    T *sCb = p; p += RC::n();
    T *lS1 = p; p += RC::n();    // adjoints of sigma1', sigma2' (incl. sig11/sig22 shares)
    T *lS2 = p; p += RC::n();
    T *lCd = p; p += RC::n();
    T *lCb = p; p += RC::n();
    T *lFv = p; p += RC::n();
    T *lFu = p; p += RC::n();
    T *lS12 = p; p += RZ2::n();
    uint32_t *sF = reinterpret_cast<uint32_t *>(p);

    const int i0 = blockIdx.y * TI, j0 = blockIdx.x * TJ;
    const int tid = threadIdx.x;
    const T cosW2 = k.halfCos;

    // ---- stage inputs, clear accumulators
    for (int idx = tid; idx < RS::n(); idx += THREADS) {
        const int li = idx / RS::W + RS::r0, lj = idx % RS::W + RS::c0;
        const int64_t o = (int64_t)d.wxt(i0 + li) * lp + d.wyt(j0 + lj);
        sU[idx] = io.u[o * io.sst];
        sV[idx] = io.v[o * io.sst];
        sUo[idx] = c.uOc[o];
        sVo[idx] = c.vOc[o];
        sF[idx] = c.flags[o];
        lU[idx] = lV[idx] = lUo[idx] = lVo[idx] = T(0);
    }
    for (int idx = tid; idx < RZ::n(); idx += THREADS) lE12[idx] = T(0);
    for (int idx = tid; idx < RB::n(); idx += THREADS) lZeta[idx] = T(0);
    for (int idx = tid; idx < RC::n(); idx += THREADS)
        lS1[idx] = lS2[idx] = lCd[idx] = lCb[idx] = lFv[idx] = lFu[idx] = T(0);
    for (int idx = tid; idx < RZ2::n(); idx += THREADS) lS12[idx] = T(0);
    __syncthreads();

#define XS(li, lj) RS::at(li, lj)
    // ---- forward A: e12 at Z
    for (int idx = tid; idx < RZ::n(); idx += THREADS) {
        const int li = idx / RZ::W + RZ::r0, lj = idx % RZ::W + RZ::c0;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const uint32_t f0 = sF[XS(li, lj)], fw = sF[XS(li - 1, lj)], fs = sF[XS(li, lj - 1)],
                       fws = sF[XS(li - 1, lj - 1)];
        const T mzh = (f0 & fw & fs & fws & F_MC) ? T(0.5) : T(0);
        const T hU = one_if<T>(f0, F_MU) - one_if<T>(fs, F_MU);
        const T hV = one_if<T>(f0, F_MV) - one_if<T>(fw, F_MV);
        const T u0 = sU[XS(li, lj)], us = sU[XS(li, lj - 1)];
        const T v0 = sV[XS(li, lj)], vw = sV[XS(li - 1, lj)];
        sE12[idx] = c.rdyU_y[gj] * (mzh * (u0 - us) + hU * (u0 + us)) +
                    c.rdxV_x[gi] * (mzh * (v0 - vw) + hV * (v0 + vw));
    }
    __syncthreads();

    // ---- forward B: Delta, zeta at C [-1, TI] x [-1, TJ]; drag on [-1, TI) x [-1, TJ)
    for (int idx = tid; idx < RB::n(); idx += THREADS) {
        const int li = idx / RB::W + RB::r0, lj = idx % RB::W + RB::c0;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const int64_t o = (int64_t)gi * lp + gj;
        const uint32_t f0 = sF[XS(li, lj)];
        const T mInC = one_if<T>(f0, F_INC);
        const T u0 = sU[XS(li, lj)], ue = sU[XS(li + 1, lj)], v0 = sV[XS(li, lj)], vn = sV[XS(li, lj + 1)];
        const T e11 = (ue - u0) * c.rdxU_x[gi] * mInC;
        const T e22 = (vn - v0) * c.rdyV_y[gj] * mInC;
        auto zq = [&](int a_, int b_) {
            const T e = sE12[RZ::at(a_, b_)];
            return c.rAz[(int64_t)d.wxt(i0 + a_) * lp + d.wyt(j0 + b_)] * (e * e);
        };
        const T e12c = c.qrA[o] * ((zq(li, lj) + zq(li + 1, lj)) + (zq(li, lj + 1) + zq(li + 1, lj + 1)));
        const T ep = e11 + e22, em = e11 - e22;
        const T delta = sqrt(ep * ep + k.rsq * (em * em + T(4) * e12c));
        sDel[idx] = delta;
        sZeta[idx] = c.Ph[o] / (delta + k.deltaMin);
        if (li < TI && lj < TJ) {
            const int q = RC::at(li, lj);
            const uint32_t fe = sF[XS(li + 1, lj)], fn = sF[XS(li, lj + 1)];
            const T mC = one_if<T>(f0, F_MC);
            const T du0 = (u0 - sUo[XS(li, lj)]) * one_if<T>(f0, F_INU);
            const T du1 = (ue - sUo[XS(li + 1, lj)]) * one_if<T>(fe, F_INU);
            const T dv0 = (v0 - sVo[XS(li, lj)]) * one_if<T>(f0, F_INV);
            const T dv1 = (vn - sVo[XS(li, lj + 1)]) * one_if<T>(fn, F_INV);
            const T t = T(0.25) * ((du0 + du1) * (du0 + du1) + (dv0 + dv1) * (dv0 + dv1));
            const bool south = f0 & F_SOUTH;
            const T dc = south ? k.dS : k.dN, dc2 = south ? k.dS2 : k.dN2;
            sCd[q] = ((dc2 * t > k.cmin2) ? dc * sqrt(t) : k.cmin) * mC;
            if (BASAL) {
                const T a1 = u0 * one_if<T>(f0, F_INU), b1 = ue * one_if<T>(fe, F_INU);
                const T c1 = v0 * one_if<T>(f0, F_INV), e1 = vn * one_if<T>(fn, F_INV);
                const T s = T(0.25) * (a1 * a1 + b1 * b1 + c1 * c1 + e1 * e1);
                sCb[q] = c.bfac[o] / sqrt(s + k.U02);
            }
        }
    }
    __syncthreads();

    // ---- reverse D: own U and V points
    for (int idx = tid; idx < TI * TJ; idx += THREADS) {
        const int li = idx / TJ, lj = idx % TJ;
        const int gi = i0 + li, gj = j0 + lj;
        if (gi >= d.NX || gj >= d.NY) continue;
        const int64_t o = (int64_t)gi * lp + gj;
        const uint32_t f0 = sF[XS(li, lj)];
        // own C and Z output adjoints
        atomic_add(&lS1[RC::at(li, lj)], io.ls1[(int64_t)gi * io.ldl + gj]);
        atomic_add(&lS2[RC::at(li, lj)], io.ls2[(int64_t)gi * io.ldl + gj]);
        atomic_add(&lS12[RZ2::at(li, lj)], io.ls12[(int64_t)gi * io.ldl + gj]);
        // transpose of the halo-image stores: the adjoints of the images
        const bool hx = h.x_fill && in_xhalo(d, h.olx, gi);
        const bool hy = h.y_fill && in_yhalo(d, h.oly, gj);
        if (hx || hy) continue;   // this point's value is an image: no own update
        T lu = io.lu[(int64_t)gi * io.ldl + gj], lv = io.lv[(int64_t)gi * io.ldl + gj];
        {
            int ix[2] = {gi, -1}, jy[2] = {gj, -1};
            if (h.x_fill) {
                if (gi + d.nx < d.NX && in_xhalo(d, h.olx, gi + d.nx)) ix[1] = gi + d.nx;
                else if (gi - d.nx >= 0 && in_xhalo(d, h.olx, gi - d.nx)) ix[1] = gi - d.nx;
            }
            if (h.y_fill) {
                if (gj + d.ny < d.NY && in_yhalo(d, h.oly, gj + d.ny)) jy[1] = gj + d.ny;
                else if (gj - d.ny >= 0 && in_yhalo(d, h.oly, gj - d.ny)) jy[1] = gj - d.ny;
            }
            for (int aa = 0; aa < 2; ++aa)
                for (int bb = 0; bb < 2; ++bb) {
                    if ((aa == 0 && bb == 0) || ix[aa] < 0 || jy[bb] < 0) continue;
                    lu += io.lu[(int64_t)ix[aa] * io.ldl + jy[bb]];
                    lv += io.lv[(int64_t)ix[aa] * io.ldl + jy[bb]];
                }
        }
        const T u0 = sU[XS(li, lj)], v0 = sV[XS(li, lj)];
        const T cd0 = sCd[RC::at(li, lj)], cdw = sCd[RC::at(li - 1, lj)], cds = sCd[RC::at(li, lj - 1)];
        const T sg = (f0 & F_SPOS) ? T(1) : ((f0 & F_SNEG) ? T(-1) : T(0));
        {   // U point
            const T AW = c.AW[o], mU = c.mU[o];
            T den = mU * k.bU1 + cosW2 * AW * (cd0 + cdw);
            if (BASAL) den += T(0.5) * AW * (sCb[RC::at(li, lj)] + sCb[RC::at(li - 1, lj)]);
            const bool guard = den == T(0);   // replaced by 1: a constant branch
            if (guard) den = T(1);
            const T un = io.un[((int64_t)gi * io.ldn + gj) * io.sst];
            const T lN = one_if<T>(f0, F_MU) * lu / den;
            const T lden = guard ? T(0) : -un * lu / den;
            atomic_add(&lU[XS(li, lj)], k.bU * mU * lN);
            a.mU[o] += k.bU * u0 * lN + k.bU1 * lden;
            a.cU[o] += lN;
            const T uo = sUo[XS(li, lj)];
            atomic_add(&lUo[XS(li, lj)], cosW2 * AW * (cd0 + cdw) * lN);
            T lAW = cosW2 * (cd0 + cdw) * uo * lN + cosW2 * (cd0 + cdw) * lden;
            const T lcd = cosW2 * AW * uo * lN + cosW2 * AW * lden;
            T lcd0 = lcd, lcdw = lcd;
            if (BASAL) {
                lAW += T(0.5) * (sCb[RC::at(li, lj)] + sCb[RC::at(li - 1, lj)]) * lden;
                atomic_add(&lCb[RC::at(li, lj)], T(0.5) * AW * lden);
                atomic_add(&lCb[RC::at(li - 1, lj)], T(0.5) * AW * lden);
            }
            if (TURN) {
                const T lm = one_if<T>(f0, F_LMU);
                const T du0 = uo - u0, dun = sUo[XS(li, lj + 1)] - sU[XS(li, lj + 1)];
                const T duw = sUo[XS(li - 1, lj)] - sU[XS(li - 1, lj)];
                const T duwn = sUo[XS(li - 1, lj + 1)] - sU[XS(li - 1, lj + 1)];
                const T g = -sg * k.sinW * T(0.5) * lm;
                lAW += g * (cd0 * T(0.5) * (du0 + dun) + cdw * T(0.5) * (duw + duwn)) * lN;
                const T q = g * AW * lN;
                lcd0 += q * T(0.5) * (du0 + dun);
                lcdw += q * T(0.5) * (duw + duwn);
                const T q0 = q * cd0 * T(0.5), qw = q * cdw * T(0.5);
                atomic_add(&lUo[XS(li, lj)], q0);
                atomic_add(&lU[XS(li, lj)], -q0);
                atomic_add(&lUo[XS(li, lj + 1)], q0);
                atomic_add(&lU[XS(li, lj + 1)], -q0);
                atomic_add(&lUo[XS(li - 1, lj)], qw);
                atomic_add(&lU[XS(li - 1, lj)], -qw);
                atomic_add(&lUo[XS(li - 1, lj + 1)], qw);
                atomic_add(&lU[XS(li - 1, lj + 1)], -qw);
            }
            a.AW[o] += lAW;
            atomic_add(&lCd[RC::at(li, lj)], lcd0);
            atomic_add(&lCd[RC::at(li - 1, lj)], lcdw);
            atomic_add(&lFv[RC::at(li, lj)], T(0.5) * lN);
            atomic_add(&lFv[RC::at(li - 1, lj)], T(0.5) * lN);
            const T r = c.rrAu[o] * lN;
            const T ldy = r * c.dyV_y[gj], ldx = r * c.dxV_x[gi];
            // sig11 = (s1 + s2)/2 at C(i) and C(i-1)
            atomic_add(&lS1[RC::at(li, lj)], T(0.5) * ldy);
            atomic_add(&lS2[RC::at(li, lj)], T(0.5) * ldy);
            atomic_add(&lS1[RC::at(li - 1, lj)], -T(0.5) * ldy);
            atomic_add(&lS2[RC::at(li - 1, lj)], -T(0.5) * ldy);
            atomic_add(&lS12[RZ2::at(li, lj + 1)], ldx);
            atomic_add(&lS12[RZ2::at(li, lj)], -ldx);
        }
        {   // V point
            const T AS = c.AS[o], mV = c.mV[o];
            T den = mV * k.bU1 + cosW2 * AS * (cd0 + cds);
            if (BASAL) den += T(0.5) * AS * (sCb[RC::at(li, lj)] + sCb[RC::at(li, lj - 1)]);
            const bool guard = den == T(0);
            if (guard) den = T(1);
            const T vnx = io.vn[((int64_t)gi * io.ldn + gj) * io.sst];
            const T lN = one_if<T>(f0, F_MV) * lv / den;
            const T lden = guard ? T(0) : -vnx * lv / den;
            atomic_add(&lV[XS(li, lj)], k.bU * mV * lN);
            a.mV[o] += k.bU * v0 * lN + k.bU1 * lden;
            a.cV[o] += lN;
            const T vo = sVo[XS(li, lj)];
            atomic_add(&lVo[XS(li, lj)], cosW2 * AS * (cd0 + cds) * lN);
            T lAS = cosW2 * (cd0 + cds) * vo * lN + cosW2 * (cd0 + cds) * lden;
            const T lcd = cosW2 * AS * vo * lN + cosW2 * AS * lden;
            T lcd0 = lcd, lcds = lcd;
            if (BASAL) {
                lAS += T(0.5) * (sCb[RC::at(li, lj)] + sCb[RC::at(li, lj - 1)]) * lden;
                atomic_add(&lCb[RC::at(li, lj)], T(0.5) * AS * lden);
                atomic_add(&lCb[RC::at(li, lj - 1)], T(0.5) * AS * lden);
            }
            if (TURN) {
                const T lm = one_if<T>(f0, F_LMV);
                const T dv0 = vo - v0, dve = sVo[XS(li + 1, lj)] - sV[XS(li + 1, lj)];
                const T dvs = sVo[XS(li, lj - 1)] - sV[XS(li, lj - 1)];
                const T dvse = sVo[XS(li + 1, lj - 1)] - sV[XS(li + 1, lj - 1)];
                const T g = sg * k.sinW * T(0.5) * lm;
                lAS += g * (cd0 * T(0.5) * (dv0 + dve) + cds * T(0.5) * (dvs + dvse)) * lN;
                const T q = g * AS * lN;
                lcd0 += q * T(0.5) * (dv0 + dve);
                lcds += q * T(0.5) * (dvs + dvse);
                const T q0 = q * cd0 * T(0.5), qs = q * cds * T(0.5);
                atomic_add(&lVo[XS(li, lj)], q0);
                atomic_add(&lV[XS(li, lj)], -q0);
                atomic_add(&lVo[XS(li + 1, lj)], q0);
                atomic_add(&lV[XS(li + 1, lj)], -q0);
                atomic_add(&lVo[XS(li, lj - 1)], qs);
                atomic_add(&lV[XS(li, lj - 1)], -qs);
                atomic_add(&lVo[XS(li + 1, lj - 1)], qs);
                atomic_add(&lV[XS(li + 1, lj - 1)], -qs);
            }
            a.AS[o] += lAS;
            atomic_add(&lCd[RC::at(li, lj)], lcd0);
            atomic_add(&lCd[RC::at(li, lj - 1)], lcds);
            atomic_add(&lFu[RC::at(li, lj)], -T(0.5) * lN);
            atomic_add(&lFu[RC::at(li, lj - 1)], -T(0.5) * lN);
            const T r = c.rrAv[o] * lN;
            const T ldx = r * c.dxU_x[gi], ldy = r * c.dyU_y[gj];
            // sig22 = (s1 - s2)/2 at C(j) and C(j-1)
            atomic_add(&lS1[RC::at(li, lj)], T(0.5) * ldx);
            atomic_add(&lS2[RC::at(li, lj)], -T(0.5) * ldx);
            atomic_add(&lS1[RC::at(li, lj - 1)], -T(0.5) * ldx);
            atomic_add(&lS2[RC::at(li, lj - 1)], T(0.5) * ldx);
            atomic_add(&lS12[RZ2::at(li + 1, lj)], ldy);
            atomic_add(&lS12[RZ2::at(li, lj)], -ldy);
        }
    }
    __syncthreads();

    // ---- reverse C: sigma12' at Z [0, TI] x [0, TJ]
    for (int idx = tid; idx < RZ2::n(); idx += THREADS) {
        const int li = idx / RZ2::W + RZ2::r0, lj = idx % RZ2::W + RZ2::c0;
        const T ls = lS12[idx];
        if (ls == T(0)) continue;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        atomic_add(&io.os12[(int64_t)gi * lp + gj], k.alpha_m1 * k.ralpha * ls);
        const int n = ((sF[XS(li, lj)] & F_MC) ? 1 : 0) + ((sF[XS(li - 1, lj)] & F_MC) ? 1 : 0) +
                      ((sF[XS(li, lj - 1)] & F_MC) ? 1 : 0) + ((sF[XS(li - 1, lj - 1)] & F_MC) ? 1 : 0);
        const T norm = n == 0 ? T(0) : T(1) / T(n);
        const T zz = norm * ((sZeta[RB::at(li, lj)] + sZeta[RB::at(li - 1, lj)]) +
                             (sZeta[RB::at(li, lj - 1)] + sZeta[RB::at(li - 1, lj - 1)]));
        const T e12 = sE12[RZ::at(li, lj)];
        const T lzz = T(0.5) * e12 * k.ralpha * ls * norm;
        atomic_add(&lZeta[RB::at(li, lj)], lzz);
        atomic_add(&lZeta[RB::at(li - 1, lj)], lzz);
        atomic_add(&lZeta[RB::at(li, lj - 1)], lzz);
        atomic_add(&lZeta[RB::at(li - 1, lj - 1)], lzz);
        atomic_add(&lE12[RZ::at(li, lj)], T(0.5) * zz * k.ralpha * ls);
    }
    __syncthreads();

    // ---- reverse B: C points [-1, TI] x [-1, TJ]
    double dragN = 0.0, dragS = 0.0;
    for (int idx = tid; idx < RB::n(); idx += THREADS) {
        const int li = idx / RB::W + RB::r0, lj = idx % RB::W + RB::c0;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const int64_t o = (int64_t)gi * lp + gj;
        const uint32_t f0 = sF[XS(li, lj)];
        const T mInC = one_if<T>(f0, F_INC), mC = one_if<T>(f0, F_MC);
        const T u0 = sU[XS(li, lj)], ue = sU[XS(li + 1, lj)], v0 = sV[XS(li, lj)], vn = sV[XS(li, lj + 1)];
        const T rdx = c.rdxU_x[gi], rdy = c.rdyV_y[gj];
        const T e11 = (ue - u0) * rdx * mInC, e22 = (vn - v0) * rdy * mInC;
        const T ep = e11 + e22, em = e11 - e22;
        const T delta = sDel[idx], zeta = sZeta[idx];
        T lz = lZeta[idx], lep = T(0), lem = T(0), ldel = T(0);
        if (li < TI && lj < TJ) {
            const int q = RC::at(li, lj);
            const T l1 = lS1[q], l2 = lS2[q];
            const T g1 = k.ralpha * mC * l1, g2 = k.ralpha * mC * l2;
            if (l1 != T(0)) atomic_add(&io.os1[o], k.alpha_m1 * g1);
            if (l2 != T(0)) atomic_add(&io.os2[o], k.alpha_m1 * g2);
            lz += (T(2) * ep - k.kp * delta) * g1 + T(0.5) * em * g2;
            lep += T(2) * zeta * g1;
            lem += T(0.5) * zeta * g2;
            ldel += -k.kp * zeta * g1;
            // ocean drag
            const T lcd = lCd[q];
            if (lcd != T(0)) {
                const uint32_t fe = sF[XS(li + 1, lj)], fn = sF[XS(li, lj + 1)];
                const T m0 = one_if<T>(f0, F_INU), m1 = one_if<T>(fe, F_INU);
                const T n0 = one_if<T>(f0, F_INV), n1 = one_if<T>(fn, F_INV);
                const T du0 = (u0 - sUo[XS(li, lj)]) * m0, du1 = (ue - sUo[XS(li + 1, lj)]) * m1;
                const T dv0 = (v0 - sVo[XS(li, lj)]) * n0, dv1 = (vn - sVo[XS(li, lj + 1)]) * n1;
                const T t = T(0.25) * ((du0 + du1) * (du0 + du1) + (dv0 + dv1) * (dv0 + dv1));
                const bool south = f0 & F_SOUTH;
                const T dc = south ? k.dS : k.dN, dc2 = south ? k.dS2 : k.dN2;
                if (dc2 * t > k.cmin2 && t > T(0)) {
                    const T st = sqrt(t);
                    const double lw = (double)(lcd * mC * rhoSea * st);
                    if (south) dragS += lw; else dragN += lw;
                    const T lt = lcd * mC * dc / (T(2) * st);
                    const T ldu = T(0.5) * (du0 + du1) * lt, ldv = T(0.5) * (dv0 + dv1) * lt;
                    atomic_add(&lU[XS(li, lj)], m0 * ldu);
                    atomic_add(&lUo[XS(li, lj)], -m0 * ldu);
                    atomic_add(&lU[XS(li + 1, lj)], m1 * ldu);
                    atomic_add(&lUo[XS(li + 1, lj)], -m1 * ldu);
                    atomic_add(&lV[XS(li, lj)], n0 * ldv);
                    atomic_add(&lVo[XS(li, lj)], -n0 * ldv);
                    atomic_add(&lV[XS(li, lj + 1)], n1 * ldv);
                    atomic_add(&lVo[XS(li, lj + 1)], -n1 * ldv);
                }
            }
            if (BASAL) {
                const T lcb = lCb[q];
                if (lcb != T(0)) {
                    const uint32_t fe = sF[XS(li + 1, lj)], fn = sF[XS(li, lj + 1)];
                    const T m0 = one_if<T>(f0, F_INU), m1 = one_if<T>(fe, F_INU);
                    const T n0 = one_if<T>(f0, F_INV), n1 = one_if<T>(fn, F_INV);
                    const T a1 = u0 * m0, b1 = ue * m1, c1 = v0 * n0, e1 = vn * n1;
                    const T s = T(0.25) * (a1 * a1 + b1 * b1 + c1 * c1 + e1 * e1) + k.U02;
                    const T rs = T(1) / sqrt(s);
                    atomic_add(&a.bfac[o], lcb * rs);
                    const T ls_ = -T(0.5) * c.bfac[o] * rs * rs * rs * lcb * T(0.25) * T(2);
                    atomic_add(&lU[XS(li, lj)], ls_ * a1 * m0);
                    atomic_add(&lU[XS(li + 1, lj)], ls_ * b1 * m1);
                    atomic_add(&lV[XS(li, lj)], ls_ * c1 * n0);
                    atomic_add(&lV[XS(li, lj + 1)], ls_ * e1 * n1);
                }
            }
            // Coriolis terms fvC = mfC (v + v_n), fuC = mfC (u + u_e)
            const T lfv = lFv[q], lfu = lFu[q];
            if (lfv != T(0) || lfu != T(0)) {
                const T mf = c.mfC[o];
                atomic_add(&a.mfC[o], (v0 + vn) * lfv + (u0 + ue) * lfu);
                atomic_add(&lV[XS(li, lj)], mf * lfv);
                atomic_add(&lV[XS(li, lj + 1)], mf * lfv);
                atomic_add(&lU[XS(li, lj)], mf * lfu);
                atomic_add(&lU[XS(li + 1, lj)], mf * lfu);
            }
        }
        if (lz != T(0)) {
            const T r = T(1) / (delta + k.deltaMin);
            atomic_add(&a.Ph[o], lz * r);
            ldel += -zeta * r * lz;
        }
        if (ldel != T(0) && delta > T(0)) {
            const T lD = ldel / (T(2) * delta);
            lep += T(2) * ep * lD;
            lem += T(2) * k.rsq * em * lD;
            const T le12c = T(4) * k.rsq * lD * c.qrA[o];
            auto put = [&](int a_, int b_) {
                const T e = sE12[RZ::at(a_, b_)];
                const T rz = c.rAz[(int64_t)d.wxt(i0 + a_) * lp + d.wyt(j0 + b_)];
                atomic_add(&lE12[RZ::at(a_, b_)], le12c * rz * T(2) * e);
            };
            put(li, lj);
            put(li + 1, lj);
            put(li, lj + 1);
            put(li + 1, lj + 1);
        }
        if (lep != T(0) || lem != T(0)) {
            const T le11 = (lep + lem) * rdx * mInC, le22 = (lep - lem) * rdy * mInC;
            atomic_add(&lU[XS(li + 1, lj)], le11);
            atomic_add(&lU[XS(li, lj)], -le11);
            atomic_add(&lV[XS(li, lj + 1)], le22);
            atomic_add(&lV[XS(li, lj)], -le22);
        }
    }
    // water-drag gradients: warp sums, one atomic per warp
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        dragN += __shfl_down_sync(0xffffffffu, dragN, off);
        dragS += __shfl_down_sync(0xffffffffu, dragS, off);
    }
    if ((tid & 31) == 0) {
        if (dragN != 0.0) atomicAdd(a.dragN, dragN);
        if (dragS != 0.0) atomicAdd(a.dragS, dragS);
    }
    __syncthreads();

    // ---- reverse A: e12 at Z
    for (int idx = tid; idx < RZ::n(); idx += THREADS) {
        const T le = lE12[idx];
        if (le == T(0)) continue;
        const int li = idx / RZ::W + RZ::r0, lj = idx % RZ::W + RZ::c0;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const uint32_t f0 = sF[XS(li, lj)], fw = sF[XS(li - 1, lj)], fs = sF[XS(li, lj - 1)],
                       fws = sF[XS(li - 1, lj - 1)];
        const T mzh = (f0 & fw & fs & fws & F_MC) ? T(0.5) : T(0);
        const T hU = one_if<T>(f0, F_MU) - one_if<T>(fs, F_MU);
        const T hV = one_if<T>(f0, F_MV) - one_if<T>(fw, F_MV);
        const T ry = c.rdyU_y[gj] * le, rx = c.rdxV_x[gi] * le;
        atomic_add(&lU[XS(li, lj)], ry * (mzh + hU));
        atomic_add(&lU[XS(li, lj - 1)], ry * (hU - mzh));
        atomic_add(&lV[XS(li, lj)], rx * (mzh + hV));
        atomic_add(&lV[XS(li - 1, lj)], rx * (hV - mzh));
    }
    __syncthreads();

    // ---- flush u, v, ocean-velocity adjoints of the staged region
    for (int idx = tid; idx < RS::n(); idx += THREADS) {
        const int li = idx / RS::W + RS::r0, lj = idx % RS::W + RS::c0;
        const int64_t o = (int64_t)d.wxt(i0 + li) * lp + d.wyt(j0 + lj);
        if (lU[idx] != T(0)) atomic_add(&io.ou[o], lU[idx]);
        if (lV[idx] != T(0)) atomic_add(&io.ov[o], lV[idx]);
        if (lUo[idx] != T(0)) atomic_add(&a.uOc[o], lUo[idx]);
        if (lVo[idx] != T(0)) atomic_add(&a.vOc[o], lVo[idx]);
    }
#undef XS
}

// Adjoint of the prep kernel: folded-constant adjoints -> field adjoints.
// Ph = 0.5 P (1 + tsf); mfC = 0.5 mC fCori; cU = mU/dt u0 + WFX;
// bfac = K2 softplus_10(h - |R| A / K1) 0.1 exp(-Cb (1 - A)) (A > 0.01).
template <class T, bool BASAL>
__global__ void prep_adjoint_kernel(VerisParams p, Fields<double> f, Dims d, int64_t lp, FastConsts<T> c,
                                    Adj<T> a, const T *lu0, const T *lv0, VerisFieldsF64 g, T *lu_init,
                                    T *lv_init) {
    const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 8 + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const int64_t o = d.raw(i, j), q = (int64_t)i * lp + j;
    auto put = [&](const double *arr, double v) {
        if (arr) *const_cast<double *>(arr + o) += v;
    };
    const double rdt = p.recip_deltatDyn;
    const double lcU = (double)a.cU[q], lcV = (double)a.cV[q];
    put(g.SeaIceStrength, 0.5 * (1.0 + p.tensileStrFac) * (double)a.Ph[q]);
    put(g.SeaIceMassC, 0.5 * f.fCori[o] * (double)a.mfC[q]);
    put(g.SeaIceMassU, (double)a.mU[q] + rdt * f.uIce[o] * lcU);
    put(g.SeaIceMassV, (double)a.mV[q] + rdt * f.vIce[o] * lcV);
    put(g.WindForcingX, lcU);
    put(g.WindForcingY, lcV);
    put(g.AreaW, (double)a.AW[q]);
    put(g.AreaS, (double)a.AS[q]);
    put(g.uOcean, (double)a.uOc[q]);
    put(g.vOcean, (double)a.vOc[q]);
    // the initial velocities: the subcycle adjoint plus the u^{n-1} term of cU
    lu_init[o] = lu0[q] + (T)(f.SeaIceMassU[o] * rdt * lcU);
    lv_init[o] = lv0[q] + (T)(f.SeaIceMassV[o] * rdt * lcV);
    if (BASAL) {
        const double A = f.Area[o];
        if (A > 0.01) {
            const double lb = (double)a.bfac[q];
            const double hcrit = fabs(f.R_low[o]) * A / p.basalDragK1;
            const double x = 10.0 * (f.hIceMean[o] - hcrit);
            const double sp = log(exp(x) + 1.0) * 0.1;          // softplus / 10
            const double sig = 1.0 / (1.0 + exp(-x));           // its derivative w.r.t. (h - hcrit)
            const double ex = exp(-p.cBasalStar * (1.0 - A));
            const double K2 = p.basalDragK2;
            // d/dh and d/dA
            put(g.hIceMean, lb * K2 * sig * ex);
            put(g.Area, lb * K2 * (sig * (-fabs(f.R_low[o]) / p.basalDragK1) * ex + sp * ex * p.cBasalStar));
        }
    }
}

template <class T>
__global__ void scale_kernel(T *x, int64_t n, T s) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        x[k] *= s;
}

template <class T, bool B, bool R, int TI>
static int launch_adj_ti(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c,
                         const FastScalars<T> &k, const Io<T> &io, const Adj<T> &a, T rhoSea, cudaStream_t st) {
    auto kern = evp_adjoint_kernel<T, B, R, TI>;
    const size_t sm = Smem<T, TI>::bytes();
    static std::atomic<bool> configured[MAX_DEVICES];
    if (!smem_configured(configured, kern, (int)sm)) return VERIS_ERR_LAUNCH;
    dim3 grid((d.NY + TJ - 1) / TJ, (d.NX + TI - 1) / TI);
    kern<<<grid, THREADS, sm, st>>>(d, lp, h, c, k, io, a, rhoSea);
    return launch_status();
}

// tile rows: 8 while 16-row tiles would leave SMs idle (fewer than two
// tiles per SM), else 16 (less recomputed ring per cell); float32 goes down
// to 4 the same way
template <class T, bool B, bool R>
static int launch_adj(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c, const FastScalars<T> &k,
                      const Io<T> &io, const Adj<T> &a, T rhoSea, cudaStream_t st) {
    int sms = sm_count();
    if (sms == 0) sms = 152;
    const long tiles16 = (long)((d.NY + TJ - 1) / TJ) * ((d.NX + 15) / 16);
    if constexpr (sizeof(T) == 4) {
        // float32 is bound by latency, not arithmetic: 4-row tiles (more
        // recomputed ring, twice the CTAs) while 8-row tiles would leave SMs
        // with fewer than two
        const long tiles8 = (long)((d.NY + TJ - 1) / TJ) * ((d.NX + 7) / 8);
        if (tiles8 < 2L * sms) return launch_adj_ti<T, B, R, 4>(d, lp, h, c, k, io, a, rhoSea, st);
    }
    if (tiles16 < 2L * sms) return launch_adj_ti<T, B, R, 8>(d, lp, h, c, k, io, a, rhoSea, st);
    return launch_adj_ti<T, B, R, 16>(d, lp, h, c, k, io, a, rhoSea, st);
}

// workspace: [fast layout][11 constant adjoints][2 scalars]
//            [checkpoints: ncp states][segment: K+1 states][2 adjoint states]
template <class T>
struct Plan {
    FastConsts<T> c;
    T *st2[2][5];
    int *status;
    Adj<T> a;
    T *cp, *seg, *lam[2][5];
    T *scr[N_SCRATCH];   // the gather passes' arrays
    size_t field;   // bytes of one internal array
    size_t total;
};

template <class T>
static size_t plan(const Dims &d, int n, int K, char *base, Plan<T> *pl, bool taped = false) {
    size_t off = fast_layout<T>(d, base, &pl->c, pl->st2, &pl->status);
    const int64_t lp = internal_pitch(d.NY);
    pl->field = rup256((size_t)d.NX * lp * sizeof(T));
    auto take = [&](size_t nb) { char *q = base ? base + off : nullptr; off += nb; return q; };
    T **arrs[11] = {&pl->a.Ph, &pl->a.mfC, &pl->a.bfac, &pl->a.mU, &pl->a.cU, &pl->a.AW, &pl->a.uOc,
                    &pl->a.mV, &pl->a.cV, &pl->a.AS, &pl->a.vOc};
    for (int q = 0; q < 11; ++q) *arrs[q] = reinterpret_cast<T *>(take(pl->field));
    double *sc = reinterpret_cast<double *>(take(256));
    pl->a.dragN = sc;
    pl->a.dragS = sc ? sc + 1 : nullptr;
    // float64 gather passes: per-cell water-drag sums, reduced after the sweep
    pl->a.dragC = reinterpret_cast<double *>(take(sizeof(T) == 8 ? rup256((size_t)d.NX * lp * sizeof(double)) : 0));
    const int ncp = taped ? 0 : (n + K - 1) / K;
    pl->cp = reinterpret_cast<T *>(take((size_t)ncp * 5 * pl->field));
    pl->seg = reinterpret_cast<T *>(take(taped ? 0 : (size_t)(K + 1) * 5 * pl->field));
    for (int b = 0; b < 2; ++b)
        for (int q = 0; q < 5; ++q) pl->lam[b][q] = reinterpret_cast<T *>(take(pl->field));
    for (int q = 0; q < N_SCRATCH; ++q) pl->scr[q] = reinterpret_cast<T *>(take(pl->field));
    pl->total = off;
    return off;
}

// field q of slot s: the checkpoints and segments hold 5 fields per slot, a
// forward's tape tape_slot_fields
template <class T>
static T *slot(T *base, size_t field, int s, int q, int width = 5) {
    return reinterpret_cast<T *>(reinterpret_cast<char *>(base) + ((size_t)s * width + q) * field);
}

template <class T>
static int copy_state(T *const dst[5], T *const src[5], size_t bytes, cudaStream_t st) {
    for (int q = 0; q < 5; ++q)
        if (cudaMemcpyAsync(dst[q], src[q], bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return VERIS_ERR_LAUNCH;
    return VERIS_OK;
}

// the float32 adjoint's form: 0 by grid size, 1 the tile kernel, 2 the gather passes, 3 the
// gather passes with P4 and P1 of consecutive subcycles in separate launches
static std::atomic<int> g_f32_form{0};
// padded cells from which the float32 adjoint takes the gather passes: a recomputed segment
// (two more passes per subcycle) from 2^19 (measured: 360 x 180 faster with the tile kernel,
// 3600 x 1800 with the passes), a tape with the walk's terms from 2^16 (360 x 180, 66,976
// padded cells: 1-degree trajectory 3.53x its forward with the passes, 3.70x with the tile
// kernel)
constexpr int64_t F32_GATHER_CELLS = 1 << 19;
constexpr int64_t F32_GATHER_CELLS_TAPED = 1 << 16;

// tape != nullptr: the forward's subcycle states (slot k = after k
// subcycles, 5 arrays per slot, plan field bytes each) replace the
// checkpoints and the recomputation
template <class T>
static int evp_adjoint(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int n, int K,
                       const T *const lout[5], T *const lin[5], const VerisFieldsF64 *lf, double *lscal, void *ws,
                       size_t wsb, veris_stream_t s, const T *tape = nullptr, size_t tape_bytes = 0) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && lf && lscal && n >= 1, VERIS_ERR_ARG);
    for (int q = 0; q < 5; ++q) VERIS_REQUIRE(lout[q] && lin[q], VERIS_ERR_ARG);
    if (fast_support(*p)) return VERIS_ERR_UNSUPPORTED;
    if (K <= 0 || K > n || tape) K = n;
    const bool taped = tape != nullptr;
    // float64: the gather passes; float32: the passes on large grids (memory-bound there), the
    // tile kernel on small ones (its one launch per subcycle beats four to six latency-bound ones)
    const int f32_form = g_f32_form.load(std::memory_order_relaxed);
    const bool gather = sizeof(T) == 8 || f32_form >= 2 ||
                        (f32_form == 0 &&
                         (int64_t)d.NX * d.NY >= (taped ? F32_GATHER_CELLS_TAPED : F32_GATHER_CELLS));
    Plan<T> pl;
    VERIS_REQUIRE(ws && wsb >= plan<T>(d, n, K, nullptr, &pl, taped), VERIS_ERR_WORKSPACE);
    plan<T>(d, n, K, static_cast<char *>(ws), &pl, taped);
    // slot width of the states the sweep reads: a tape's, or the segment's
    const int W = taped ? tape_slot_fields<T>() : 5;
    if (taped) VERIS_REQUIRE(tape_bytes >= (size_t)(n + 1) * W * pl.field, VERIS_ERR_WORKSPACE);
    cudaStream_t st = (cudaStream_t)s;
    const int64_t lp = internal_pitch(d.NY);
    const Fields<double> &f = *reinterpret_cast<const Fields<double> *>(vs);
    const bool basal = p->basalDragK2 != 0.0, turn = p->sinWat != 0.0;
    const HaloFill h = halo_fill_of(*p);
    const FastScalars<T> k = fast_scalars<T>(*p);
    int stt;
    // zero the constant adjoints and the scalars
    T *zero_list[11] = {pl.a.Ph, pl.a.mfC, pl.a.bfac, pl.a.mU, pl.a.cU, pl.a.AW, pl.a.uOc,
                        pl.a.mV, pl.a.cV, pl.a.AS, pl.a.vOc};
    for (int q = 0; q < 11; ++q)
        if (cudaMemsetAsync(zero_list[q], 0, pl.field, st) != cudaSuccess) return VERIS_ERR_LAUNCH;
    if (cudaMemsetAsync(pl.a.dragN, 0, 2 * sizeof(double), st) != cudaSuccess) return VERIS_ERR_LAUNCH;
    if (sizeof(T) == 8 &&
        cudaMemsetAsync(pl.a.dragC, 0, (size_t)d.NX * lp * sizeof(double), st) != cudaSuccess)
        return VERIS_ERR_LAUNCH;

    // forward sweep: state 0 from the prep, checkpoints every K subcycles
    T *cp0[5];
    for (int q = 0; q < 5; ++q) cp0[q] = taped ? pl.st2[0][q] : slot(pl.cp, pl.field, 0, q);
    if ((stt = fast_prep<T>(d, *p, f, pl.c, cp0, st)) != VERIS_OK) return stt;   // constants (+ state 0)
    const int ncp = taped ? 1 : (n + K - 1) / K;
    if (!taped) {
        // states K, 2K, ... (ncp-1)K go to checkpoint slots; the ones between to scratch
        const int last = (ncp - 1) * K;
        const T *cur[5] = {cp0[0], cp0[1], cp0[2], cp0[3], cp0[4]};
        for (int nx = 1; nx <= last; ++nx) {
            T *dst[5];
            for (int q = 0; q < 5; ++q) dst[q] = (nx % K == 0) ? slot(pl.cp, pl.field, nx / K, q) : pl.st2[nx % 2][q];
            FastIO<T> io{cur[0], cur[1], cur[2], cur[3], cur[4], dst[0], dst[1], dst[2], dst[3], dst[4], lp};
            if ((stt = fast_subcycle<T>(d, h, pl.c, k, io, basal, turn, st)) != VERIS_OK) return stt;
            for (int q = 0; q < 5; ++q) cur[q] = dst[q];
        }
    }
    // reverse sweep, segment by segment
    int lb = 0;   // the adjoint buffer holding lambda_{s+1} (after the first subcycle)
    for (int m = ncp - 1; m >= 0; --m) {
        const int s0 = m * K, s1 = (s0 + K < n) ? s0 + K : n;
        // segment states: recomputed from the checkpoint, or the forward's tape
        T *const segb = taped ? const_cast<T *>(tape) : pl.seg;
        if (!taped) {
            T *segs[5];
            for (int q = 0; q < 5; ++q) segs[q] = slot(pl.seg, pl.field, 0, q);
            T *cps[5];
            for (int q = 0; q < 5; ++q) cps[q] = slot(pl.cp, pl.field, m, q);
            if constexpr (sizeof(T) == 8) {
                // float64 segment slots hold (u, v, Delta, zeta, cDrag); the
                // stresses run in the workspace's state buffers
                T *to[5] = {segs[0], segs[1], pl.st2[0][2], pl.st2[0][3], pl.st2[0][4]};
                if ((stt = copy_state<T>(to, cps, pl.field, st)) != VERIS_OK) return stt;
            } else {
                if ((stt = copy_state<T>(segs, cps, pl.field, st)) != VERIS_OK) return stt;
            }
        }
        for (int ss = s0; ss < s1 && !taped; ++ss) {
            const T *cur[5];
            T *dst[5];
            for (int q = 0; q < 5; ++q) {
                cur[q] = slot(pl.seg, pl.field, ss - s0, q);
                dst[q] = slot(pl.seg, pl.field, ss - s0 + 1, q);
            }
            FastIO<T> io{cur[0], cur[1], cur[2], cur[3], cur[4], dst[0], dst[1], dst[2], dst[3], dst[4], lp};
            if constexpr (sizeof(T) == 8) {
                T *const *a = pl.st2[(ss - s0) % 2], *const *b = pl.st2[(ss - s0 + 1) % 2];
                io.s1 = a[2]; io.s2 = a[3]; io.s12 = a[4];
                io.s1o = b[2]; io.s2o = b[3]; io.s12o = b[4];
                io.tDel = slot(pl.seg, pl.field, ss - s0, 2);
                io.tZeta = slot(pl.seg, pl.field, ss - s0, 3);
                io.tCd = slot(pl.seg, pl.field, ss - s0, 4);
            }
            if ((stt = fast_subcycle<T>(d, h, pl.c, k, io, basal, turn, st)) != VERIS_OK) return stt;
        }
        for (int ss = s1 - 1; ss >= s0; --ss) {
            const bool first = ss == n - 1;
            T *out[5];
            for (int q = 0; q < 5; ++q) out[q] = pl.lam[first ? 0 : lb ^ 1][q];
            const int rs = taped ? ss : ss - s0;   // slot of this subcycle's input state
            if (gather) {
                // gather passes: every adjoint array written whole, nothing to clear.  A float64
                // slot holds (u, v, Delta, zeta, cDrag); a float32 tape the walk's (u, v, sigma1,
                // sigma2) layout and its Delta, zeta, cDrag; a float32 segment five planar state
                // arrays: the passes recompute Delta, zeta and cDrag
                const bool quad = taped && sizeof(T) == 4;
                auto tape_of = [&](int sub) {
                    const int r = taped ? sub : sub - s0;   // slot of the subcycle's input state
                    TapeG<T> tt;
                    tt.u = slot(segb, pl.field, r, 0, W);
                    tt.v = quad ? tt.u + 1 : slot(segb, pl.field, r, 1, W);
                    tt.un = slot(segb, pl.field, r + 1, 0, W);
                    tt.vn = quad ? tt.un + 1 : slot(segb, pl.field, r + 1, 1, W);
                    tt.sst = quad ? 4 : 1;
                    const int qd = sizeof(T) == 8 ? 2 : 5;
                    const bool rich = sizeof(T) == 8 || quad;
                    tt.del = rich ? slot(segb, pl.field, r, qd, W) : nullptr;
                    tt.zeta = rich ? slot(segb, pl.field, r, qd + 1, W) : nullptr;
                    tt.cd = rich ? slot(segb, pl.field, r, qd + 2, W) : nullptr;
                    return tt;
                };
                // the adjoints of subcycle `sub`: in from its result's buffer (the caller's at the
                // last subcycle), out to the other of the two
                auto lam_of = [&](int sub, int b) {
                    LamG<T> ll;
                    if (sub == n - 1) {
                        ll.lu = lout[0]; ll.lv = lout[1]; ll.ls1 = lout[2]; ll.ls2 = lout[3]; ll.ls12 = lout[4];
                        ll.ldl = d.ld;
                    } else {
                        ll.lu = pl.lam[b][0]; ll.lv = pl.lam[b][1]; ll.ls1 = pl.lam[b][2];
                        ll.ls2 = pl.lam[b][3]; ll.ls12 = pl.lam[b][4];
                        ll.ldl = lp;
                    }
                    T *const *o5 = pl.lam[sub == n - 1 ? 0 : b ^ 1];
                    ll.ou = o5[0]; ll.ov = o5[1]; ll.os1 = o5[2]; ll.os2 = o5[3]; ll.os12 = o5[4];
                    return ll;
                };
                const TapeG<T> tt = tape_of(ss);
                const LamG<T> ll = lam_of(ss, lb);
                const int lb_next = first ? 0 : lb ^ 1;
                bool done = false;
                if constexpr (sizeof(T) == 4) {
                    // float32 without turning angle: P4 of each subcycle fused with P1 of the one
                    // before it in the segment
                    if (!turn && f32_form != 3) {
                        const bool head = ss == s1 - 1;
                        if (ss > s0) {
                            const TapeG<T> tp = tape_of(ss - 1);
                            const LamG<T> lpv = lam_of(ss - 1, lb_next);
                            stt = adjoint_gather_chain<T>(d, lp, h, pl.c, k, p->rhoSea, tt, ll, pl.a, pl.scr, basal,
                                                          head, &tp, &lpv, st);
                        } else {
                            stt = adjoint_gather_chain<T>(d, lp, h, pl.c, k, p->rhoSea, tt, ll, pl.a, pl.scr, basal,
                                                          head, nullptr, nullptr, st);
                        }
                        done = true;
                    }
                }
                if (!done)
                    stt = adjoint_gather_subcycle<T>(d, lp, h, pl.c, k, p->rhoSea, tt, ll, pl.a, pl.scr, basal, turn,
                                                     st);
                if (stt != VERIS_OK) return stt;
                lb = lb_next;
                continue;
            }
            if constexpr (sizeof(T) == 4) {   // the float32 tile kernel (float64 always gathers)
                // the five adjoint arrays of a buffer are contiguous: one memset
                if (cudaMemsetAsync(out[0], 0, 5 * pl.field, st) != cudaSuccess) return VERIS_ERR_LAUNCH;
                Io<T> io;
                // a float32 tape is written by the register walk in its own
                // layout: (u, v, sigma1, sigma2) per point over the slot's first
                // four fields
                const bool quad = taped && sizeof(T) == 4;
                io.u = slot(segb, pl.field, rs, 0, W);
                io.v = quad ? io.u + 1 : slot(segb, pl.field, rs, 1, W);
                io.s1 = slot(segb, pl.field, rs, 2, W);
                io.s2 = slot(segb, pl.field, rs, 3, W);
                io.s12 = slot(segb, pl.field, rs, 4, W);
                io.un = slot(segb, pl.field, rs + 1, 0, W);
                io.vn = quad ? io.un + 1 : slot(segb, pl.field, rs + 1, 1, W);
                io.sst = quad ? 4 : 1;
                io.ldn = lp;
                if (first) {
                    io.lu = lout[0]; io.lv = lout[1]; io.ls1 = lout[2]; io.ls2 = lout[3]; io.ls12 = lout[4];
                    io.ldl = d.ld;
                } else {
                    io.lu = pl.lam[lb][0]; io.lv = pl.lam[lb][1]; io.ls1 = pl.lam[lb][2];
                    io.ls2 = pl.lam[lb][3]; io.ls12 = pl.lam[lb][4];
                    io.ldl = lp;
                }
                io.ou = out[0]; io.ov = out[1]; io.os1 = out[2]; io.os2 = out[3]; io.os12 = out[4];
                const T rho = (T)p->rhoSea;
                if (basal)
                    stt = turn ? launch_adj<T, true, true>(d, lp, h, pl.c, k, io, pl.a, rho, st)
                               : launch_adj<T, true, false>(d, lp, h, pl.c, k, io, pl.a, rho, st);
                else
                    stt = turn ? launch_adj<T, false, true>(d, lp, h, pl.c, k, io, pl.a, rho, st)
                               : launch_adj<T, false, false>(d, lp, h, pl.c, k, io, pl.a, rho, st);
                if (stt != VERIS_OK) return stt;
                lb = first ? 0 : lb ^ 1;
            }
        }
    }
    if (sizeof(T) == 8) {   // the water-drag gradients of the gather passes
        const double wN = k.dN != 0 ? p->rhoSea / (double)k.dN : 0.0, wS = k.dS != 0 ? p->rhoSea / (double)k.dS : 0.0;
        if ((stt = reduce_drag(d, lp, pl.c.flags, pl.a.dragC, wN, wS, pl.a.dragN, pl.a.dragS, st)) != VERIS_OK)
            return stt;
    }
    // fold the constant adjoints back onto the fields; initial-state adjoints
    dim3 g2((d.NY + 31) / 32, (d.NX + 7) / 8);
    T *const *l0 = pl.lam[lb];
    if (basal)
        prep_adjoint_kernel<T, true><<<g2, dim3(32, 8), 0, st>>>(*p, f, d, lp, pl.c, pl.a, l0[0], l0[1], *lf, lin[0],
                                                                 lin[1]);
    else
        prep_adjoint_kernel<T, false><<<g2, dim3(32, 8), 0, st>>>(*p, f, d, lp, pl.c, pl.a, l0[0], l0[1], *lf, lin[0],
                                                                  lin[1]);
    if ((stt = launch_status()) != VERIS_OK) return stt;
    for (int q = 2; q < 5; ++q)
        if (cudaMemcpy2DAsync(lin[q], d.ld * sizeof(T), l0[q], lp * sizeof(T), d.NY * sizeof(T), d.NX,
                              cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return VERIS_ERR_LAUNCH;
    // scalar gradients: written to the caller's two values
    if (cudaMemcpyAsync(lscal, pl.a.dragN, 2 * sizeof(double), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return VERIS_ERR_LAUNCH;
    return VERIS_OK;
}

}  // namespace adj

}  // namespace veris

using namespace veris;

extern "C" {

size_t veris_evp_adjoint_workspace_bytes(const VerisGrid *g, int32_t elem_size, int32_t n, int32_t K) {
    Dims d;
    if (check_grid(g, &d) != VERIS_OK || n < 1) return 0;
    if (K <= 0 || K > n) K = n;
    if (elem_size == 8) {
        adj::Plan<double> pl;
        return adj::plan<double>(d, n, K, nullptr, &pl);
    }
    if (elem_size == 4) {
        adj::Plan<float> pl;
        return adj::plan<float>(d, n, K, nullptr, &pl);
    }
    return 0;
}

size_t veris_evp_adjoint_taped_workspace_bytes(const VerisGrid *g, int32_t n) {
    Dims d;
    if (check_grid(g, &d) != VERIS_OK || n < 1) return 0;
    adj::Plan<double> pl;
    return adj::plan<double>(d, n, n, nullptr, &pl, true);
}

int veris_evp_adjoint_taped_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                                const double *tape, size_t tape_bytes, const double *lu, const double *lv,
                                const double *ls1, const double *ls2, const double *ls12, double *lu0,
                                double *lv0, double *ls10, double *ls20, double *ls120,
                                const VerisFieldsF64 *lfields, double *lscalars, void *ws, size_t wsb,
                                veris_stream_t s) {
    VERIS_REQUIRE(tape, VERIS_ERR_ARG);
    const double *lout[5] = {lu, lv, ls1, ls2, ls12};
    double *lin[5] = {lu0, lv0, ls10, ls20, ls120};
    return adj::evp_adjoint<double>(g, p, vs, n, n, lout, lin, lfields, lscalars, ws, wsb, s, tape, tape_bytes);
}

size_t veris_evp_adjoint_taped_workspace_bytes_f32(const VerisGrid *g, int32_t n) {
    Dims d;
    if (check_grid(g, &d) != VERIS_OK || n < 1) return 0;
    adj::Plan<float> pl;
    return adj::plan<float>(d, n, n, nullptr, &pl, true);
}

int veris_evp_adjoint_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                          int32_t K, const float *lu, const float *lv, const float *ls1, const float *ls2,
                          const float *ls12, float *lu0, float *lv0, float *ls10, float *ls20, float *ls120,
                          const VerisFieldsF64 *lfields, double *lscalars, void *ws, size_t wsb, veris_stream_t s) {
    const float *lout[5] = {lu, lv, ls1, ls2, ls12};
    float *lin[5] = {lu0, lv0, ls10, ls20, ls120};
    return adj::evp_adjoint<float>(g, p, vs, n, K, lout, lin, lfields, lscalars, ws, wsb, s);
}

int veris_evp_adjoint_taped_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                                const float *tape, size_t tape_bytes, const float *lu, const float *lv,
                                const float *ls1, const float *ls2, const float *ls12, float *lu0, float *lv0,
                                float *ls10, float *ls20, float *ls120, const VerisFieldsF64 *lfields,
                                double *lscalars, void *ws, size_t wsb, veris_stream_t s) {
    VERIS_REQUIRE(tape, VERIS_ERR_ARG);
    const float *lout[5] = {lu, lv, ls1, ls2, ls12};
    float *lin[5] = {lu0, lv0, ls10, ls20, ls120};
    return adj::evp_adjoint<float>(g, p, vs, n, n, lout, lin, lfields, lscalars, ws, wsb, s, tape, tape_bytes);
}

int veris_evp_adjoint_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                          int32_t K, const double *lu, const double *lv, const double *ls1, const double *ls2,
                          const double *ls12, double *lu0, double *lv0, double *ls10, double *ls20,
                          double *ls120, const VerisFieldsF64 *lfields, double *lscalars, void *ws, size_t wsb,
                          veris_stream_t s) {
    const double *lout[5] = {lu, lv, ls1, ls2, ls12};
    double *lin[5] = {lu0, lv0, ls10, ls20, ls120};
    return adj::evp_adjoint<double>(g, p, vs, n, K, lout, lin, lfields, lscalars, ws, wsb, s);
}

int veris_evp_adjoint_f32_form(int32_t form) {
    VERIS_REQUIRE(form >= 0 && form <= 3, VERIS_ERR_ARG);
    adj::g_f32_form.store(form, std::memory_order_relaxed);
    return VERIS_OK;
}

}  // extern "C"
