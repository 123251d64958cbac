// The mEVP subcycle loop, fast forms (veris/evp_solver.py:21-319).
//
// Same algorithm and the same wrap/halo semantics as the plain form,
// restructured for GB300:
//
// * once per step a prep kernel folds every step-constant input of the
//   subcycle into compact arrays (ice strength factor, Coriolis factor, area
//   weights, mass-weighted previous velocity plus wind forcing, ...), packs
//   the six masks, the hemisphere and the "mass != 0" switches into one
//   32-bit flag word per cell, and reduces the grid lengths (which vary along
//   one axis only on the host model's grids) to 1-D vectors;
// * float32: per subcycle the register-walking kernel (evp_walk.cu) or the
//   TMA-staged kernel (evp_tma.cu); where tensor maps cannot be built, the
//   shared-memory kernel below, which stages u, v, the ocean velocities and
//   the flags of its tile plus a 2-cell ring and reads every other array
//   once per point it needs;
// * float64: the float64 tile kernel (evp_fast64.cu), arranged for GB300's
//   float64 pipe;
// * float32 instantiations contain no float64 arithmetic.
//
// Covers the default rheology (noSlip without second-order terms, no
// adaptive relaxation, replacement pressure on, metric terms k1/k2 zero,
// masks 0/1, 1-D grid lengths); veris_evp_fast_check reports what a state
// breaks, and callers use the plain form for those.
#include "evp_tile.cuh"

namespace veris {

int fast_support(const VerisParams &p) {
    int v = 0;
    if (p.useAdaptiveEVP) v |= V_ADAPT;
    if (!p.noSlip) v |= V_SLIP;
    if (p.secondOrderBC) v |= V_SECOND;
    if (p.pressReplFac != 1.0) v |= V_PRESS;
    return v;
}

// ------------------------------------------------------------------ checks
__global__ void fast_check_kernel(Fields<double> f, Dims d, int *viol) {
    const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 8 + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const int64_t o = d.raw(i, j), o0 = d.raw(i, 0), oj = d.raw(0, j);
    int v = 0;
    if (f.k1AtC[o] != 0.0 || f.k2AtC[o] != 0.0 || f.k1AtZ[o] != 0.0 || f.k2AtZ[o] != 0.0) v |= V_KTERMS;
    const double *m[6] = {f.iceMask, f.iceMaskU, f.iceMaskV, f.maskInC, f.maskInU, f.maskInV};
    for (int q = 0; q < 6; ++q)
        if (m[q][o] != 0.0 && m[q][o] != 1.0) v |= V_MASKS;
    if (f.recip_dxU[o] != f.recip_dxU[o0] || f.recip_dxV[o] != f.recip_dxV[o0] || f.dxV[o] != f.dxV[o0] ||
        f.dxU[o] != f.dxU[o0])
        v |= V_METRIC;
    if (f.recip_dyV[o] != f.recip_dyV[oj] || f.recip_dyU[o] != f.recip_dyU[oj] || f.dyV[o] != f.dyV[oj] ||
        f.dyU[o] != f.dyU[oj])
        v |= V_METRIC;
    if (f.recip_rA[o] != f.recip_rA[oj] || f.rAz[o] != f.rAz[oj] || f.recip_rAu[o] != f.recip_rAu[oj] ||
        f.recip_rAv[o] != f.recip_rAv[oj])
        v |= V_AREA2D;
    if (v) atomicOr(viol, v);
}

// ------------------------------------------------------------------- prep
template <class T, bool BASAL>
__global__ void fast_prep_kernel(VerisParams p, Fields<double> f, Dims d, int64_t lp, FastConsts<T> c, T *u, T *v,
                                 T *s1, T *s2, T *s12, int paired) {
    const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 8 + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const int64_t o = d.raw(i, j);
    const int64_t q = (int64_t)i * lp + j;
    const double rdt = p.recip_deltatDyn;
    const double P = f.SeaIceStrength[o];
    c.Ph[q] = (T)(0.5 * P * (1.0 + p.tensileStrFac));
    c.mfC[q] = (T)(f.SeaIceMassC[o] * f.fCori[o] * 0.5);
    c.qrA[q] = (T)(0.25 * f.recip_rA[o]);
    c.rAz[q] = (T)f.rAz[o];
    const double mU = f.SeaIceMassU[o], mV = f.SeaIceMassV[o];
    c.mU[q] = (T)mU;
    c.mV[q] = (T)mV;
    c.cU[q] = (T)(mU * rdt * f.uIce[o] + f.WindForcingX[o]);
    c.cV[q] = (T)(mV * rdt * f.vIce[o] + f.WindForcingY[o]);
    c.AW[q] = (T)f.AreaW[o];
    c.AS[q] = (T)f.AreaS[o];
    c.uOc[q] = (T)f.uOcean[o];
    c.vOc[q] = (T)f.vOcean[o];
    c.rrAu[q] = (T)f.recip_rAu[o];
    c.rrAv[q] = (T)f.recip_rAv[o];
    if constexpr (sizeof(T) == 4) {   // the register walk's grouped inputs
        c.q4U[4 * q] = c.cU[q];
        c.q4U[4 * q + 1] = c.cV[q];
        c.q4U[4 * q + 2] = c.AW[q];
        c.q4U[4 * q + 3] = c.AS[q];
        c.pMUV[2 * q] = c.mU[q];
        c.pMUV[2 * q + 1] = c.mV[q];
        c.q4M[4 * q] = c.mU[q];
        c.q4M[4 * q + 1] = c.mV[q];
        c.q4M[4 * q + 2] = c.rrAu[q];
        c.q4M[4 * q + 3] = c.rrAv[q];
        c.q4O[4 * q] = c.uOc[q];
        c.q4O[4 * q + 1] = c.vOc[q];
        c.q4O[4 * q + 2] = c.mfC[q];
        c.q4O[4 * q + 3] = c.Ph[q];
        c.pQrRz[2 * q] = c.qrA[q];
        c.pQrRz[2 * q + 1] = c.rAz[q];
    }
    if (p.useAdaptiveEVP)   // veris/evp_solver.py:65-73, the state-only factor of alphaC
        c.acf[q] = (T)(p.EVPcFac * f.recip_rA[o] / fmax(f.SeaIceMassC[o], 1e-4));
    if constexpr (sizeof(T) == 8) {   // the float64 subcycle's folded products
        const double bU = p.evpBeta * rdt, bU1 = bU + rdt;
        c.rsqrA[q] = f.recip_rA[o] / (p.PlasDefCoeff * p.PlasDefCoeff);
        c.mf4[q] = 0.25 * f.SeaIceMassC[o] * f.fCori[o];
        c.mUb1[q] = mU * bU1;
        c.mVb1[q] = mV * bU1;
        c.mUb[q] = bU * mU;
        c.mVb[q] = bU * mV;
        c.hAW[q] = 0.5 * p.cosWat * f.AreaW[o];
        c.hAS[q] = 0.5 * p.cosWat * f.AreaS[o];
        c.Phh[q] = c.Ph[q] * (0.5 / p.evpAlpha);
        if (j == 0) {
            c.rdxVh_x[i] = 0.5 * f.recip_dxV[o];
            c.dxUh_x[i] = 0.5 * f.dxU[o];
        }
        if (i == 0) {
            c.rdyUh_y[j] = 0.5 * f.recip_dyU[o];
            c.dyVh_y[j] = 0.5 * f.dyV[o];
        }
    }
    if (BASAL) {
        const double A = f.Area[o];
        double b = 0.0;
        if (A > 0.01) {
            const double hcrit = fabs(f.R_low[o]) * A / p.basalDragK1;
            b = p.basalDragK2 * log(exp(10.0 * (f.hIceMean[o] - hcrit)) + 1.0) * 0.1 *
                exp(-p.cBasalStar * (1.0 - A));
        }
        c.bfac[q] = (T)b;
    }
    const double fc = f.fCori[o];
    uint32_t fl = 0;
    fl |= f.iceMask[o] != 0.0 ? F_MC : 0;
    fl |= f.maskInC[o] != 0.0 ? F_INC : 0;
    fl |= f.iceMaskU[o] != 0.0 ? F_MU : 0;
    fl |= f.maskInU[o] != 0.0 ? F_INU : 0;
    fl |= f.iceMaskV[o] != 0.0 ? F_MV : 0;
    fl |= f.maskInV[o] != 0.0 ? F_INV : 0;
    fl |= mU != 0.0 ? F_LMU : 0;
    fl |= mV != 0.0 ? F_LMV : 0;
    fl |= fc < 0.0 ? F_SOUTH : 0;
    fl |= fc > 0.0 ? F_SPOS : 0;
    fl |= fc < 0.0 ? F_SNEG : 0;
    c.flags[q] = fl;
    c.flags16[q] = (uint16_t)fl;   // the flags use bits 0..10
    if (j == 0) {
        c.rdxU_x[i] = (T)f.recip_dxU[o];
        c.rdxV_x[i] = (T)f.recip_dxV[o];
        c.dxV_x[i] = (T)f.dxV[o];
        c.dxU_x[i] = (T)f.dxU[o];
        c.xm4[4 * i] = (T)f.recip_dxV[o];
        c.xm4[4 * i + 1] = (T)f.recip_dxU[o];
        c.xm4[4 * i + 2] = (T)f.dxU[o];
        c.xm4[4 * i + 3] = (T)f.dxV[o];
    }
    if (i == 0) {
        c.rdyV_y[j] = (T)f.recip_dyV[o];
        c.rdyU_y[j] = (T)f.recip_dyU[o];
        c.dyV_y[j] = (T)f.dyV[o];
        c.dyU_y[j] = (T)f.dyU[o];
        c.qrA_y[j] = (T)(0.25 * f.recip_rA[o]);
        c.rAz_y[j] = (T)f.rAz[o];
        c.rrAu_y[j] = (T)f.recip_rAu[o];
        c.rrAv_y[j] = (T)f.recip_rAv[o];
    }
    if (paired) {   // the register walk's layout: (u, v, sigma1, sigma2) over the four buffers
        u[4 * q] = (T)f.uIce[o];
        u[4 * q + 1] = (T)f.vIce[o];
        u[4 * q + 2] = (T)f.sigma1[o];
        u[4 * q + 3] = (T)f.sigma2[o];
    } else {
        u[q] = (T)f.uIce[o];
        v[q] = (T)f.vIce[o];
        s1[q] = (T)f.sigma1[o];
        s2[q] = (T)f.sigma2[o];
    }
    s12[q] = (T)f.sigma12[o];
}

// ------------------------------------------------ shared-memory subcycle
template <class T>
struct FastTile;
template <>
struct FastTile<float> { static constexpr int TI = 32, TJ = 32, MINB = 3; };

template <class T>
using FastSmem = TileSmem<T, FastTile<T>::TI, FastTile<T>::TJ>;

// d: caller's grid (wrap extents); reads of internal arrays use pitch lp
template <class T, bool BASAL, bool TURN>
__global__ void __launch_bounds__(FAST_THREADS, FastTile<T>::MINB)
evp_fast_kernel(Dims d, int64_t lp, HaloFill h, FastConsts<T> c, FastScalars<T> k, FastIO<T> io) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int TI = FastTile<T>::TI, TJ = FastTile<T>::TJ;
    fast_tile<T, TI, TJ, BASAL, TURN>(smem_raw, d, lp, h, c, k, io, blockIdx.y * TI, blockIdx.x * TJ);
}

template <class T, bool B, bool R>
static int launch_fast(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c,
                       const FastScalars<T> &k, const FastIO<T> &io, cudaStream_t st) {
    auto kern = evp_fast_kernel<T, B, R>;
    static_assert(sizeof(T) == 4, "float64 subcycles run the float64 tile kernel (evp_fast64.cu)");
    const size_t sm = FastSmem<T>::bytes();
    static std::atomic<bool> configured[MAX_DEVICES];
    if (!smem_configured(configured, kern, (int)sm)) return VERIS_ERR_LAUNCH;
    dim3 grid((d.NY + FastTile<T>::TJ - 1) / FastTile<T>::TJ, (d.NX + FastTile<T>::TI - 1) / FastTile<T>::TI);
    kern<<<grid, FAST_THREADS, sm, st>>>(d, lp, h, c, k, io);
    return launch_status();
}

template <class T>
int fast_prep(const Dims &d, const VerisParams &p, const Fields<double> &f, const FastConsts<T> &c,
              T *const state0[5], cudaStream_t st) {
    const int64_t lp = internal_pitch(d.NY);
    dim3 g2((d.NY + 31) / 32, (d.NX + 7) / 8);
    if (p.basalDragK2 != 0.0)
        fast_prep_kernel<T, true><<<g2, dim3(32, 8), 0, st>>>(p, f, d, lp, c, state0[0], state0[1], state0[2],
                                                              state0[3], state0[4], 0);
    else
        fast_prep_kernel<T, false><<<g2, dim3(32, 8), 0, st>>>(p, f, d, lp, c, state0[0], state0[1], state0[2],
                                                               state0[3], state0[4], 0);
    return launch_status();
}

template <class T>
int fast_subcycle(const Dims &d, const HaloFill &h, const FastConsts<T> &c, const FastScalars<T> &k,
                  const FastIO<T> &io, bool basal, bool turn, cudaStream_t st) {
    if constexpr (sizeof(T) == 8) {
        return fast64_subcycle(d, h, c, k, io, basal, turn, st);
    } else {
        const int64_t lp = internal_pitch(d.NY);
        if (basal)
            return turn ? launch_fast<T, true, true>(d, lp, h, c, k, io, st)
                        : launch_fast<T, true, false>(d, lp, h, c, k, io, st);
        return turn ? launch_fast<T, false, true>(d, lp, h, c, k, io, st)
                    : launch_fast<T, false, false>(d, lp, h, c, k, io, st);
    }
}

template int fast_prep<float>(const Dims &, const VerisParams &, const Fields<double> &, const FastConsts<float> &,
                              float *const[5], cudaStream_t);
template int fast_prep<double>(const Dims &, const VerisParams &, const Fields<double> &, const FastConsts<double> &,
                               double *const[5], cudaStream_t);
template int fast_subcycle<float>(const Dims &, const HaloFill &, const FastConsts<float> &, const FastScalars<float> &,
                                  const FastIO<float> &, bool, bool, cudaStream_t);
template int fast_subcycle<double>(const Dims &, const HaloFill &, const FastConsts<double> &,
                                   const FastScalars<double> &, const FastIO<double> &, bool, bool, cudaStream_t);

template <class T>
static size_t tape_field(const Dims &d) { return rup256((size_t)d.NX * internal_pitch(d.NY) * sizeof(T)); }

// tape != nullptr: every subcycle is kept, slot k (tape_slot_fields arrays
// of tape_field bytes each, pitch lp) holding the state after k subcycles;
// in float64 slot k holds (u_k, v_k, Delta_k, zeta_k, cDrag_k), the
// velocities after k subcycles and the viscosity and drag terms subcycle
// k + 1 computes from them (the adjoint needs no stresses; they run in the
// workspace's state buffers); in float32 the register walk's state after k
// subcycles, then Delta_k, zeta_k, cDrag_k (constant alpha)
template <class T>
static int evp_fast(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs64, int n, T *uo, T *vo,
                    T *s1o, T *s2o, T *s12o, void *ws, size_t wsb, int allow_tma, veris_stream_t s,
                    T *tape = nullptr, size_t tape_bytes = 0, int walk_variant = 0) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs64 && uo && vo && s1o && s2o && s12o, VERIS_ERR_ARG);
    VERIS_REQUIRE(n >= 1, VERIS_ERR_ARG);
    const bool walker = sizeof(T) == 4 && (allow_tma >= 4 || allow_tma < 0);
    // the walk's own subcycle chain runs on its state layout; a float32 tape
    // keeps that layout in every slot (the adjoint reads it so)
    const bool paired = walker;
    if (walker ? walk_support(*p) : fast_support(*p)) return VERIS_ERR_UNSUPPORTED;
    const bool adapt = p->useAdaptiveEVP != 0;
    FastConsts<T> c;
    T *state[2][5];
    int *status = nullptr;
    const size_t need = fast_layout<T>(d, nullptr, &c, state, &status);
    VERIS_REQUIRE(ws && wsb >= need, VERIS_ERR_WORKSPACE);
    fast_layout<T>(d, static_cast<char *>(ws), &c, state, &status);
    const int64_t lp = internal_pitch(d.NY);
    cudaStream_t st = (cudaStream_t)s;
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return VERIS_ERR_LAUNCH;
    const Fields<double> &f = *reinterpret_cast<const Fields<double> *>(vs64);
    const bool basal = p->basalDragK2 != 0.0, turn = p->sinWat != 0.0;
    const size_t tf = tape_field<T>(d);
    constexpr int W = tape_slot_fields<T>();
    if (tape) VERIS_REQUIRE(tape_bytes >= (size_t)(n + 1) * W * tf, VERIS_ERR_WORKSPACE);
    auto tslot = [&](int sl, int q) { return reinterpret_cast<T *>(reinterpret_cast<char *>(tape) + ((size_t)sl * W + q) * tf); };
    // float64 tapes: the stresses stay in the workspace's state buffers
    constexpr bool rich = sizeof(T) == 8;
    T *s0[5];
    for (int q = 0; q < 5; ++q) s0[q] = tape && !(rich && q >= 2) ? tslot(0, q) : state[0][q];
    dim3 g2((d.NY + 31) / 32, (d.NX + 7) / 8);
    if (basal)
        fast_prep_kernel<T, true><<<g2, dim3(32, 8), 0, st>>>(*p, f, d, lp, c, s0[0], s0[1], s0[2], s0[3], s0[4],
                                                              paired ? 1 : 0);
    else
        fast_prep_kernel<T, false><<<g2, dim3(32, 8), 0, st>>>(*p, f, d, lp, c, s0[0], s0[1], s0[2], s0[3], s0[4],
                                                               paired ? 1 : 0);
    int stt = launch_status();
    if (stt != VERIS_OK) return stt;
    const FastScalars<T> k = fast_scalars<T>(*p);
    const HaloFill h = halo_fill_of(*p);
    T *outs[5] = {uo, vo, s1o, s2o, s12o};
    if (tape) {
        for (int it = 0; it < n; ++it) {
            bool done = false;
            if constexpr (sizeof(T) == 4) {
                if (allow_tma >= 4 || allow_tma < 0) {   // float32 tape written by the register-walking kernel
                    float *const from[2][5] = {{tslot(it, 0), tslot(it, 1), tslot(it, 2), tslot(it, 3), tslot(it, 4)},
                                               {nullptr, nullptr, nullptr, nullptr, nullptr}};
                    float *const to[5] = {tslot(it + 1, 0), tslot(it + 1, 1), tslot(it + 1, 2), tslot(it + 1, 3),
                                          tslot(it + 1, 4)};
                    float *const rich[3] = {tslot(it, 5), tslot(it, 6), tslot(it, 7)};
                    if ((stt = evp_walk_subcycles(adapt, true, d, h, c, k, from, to, lp, 1, basal, turn,
                                                  allow_tma < 0 ? 0 : allow_tma, walk_variant, st, true, nullptr,
                                                  adapt ? nullptr : rich)) != VERIS_OK)
                        return stt;
                    done = true;
                }
            }
            if (!done) {
                FastIO<T> io{tslot(it, 0), tslot(it, 1), tslot(it, 2), tslot(it, 3), tslot(it, 4),
                             tslot(it + 1, 0), tslot(it + 1, 1), tslot(it + 1, 2), tslot(it + 1, 3), tslot(it + 1, 4),
                             lp};
                if constexpr (rich) {
                    T *const *a = state[it % 2], *const *b = state[(it + 1) % 2];
                    io.s1 = a[2]; io.s2 = a[3]; io.s12 = a[4];
                    io.s1o = b[2]; io.s2o = b[3]; io.s12o = b[4];
                    io.tDel = tslot(it, 2); io.tZeta = tslot(it, 3); io.tCd = tslot(it, 4);
                }
                if ((stt = fast_subcycle<T>(d, h, c, k, io, basal, turn, st)) != VERIS_OK) return stt;
            }
        }
        if constexpr (sizeof(T) == 4) {
            if (walker) {   // the last slot in the walk's layout
                float *const o5[5] = {outs[0], outs[1], outs[2], outs[3], outs[4]};
                return evp_walk_unpack(d, tslot(n, 0), tslot(n, 4), o5, d.ld, st);
            }
        }
        for (int q = 0; q < 5; ++q) {
            const T *from = rich && q >= 2 ? state[n % 2][q] : tslot(n, q);
            if (cudaMemcpy2DAsync(outs[q], d.ld * sizeof(T), from, lp * sizeof(T), d.NY * sizeof(T), d.NX,
                                  cudaMemcpyDeviceToDevice, st) != cudaSuccess)
                return VERIS_ERR_LAUNCH;
        }
        return VERIS_OK;
    }
    if constexpr (sizeof(T) == 4) {
        if (allow_tma >= 4 || allow_tma < 0)   // register-walking kernel, allow_tma rows per walk (< 0: auto)
            return evp_walk_subcycles(adapt, paired, d, h, c, k, state, outs, d.ld, n, basal, turn,
                                      allow_tma < 0 ? 0 : allow_tma, walk_variant, st, false, status);
        if (allow_tma) {
            stt = evp_tma_subcycles(d, h, c, k, state, outs, d.ld, n, status, basal, turn, st);
            if (stt != VERIS_ERR_UNSUPPORTED) return stt;
        }
    }
    const T *cur[5] = {state[0][0], state[0][1], state[0][2], state[0][3], state[0][4]};
    for (int it = 0; it < n; ++it) {
        const bool last = it == n - 1;
        T *const *dst = last ? outs : state[(it + 1) % 2];
        FastIO<T> io{cur[0], cur[1], cur[2], cur[3], cur[4], dst[0], dst[1], dst[2], dst[3], dst[4],
                     last ? d.ld : lp};
        if constexpr (sizeof(T) == 8)
            stt = fast64_subcycle(d, h, c, k, io, basal, turn, st);
        else if (basal)
            stt = turn ? launch_fast<T, true, true>(d, lp, h, c, k, io, st) : launch_fast<T, true, false>(d, lp, h, c, k, io, st);
        else
            stt = turn ? launch_fast<T, false, true>(d, lp, h, c, k, io, st) : launch_fast<T, false, false>(d, lp, h, c, k, io, st);
        if (stt != VERIS_OK) return stt;
        for (int q = 0; q < 5; ++q) cur[q] = dst[q];
    }
    return VERIS_OK;
}

}  // namespace veris

using namespace veris;

extern "C" {

size_t veris_evp_fast_workspace_bytes(const VerisGrid *g, int32_t elem_size) {
    Dims d;
    if (check_grid(g, &d) != VERIS_OK) return 0;
    int *status;
    if (elem_size == 4) {
        FastConsts<float> c;
        float *s[2][5];
        return fast_layout<float>(d, nullptr, &c, s, &status);
    }
    if (elem_size == 8) {
        FastConsts<double> c;
        double *s[2][5];
        return fast_layout<double>(d, nullptr, &c, s, &status);
    }
    return 0;
}

int veris_evp_fast_settings_check(const VerisParams *p) { return p ? fast_support(*p) : V_ADAPT; }

int veris_evp_walk_settings_check(const VerisParams *p) { return p ? walk_support(*p) : V_SLIP; }

int veris_evp_fast_check(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t *viol_device,
                         veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && viol_device, VERIS_ERR_ARG);
    cudaStream_t st = (cudaStream_t)s;
    if (cudaMemsetAsync(viol_device, 0, sizeof(int32_t), st) != cudaSuccess) return VERIS_ERR_LAUNCH;
    dim3 g2((d.NY + 31) / 32, (d.NX + 7) / 8);
    fast_check_kernel<<<g2, dim3(32, 8), 0, st>>>(*reinterpret_cast<const Fields<double> *>(vs), d, viol_device);
    return launch_status();
}

int veris_evp_fast_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                              float *u, float *v, float *s1, float *s2, float *s12, void *ws, size_t wsb,
                              veris_stream_t s) {
    return evp_fast<float>(g, p, vs, n, u, v, s1, s2, s12, ws, wsb, 1, s);
}

int veris_evp_walk_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                              int32_t rows, int32_t variant, float *u, float *v, float *s1, float *s2, float *s12,
                              void *ws, size_t wsb, veris_stream_t s) {
    VERIS_REQUIRE((rows == 0 || (rows >= 4 && rows <= 4096)) && variant >= 0 && variant < N_WALK_VARIANTS, VERIS_ERR_ARG);
    return evp_fast<float>(g, p, vs, n, u, v, s1, s2, s12, ws, wsb, rows == 0 ? -1 : rows, s, nullptr, 0, variant);
}

int veris_evp_smem_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                              float *u, float *v, float *s1, float *s2, float *s12, void *ws, size_t wsb,
                              veris_stream_t s) {
    return evp_fast<float>(g, p, vs, n, u, v, s1, s2, s12, ws, wsb, 0, s);
}

int veris_evp_fast_solver_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                              double *u, double *v, double *s1, double *s2, double *s12, void *ws, size_t wsb,
                              veris_stream_t s) {
    return evp_fast<double>(g, p, vs, n, u, v, s1, s2, s12, ws, wsb, 0, s);
}

size_t veris_evp_tape_bytes(const VerisGrid *g, int32_t elem_size, int32_t n) {
    Dims d;
    if (check_grid(g, &d) != VERIS_OK || n < 1) return 0;
    if (elem_size == 8) return (size_t)(n + 1) * tape_slot_fields<double>() * tape_field<double>(d);
    if (elem_size == 4) return (size_t)(n + 1) * tape_slot_fields<float>() * tape_field<float>(d);
    return 0;
}

int veris_evp_fast_tape_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                            double *u, double *v, double *s1, double *s2, double *s12, double *tape,
                            size_t tape_bytes, void *ws, size_t wsb, veris_stream_t s) {
    VERIS_REQUIRE(tape, VERIS_ERR_ARG);
    return evp_fast<double>(g, p, vs, n, u, v, s1, s2, s12, ws, wsb, 0, s, tape, tape_bytes);
}

int veris_evp_fast_tape_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                            float *u, float *v, float *s1, float *s2, float *s12, float *tape, size_t tape_bytes,
                            void *ws, size_t wsb, veris_stream_t s) {
    VERIS_REQUIRE(tape, VERIS_ERR_ARG);
    return evp_fast<float>(g, p, vs, n, u, v, s1, s2, s12, ws, wsb, -1, s, tape, tape_bytes);   // walking kernel
}

int veris_evp_fast_status(const void *ws, int32_t *status_host, veris_stream_t s) {
    VERIS_REQUIRE(ws && status_host, VERIS_ERR_ARG);
    cudaStream_t st = (cudaStream_t)s;
    if (cudaMemcpyAsync(status_host, ws, sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return VERIS_ERR_LAUNCH;
    if (cudaStreamSynchronize(st) != cudaSuccess) return VERIS_ERR_LAUNCH;
    return VERIS_OK;
}

}  // extern "C"
