// Shared pieces of the fast EVP forms (veris/evp_solver.py:21-319): the
// folded step constants, their once-per-step prep kernel, the support check
// and the launch interface of the TMA-staged kernel.
//
// Internal arrays (constants and the ping-pong state) use their own pitch
// `lp`, a multiple of 8 elements, so that every row starts on a 32-byte
// boundary (TMA needs 16); the caller's arrays keep the caller's pitch.
#pragma once

#include "stencil.cuh"

namespace veris {

// flag bits of the per-cell 32-bit word
enum : uint32_t {
    F_MC = 1u << 0,    // iceMask
    F_INC = 1u << 1,   // maskInC
    F_MU = 1u << 2,    // iceMaskU
    F_INU = 1u << 3,   // maskInU
    F_MV = 1u << 4,    // iceMaskV
    F_INV = 1u << 5,   // maskInV
    F_LMU = 1u << 6,   // SeaIceMassU != 0
    F_LMV = 1u << 7,   // SeaIceMassV != 0
    F_SOUTH = 1u << 8, // fCori < 0
    F_SPOS = 1u << 9,  // sign(fCori) = +1
    F_SNEG = 1u << 10, // sign(fCori) = -1
};

// settings and state properties the fast forms do not cover
enum : int {
    V_ADAPT = 1, V_SLIP = 2, V_SECOND = 4, V_PRESS = 8, V_KTERMS = 16, V_MASKS = 32, V_METRIC = 64,
    V_AREA2D = 128   // cell areas vary along both axes: the register walk (not the tile forms) needs them along j only
};

// device status word bits (first word of the fast workspace)
enum : int { S_TMA_TIMEOUT = 1, S_WALK_TIMEOUT = 2 };

template <class T>
struct FastConsts {
    // C points
    T *Ph;     // 0.5 * P * (1 + tensileStrFac)
    T *mfC;    // 0.5 * SeaIceMassC * fCori
    T *qrA;    // 0.25 / rA
    T *rAz;    // rAz (Z points)
    T *bfac;   // basal drag factor (only with basalDragK2 != 0)
    // U points
    T *mU, *cU, *AW, *uOc, *rrAu;   // cU = mU/dt * u^{n-1} + WindForcingX
    // V points
    T *mV, *cV, *AS, *vOc, *rrAv;
    T *acf;    // adaptive EVP: EVPcFac * recip_rA / max(SeaIceMassC, 1e-4) (alphaC = sqrt(zeta * acf))
    uint32_t *flags;
    T *rdxU_x, *rdxV_x, *dxV_x, *dxU_x;   // grid lengths varying with i
    T *xm4;    // the same four per row, interleaved (rdxV, rdxU, dxU, dxV): one 16-byte load
    // the register walk's inputs in 16- and 8-byte groups, pitch lp:
    // (cU, cV, AW, AS), (mU, mV, rrAu, rrAv), (uOc, vOc, mfC, Ph), (qrA, rAz)
    T *q4U, *q4M, *q4O, *pQrRz;
    T *rdyV_y, *rdyU_y, *dyV_y, *dyU_y;   // grid lengths varying with j
    T *qrA_y, *rAz_y, *rrAu_y, *rrAv_y;   // the register walk's cell areas (0.25/rA, rAz, 1/rAu, 1/rAv), along j
    T *pMUV;   // (mU, mV) pairs, pitch lp: the register walk's U/V masses when its areas are 1-D
    uint16_t *flags16;   // the flag word's 11 bits, pitch lp: the register walk's copy
    int *wprog;          // the persistent walk's progress counters, one per walk (MAX_WALKS)
    // float64 only (evp_fast64.cu): products the float64 subcycle would
    // otherwise form on every subcycle, folded once per step
    T *rsqrA;        // recip_rA / e^2 (C points)
    T *mf4;          // 0.25 * SeaIceMassC * fCori
    T *mUb1, *mVb1;  // mass * (beta + 1) / dt (U, V points)
    T *mUb, *mVb;    // mass * beta / dt
    T *hAW, *hAS;    // 0.5 * cos(water turning angle) * AreaW, AreaS
    T *Phh;          // Ph / (2 alpha): its division by Delta + Delta_min gives zeta / (2 alpha)
    T *rdxVh_x, *dxUh_x;   // 0.5 * recip_dxV, 0.5 * dxU (along i)
    T *rdyUh_y, *dyVh_y;   // 0.5 * recip_dyU, 0.5 * dyV (along j)
};
constexpr int N_FAST_2D = 16;
constexpr int MAX_WALKS = 16384;   // walks of one persistent float32 launch (resident warps bound it)
constexpr int N_F64_2D = 9;

__host__ __device__ inline int64_t internal_pitch(int NY) { return ((int64_t)NY + 7) / 8 * 8; }

inline size_t rup256(size_t x) { return (x + 255) / 256 * 256; }

// Carves the fast workspace: status word, constants, two state buffers.
template <class T>
size_t fast_layout(const Dims &d, char *base, FastConsts<T> *c, T *state[2][5], int **status) {
    const int64_t lp = internal_pitch(d.NY);
    const size_t f2 = rup256((size_t)d.NX * lp * sizeof(T));
    const size_t fl = rup256((size_t)d.NX * lp * sizeof(uint32_t));
    const size_t fx = rup256((size_t)d.NX * sizeof(T)), fy = rup256((size_t)d.NY * sizeof(T));
    size_t off = 0;
    auto take = [&](size_t n) { char *p = base ? base + off : nullptr; off += n; return p; };
    *status = reinterpret_cast<int *>(take(256));
    T **two[N_FAST_2D] = {&c->Ph, &c->mfC, &c->qrA, &c->rAz, &c->bfac, &c->mU, &c->cU, &c->AW,
                          &c->uOc, &c->rrAu, &c->mV, &c->cV, &c->AS, &c->vOc, &c->rrAv, &c->acf};
    for (int q = 0; q < N_FAST_2D; ++q) *two[q] = reinterpret_cast<T *>(take(f2));
    c->flags = reinterpret_cast<uint32_t *>(take(fl));
    T **xs[4] = {&c->rdxU_x, &c->rdxV_x, &c->dxV_x, &c->dxU_x};
    T **ys[8] = {&c->rdyV_y, &c->rdyU_y, &c->dyV_y, &c->dyU_y, &c->qrA_y, &c->rAz_y, &c->rrAu_y, &c->rrAv_y};
    for (int q = 0; q < 4; ++q) *xs[q] = reinterpret_cast<T *>(take(fx));
    c->xm4 = reinterpret_cast<T *>(take(rup256((size_t)d.NX * 4 * sizeof(T))));
    T **quads[3] = {&c->q4U, &c->q4M, &c->q4O};
    for (int q = 0; q < 3; ++q) *quads[q] = reinterpret_cast<T *>(take(4 * f2));
    c->pQrRz = reinterpret_cast<T *>(take(2 * f2));
    c->pMUV = reinterpret_cast<T *>(take(2 * f2));
    c->flags16 = reinterpret_cast<uint16_t *>(take(rup256((size_t)d.NX * lp * sizeof(uint16_t))));
    c->wprog = reinterpret_cast<int *>(take(rup256((size_t)MAX_WALKS * sizeof(int))));
    for (int q = 0; q < 8; ++q) *ys[q] = reinterpret_cast<T *>(take(fy));
    // the float64 subcycle's folded products (no space for float32)
    const bool f64 = sizeof(T) == 8;
    T **f64s[N_F64_2D] = {&c->rsqrA, &c->mf4, &c->mUb1, &c->mVb1, &c->mUb, &c->mVb, &c->hAW, &c->hAS, &c->Phh};
    for (int q = 0; q < N_F64_2D; ++q) *f64s[q] = reinterpret_cast<T *>(take(f64 ? f2 : 0));
    c->rdxVh_x = reinterpret_cast<T *>(take(f64 ? fx : 0));
    c->dxUh_x = reinterpret_cast<T *>(take(f64 ? fx : 0));
    c->rdyUh_y = reinterpret_cast<T *>(take(f64 ? fy : 0));
    c->dyVh_y = reinterpret_cast<T *>(take(f64 ? fy : 0));
    for (int b = 0; b < 2; ++b)
        for (int q = 0; q < 5; ++q) state[b][q] = reinterpret_cast<T *>(take(f2));
    return off;
}

template <class T>
struct FastScalars {
    T alpha_m1, ralpha, rsq, deltaMin, kp;   // rheology
    T bU, bU1;                               // beta/dt, (beta+1)/dt
    T halfCos, sinW;                         // 0.5 cos(turning angle), sin(turning angle)
    T dN, dS, dN2, dS2, cmin, cmin2;         // ocean drag
    T U02;                                   // basal U0^2
    T rdt, aMin;                             // 1/dt, aEVPalphaMin (adaptive EVP)
};

template <class T>
FastScalars<T> fast_scalars(const VerisParams &p) {
    FastScalars<T> s;
    s.alpha_m1 = (T)(p.evpAlpha - 1.0);
    s.ralpha = (T)(1.0 / p.evpAlpha);
    s.rsq = (T)(1.0 / (p.PlasDefCoeff * p.PlasDefCoeff));
    s.deltaMin = (T)p.deltaMin;
    s.kp = (T)(2.0 * (1.0 - p.tensileStrFac) / (1.0 + p.tensileStrFac));
    s.bU = (T)(p.evpBeta * p.recip_deltatDyn);
    s.bU1 = (T)(p.evpBeta * p.recip_deltatDyn + p.recip_deltatDyn);
    s.halfCos = (T)(0.5 * p.cosWat);
    s.sinW = (T)p.sinWat;
    const double dN = p.waterIceDrag * p.rhoSea, dS = p.waterIceDrag_south * p.rhoSea;
    s.dN = (T)dN;
    s.dS = (T)dS;
    s.dN2 = (T)(dN * dN);
    s.dS2 = (T)(dS * dS);
    s.cmin = (T)p.cDragMin;
    s.cmin2 = (T)(p.cDragMin * p.cDragMin);
    s.U02 = (T)(p.basalDragU0 * p.basalDragU0);
    s.rdt = (T)p.recip_deltatDyn;
    s.aMin = (T)p.aEVPalphaMin;
    return s;
}

template <class T>
struct FastIO {
    const T *u, *v, *s1, *s2, *s12;   // state at the start of the subcycle (internal pitch)
    T *uo, *vo, *s1o, *s2o, *s12o;    // state at its end
    int64_t ldo;                      // pitch of the outputs
    // float64 tapes (pitch ldo, C points; all three or none): Delta and
    // zeta of the subcycle's viscosities and its ocean-drag coefficient,
    // which the adjoint reads instead of recomputing
    T *tDel = nullptr, *tZeta = nullptr, *tCd = nullptr;
};

int fast_support(const VerisParams &p);
// the settings the register-walking kernel does not cover (it runs adaptive EVP)
inline int walk_support(const VerisParams &p) { return fast_support(p) & ~V_ADAPT; }

// Host helpers of the fast forms (instantiated for float and double):
// the once-per-step fold of the constants (and of the initial state into
// state0), and one shared-memory-form subcycle.
template <class T>
int fast_prep(const Dims &d, const VerisParams &p, const Fields<double> &f, const FastConsts<T> &c,
              T *const state0[5], cudaStream_t st);
template <class T>
int fast_subcycle(const Dims &d, const HaloFill &h, const FastConsts<T> &c, const FastScalars<T> &k,
                  const FastIO<T> &io, bool basal, bool turn, cudaStream_t st);
// one float64 subcycle with the float64 tile kernel (evp_fast64.cu)
int fast64_subcycle(const Dims &d, const HaloFill &h, const FastConsts<double> &c, const FastScalars<double> &k,
                    const FastIO<double> &io, bool basal, bool turn, cudaStream_t st);

// n float32 subcycles with the TMA-staged kernel, reading state[0] first and
// writing the last subcycle into outs.  Returns VERIS_ERR_UNSUPPORTED (having
// launched nothing) when the tensor maps cannot be built; the caller then
// uses the shared-memory form.
int evp_tma_subcycles(const Dims &d, const HaloFill &h, const FastConsts<float> &c, const FastScalars<float> &k,
                      float *const state[2][5], float *const outs[5], int64_t ldo, int n, int *status, bool basal,
                      bool turn, cudaStream_t st);
bool evp_tma_available();
// the same with the register-walking kernel: one warp per 28-column strip
// walking `rows` output rows, compiled form `variant` (loop unroll x register
// budget), reading state[0] first
// compiled forms of the register-walking kernel (evp_walk.cu)
constexpr int N_WALK_VARIANTS = 4;
// paired: the state buffers hold the walk's own layout ((u, v, sigma1,
// sigma2) in 16 bytes per point over the four buffers, sigma12 alone; the
// prep writes the first state so); the last subcycle writes planar `outs`
// unless paired_outs.  `rich` (one paired subcycle with paired outs,
// constant alpha): the subcycle's Delta, zeta and ocean-drag coefficient at
// every point, pitch lp, into rich[0..2] (a float32 tape slot's last three
// fields)
int evp_walk_subcycles(bool adapt, bool paired, const Dims &d, const HaloFill &h, const FastConsts<float> &c,
                       const FastScalars<float> &k,
                       float *const state[2][5], float *const outs[5], int64_t ldo, int n, bool basal, bool turn,
                       int rows, int variant, cudaStream_t st, bool paired_outs = false, int *status = nullptr,
                       float *const *rich = nullptr);

// Fields per slot of an EVP tape (each the size of one internal array):
// float64 (u, v, Delta, zeta, cDrag), the stresses staying in the
// workspace; float32 the register walk's state, (u, v, sigma1, sigma2) per
// point over four fields and sigma12, then Delta, zeta and cDrag
template <class T>
constexpr int tape_slot_fields() { return sizeof(T) == 8 ? 5 : 8; }
// the walk's layout (its first four fields at `quad`, sigma12 at `s12`, pitch
// lp) -> five planar arrays of pitch ldo
int evp_walk_unpack(const Dims &d, const float *quad, const float *s12, float *const outs[5], int64_t ldo,
                    cudaStream_t st);

template <class T>
__device__ __forceinline__ T one_if(uint32_t f, uint32_t bit) { return (f & bit) ? T(1) : T(0); }

}  // namespace veris
