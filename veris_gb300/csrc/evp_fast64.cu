// Float64 fast-form mEVP subcycle (veris/evp_solver.py:21-254), arranged for
// GB300's float64 pipe.
//
// GB300 executes float64 arithmetic at 2 lanes per SM and cycle, 1/64 of its
// float32 rate, so a float64 subcycle is bound by the number of float64-pipe
// instructions per cell (the HBM traffic is ~0.06 of the roofline).  The
// kernel computes the subcycle of the shared-memory tile in evp_tile.cuh
// (same stages, same wrap and halo semantics) with about half the float64
// instructions:
//
// * the 0/1 masks are applied as selects on the integer pipe, not as
//   multiplications; the wet-point count of the sigma12 average selects a
//   precomputed coefficient;
// * products of step constants are folded once per step by the prep
//   (recip_rA/e^2, mass*(beta+1)/dt, mass*beta/dt, 0.5*cos*Area, 0.25*m*f,
//   halved grid lengths, and 1/(2 alpha) into the ice strength factor, so
//   that its division by Delta + Delta_min gives zeta/(2 alpha), the stress
//   update's coefficient), one multiplication fewer per use; the drag
//   coefficient is the square root of the product the drag floor's test
//   forms;
// * divisions and square roots start from the hardware's approximate
//   reciprocal and reciprocal square root (rcp/rsqrt.approx.ftz.f64) and
//   add the first terms of the series of the exact correction: with
//   e = 1 - b*r0, 1/b = r0/(1 - e) = r0*(1 + e + e^2 + ...); with
//   s0 = x*y and r = 1 - s0*y, sqrt(x) = s0*(1 - r)^(-1/2) = s0*(1 + r/2 +
//   3r^2/8 + ...) (the Newton-Raphson correction taken to second order,
//   P. Markstein, IBM J. Res. Dev. 34 (1990) 111).  Four and five float64
//   instructions, no slow path; a warp whose operands leave a safe exponent
//   range uses IEEE division or square root instead;
// * warps whose cells all have zero ice strength skip the viscosity's
//   square root and division (zeta = 0, which the formula gives), warps on
//   land skip the velocity division;
// * work units of at most 24 rows x 32 columns by default, three 256-thread
//   CTAs per SM (16 and 32 rows: four and two; the larger the unit, the
//   less ring work but the fewer resident warps to cover the float64 pipe's
//   latency), the launch ending on a round of small units so that the SMs
//   run out of work together.
#include "evp_fast.cuh"
#include "f64math.cuh"

namespace veris {

struct F64Scalars {
    double am1r;             // (alpha - 1) / alpha
    double kp2;              // 2 * (press factor 2(1 - tsf)/(1 + tsf))
    double rsq, deltaMin;    // 1/e^2, Delta_min
    double dcq2N, dcq2S;     // 0.25 * (rhoSea * waterIceDrag)^2, north and south
    double cmin, cmin2;      // cDragMin, its square
    double U02;              // basal drag U0^2
    double sinW;             // sin(water turning angle)
    double nh1, nh2, nh3, nh4;   // 1 / n: the sigma12 average over n wet C points (of zeta / (2 alpha))
    double twoAlpha;             // 2 alpha: zeta from zeta / (2 alpha), for the tape
};

static F64Scalars f64_scalars(const FastScalars<double> &k) {
    F64Scalars s;
    s.am1r = k.alpha_m1 * k.ralpha;
    s.kp2 = 2.0 * k.kp;
    s.rsq = k.rsq;
    s.deltaMin = k.deltaMin;
    s.dcq2N = 0.25 * k.dN2;
    s.dcq2S = 0.25 * k.dS2;
    s.cmin = k.cmin;
    s.cmin2 = k.cmin2;
    s.U02 = k.U02;
    s.sinW = k.sinW;
    s.nh1 = 1.0;
    s.nh2 = 0.5;
    s.nh3 = 1.0 / 3.0;
    s.nh4 = 0.25;
    s.twoAlpha = 2.0 / k.ralpha;
    return s;
}

// ------------------------------------------------------------------ tile
constexpr int F64_THREADS = 256;

// TI output rows x 32 columns per CTA; 16-, 24- and 32-row tiles fit 4, 3
// and 2 CTAs per SM (smaller tiles: more resident warps, more ring work)
template <int TI_>
struct Smem64 {
    static constexpr int TI = TI_, TJ = 32;
    static constexpr int WS = TJ + 4, HS = TI + 4, NS = WS * HS;   // u, v, flags: origin -2
    static constexpr int WZ = TJ + 3, HZ = TI + 3, NZ = WZ * HZ;   // e12 and rAz*e12^2: origin -1
    static constexpr int WB = TJ + 2, HB = TI + 2, NB = WB * HB;   // zeta: origin -1
    static constexpr int WC = TJ + 1, HC = TI + 1, NC = WC * HC;   // C ring (origin -1), Z (origin 0)
    static constexpr size_t bytes(bool basal) {
        return sizeof(double) * (size_t)(2 * NS + 2 * NZ + NB + (basal ? 6 : 5) * NC) + sizeof(uint32_t) * NS;
    }
};
constexpr int f64_min_blocks(int ti) { return ti <= 16 ? 4 : (ti <= 24 ? 3 : 2); }
static_assert(2 * (Smem64<32>::bytes(true) + 1024) <= 228 * 1024, "two 32-row CTAs per SM");
static_assert(3 * (Smem64<24>::bytes(false) + 1024) <= 228 * 1024, "three 24-row CTAs per SM");
static_assert(4 * (Smem64<16>::bytes(true) + 1024) <= 228 * 1024, "four 16-row CTAs per SM");

// Work units, one per CTA, in dispatch order: first the P1 pieces of rows
// [0, R1) of every 32-column strip, then the P2 smaller pieces of rows
// [R1, NX) of every strip (at most TI rows each, for which the shared memory
// is sized).  The hardware hands CTAs to SMs in block order as slots free up,
// so the launch ends on the small pieces and the SMs run out of work
// together instead of on a thin last wave of full tiles.
struct F64Units {
    int P1, R1, P2, U1;
};

template <int TI, bool BASAL, bool TURN, bool TAPE>
__global__ void __launch_bounds__(F64_THREADS, f64_min_blocks(TI))
evp_f64_kernel(Dims d, int64_t lp, HaloFill h, FastConsts<double> c, F64Scalars k, FastIO<double> io,
               F64Units w) {
    using S = Smem64<TI>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sU = reinterpret_cast<double *>(smem_raw);
    double *sV = sU + S::NS;
    double *sE12 = sV + S::NS;
    double *sZq = sE12 + S::NZ;   // rAz*e12^2 in stages A/B, then sigma12 (origin 0, pitch WC)
    double *sZeta = sZq + S::NZ;
    double *sS11 = sZeta + S::NB;
    double *sS22 = sS11 + S::NC;
    double *sCd = sS22 + S::NC;
    double *sFv = sCd + S::NC;
    double *sFu = sFv + S::NC;
    double *sCb = sFu + S::NC;    // basal drag only
    uint32_t *sF = reinterpret_cast<uint32_t *>(sCb + (BASAL ? S::NC : 0));
    double *sS12 = sZq;
    int i0, ti, j0;
    {
        const int unit = blockIdx.x;
        const bool big = unit < w.U1;
        const int P = big ? w.P1 : w.P2, v = big ? unit : unit - w.U1;
        const int r0 = big ? 0 : w.R1, rows = big ? w.R1 : d.NX - w.R1, pc = v % P;
        i0 = r0 + (int)((int64_t)pc * rows / P);
        ti = r0 + (int)((int64_t)(pc + 1) * rows / P) - i0;
        j0 = (v / P) * S::TJ;
    }
    // the unit's region sizes (ti <= TI rows)
    const int nS = (ti + 4) * S::WS, nZ = (ti + 3) * S::WZ, nB = (ti + 2) * S::WB, nC = (ti + 1) * S::WC;
    const int tid = threadIdx.x;
    constexpr unsigned ALL = 0xffffffffu;
#define IS(li, lj) (((li) + 2) * S::WS + ((lj) + 2))
#define IZ(li, lj) (((li) + 1) * S::WZ + ((lj) + 1))
#define IB(li, lj) (((li) + 1) * S::WB + ((lj) + 1))
#define IC(li, lj) (((li) + 1) * S::WC + ((lj) + 1))
#define IZZ(li, lj) ((li) * S::WC + (lj))
    // ocean velocities at tile offsets (read through L1; not staged)
    auto uoc = [&](int li, int lj) { return __ldg(c.uOc + (int64_t)d.wxt(i0 + li) * lp + d.wyt(j0 + lj)); };
    auto voc = [&](int li, int lj) { return __ldg(c.vOc + (int64_t)d.wxt(i0 + li) * lp + d.wyt(j0 + lj)); };

    // ---- stage u, v and the flags of the tile plus a 2-cell ring
    for (int idx = tid; idx < nS; idx += F64_THREADS) {
        const int li = idx / S::WS - 2, lj = idx % S::WS - 2;
        const int64_t o = (int64_t)d.wxt(i0 + li) * lp + d.wyt(j0 + lj);
        sU[idx] = __ldg(io.u + o);
        sV[idx] = __ldg(io.v + o);
        sF[idx] = __ldg(c.flags + o);
    }
    __syncthreads();

    // ---- A: e12 at Z points [-1, TI+1] x [-1, TJ+1] (veris/dynamics_routines.py:160-175)
    for (int base = 0; base < nZ; base += F64_THREADS) {
        const int idx = base + tid;
        const unsigned m = __ballot_sync(ALL, idx < nZ);
        if (idx >= nZ) continue;
        const int li = idx / S::WZ - 1, lj = idx % S::WZ - 1;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const uint32_t f0 = sF[IS(li, lj)], fw = sF[IS(li - 1, lj)], fs = sF[IS(li, lj - 1)],
                       fws = sF[IS(li - 1, lj - 1)];
        const bool mz = (f0 & fw & fs & fws & F_MC) != 0;
        // no-slip boundary terms: (iceMaskU - its southern neighbour) and (iceMaskV - its western one)
        const int hU = (int)((f0 & F_MU) != 0) - (int)((fs & F_MU) != 0);
        const int hV = (int)((f0 & F_MV) != 0) - (int)((fw & F_MV) != 0);
        const double u0 = sU[IS(li, lj)], us = sU[IS(li, lj - 1)];
        const double v0 = sV[IS(li, lj)], vw = sV[IS(li - 1, lj)];
        const double ry = __ldg(c.rdyUh_y + gj), rx = __ldg(c.rdxVh_x + gi);
        double e;
        if (__any_sync(m, (hU | hV) != 0)) {
            const double hu2 = hU == 0 ? 0.0 : (hU > 0 ? 2.0 : -2.0);
            const double hv2 = hV == 0 ? 0.0 : (hV > 0 ? 2.0 : -2.0);
            const double tu = fma(hu2, u0 + us, mz ? u0 - us : 0.0);
            const double tv = fma(hv2, v0 + vw, mz ? v0 - vw : 0.0);
            e = fma(ry, tu, rx * tv);
        } else {
            e = mz ? fma(ry, u0 - us, rx * (v0 - vw)) : 0.0;
        }
        sE12[idx] = e;
        sZq[idx] = __ldg(c.rAz + (int64_t)gi * lp + gj) * (e * e);
    }
    __syncthreads();

    // ---- B: viscosities at C [-1, TI] x [-1, TJ] (veris/dynamics_routines.py:220-268);
    //      stresses, drag and Coriolis terms on [-1, TI) x [-1, TJ) (veris/evp_solver.py:80-145)
    for (int base = 0; base < nB; base += F64_THREADS) {
        const int idx = base + tid;
        const unsigned m = __ballot_sync(ALL, idx < nB);
        if (idx >= nB) continue;
        const int li = idx / S::WB - 1, lj = idx % S::WB - 1;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const int64_t o = (int64_t)gi * lp + gj;
        const uint32_t f0 = sF[IS(li, lj)];
        const bool inC = f0 & F_INC;
        const double u0 = sU[IS(li, lj)], ue = sU[IS(li + 1, lj)];
        const double v0 = sV[IS(li, lj)], vn = sV[IS(li, lj + 1)];
        const double e11 = inC ? (ue - u0) * __ldg(c.rdxU_x + gi) : 0.0;
        const double e22 = inC ? (vn - v0) * __ldg(c.rdyV_y + gj) : 0.0;
        const double ep = e11 + e22, em = e11 - e22;
        const double Ph = __ldg(c.Phh + o);   // Ph / (2 alpha): zeta below is zeta / (2 alpha)
        double zeta = 0.0, delta = 0.0;
        // (a taped subcycle keeps Delta where zeta = 0 too: the adjoint needs it)
        const bool strong = __any_sync(m, !is_zero(Ph));
        if (TAPE || strong) {
            const double zs =
                (sZq[IZ(li, lj)] + sZq[IZ(li + 1, lj)]) + (sZq[IZ(li, lj + 1)] + sZq[IZ(li + 1, lj + 1)]);
            // Delta^2 = ep^2 + (em^2 + 4 * 0.25/rA * sum rAz e12^2) / e^2
            const double d2 = fma(__ldg(c.rsqrA + o), zs, fma(k.rsq * em, em, ep * ep));
            delta = sqrt64(d2, m);
            if (strong) zeta = div64(Ph, delta + k.deltaMin, m);
        }
        sZeta[idx] = zeta;
        const bool in2 = li < ti && lj < S::TJ;
        const unsigned m2 = __ballot_sync(m, in2);
        if (in2) {
            const int q = IC(li, lj);
            const bool mC = f0 & F_MC;
            // sigma_k = sigma_k (alpha-1)/alpha + zeta/(2 alpha) * (4 ep - 2 kp Delta | em)
            const double zh = zeta;
            const double s1 = mC ? fma(__ldg(io.s1 + o), k.am1r, zh * fma(4.0, ep, -(k.kp2 * delta))) : 0.0;
            const double s2 = mC ? fma(__ldg(io.s2 + o), k.am1r, zh * em) : 0.0;
            sS11[q] = (s1 + s2) * __ldg(c.dyVh_y + gj);
            sS22[q] = (s1 - s2) * __ldg(c.dxUh_x + gi);
            const bool own = li >= 0 && lj >= 0 && i0 + li < d.NX && j0 + lj < d.NY;
            if (own) {
                const int64_t w = (int64_t)gi * io.ldo + gj;
                io.s1o[w] = s1;
                io.s2o[w] = s2;
            }
            // ocean drag at C (veris/dynamics_routines.py:21-52): with X = 4 t and
            // Y = (dc^2/4) X, dc^2 t > cmin^2 <=> Y > cmin^2 and dc sqrt(t) = sqrt(Y)
            const uint32_t fe = sF[IS(li + 1, lj)], fn = sF[IS(li, lj + 1)];
            const double du0 = (f0 & F_INU) ? u0 - __ldg(c.uOc + o) : 0.0;
            const double du1 = (fe & F_INU) ? ue - uoc(li + 1, lj) : 0.0;
            const double dv0 = (f0 & F_INV) ? v0 - __ldg(c.vOc + o) : 0.0;
            const double dv1 = (fn & F_INV) ? vn - voc(li, lj + 1) : 0.0;
            const double a = du0 + du1, b = dv0 + dv1;
            const double X = fma(b, b, a * a);
            const bool south = f0 & F_SOUTH;
            const double Y = (south ? k.dcq2S : k.dcq2N) * X;
            const bool fast = gt_nonneg(Y, k.cmin2);
            double cd = k.cmin;
            if (__any_sync(m2, fast)) {
                const double sy = sqrt64(Y, m2);
                if (fast) cd = sy;
            }
            sCd[q] = mC ? cd : 0.0;
            if (TAPE && own) {
                const int64_t w = (int64_t)gi * io.ldo + gj;
                io.tDel[w] = delta;
                io.tZeta[w] = zeta * k.twoAlpha;
                io.tCd[w] = mC ? cd : 0.0;
            }
            if (BASAL) {   // veris/dynamics_routines.py:55-96 with the step factor folded by the prep
                const double a_ = (f0 & F_INU) ? u0 : 0.0, b_ = (fe & F_INU) ? ue : 0.0;
                const double c_ = (f0 & F_INV) ? v0 : 0.0, e_ = (fn & F_INV) ? vn : 0.0;
                const double s = 0.25 * (a_ * a_ + b_ * b_ + c_ * c_ + e_ * e_);
                sCb[q] = div64(__ldg(c.bfac + o), sqrt64(s + k.U02, m2), m2);
            }
            const double mf = __ldg(c.mf4 + o);
            sFv[q] = mf * (v0 + vn);
            sFu[q] = mf * (u0 + ue);
        }
    }
    __syncthreads();

    // ---- C: sigma12 at Z [0, TI] x [0, TJ] (veris/evp_solver.py:101-103 with
    //      veris/averaging.py:4-19); sZq is dead: it takes sigma12
    for (int idx = tid; idx < nC; idx += F64_THREADS) {
        const int li = idx / S::WC, lj = idx % S::WC;
        const int gi = d.wxt(i0 + li), gj = d.wyt(j0 + lj);
        const uint32_t n = (sF[IS(li, lj)] & F_MC) + (sF[IS(li - 1, lj)] & F_MC) + (sF[IS(li, lj - 1)] & F_MC) +
                           (sF[IS(li - 1, lj - 1)] & F_MC);
        const double nh = n == 4 ? k.nh4 : (n == 3 ? k.nh3 : (n == 2 ? k.nh2 : (n == 1 ? k.nh1 : 0.0)));
        const double zs = (sZeta[IB(li, lj)] + sZeta[IB(li - 1, lj)]) +
                          (sZeta[IB(li, lj - 1)] + sZeta[IB(li - 1, lj - 1)]);
        const double s12 = fma(__ldg(io.s12 + (int64_t)gi * lp + gj), k.am1r, (nh * zs) * sE12[IZ(li, lj)]);
        sS12[idx] = s12;
        if (li < ti && lj < S::TJ && i0 + li < d.NX && j0 + lj < d.NY) io.s12o[(int64_t)gi * io.ldo + gj] = s12;
    }
    __syncthreads();

    // ---- D: u, v at the tile's U and V points (veris/evp_solver.py:105-187)
    for (int base = 0; base < ti * S::TJ; base += F64_THREADS) {
        const int idx = base + tid;
        const int li = idx / S::TJ, lj = idx % S::TJ;
        const int gi = i0 + li, gj = j0 + lj;
        const bool act = idx < ti * S::TJ && gi < d.NX && gj < d.NY;
        const unsigned m = __ballot_sync(ALL, act);
        if (!act) continue;
        const int64_t o = (int64_t)gi * lp + gj;
        const uint32_t f0 = sF[IS(li, lj)];
        const double u0 = sU[IS(li, lj)], v0 = sV[IS(li, lj)];
        const double cd0 = sCd[IC(li, lj)], cdw = sCd[IC(li - 1, lj)], cds = sCd[IC(li, lj - 1)];
        {   // U point
            const double kU = __ldg(c.hAW + o) * (cd0 + cdw);
            const double uo0 = __ldg(c.uOc + o);
            double fx = fma(kU, uo0, __ldg(c.cU + o)) + (sFv[IC(li, lj)] + sFv[IC(li - 1, lj)]);
            if (TURN) {
                const double sg = (f0 & F_SPOS) ? 1.0 : ((f0 & F_SNEG) ? -1.0 : 0.0);
                const double du0 = uo0 - u0, dun = uoc(li, lj + 1) - sU[IS(li, lj + 1)];
                const double duw = uoc(li - 1, lj) - sU[IS(li - 1, lj)];
                const double duwn = uoc(li - 1, lj + 1) - sU[IS(li - 1, lj + 1)];
                const double t = (cd0 * 0.5 * (du0 + dun) + cdw * 0.5 * (duw + duwn)) * __ldg(c.AW + o);
                if (f0 & F_LMU) fx -= sg * k.sinW * 0.5 * t;
            }
            const double sdx = __ldg(c.rrAu + o) * fma(__ldg(c.dxV_x + gi), sS12[IZZ(li, lj + 1)] - sS12[IZZ(li, lj)],
                                                       sS11[IC(li, lj)] - sS11[IC(li - 1, lj)]);
            double den = __ldg(c.mUb1 + o) + kU;
            if (BASAL) den = fma(0.5 * __ldg(c.AW + o), sCb[IC(li, lj)] + sCb[IC(li - 1, lj)], den);
            den = is_zero(den) ? 1.0 : den;
            const double num = fma(__ldg(c.mUb + o), u0, fx) + sdx;
            const bool wet = f0 & F_MU;
            double un = 0.0;
            if (__any_sync(m, wet)) {
                const double q = div64(num, den, m);
                un = wet ? q : 0.0;
            }
            store_filled_ld(io.uo, io.ldo, d, h, gi, gj, un);
        }
        {   // V point
            const double kV = __ldg(c.hAS + o) * (cd0 + cds);
            const double vo0 = __ldg(c.vOc + o);
            double fy = fma(kV, vo0, __ldg(c.cV + o)) - (sFu[IC(li, lj)] + sFu[IC(li, lj - 1)]);
            if (TURN) {
                const double sg = (f0 & F_SPOS) ? 1.0 : ((f0 & F_SNEG) ? -1.0 : 0.0);
                const double dv0 = vo0 - v0, dve = voc(li + 1, lj) - sV[IS(li + 1, lj)];
                const double dvs = voc(li, lj - 1) - sV[IS(li, lj - 1)];
                const double dvse = voc(li + 1, lj - 1) - sV[IS(li + 1, lj - 1)];
                const double t = (cd0 * 0.5 * (dv0 + dve) + cds * 0.5 * (dvs + dvse)) * __ldg(c.AS + o);
                if (f0 & F_LMV) fy += sg * k.sinW * 0.5 * t;
            }
            const double sdy = __ldg(c.rrAv + o) * fma(__ldg(c.dyU_y + gj), sS12[IZZ(li + 1, lj)] - sS12[IZZ(li, lj)],
                                                       sS22[IC(li, lj)] - sS22[IC(li, lj - 1)]);
            double den = __ldg(c.mVb1 + o) + kV;
            if (BASAL) den = fma(0.5 * __ldg(c.AS + o), sCb[IC(li, lj)] + sCb[IC(li, lj - 1)], den);
            den = is_zero(den) ? 1.0 : den;
            const double num = fma(__ldg(c.mVb + o), v0, fy) + sdy;
            const bool wet = f0 & F_MV;
            double vnew = 0.0;
            if (__any_sync(m, wet)) {
                const double q = div64(num, den, m);
                vnew = wet ? q : 0.0;
            }
            store_filled_ld(io.vo, io.ldo, d, h, gi, gj, vnew);
        }
    }
#undef IS
#undef IZ
#undef IB
#undef IC
#undef IZZ
}

// The units of a launch: when all full pieces fit the resident CTAs' slots
// at once, the fewest pieces of at most TI rows; otherwise a last round of
// about one small piece (TI/4 rows) per slot at the bottom of every strip,
// the rest in full pieces.  (Equal full tiles left a thin last wave: 12 % of
// the SM cycles idle on 1440 x 720 with 24-row tiles; third-height last
// pieces took 197.2 us a launch there, quarter-height 193.0, fifth- and
// sixth-height 193.8.)
static F64Units f64_units(const Dims &d, int TI, int slots) {
    const int strips = (d.NY + 31) / 32;
    F64Units w;
    const int minP = (d.NX + TI - 1) / TI;
    w.P2 = 0;
    w.R1 = d.NX;
    if ((int64_t)strips * minP > slots) {
        const int small = TI / 4 > 4 ? TI / 4 : 4;
        w.P2 = (slots + strips - 1) / strips;
        const int r2 = w.P2 * small;
        if (r2 < d.NX / 2) w.R1 = d.NX - r2;
        else w.P2 = 0;
    }
    w.P1 = (w.R1 + TI - 1) / TI;
    w.U1 = strips * w.P1;
    return w;
}

template <int TI, bool B, bool R, bool TP>
static int launch64(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<double> &c, const F64Scalars &k,
                    const FastIO<double> &io, cudaStream_t st) {
    using S = Smem64<TI>;
    auto kern = evp_f64_kernel<TI, B, R, TP>;
    const size_t sm = S::bytes(B);
    static std::atomic<bool> configured[MAX_DEVICES];
    if (!smem_configured(configured, kern, (int)sm)) return VERIS_ERR_LAUNCH;
    static std::atomic<int> resident[MAX_DEVICES];   // CTAs per SM (0: not queried yet)
    const int dev = current_device();
    if (dev < 0) return VERIS_ERR_LAUNCH;
    int per = resident[dev].load(std::memory_order_acquire);
    if (per == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, F64_THREADS, sm) != cudaSuccess || per < 1) {
            cudaGetLastError();
            return VERIS_ERR_LAUNCH;
        }
        resident[dev].store(per, std::memory_order_release);
    }
    const int sms = sm_count();
    if (sms <= 0) return VERIS_ERR_LAUNCH;
    const F64Units w = f64_units(d, TI, per * sms);
    const int units = w.U1 + ((d.NY + S::TJ - 1) / S::TJ) * w.P2;
    kern<<<units, F64_THREADS, sm, st>>>(d, lp, h, c, k, io, w);
    return launch_status();
}

// a taped subcycle (io.tDel set) also writes Delta, zeta and cDrag
template <int TI, bool B, bool R>
static int launch64_tape(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<double> &c,
                         const F64Scalars &k, const FastIO<double> &io, cudaStream_t st) {
    return io.tDel ? launch64<TI, B, R, true>(d, lp, h, c, k, io, st) : launch64<TI, B, R, false>(d, lp, h, c, k, io, st);
}

template <int TI>
static int launch64_rows(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<double> &c,
                         const F64Scalars &k, const FastIO<double> &io, bool basal, bool turn, cudaStream_t st) {
    if (basal)
        return turn ? launch64_tape<TI, true, true>(d, lp, h, c, k, io, st)
                    : launch64_tape<TI, true, false>(d, lp, h, c, k, io, st);
    return turn ? launch64_tape<TI, false, true>(d, lp, h, c, k, io, st)
                : launch64_tape<TI, false, false>(d, lp, h, c, k, io, st);
}

// rows per tile of later float64 subcycles (0: the default); process-wide
static std::atomic<int> g_tile_rows{0};
// measured on GB300 (ordered units): 24 rows 204.0 / 1153.0 us per subcycle
// on 1440x720 / 3600x1800, against 202.6 / 1173.3 (16) and 222.7 / 1240.8
// (32); the bench's tuner picks per workload
constexpr int F64_DEFAULT_ROWS = 24;

int fast64_subcycle(const Dims &d, const HaloFill &h, const FastConsts<double> &c, const FastScalars<double> &ks,
                    const FastIO<double> &io, bool basal, bool turn, cudaStream_t st) {
    const int64_t lp = internal_pitch(d.NY);
    const F64Scalars k = f64_scalars(ks);
    const int rows = g_tile_rows.load(std::memory_order_relaxed);
    switch (rows ? rows : F64_DEFAULT_ROWS) {
        case 16: return launch64_rows<16>(d, lp, h, c, k, io, basal, turn, st);
        case 24: return launch64_rows<24>(d, lp, h, c, k, io, basal, turn, st);
        default: return launch64_rows<32>(d, lp, h, c, k, io, basal, turn, st);
    }
}

}  // namespace veris

using namespace veris;

extern "C" int veris_evp_f64_tile_rows(int32_t rows) {
    VERIS_REQUIRE(rows == 0 || rows == 16 || rows == 24 || rows == 32, VERIS_ERR_ARG);
    g_tile_rows.store(rows, std::memory_order_relaxed);
    return VERIS_OK;
}
