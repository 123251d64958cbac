// The mEVP subcycle loop (veris/evp_solver.py:21-319), plain form: one tiled
// kernel per subcycle.
//
// A CTA owns a TI x TJ tile of padded points (x rows by y columns, y
// contiguous).  It recomputes the intermediates it needs on a thin ring
// around the tile into shared memory, so one launch does the whole subcycle:
//
//   A  e12 (and rAz*e12^2) at Z points  [-1, TI+1] x [-1, TJ+1]
//   B  e11, e22, Delta, zeta, press at C [-1, TI] x [-1, TJ]; on [-1, TI) x
//      [-1, TJ) also the new sigma1/sigma2, sig11/sig22, the drag
//      coefficients and the Coriolis terms at C
//   C  zeta at Z and the new sigma12      [0, TI] x [0, TJ]
//   D  stress divergence, forcing, implicit drag and the new u, v on the tile
//
// The new u, v are stored together with their periodic images in the halo
// columns (and rows) that the reference's fill_overlap_uv refreshes
// (veris/evp_solver.py:190).  Stresses are not halo-filled, as in the
// reference.  Inputs and outputs alternate between the caller's output
// arrays and the workspace (ping-pong), so no CTA reads a value another CTA
// of the same launch writes.
#include <mutex>

#include "stencil.cuh"

namespace veris {

constexpr int EVP_TI = 32, EVP_TJ = 32, EVP_THREADS = 256;

template <class T>
struct EvpIO {
    const T *u, *v, *s1, *s2, *s12;   // state at the start of the subcycle
    T *uo, *vo, *s1o, *s2o, *s12o;    // state at its end
    const T *uNm1, *vNm1;             // velocities of the previous time step
    T *aCo = nullptr;                 // adaptive EVP: alphaC of the subcycle, when not null
};

template <class T>
struct EvpSmem {
    // widths of the regions
    static constexpr int WZ = EVP_TJ + 3, HZ = EVP_TI + 3;   // stage A
    static constexpr int WB = EVP_TJ + 2, HB = EVP_TI + 2;   // stage B (zeta, alphaC)
    static constexpr int WC = EVP_TJ + 1, HC = EVP_TI + 1;   // R_C arrays and sigma12
    static constexpr int NZ = WZ * HZ, NB = WB * HB, NC = WC * HC;
    static constexpr int N_C_ARRAYS = 8;  // sig11 sig22 cd cb fvC fuC sp s12
    static constexpr size_t bytes() {
        return sizeof(T) * (size_t)(2 * NZ + 2 * NB + N_C_ARRAYS * NC);
    }
};

template <class T, bool ADAPT, bool SIDE, bool BASAL>
__global__ void __launch_bounds__(EVP_THREADS, 2)
evp_subcycle_kernel(Ctx<T> c, HaloFill h, EvpIO<T> io) {
    using S = EvpSmem<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *e12s = reinterpret_cast<T *>(smem_raw);
    T *zqs = e12s + S::NZ;
    T *zeta = zqs + S::NZ;
    T *aCs = zeta + S::NB;
    T *sig11 = aCs + S::NB;
    T *sig22 = sig11 + S::NC;
    T *cds = sig22 + S::NC;
    T *cbs = cds + S::NC;
    T *fvC = cbs + S::NC;
    T *fuC = fvC + S::NC;
    T *sps = fuC + S::NC;
    T *s12s = sps + S::NC;

    const Fields<T> &f = c.f;
    const Dims &d = c.d;
    const int i0 = blockIdx.y * EVP_TI, j0 = blockIdx.x * EVP_TJ;
    const int tid = threadIdx.x;

    // index helpers: stage A / B arrays are offset by one, R_C arrays by one,
    // R_Z (sigma12) by zero
#define ZA(li, lj) ((li) + 1) * S::WZ + ((lj) + 1)
#define ZB(li, lj) ((li) + 1) * S::WB + ((lj) + 1)
#define ZC(li, lj) ((li) + 1) * S::WC + ((lj) + 1)
#define ZZ(li, lj) (li) * S::WC + (lj)

    // ---- stage A: e12 at Z points
    for (int idx = tid; idx < S::NZ; idx += EVP_THREADS) {
        const int li = idx / S::WZ - 1, lj = idx % S::WZ - 1;
        const int gi = i0 + li, gj = j0 + lj;
        if (gi >= d.NX + 2 || gj >= d.NY + 2) continue;   // feeds no stored point; keeps the wrap within one period
        const T e = strain_z(c, io.u, io.v, gi, gj);
        e12s[idx] = e;
        zqs[idx] = c.ld(f.rAz, gi, gj) * (e * e);
    }
    __syncthreads();

    // ---- stage B: viscosities and the C-point stress update
    const T alpha = T(c.p.evpAlpha);
    const T rdenom = T(1.0 / c.p.evpAlpha);
    for (int idx = tid; idx < S::NB; idx += EVP_THREADS) {
        const int li = idx / S::WB - 1, lj = idx % S::WB - 1;
        const int gi = i0 + li, gj = j0 + lj;
        if (gi >= d.NX + 2 || gj >= d.NY + 2) continue;   // feeds no stored point; keeps the wrap within one period
        T e11, e22;
        strain_c(c, io.u, io.v, gi, gj, e11, e22);
        T zt, et, pr, dl;
        viscosity_c(c, gi, gj, e11, e22, zqs[ZA(li, lj)], zqs[ZA(li + 1, lj)], zqs[ZA(li, lj + 1)],
                    zqs[ZA(li + 1, lj + 1)], zt, et, pr, dl);
        zeta[idx] = zt;
        const T mC = c.ld(f.iceMask, gi, gj);
        T aC = alpha, d1 = rdenom;
        if (ADAPT) {
            const T mass = c.ld(f.SeaIceMassC, gi, gj);
            aC = sqrt(zt * T(c.p.EVPcFac) / (mass > T(1e-4) ? mass : T(1e-4)) * c.ld(f.recip_rA, gi, gj)) * mC;
            aC = aC > T(c.p.aEVPalphaMin) ? aC : T(c.p.aEVPalphaMin);
            aCs[idx] = aC;
            d1 = T(1.0) / aC;
        }
        if (li < EVP_TI && lj < EVP_TJ) {
            const int k = ZC(li, lj);
            const T ep = e11 + e22, em = e11 - e22;
            const T div = T(2) * zt * ep - pr;
            const T ten = T(2) * zt * em;
            const T s1 = (c.ld(io.s1, gi, gj) * (aC - T(1)) + div) * d1 * mC;
            const T s2 = (c.ld(io.s2, gi, gj) * (aC - T(1)) + ten * T(0.25)) * d1 * mC;
            sig11[k] = T(0.5) * (s1 + s2);
            sig22[k] = T(0.5) * (s1 - s2);
            if (li >= 0 && lj >= 0 && gi < d.NX && gj < d.NY) {
                const int64_t o = d.raw(gi, gj);
                io.s1o[o] = s1;
                io.s2o[o] = s2;
                if (ADAPT && io.aCo) io.aCo[o] = aC;
            }
            cds[k] = ocean_drag_c(c, io.u, io.v, gi, gj);
            if (BASAL) cbs[k] = basal_drag_c(c, io.u, io.v, gi, gj);
            const T mf = c.ld(f.SeaIceMassC, gi, gj) * c.ld(f.fCori, gi, gj) * T(0.5);
            fvC[k] = mf * (c.ld(io.v, gi, gj) + c.ld(io.v, gi, gj + 1));
            fuC[k] = mf * (c.ld(io.u, gi, gj) + c.ld(io.u, gi + 1, gj));
            if (SIDE) sps[k] = ice_speed_c(c, io.u, io.v, gi, gj);
        }
    }
    __syncthreads();

    // ---- stage C: sigma12 at Z points
    for (int idx = tid; idx < S::NC; idx += EVP_THREADS) {
        const int li = idx / S::WC, lj = idx % S::WC;
        const int gi = i0 + li, gj = j0 + lj;
        if (gi >= d.NX + 2 || gj >= d.NY + 2) continue;   // feeds no stored point; keeps the wrap within one period
        const T zz = c2z_norm(c, gi, gj, true) *
                     ((zeta[ZB(li, lj)] + zeta[ZB(li - 1, lj)]) + (zeta[ZB(li, lj - 1)] + zeta[ZB(li - 1, lj - 1)]));
        T aZ = alpha, d2 = rdenom;
        if (ADAPT) {
            aZ = T(0.5) * (T(0.5) * (aCs[ZB(li, lj)] + aCs[ZB(li, lj - 1)]) +
                           T(0.5) * (aCs[ZB(li - 1, lj)] + aCs[ZB(li - 1, lj - 1)]));
            d2 = T(1.0) / aZ;
        }
        const T shr = T(2) * zz * e12s[ZA(li, lj)];
        const T s12 = (c.ld(io.s12, gi, gj) * (aZ - T(1)) + shr * T(0.25)) * d2;
        s12s[idx] = s12;
        if (li < EVP_TI && lj < EVP_TJ && gi < d.NX && gj < d.NY) io.s12o[d.raw(gi, gj)] = s12;
    }
    __syncthreads();

    // ---- stage D: momentum update at U and V points of the tile
    const T rdt = T(c.p.recip_deltatDyn);
    const T cosW = T(c.p.cosWat), sinW = T(c.p.sinWat);
    const T beta = T(c.p.evpBeta);
    for (int idx = tid; idx < EVP_TI * EVP_TJ; idx += EVP_THREADS) {
        const int li = idx / EVP_TJ, lj = idx % EVP_TJ;
        const int gi = i0 + li, gj = j0 + lj;
        if (gi >= d.NX || gj >= d.NY) continue;
        const int64_t o = d.raw(gi, gj);
        const T sg = sgn(__ldg(f.fCori + o));
        const T cd0 = cds[ZC(li, lj)], cdw = cds[ZC(li - 1, lj)], cdsou = cds[ZC(li, lj - 1)];
        const T cb0 = BASAL ? cbs[ZC(li, lj)] : T(0);
        const T cbw = BASAL ? cbs[ZC(li - 1, lj)] : T(0);
        const T cbs_ = BASAL ? cbs[ZC(li, lj - 1)] : T(0);
        const T u0 = __ldg(io.u + o), v0 = __ldg(io.v + o);

        // U point
        {
            const T sdx = (sig11[ZC(li, lj)] * __ldg(f.dyV + o) - sig11[ZC(li - 1, lj)] * c.ld(f.dyV, gi - 1, gj) -
                           s12s[ZZ(li, lj)] * __ldg(f.dxV + o) + s12s[ZZ(li, lj + 1)] * c.ld(f.dxV, gi, gj + 1)) *
                          __ldg(f.recip_rAu + o);
            const T mU = __ldg(f.SeaIceMassU + o);
            const T lm = mU != T(0) ? T(1) : mU;
            const T uo = __ldg(f.uOcean + o);
            const T du0 = uo - u0;
            const T dun = c.ld(f.uOcean, gi, gj + 1) - c.ld(io.u, gi, gj + 1);
            const T duw = c.ld(f.uOcean, gi - 1, gj) - c.ld(io.u, gi - 1, gj);
            const T duwn = c.ld(f.uOcean, gi - 1, gj + 1) - c.ld(io.u, gi - 1, gj + 1);
            const T AW = __ldg(f.AreaW + o);
            T fx = __ldg(f.WindForcingX + o) +
                   (T(0.5) * (cd0 + cdw) * cosW * uo -
                    sg * sinW * T(0.5) * (cd0 * T(0.5) * (du0 + dun) + cdw * T(0.5) * (duw + duwn)) * lm) * AW;
            fx = fx + T(0.5) * (fvC[ZC(li, lj)] + fvC[ZC(li - 1, lj)]);
            const T bU = (ADAPT ? T(0.5) * (aCs[ZB(li, lj)] + aCs[ZB(li - 1, lj)]) : beta) * rdt;
            const T bU1 = bU + rdt;
            T den = mU * bU1 + AW * (T(0.5) * (cd0 + cdw) * cosW + T(0.5) * (cb0 + cbw));
            den = den == T(0) ? T(1) : den;
            if (SIDE) den = den + side_drag_u(c, gi, gj, sps[ZC(li, lj)], sps[ZC(li - 1, lj)]);
            const T un = __ldg(f.iceMaskU + o) * (bU * mU * u0 + mU * rdt * __ldg(io.uNm1 + o) + fx + sdx) / den;
            store_filled(io.uo, d, h, gi, gj, un);
        }
        // V point
        {
            const T sdy = (sig22[ZC(li, lj)] * __ldg(f.dxU + o) - sig22[ZC(li, lj - 1)] * c.ld(f.dxU, gi, gj - 1) -
                           s12s[ZZ(li, lj)] * __ldg(f.dyU + o) + s12s[ZZ(li + 1, lj)] * c.ld(f.dyU, gi + 1, gj)) *
                          __ldg(f.recip_rAv + o);
            const T mV = __ldg(f.SeaIceMassV + o);
            const T lm = mV != T(0) ? T(1) : mV;
            const T vo = __ldg(f.vOcean + o);
            const T dv0 = vo - v0;
            const T dve = c.ld(f.vOcean, gi + 1, gj) - c.ld(io.v, gi + 1, gj);
            const T dvs = c.ld(f.vOcean, gi, gj - 1) - c.ld(io.v, gi, gj - 1);
            const T dvse = c.ld(f.vOcean, gi + 1, gj - 1) - c.ld(io.v, gi + 1, gj - 1);
            const T AS = __ldg(f.AreaS + o);
            T fy = __ldg(f.WindForcingY + o) +
                   (T(0.5) * (cd0 + cdsou) * cosW * vo +
                    sg * sinW * T(0.5) * (cd0 * T(0.5) * (dv0 + dve) + cdsou * T(0.5) * (dvs + dvse)) * lm) * AS;
            fy = fy - T(0.5) * (fuC[ZC(li, lj)] + fuC[ZC(li, lj - 1)]);
            const T bV = (ADAPT ? T(0.5) * (aCs[ZB(li, lj)] + aCs[ZB(li, lj - 1)]) : beta) * rdt;
            const T bV1 = bV + rdt;
            T den = mV * bV1 + AS * (T(0.5) * (cd0 + cdsou) * cosW + T(0.5) * (cb0 + cbs_));
            den = den == T(0) ? T(1) : den;
            if (SIDE) den = den + side_drag_v(c, gi, gj, sps[ZC(li, lj)], sps[ZC(li, lj - 1)]);
            const T vn = __ldg(f.iceMaskV + o) * (bV * mV * v0 + mV * rdt * __ldg(io.vNm1 + o) + fy + sdy) / den;
            store_filled(io.vo, d, h, gi, gj, vn);
        }
    }
#undef ZA
#undef ZB
#undef ZC
#undef ZZ
}

template <class T, bool A, bool Sd, bool B>
static int launch_subcycle(const Ctx<T> &c, const HaloFill &h, const EvpIO<T> &io, cudaStream_t st) {
    auto kern = evp_subcycle_kernel<T, A, Sd, B>;
    const size_t sm = EvpSmem<T>::bytes();
    static std::atomic<bool> configured[MAX_DEVICES];
    if (!smem_configured(configured, kern, (int)sm)) return VERIS_ERR_LAUNCH;
    dim3 grid((c.d.NY + EVP_TJ - 1) / EVP_TJ, (c.d.NX + EVP_TI - 1) / EVP_TI);
    kern<<<grid, EVP_THREADS, sm, st>>>(c, h, io);
    return launch_status();
}

template <class T>
static int dispatch_subcycle(const Ctx<T> &c, const HaloFill &h, const EvpIO<T> &io, cudaStream_t st) {
    const bool A = c.p.useAdaptiveEVP != 0, Sd = c.p.noSlip == 0, B = c.p.basalDragK2 != 0.0;
    if (A) {
        if (Sd) return B ? launch_subcycle<T, true, true, true>(c, h, io, st) : launch_subcycle<T, true, true, false>(c, h, io, st);
        return B ? launch_subcycle<T, true, false, true>(c, h, io, st) : launch_subcycle<T, true, false, false>(c, h, io, st);
    }
    if (Sd) return B ? launch_subcycle<T, false, true, true>(c, h, io, st) : launch_subcycle<T, false, true, false>(c, h, io, st);
    return B ? launch_subcycle<T, false, false, true>(c, h, io, st) : launch_subcycle<T, false, false, false>(c, h, io, st);
}

static size_t field_bytes(const Dims &d, size_t elem) { return (size_t)d.NX * (size_t)d.ld * elem; }

static size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <class T>
static int evp_solver(const VerisGrid *g, const VerisParams *p, const Fields<T> *vs, int n, T *u, T *v,
                      T *s1, T *s2, T *s12, void *ws, size_t ws_bytes, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && u && v && s1 && s2 && s12, VERIS_ERR_ARG);
    VERIS_REQUIRE(n >= 0, VERIS_ERR_ARG);
    cudaStream_t st = (cudaStream_t)s;
    const size_t fb = round_up(field_bytes(d, sizeof(T)), 256);
    if (n == 0) {
        const T *src[5] = {vs->uIce, vs->vIce, vs->sigma1, vs->sigma2, vs->sigma12};
        T *dst[5] = {u, v, s1, s2, s12};
        for (int q = 0; q < 5; ++q)
            if (cudaMemcpyAsync(dst[q], src[q], field_bytes(d, sizeof(T)), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
                return VERIS_ERR_LAUNCH;
        return VERIS_OK;
    }
    if (n > 1) VERIS_REQUIRE(ws && ws_bytes >= 5 * fb, VERIS_ERR_WORKSPACE);
    Ctx<T> c;
    c.f = *vs;
    c.d = d;
    c.p = *p;
    const HaloFill h = halo_fill_of(*p);
    T *buf[2][5] = {{u, v, s1, s2, s12}, {nullptr, nullptr, nullptr, nullptr, nullptr}};
    if (n > 1)
        for (int q = 0; q < 5; ++q) buf[1][q] = reinterpret_cast<T *>(static_cast<char *>(ws) + q * fb);
    const T *cur[5] = {vs->uIce, vs->vIce, vs->sigma1, vs->sigma2, vs->sigma12};
    for (int it = 0; it < n; ++it) {
        T **dst = buf[(n - 1 - it) % 2];
        EvpIO<T> io{cur[0], cur[1], cur[2], cur[3], cur[4], dst[0], dst[1], dst[2], dst[3], dst[4],
                    vs->uIce, vs->vIce};
        const int stt = dispatch_subcycle<T>(c, h, io, st);
        if (stt != VERIS_OK) return stt;
        for (int q = 0; q < 5; ++q) cur[q] = dst[q];
    }
    return VERIS_OK;
}

// ---------------------------------------------------------------------------
// Residual diagnostics (veris/evp_solver.py:193-234, computeEvpResidual), as
// that branch means them (it reads names it never binds): after subcycle k,
// over the interior points,
//   resSig[k] = sum (d sig11 alphaC iceMask)^2 + (d sig22 alphaC iceMask)^2 + (d sigma12 alphaZ)^2
//   resU[k]   = sum (iceMaskU d uIce betaU)^2 + (iceMaskV d vIce betaV)^2
// with sig11, sig22 = (sigma1 +- sigma2) / 2 and d the change over the
// subcycle.  The ping-pong keeps the state before the subcycle intact, so the
// residual kernel reads both states directly.  The sums are in float64 and
// deterministic: a fixed grid (a function of the interior size only), warp
// shuffles and one partial pair per block, then one block per subcycle adds
// the partials in index order.

constexpr int RES_THREADS = 256, RES_MAX_BLOCKS = 2048;

// one block per interior row (rows beyond RES_MAX_BLOCKS go round again)
static int res_blocks(const Dims &d) { return d.nx < RES_MAX_BLOCKS ? d.nx : RES_MAX_BLOCKS; }

template <class T>
struct ResIO {
    const T *u0, *v0, *s10, *s20, *s120;   // before the subcycle
    const T *u1, *v1, *s11, *s21, *s121;   // after it
    const T *mC, *mU, *mV;
    const T *aC;                            // adaptive alphaC, or null: alpha and beta are constants
    double alpha, beta;
};

__device__ __forceinline__ double warp_sum(double x) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

template <class T>
__global__ void __launch_bounds__(RES_THREADS) evp_residual_kernel(Dims d, ResIO<T> r, double *partial) {
    __shared__ double red[2][RES_THREADS / 32];
    const int ox = (d.NX - d.nx) / 2, oy = (d.NY - d.ny) / 2;
    double su = 0.0, ss = 0.0;
    for (int row = blockIdx.x; row < d.nx; row += gridDim.x)
    for (int col = threadIdx.x; col < d.ny; col += RES_THREADS) {
        const int64_t o = d.raw(ox + row, oy + col);
        // (d sig11)^2 + (d sig22)^2 = 0.5 ((d sigma1)^2 + (d sigma2)^2); with
        // constant alpha and beta their squares multiply the block sums instead
        const double d1 = (double)r.s11[o] - (double)r.s10[o], d2 = (double)r.s21[o] - (double)r.s20[o];
        const double d12 = (double)r.s121[o] - (double)r.s120[o];
        const double du = (double)r.mU[o] * ((double)r.u1[o] - (double)r.u0[o]);
        const double dv = (double)r.mV[o] * ((double)r.v1[o] - (double)r.v0[o]);
        const double mC = r.mC[o];
        const double c2 = fma(d1, d1, d2 * d2) * (0.5 * (mC * mC));
        if (r.aC) {
            const double a0 = r.aC[o], aw = r.aC[o - d.ld], as = r.aC[o - 1], asw = r.aC[o - d.ld - 1];
            const double aZ = 0.5 * (0.5 * (a0 + as) + 0.5 * (aw + asw));
            const double bU = 0.5 * (a0 + aw), bV = 0.5 * (a0 + as);
            ss += c2 * (a0 * a0) + (d12 * aZ) * (d12 * aZ);
            su += (du * bU) * (du * bU) + (dv * bV) * (dv * bV);
        } else {
            ss += fma(d12, d12, c2);
            su += fma(du, du, dv * dv);
        }
    }
    if (!r.aC) {
        su *= r.beta * r.beta;
        ss *= r.alpha * r.alpha;
    }
    su = warp_sum(su);
    ss = warp_sum(ss);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = su;
        red[1][w] = ss;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        su = threadIdx.x < RES_THREADS / 32 ? red[0][threadIdx.x] : 0.0;
        ss = threadIdx.x < RES_THREADS / 32 ? red[1][threadIdx.x] : 0.0;
        su = warp_sum(su);
        ss = warp_sum(ss);
        if (threadIdx.x == 0) {
            partial[2 * blockIdx.x] = su;
            partial[2 * blockIdx.x + 1] = ss;
        }
    }
}

// one block per subcycle: the partials of that subcycle in index order
__global__ void __launch_bounds__(RES_THREADS) evp_residual_finish_kernel(const double *partial, int nblk,
                                                                          double *resU, double *resSig) {
    __shared__ double red[2][RES_THREADS / 32];
    const double *pk = partial + (int64_t)blockIdx.x * 2 * nblk;
    double su = 0.0, ss = 0.0;
    for (int b = threadIdx.x; b < nblk; b += RES_THREADS) {
        su += pk[2 * b];
        ss += pk[2 * b + 1];
    }
    su = warp_sum(su);
    ss = warp_sum(ss);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = su;
        red[1][w] = ss;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        su = threadIdx.x < RES_THREADS / 32 ? red[0][threadIdx.x] : 0.0;
        ss = threadIdx.x < RES_THREADS / 32 ? red[1][threadIdx.x] : 0.0;
        su = warp_sum(su);
        ss = warp_sum(ss);
        if (threadIdx.x == 0) {
            resU[blockIdx.x] = su;
            resSig[blockIdx.x] = ss;
        }
    }
}

static size_t residual_workspace_bytes(const Dims &d, size_t elem, int n) {
    return 6 * round_up(field_bytes(d, elem), 256) + (size_t)(n > 0 ? n : 0) * 2 * res_blocks(d) * sizeof(double);
}

template <class T>
static int evp_residual_solver(const VerisGrid *g, const VerisParams *p, const Fields<T> *vs, int n, T *u, T *v,
                               T *s1, T *s2, T *s12, double *resU, double *resSig, void *ws, size_t ws_bytes,
                               veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(p && vs && u && v && s1 && s2 && s12, VERIS_ERR_ARG);
    VERIS_REQUIRE(n >= 0, VERIS_ERR_ARG);
    if (n == 0) return evp_solver<T>(g, p, vs, 0, u, v, s1, s2, s12, ws, ws_bytes, s);
    VERIS_REQUIRE(resU && resSig, VERIS_ERR_ARG);
    VERIS_REQUIRE(ws && ws_bytes >= residual_workspace_bytes(d, sizeof(T), n), VERIS_ERR_WORKSPACE);
    cudaStream_t st = (cudaStream_t)s;
    const size_t fb = round_up(field_bytes(d, sizeof(T)), 256);
    Ctx<T> c;
    c.f = *vs;
    c.d = d;
    c.p = *p;
    const HaloFill h = halo_fill_of(*p);
    const bool adapt = p->useAdaptiveEVP != 0;
    char *base = static_cast<char *>(ws);
    T *buf[2][5] = {{u, v, s1, s2, s12}, {nullptr, nullptr, nullptr, nullptr, nullptr}};
    for (int q = 0; q < 5; ++q) buf[1][q] = reinterpret_cast<T *>(base + q * fb);
    T *aC = reinterpret_cast<T *>(base + 5 * fb);
    double *partial = reinterpret_cast<double *>(base + 6 * fb);
    const int nblk = res_blocks(d);
    const T *cur[5] = {vs->uIce, vs->vIce, vs->sigma1, vs->sigma2, vs->sigma12};
    for (int it = 0; it < n; ++it) {
        T **dst = buf[(n - 1 - it) % 2];
        EvpIO<T> io{cur[0], cur[1], cur[2], cur[3], cur[4], dst[0], dst[1], dst[2], dst[3], dst[4],
                    vs->uIce, vs->vIce, adapt ? aC : nullptr};
        int stt = dispatch_subcycle<T>(c, h, io, st);
        if (stt != VERIS_OK) return stt;
        ResIO<T> r{cur[0], cur[1], cur[2], cur[3], cur[4], dst[0], dst[1], dst[2], dst[3], dst[4],
                   vs->iceMask, vs->iceMaskU, vs->iceMaskV, adapt ? aC : nullptr, p->evpAlpha, p->evpBeta};
        evp_residual_kernel<T><<<nblk, RES_THREADS, 0, st>>>(d, r, partial + (int64_t)it * 2 * nblk);
        stt = launch_status();
        if (stt != VERIS_OK) return stt;
        for (int q = 0; q < 5; ++q) cur[q] = dst[q];
    }
    evp_residual_finish_kernel<<<n, RES_THREADS, 0, st>>>(partial, nblk, resU, resSig);
    return launch_status();
}

}  // namespace veris

using namespace veris;

extern "C" {

size_t veris_evp_residual_workspace_bytes(const VerisGrid *g, int32_t elem_size, int32_t n_subcycles) {
    Dims d;
    if (check_grid(g, &d) != VERIS_OK || (elem_size != 4 && elem_size != 8) || n_subcycles < 0) return 0;
    return residual_workspace_bytes(d, (size_t)elem_size, n_subcycles);
}

int veris_evp_residual_solver_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                  int32_t n, double *u, double *v, double *s1, double *s2, double *s12,
                                  double *resU, double *resSig, void *ws, size_t ws_bytes, veris_stream_t s) {
    return evp_residual_solver<double>(g, p, reinterpret_cast<const Fields<double> *>(vs), n, u, v, s1, s2, s12,
                                       resU, resSig, ws, ws_bytes, s);
}

int veris_evp_residual_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF32 *vs,
                                  int32_t n, float *u, float *v, float *s1, float *s2, float *s12,
                                  double *resU, double *resSig, void *ws, size_t ws_bytes, veris_stream_t s) {
    return evp_residual_solver<float>(g, p, reinterpret_cast<const Fields<float> *>(vs), n, u, v, s1, s2, s12,
                                      resU, resSig, ws, ws_bytes, s);
}

size_t veris_evp_workspace_bytes(const VerisGrid *g, int32_t elem_size) {
    Dims d;
    if (check_grid(g, &d) != VERIS_OK || (elem_size != 4 && elem_size != 8)) return 0;
    return 5 * round_up(field_bytes(d, (size_t)elem_size), 256);
}

int veris_evp_solver_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs, int32_t n,
                         double *u, double *v, double *s1, double *s2, double *s12, void *ws,
                         size_t ws_bytes, veris_stream_t s) {
    return evp_solver<double>(g, p, reinterpret_cast<const Fields<double> *>(vs), n, u, v, s1, s2, s12, ws,
                              ws_bytes, s);
}

int veris_evp_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF32 *vs, int32_t n,
                         float *u, float *v, float *s1, float *s2, float *s12, void *ws, size_t ws_bytes,
                         veris_stream_t s) {
    return evp_solver<float>(g, p, reinterpret_cast<const Fields<float> *>(vs), n, u, v, s1, s2, s12, ws,
                             ws_bytes, s);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free form of veris_evp_solver_f64 (no counterpart in the
// reference).  Some callers cannot allocate device memory: a host ocean
// model's time loop that drives the sea-ice step through this C ABI has no
// device allocator of its own, and a caller running under a device-memory
// budget fixed at start-up must not grow it per step.  For them the
// ping-pong half of the subcycle loop lives in this file-scope array instead
// of a caller-provided workspace.  Every GPU that loads the library holds the
// array until the process exits.  Nothing in it has to start at zero: each
// subcycle writes every point of the buffer before the next one reads it.
// Calls share the array, so calls that overlap on the GPU race on it.
namespace {

constexpr int64_t NOALLOC_MAX_CELLS = VERIS_NOALLOC_MAX_CELLS;
static __device__ __align__(256) double g_noalloc_scratch[5 * NOALLOC_MAX_CELLS];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// device address of the scratch for the current device, looked up once per
// device with that device current
int noalloc_scratch(double **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        cudaGetLastError();
        return VERIS_ERR_LAUNCH;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
            cudaGetLastError();
            return VERIS_ERR_LAUNCH;
        }
        g_noalloc_ptr[dev] = static_cast<double *>(ptr);
    }
    *out = g_noalloc_ptr[dev];
    return VERIS_OK;
}

}  // namespace

extern "C" int veris_evp_solver_f64_noalloc(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                            int32_t n, double *u, double *v, double *s1, double *s2, double *s12,
                                            veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    if ((int64_t)d.NX * d.ld > NOALLOC_MAX_CELLS) return VERIS_ERR_TOO_LARGE;
    VERIS_REQUIRE(p && vs && u && v && s1 && s2 && s12, VERIS_ERR_ARG);
    VERIS_REQUIRE(n >= 0, VERIS_ERR_ARG);
    double *scratch = nullptr;
    const int st = noalloc_scratch(&scratch);
    if (st != VERIS_OK) return st;
    // the five scratch buffers follow each other at NX * ld elements
    const size_t per = (size_t)d.NX * d.ld;
    const size_t need = 5 * round_up(per * sizeof(double), 256);
    return evp_solver<double>(g, p, reinterpret_cast<const Fields<double> *>(vs), n, u, v, s1, s2, s12, scratch,
                              need <= sizeof(g_noalloc_scratch) ? need : 0, s);
}
