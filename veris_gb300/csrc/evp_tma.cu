// TMA-staged float32 mEVP subcycle (veris/evp_solver.py:21-254).
//
// Persistent form: one 1024-thread CTA per SM walks its share of 28 x 28
// output tiles with a two-stage pipeline.  While the CTA computes tile k from
// one shared-memory stage, the tensor-memory-access unit fills the other
// stage with tile k+1: the tile plus a 2-cell ring (32 x 32 points) of every
// input the stencils reach, and the eight per-point constants of the 28 x 28
// tile, all tiled cp.async.bulk.tensor loads issued by one thread and
// completing on that stage's mbarrier.  After a bounded wait the few staged
// cells that wrap around the padded array are patched (TMA fills out-of-range
// cells with zeros; the reference's roll wraps), then four stages run from
// shared memory:
//
//   lane = staged column, warp w = staged row w, so every stencil
//   neighbour is a fixed offset (+-1 column, +-ROW row) into one common
//   32 x 40 layout; no index is divided or wrapped per point.
//
// Intermediates are written in place over staged inputs that are dead by
// then; before a stage is refilled every thread fences its generic writes
// against the async proxy.  Box origins along the contiguous axis are 16-byte
// aligned (x = j0 - 4 or j0, j0 a multiple of 28); rows may start at -2 or run
// past the last row, where TMA reads the zero fill.  Division and square root
// use the approximate hardware forms (relative error ~2^-22), well inside
// the float32 path's stated error.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "evp_fast.cuh"

namespace veris {

namespace tma {

constexpr int TO = 28;            // output tile: rows and columns
constexpr int SR = 32;            // staged rows and columns (tile + ring)
constexpr int ROW = 40;           // ring-box row length: columns j0-4 .. j0+35
constexpr int THREADS = 1024;     // 32 warps x 1 staged row
constexpr int RPW = 1;            // staged rows per warp
constexpr int RING_BYTES = SR * ROW * 4;          // 5120, a multiple of 128
constexpr int OWN_BYTES = TO * TO * 4;            // 3136
constexpr int OWN_STRIDE = (OWN_BYTES + 127) / 128 * 128;

// ring arrays of one pipeline stage (box ROW x SR at x = j0 - 4, y = i0 - 2)
enum { R_U, R_V, R_UOC, R_VOC, R_FLG, R_S1, R_S2, R_MFC, R_PH, R_QRA, R_S12, R_RAZ, R_BFAC, R_STAGE };
constexpr int N_RING_LOADS = 12;  // R_U .. R_RAZ (+ R_BFAC with basal drag)
// own-point arrays (box TO x TO at x = j0, y = i0)
enum { O_CU, O_CV, O_AW, O_AS, O_MU, O_MV, O_RRAU, O_RRAV, O_COUNT };

constexpr int STAGE_BYTES = R_STAGE * RING_BYTES + O_COUNT * OWN_STRIDE;   // 92160
constexpr int OFF_E12 = 2 * STAGE_BYTES;
constexpr int OFF_FU = OFF_E12 + RING_BYTES;
constexpr int OFF_BAR = OFF_FU + RING_BYTES;
constexpr int SMEM_BYTES = OFF_BAR + 128;                                   // 194688

// tensor maps: 5 state arrays x 2 ping-pong buffers, then the constants
enum {
    M_U0, M_V0, M_S10, M_S20, M_S120,
    M_U1, M_V1, M_S11, M_S21, M_S121,
    M_UOC, M_VOC, M_FLG, M_MFC, M_PH, M_QRA, M_RAZ, M_BFAC,
    M_CU, M_CV, M_AW, M_AS, M_MU, M_MV, M_RRAU, M_RRAV,
    M_COUNT
};

struct __align__(64) Maps {
    CUtensorMap m[M_COUNT];
};

__device__ __forceinline__ uint32_t saddr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (TMA) accesses of the same memory
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     saddr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: false after `limit` unsuccessful polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            saddr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(saddr(bar))
        : "memory");
}

__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

constexpr uint32_t WAIT_LIMIT = 1u << 20;

// staged point (r, l) of a ring array
__device__ __forceinline__ int ring(int r, int l) { return r * ROW + l + 2; }

// overwrite staged cells whose padded coordinates fall outside the array
// with the wrapped values
template <class E>
__device__ void patch(E *s, const E *g, int64_t lp, const Dims &d, int i0, int j0) {
    for (int idx = threadIdx.x; idx < SR * SR; idx += THREADS) {
        const int r = idx / SR, l = idx % SR;
        const int gi = i0 + r - 2, gj = j0 + l - 2;
        if (gi >= 0 && gi < d.NX && gj >= 0 && gj < d.NY) continue;
        s[ring(r, l)] = __ldg(g + (int64_t)d.wx(gi) * lp + d.wy(gj));
    }
}

struct Src {
    const float *u, *v, *s1, *s2, *s12;   // the state buffer this launch reads
};

__device__ __forceinline__ void store_out(float *out, int64_t ldo, const Dims &d, const HaloFill &h, bool images,
                                          int i, int j, float val) {
    if (images) store_filled_ld(out, ldo, d, h, i, j, val);
    else out[(int64_t)i * ldo + j] = val;
}

template <bool BASAL, bool TURN>
__global__ void __launch_bounds__(THREADS, 1)
evp_tma_kernel(const __grid_constant__ Maps maps, Dims d, int64_t lp, HaloFill h, FastConsts<float> c,
               FastScalars<float> k, Src src, int buf, int ntx, int ntiles, float *uo, float *vo, float *s1o,
               float *s2o, float *s12o, int64_t ldo, int *status) {
    extern __shared__ __align__(128) unsigned char sm[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + OFF_BAR);
    float *sE12 = reinterpret_cast<float *>(sm + OFF_E12);
    float *sFu = reinterpret_cast<float *>(sm + OFF_FU);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int sb = 5 * buf;

    // issue the loads of tile t into pipeline stage s
    auto issue = [&](int t, int s) {
        unsigned char *base = sm + s * STAGE_BYTES;
        const int i0 = (t / ntx) * TO, j0 = (t % ntx) * TO;
        const uint32_t bytes = (N_RING_LOADS + (BASAL ? 1 : 0)) * RING_BYTES + O_COUNT * OWN_BYTES;
        mbar_arrive_expect_tx(&bar[s], bytes);
        const int xr = j0 - 4, yr = i0 - 2;
        auto ringp = [&](int q) { return base + q * RING_BYTES; };
        tma_load_2d(ringp(R_U), &maps.m[M_U0 + sb], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_V), &maps.m[M_V0 + sb], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_S1), &maps.m[M_S10 + sb], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_S2), &maps.m[M_S20 + sb], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_S12), &maps.m[M_S120 + sb], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_UOC), &maps.m[M_UOC], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_VOC), &maps.m[M_VOC], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_FLG), &maps.m[M_FLG], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_MFC), &maps.m[M_MFC], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_PH), &maps.m[M_PH], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_QRA), &maps.m[M_QRA], xr, yr, &bar[s]);
        tma_load_2d(ringp(R_RAZ), &maps.m[M_RAZ], xr, yr, &bar[s]);
        if (BASAL) tma_load_2d(ringp(R_BFAC), &maps.m[M_BFAC], xr, yr, &bar[s]);
#pragma unroll
        for (int q = 0; q < O_COUNT; ++q)
            tma_load_2d(base + R_STAGE * RING_BYTES + q * OWN_STRIDE, &maps.m[M_CU + q], j0, i0, &bar[s]);
    };

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
        fence_proxy_async();
    }
    __syncthreads();
    int t = blockIdx.x;
    if (tid == 0 && t < ntiles) issue(t, 0);
    uint32_t phase[2] = {0u, 0u};

    for (int kk = 0; t < ntiles; ++kk, t += gridDim.x) {
        const int s = kk & 1;
        const int tn = t + gridDim.x;
        if (tid == 0 && tn < ntiles) issue(tn, s ^ 1);   // stage s^1 was released at the end of tile kk-1

        const bool ok = mbar_wait_bounded(&bar[s], phase[s], WAIT_LIMIT);
        phase[s] ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(status, S_TMA_TIMEOUT);
            // let the copies in flight land before the CTA leaves
            mbar_wait_bounded(&bar[s], phase[s] ^ 1u, WAIT_LIMIT);
            if (tn < ntiles) mbar_wait_bounded(&bar[s ^ 1], phase[s ^ 1], WAIT_LIMIT);
            return;
        }

        unsigned char *base = sm + s * STAGE_BYTES;
        float *R[R_STAGE];
#pragma unroll
        for (int q = 0; q < R_STAGE; ++q) R[q] = reinterpret_cast<float *>(base + q * RING_BYTES);
        float *sU = R[R_U], *sV = R[R_V], *sUo = R[R_UOC], *sVo = R[R_VOC];
        const uint32_t *sF = reinterpret_cast<const uint32_t *>(R[R_FLG]);
        float *sS1 = R[R_S1], *sS2 = R[R_S2], *sMf = R[R_MFC], *sPh = R[R_PH], *sQr = R[R_QRA];
        float *sS12 = R[R_S12], *sRz = R[R_RAZ], *sBf = R[R_BFAC];
        const float *O = reinterpret_cast<const float *>(base + R_STAGE * RING_BYTES);
        constexpr int OS = OWN_STRIDE / 4;

        const int i0 = (t / ntx) * TO, j0 = (t % ntx) * TO;
        if (i0 < 2 || i0 + TO + 2 > d.NX || j0 < 2 || j0 + TO + 2 > d.NY) {
            patch(sU, src.u, lp, d, i0, j0);
            patch(sV, src.v, lp, d, i0, j0);
            patch(sS1, src.s1, lp, d, i0, j0);
            patch(sS2, src.s2, lp, d, i0, j0);
            patch(sS12, src.s12, lp, d, i0, j0);
            patch(sUo, (const float *)c.uOc, lp, d, i0, j0);
            patch(sVo, (const float *)c.vOc, lp, d, i0, j0);
            patch(reinterpret_cast<uint32_t *>(R[R_FLG]), (const uint32_t *)c.flags, lp, d, i0, j0);
            patch(sMf, (const float *)c.mfC, lp, d, i0, j0);
            patch(sPh, (const float *)c.Ph, lp, d, i0, j0);
            patch(sQr, (const float *)c.qrA, lp, d, i0, j0);
            patch(sRz, (const float *)c.rAz, lp, d, i0, j0);
            if (BASAL) patch(sBf, (const float *)c.bfac, lp, d, i0, j0);
            __syncthreads();
        }
        // halo-image stores are only needed near the refreshed halos
        const bool images = (h.x_fill && (i0 < 4 || i0 + TO > d.NX - 4)) ||
                            (h.y_fill && (j0 < 4 || j0 + TO > d.NY - 4));

        const int gj = d.wy(j0 + lane - 2);
        const float rdyU = __ldg(c.rdyU_y + gj), rdyV = __ldg(c.rdyV_y + gj);
        const float dyV = __ldg(c.dyV_y + gj), dyU = __ldg(c.dyU_y + gj);
        const int r0 = warp * RPW;
        // per-row grid lengths of this warp's staged rows, loaded up front
        float rdxV_r[RPW], rdxU_r[RPW], dxU_r[RPW], dxV_r[RPW];
#pragma unroll
        for (int q = 0; q < RPW; ++q) {
            const int gi = d.wx(i0 + r0 + q - 2);
            rdxV_r[q] = __ldg(c.rdxV_x + gi);
            rdxU_r[q] = __ldg(c.rdxU_x + gi);
            dxU_r[q] = __ldg(c.dxU_x + gi);
            dxV_r[q] = __ldg(c.dxV_x + gi);
        }

        // ---- A: e12 at Z points, staged rows/cols [1, 32); rAz*e12^2 in place of rAz
#pragma unroll
        for (int q = 0; q < RPW; ++q) {
            const int r = r0 + q;
            if (r < 1 || lane < 1) continue;
            const int x = ring(r, lane);
            const float rdxV = rdxV_r[q];
            const uint32_t f0 = sF[x], fw = sF[x - ROW], fs = sF[x - 1], fws = sF[x - ROW - 1];
            const float mzh = (f0 & fw & fs & fws & F_MC) ? 0.5f : 0.f;
            const float hU = one_if<float>(f0, F_MU) - one_if<float>(fs, F_MU);
            const float hV = one_if<float>(f0, F_MV) - one_if<float>(fw, F_MV);
            const float u0 = sU[x], us = sU[x - 1], v0 = sV[x], vw = sV[x - ROW];
            const float e = rdyU * (mzh * (u0 - us) + hU * (u0 + us)) + rdxV * (mzh * (v0 - vw) + hV * (v0 + vw));
            sE12[x] = e;
            sRz[x] = sRz[x] * (e * e);
        }
        __syncthreads();

        // ---- B: viscosities at C points [1, 31); stresses, drag, Coriolis on [1, 30)
#pragma unroll
        for (int q = 0; q < RPW; ++q) {
            const int r = r0 + q;
            if (r < 1 || r > 30 || lane < 1 || lane > 30) continue;
            const int x = ring(r, lane);
            const uint32_t f0 = sF[x];
            const float mInC = one_if<float>(f0, F_INC);
            const float u0 = sU[x], ue = sU[x + ROW], v0 = sV[x], vn = sV[x + 1];
            const float e11 = (ue - u0) * rdxU_r[q] * mInC;
            const float e22 = (vn - v0) * rdyV * mInC;
            const float e12c = sQr[x] * ((sRz[x] + sRz[x + ROW]) + (sRz[x + 1] + sRz[x + ROW + 1]));
            const float ep = e11 + e22, em = e11 - e22;
            const float delta = sqrt_approx(ep * ep + k.rsq * (em * em + 4.f * e12c));
            const float zeta = __fdividef(sPh[x], delta + k.deltaMin);
            sPh[x] = zeta;
            if (r > 29 || lane > 29) continue;
            const float mC = one_if<float>(f0, F_MC);
            const float press = k.kp * zeta * delta;
            const float s1 = (sS1[x] * k.alpha_m1 + (2.f * zeta * ep - press)) * k.ralpha * mC;
            const float s2 = (sS2[x] * k.alpha_m1 + 0.5f * zeta * em) * k.ralpha * mC;
            sS1[x] = 0.5f * (s1 + s2) * dyV;
            sS2[x] = 0.5f * (s1 - s2) * dxU_r[q];
            if (r >= 2 && lane >= 2) {
                const int oi = i0 + r - 2, oj = j0 + lane - 2;
                if (oi < d.NX && oj < d.NY) {
                    const int64_t w = (int64_t)oi * ldo + oj;
                    s1o[w] = s1;
                    s2o[w] = s2;
                }
            }
            const uint32_t fe = sF[x + ROW], fn = sF[x + 1];
            const float du0 = (u0 - sUo[x]) * one_if<float>(f0, F_INU);
            const float du1 = (ue - sUo[x + ROW]) * one_if<float>(fe, F_INU);
            const float dv0 = (v0 - sVo[x]) * one_if<float>(f0, F_INV);
            const float dv1 = (vn - sVo[x + 1]) * one_if<float>(fn, F_INV);
            const float tt = 0.25f * ((du0 + du1) * (du0 + du1) + (dv0 + dv1) * (dv0 + dv1));
            const bool south = f0 & F_SOUTH;
            const float dc = south ? k.dS : k.dN, dc2 = south ? k.dS2 : k.dN2;
            sQr[x] = ((dc2 * tt > k.cmin2) ? dc * sqrt_approx(tt) : k.cmin) * mC;
            if (BASAL) {
                const float a = u0 * one_if<float>(f0, F_INU), b = ue * one_if<float>(fe, F_INU);
                const float cc = v0 * one_if<float>(f0, F_INV), e = vn * one_if<float>(fn, F_INV);
                const float sq2 = 0.25f * (a * a + b * b + cc * cc + e * e);
                sBf[x] = __fdividef(sBf[x], sqrt_approx(sq2 + k.U02));
            }
            const float mf = sMf[x];
            sMf[x] = mf * (v0 + vn);
            sFu[x] = mf * (u0 + ue);
        }
        __syncthreads();

        // ---- C: sigma12 at Z points [2, 31), in place of the old sigma12
#pragma unroll
        for (int q = 0; q < RPW; ++q) {
            const int r = r0 + q;
            if (r < 2 || r > 30 || lane < 2 || lane > 30) continue;
            const int x = ring(r, lane);
            const int n = ((sF[x] & F_MC) ? 1 : 0) + ((sF[x - ROW] & F_MC) ? 1 : 0) + ((sF[x - 1] & F_MC) ? 1 : 0) +
                          ((sF[x - ROW - 1] & F_MC) ? 1 : 0);
            const float norm = n == 0 ? 0.f : (n == 1 ? 1.f : (n == 2 ? 0.5f : (n == 3 ? 1.f / 3.f : 0.25f)));
            const float zz = norm * ((sPh[x] + sPh[x - ROW]) + (sPh[x - 1] + sPh[x - ROW - 1]));
            const float s12 = (sS12[x] * k.alpha_m1 + 0.5f * zz * sE12[x]) * k.ralpha;
            sS12[x] = s12;
            if (r < 30 && lane < 30) {
                const int oi = i0 + r - 2, oj = j0 + lane - 2;
                if (oi < d.NX && oj < d.NY) s12o[(int64_t)oi * ldo + oj] = s12;
            }
        }
        __syncthreads();

        // ---- D: u and v at the tile's U and V points, staged [2, 30)
#pragma unroll
        for (int q = 0; q < RPW; ++q) {
            const int r = r0 + q;
            if (r < 2 || r > 29 || lane < 2 || lane > 29) continue;
            const int gi = i0 + r - 2, gjo = j0 + lane - 2;
            if (gi >= d.NX || gjo >= d.NY) continue;
            const int x = ring(r, lane);
            const int xo = (r - 2) * TO + (lane - 2);
            const uint32_t f0 = sF[x];
            const float u0 = sU[x], v0 = sV[x];
            const float cd0 = sQr[x], cdw = sQr[x - ROW], cds = sQr[x - 1];
            const float dxV = dxV_r[q];
            {   // U point
                const float AW = O[O_AW * OS + xo], mU = O[O_MU * OS + xo];
                const float kU = k.halfCos * AW * (cd0 + cdw);
                float fx = O[O_CU * OS + xo] + kU * sUo[x] + 0.5f * (sMf[x] + sMf[x - ROW]);
                if (TURN) {
                    const float sg = (f0 & F_SPOS) ? 1.f : ((f0 & F_SNEG) ? -1.f : 0.f);
                    const float du0 = sUo[x] - u0, dun = sUo[x + 1] - sU[x + 1];
                    const float duw = sUo[x - ROW] - sU[x - ROW], duwn = sUo[x - ROW + 1] - sU[x - ROW + 1];
                    fx -= sg * k.sinW * 0.5f * (cd0 * 0.5f * (du0 + dun) + cdw * 0.5f * (duw + duwn)) *
                          one_if<float>(f0, F_LMU) * AW;
                }
                const float sdx = O[O_RRAU * OS + xo] * ((sS1[x] - sS1[x - ROW]) + dxV * (sS12[x + 1] - sS12[x]));
                float den = mU * k.bU1 + kU;
                if (BASAL) den += 0.5f * AW * (sBf[x] + sBf[x - ROW]);
                den = den == 0.f ? 1.f : den;
                store_out(uo, ldo, d, h, images, gi, gjo,
                          one_if<float>(f0, F_MU) * __fdividef(k.bU * mU * u0 + fx + sdx, den));
            }
            {   // V point
                const float AS = O[O_AS * OS + xo], mV = O[O_MV * OS + xo];
                const float kV = k.halfCos * AS * (cd0 + cds);
                float fy = O[O_CV * OS + xo] + kV * sVo[x] - 0.5f * (sFu[x] + sFu[x - 1]);
                if (TURN) {
                    const float sg = (f0 & F_SPOS) ? 1.f : ((f0 & F_SNEG) ? -1.f : 0.f);
                    const float dv0 = sVo[x] - v0, dve = sVo[x + ROW] - sV[x + ROW];
                    const float dvs = sVo[x - 1] - sV[x - 1], dvse = sVo[x + ROW - 1] - sV[x + ROW - 1];
                    fy += sg * k.sinW * 0.5f * (cd0 * 0.5f * (dv0 + dve) + cds * 0.5f * (dvs + dvse)) *
                          one_if<float>(f0, F_LMV) * AS;
                }
                const float sdy = O[O_RRAV * OS + xo] * ((sS2[x] - sS2[x - 1]) + dyU * (sS12[x + ROW] - sS12[x]));
                float den = mV * k.bU1 + kV;
                if (BASAL) den += 0.5f * AS * (sBf[x] + sBf[x - 1]);
                den = den == 0.f ? 1.f : den;
                store_out(vo, ldo, d, h, images, gi, gjo,
                          one_if<float>(f0, F_MV) * __fdividef(k.bU * mV * v0 + fy + sdy, den));
            }
        }
        // release stage s: generic writes ordered before the TMA refill of tile kk+2
        fence_proxy_async();
        __syncthreads();
    }
}

// ------------------------------------------------------------------ host
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// a 2-D map over an internal array (NY columns of 4-byte elements, pitch lp)
static bool encode(CUtensorMap *m, const void *base, bool is_uint, const Dims &d, int64_t lp, int box_w, int box_h) {
    auto fn = encode_fn();
    if (!fn) return false;
    if (reinterpret_cast<uintptr_t>(base) % 16 != 0 || (lp * 4) % 16 != 0) return false;
    cuuint64_t dims[2] = {(cuuint64_t)d.NY, (cuuint64_t)d.NX};
    cuuint64_t strides[1] = {(cuuint64_t)(lp * 4)};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult res = fn(m, is_uint ? CU_TENSOR_MAP_DATA_TYPE_UINT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                      const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return res == CUDA_SUCCESS;
}

// persistent grid: one CTA per SM (1 when the count is unavailable)
static int persistent_ctas() {
    const int n = sm_count();
    return n > 0 ? n : 1;
}

template <bool B, bool R>
static int launch(const Maps &maps, const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<float> &c,
                  const FastScalars<float> &k, const Src &src, int buf, float *const dst[5], int64_t ldo,
                  int *status, cudaStream_t st) {
    auto kern = evp_tma_kernel<B, R>;
    static std::atomic<bool> configured[MAX_DEVICES];
    if (!smem_configured(configured, kern, SMEM_BYTES)) return VERIS_ERR_LAUNCH;
    const int ntx = (d.NY + TO - 1) / TO, nti = (d.NX + TO - 1) / TO;
    const int ntiles = ntx * nti;
    const int grid = ntiles < persistent_ctas() ? ntiles : persistent_ctas();
    kern<<<grid, THREADS, SMEM_BYTES, st>>>(maps, d, lp, h, c, k, src, buf, ntx, ntiles, dst[0], dst[1], dst[2],
                                            dst[3], dst[4], ldo, status);
    return launch_status();
}

}  // namespace tma

bool evp_tma_available() { return tma::encode_fn() != nullptr; }

int evp_tma_subcycles(const Dims &d, const HaloFill &h, const FastConsts<float> &c, const FastScalars<float> &k,
                      float *const state[2][5], float *const outs[5], int64_t ldo, int n, int *status, bool basal,
                      bool turn, cudaStream_t st) {
    using namespace tma;
    // the tiles' rings wrap within one period only on grids wider than a tile
    // plus its ring: smaller grids take the shared-memory form
    if (d.NX < SR + 2 || d.NY < SR + 2) return VERIS_ERR_UNSUPPORTED;
    const int64_t lp = internal_pitch(d.NY);
    Maps maps;
    bool ok = true;
    for (int b = 0; b < 2; ++b)
        for (int q = 0; q < 5; ++q) ok = ok && encode(&maps.m[M_U0 + 5 * b + q], state[b][q], false, d, lp, ROW, SR);
    const void *ring_src[8] = {c.uOc, c.vOc, c.flags, c.mfC, c.Ph, c.qrA, c.rAz, c.bfac};
    for (int q = 0; q < 8; ++q) ok = ok && encode(&maps.m[M_UOC + q], ring_src[q], q == 2, d, lp, ROW, SR);
    const void *own_src[8] = {c.cU, c.cV, c.AW, c.AS, c.mU, c.mV, c.rrAu, c.rrAv};
    for (int q = 0; q < 8; ++q) ok = ok && encode(&maps.m[M_CU + q], own_src[q], false, d, lp, TO, TO);
    if (!ok) return VERIS_ERR_UNSUPPORTED;
    for (int it = 0; it < n; ++it) {
        const bool last = it == n - 1;
        const int buf = it % 2;
        const Src src{state[buf][0], state[buf][1], state[buf][2], state[buf][3], state[buf][4]};
        float *const *dst = last ? outs : state[(it + 1) % 2];
        const int64_t lo = last ? ldo : lp;
        int stt;
        if (basal)
            stt = turn ? launch<true, true>(maps, d, lp, h, c, k, src, buf, dst, lo, status, st)
                       : launch<true, false>(maps, d, lp, h, c, k, src, buf, dst, lo, status, st);
        else
            stt = turn ? launch<false, true>(maps, d, lp, h, c, k, src, buf, dst, lo, status, st)
                       : launch<false, false>(maps, d, lp, h, c, k, src, buf, dst, lo, status, st);
        if (stt != VERIS_OK) return stt;
    }
    return VERIS_OK;
}

}  // namespace veris

// ---------------------------------------------------------------------------
// Probe of the bounded mbarrier wait the TMA kernel uses (failure detection
// without a fault): one warp initialises an mbarrier expecting one arrival,
// arrives on it or not, and waits on it with mbar_wait_bounded.  When nothing
// arrives the wait gives up after `limit` polls and the probe sets the same
// status bit the TMA kernel sets (S_TMA_TIMEOUT) in *status; the kernel then
// returns normally and the context stays usable.
namespace veris {
namespace tma {

__global__ void mbar_wait_probe_kernel(int arrive, uint32_t limit, int *status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    fence_barrier_init();
    __syncthreads();
    if (arrive && threadIdx.x == 0)
        asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(saddr(&bar))
                     : "memory");
    const bool ok = mbar_wait_bounded(&bar, 0u, limit);
    __syncthreads();
    if (threadIdx.x == 0) {
        *status = ok ? 0 : S_TMA_TIMEOUT;
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(saddr(&bar)) : "memory");
    }
}

}  // namespace tma
}  // namespace veris

extern "C" int veris_mbarrier_wait_probe(int32_t arrive, uint32_t limit, int32_t *status_device, veris_stream_t s) {
    using namespace veris;
    VERIS_REQUIRE(status_device && limit > 0 && limit <= tma::WAIT_LIMIT, VERIS_ERR_ARG);
    tma::mbar_wait_probe_kernel<<<1, 32, 0, (cudaStream_t)s>>>(arrive ? 1 : 0, limit, status_device);
    return launch_status();
}
