// Register-walking float32 mEVP subcycle kernels (the walk is in
// evp_walk.cuh): one launch per subcycle, one warp per walk, and the host
// loop with the walk-length choice.
#include <atomic>

#include "evp_walk.cuh"

namespace veris {
namespace walk {

constexpr int WARPS = 4;    // warps per CTA
// kernel variants: (loop unroll, CTAs per SM the register budget must allow,
// own-point constants loaded a step early)
template <int V>
struct Variant;
template <>
struct Variant<0> { static constexpr int UNROLL = 1, MINB = 1; static constexpr bool PRE = false; };
template <>
struct Variant<1> { static constexpr int UNROLL = 1, MINB = 5; static constexpr bool PRE = false; };
template <>
struct Variant<2> { static constexpr int UNROLL = 1, MINB = 4; static constexpr bool PRE = false; };
template <>
struct Variant<3> { static constexpr int UNROLL = 1, MINB = 4; static constexpr bool PRE = true; };
constexpr int N_VARIANTS = N_WALK_VARIANTS;

template <bool BASAL, bool TURN, int V, bool ADAPT, int L>
__global__ void __launch_bounds__(WARPS * 32, Variant<V>::MINB)
evp_walk_kernel(Dims d, int64_t lp, HaloFill h, FastConsts<float> c, FastScalars<float> k, FastIO<float> io,
                int nstrips, int nwalks, int H) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * WARPS + (threadIdx.x >> 5);
    if (w >= nwalks) return;   // whole warps only
    const int strip = w % nstrips, rb = w / nstrips;
    // the single-domain walk takes the cell areas along j (the caller has
    // checked that the state's areas vary along j only: V_AREA2D clear)
    walk_strip<BASAL, TURN, Variant<V>::UNROLL, Variant<V>::PRE, ADAPT, (L != 0), (L == 1 || L == 3), true, false,
               (L == 3)>(d, lp, h, c, k, io, rb * H, strip * TW, H, lane);
}

// ---------------------------------------------------------------- persistent
// Several subcycles per launch.  Every walk is resident for the whole launch
// (a cooperative launch guarantees it) and runs its strip and rows for
// subcycle after subcycle on the walk's ping-pong state.  Before subcycle k
// it waits until the walks whose rows and columns its stencil reads, and
// those that read its own, have finished subcycle k - 1: the neighbouring
// row blocks and strips, and where a filled halo makes the opposite edge's
// images part of the stencil, the two blocks (strips) at each edge.  The
// wait is on per-walk progress counters (release after the walk's stores,
// acquire before its loads); it gives up after about half a second, sets
// S_WALK_TIMEOUT in the status word and ends the walk, and every walk that
// waits on it ends the same way.  No grid-wide barrier.

__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// true once *flag >= target; false (S_WALK_TIMEOUT set) after 2^22 polls
// or when another walk has given up
__device__ bool wait_progress(const int *flag, int target, int *status) {
    for (int spin = 0; spin < (1 << 22); ++spin) {
        if (ld_acquire(flag) >= target) return true;
        if ((spin & 255) == 255) {
            if (ld_acquire(status) & S_WALK_TIMEOUT) return false;
            __nanosleep(64);
        }
    }
    atomicOr(status, S_WALK_TIMEOUT);
    return false;
}

// the blocks a walk depends on along one axis: b-1, b, b+1 (wrapping), and
// with a filled halo near an edge the first two and last two blocks
__device__ __forceinline__ int axis_neighbours(int b, int nb, bool filled, int out[7]) {
    int n = 0;
    auto add = [&](int x) {
        x = ((x % nb) + nb) % nb;
        for (int q = 0; q < n; ++q)
            if (out[q] == x) return;
        out[n++] = x;
    };
    add(b - 1);
    add(b);
    add(b + 1);
    if (filled && (b <= 1 || b >= nb - 2)) {
        add(0);
        add(1);
        add(nb - 2);
        add(nb - 1);
    }
    return n;
}

template <bool BASAL, bool TURN, int V, bool ADAPT>
__global__ void __launch_bounds__(WARPS * 32, Variant<V>::MINB)
evp_walk_persistent_kernel(Dims d, int64_t lp, HaloFill h, FastConsts<float> c, FastScalars<float> k,
                           FastIO<float> io0, FastIO<float> io1, int n, int nstrips, int nblk, int H, int *status) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * WARPS + (threadIdx.x >> 5);
    if (w >= nstrips * nblk) return;   // whole warps only
    const int strip = w % nstrips, rb = w / nstrips;
    int rbs[7], sts[7];
    const int nr = axis_neighbours(rb, nblk, h.x_fill, rbs), ns = axis_neighbours(strip, nstrips, h.y_fill, sts);
    for (int it = 0; it < n; ++it) {
        if (it > 0) {
            bool ok = true;
            for (int q = lane; q < nr * ns; q += 32)
                ok = ok && wait_progress(c.wprog + rbs[q / ns] * nstrips + sts[q % ns], it, status);
            if (!__all_sync(0xffffffffu, ok)) return;
        }
        walk_strip<BASAL, TURN, Variant<V>::UNROLL, Variant<V>::PRE, ADAPT, true, true, true, true>(
            d, lp, h, c, k, (it & 1) ? io1 : io0, rb * H, strip * TW, H, lane);
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(c.wprog + w, it + 1);
    }
}

template <bool B, bool R, int V, bool A, int L>
static int launch(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<float> &c,
                  const FastScalars<float> &k, const FastIO<float> &io, int H, cudaStream_t st) {
    const int nstrips = (d.NY + TW - 1) / TW, nblk = (d.NX + H - 1) / H;
    const int nwalks = nstrips * nblk;
    evp_walk_kernel<B, R, V, A, L><<<(nwalks + WARPS - 1) / WARPS, WARPS * 32, 0, st>>>(d, lp, h, c, k, io,
                                                                                   nstrips, nwalks, H);
    return launch_status();
}

// walk length: the most rows per walk that still fits all walks in one wave
// of resident warps (rows >= 8); ring overhead per walk is 4 rows
template <bool B, bool R, int V, bool A, int L>
static int auto_rows(const Dims &d) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, evp_walk_kernel<B, R, V, A, L>, WARPS * 32, 0) !=
            cudaSuccess || sms <= 0 || per_sm <= 0) {
        cudaGetLastError();
        return 16;
    }
    const int strips = (d.NY + TW - 1) / TW;
    const int blocks_per_wave = (sms * per_sm * WARPS) / strips;   // row blocks that fit next to each other
    if (blocks_per_wave < 1) return 16;
    int rows = (d.NX + blocks_per_wave - 1) / blocks_per_wave;
    return rows < 8 ? 8 : (rows > 4096 ? 4096 : rows);
}

template <int V, bool A, int L>
static int launch_val(bool basal, bool turn, const Dims &d, int64_t lp, const HaloFill &h,
                      const FastConsts<float> &c, const FastScalars<float> &k, const FastIO<float> &io, int H,
                      cudaStream_t st) {
    if (H <= 0)
        H = basal ? (turn ? auto_rows<true, true, V, A, L>(d) : auto_rows<true, false, V, A, L>(d))
                  : (turn ? auto_rows<false, true, V, A, L>(d) : auto_rows<false, false, V, A, L>(d));
    if (basal)
        return turn ? launch<true, true, V, A, L>(d, lp, h, c, k, io, H, st)
                    : launch<true, false, V, A, L>(d, lp, h, c, k, io, H, st);
    return turn ? launch<false, true, V, A, L>(d, lp, h, c, k, io, H, st)
                : launch<false, false, V, A, L>(d, lp, h, c, k, io, H, st);
}

// layout L: 0 planar state in and out, 1 paired in and out, 2 paired in, planar out,
// 3 paired in and out with Delta, zeta and cDrag written (a float32 tape slot)
template <int V, int L>
static int launch_vl(bool adapt, bool basal, bool turn, const Dims &d, int64_t lp, const HaloFill &h,
                     const FastConsts<float> &c, const FastScalars<float> &k, const FastIO<float> &io, int H,
                     cudaStream_t st) {
    return adapt ? launch_val<V, true, L>(basal, turn, d, lp, h, c, k, io, H, st)
                 : launch_val<V, false, L>(basal, turn, d, lp, h, c, k, io, H, st);
}

template <int V>
static int launch_v(int layout, bool adapt, bool basal, bool turn, const Dims &d, int64_t lp, const HaloFill &h,
                    const FastConsts<float> &c, const FastScalars<float> &k, const FastIO<float> &io, int H,
                    cudaStream_t st) {
    if (layout == 1) return launch_vl<V, 1>(adapt, basal, turn, d, lp, h, c, k, io, H, st);
    if (layout == 2) return launch_vl<V, 2>(adapt, basal, turn, d, lp, h, c, k, io, H, st);
    if (layout == 3) {   // the tape's kernels: variant 0, constant alpha
        if constexpr (V == 0)
            if (!adapt) return launch_val<0, false, 3>(basal, turn, d, lp, h, c, k, io, H, st);
        return VERIS_ERR_UNSUPPORTED;
    }
    return launch_vl<V, 0>(adapt, basal, turn, d, lp, h, c, k, io, H, st);
}

// n subcycles in one persistent launch on the walk's ping-pong state
// (state[0] -> state[1] -> state[0] ...); VERIS_ERR_UNSUPPORTED when the
// walks cannot all be resident at once
template <bool B, bool R, int V, bool A>
static int launch_persistent(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<float> &c,
                             const FastScalars<float> &k, float *const state[2][5], int n, int H, int *status,
                             cudaStream_t st) {
    auto kern = evp_walk_persistent_kernel<B, R, V, A>;
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess ||
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WARPS * 32, 0) != cudaSuccess) {
        cudaGetLastError();
        return VERIS_ERR_LAUNCH;
    }
    if (!coop || sms <= 0 || per_sm <= 0) return VERIS_ERR_UNSUPPORTED;
    const int nstrips = (d.NY + TW - 1) / TW;
    if (H <= 0) {   // the shortest walks that still fit all of them in one wave of resident warps
        const int blocks_per_wave = (sms * per_sm * WARPS) / nstrips;
        if (blocks_per_wave < 1) return VERIS_ERR_UNSUPPORTED;
        H = (d.NX + blocks_per_wave - 1) / blocks_per_wave;
        H = H < 8 ? 8 : H;
    }
    const int nblk = (d.NX + H - 1) / H, nwalks = nstrips * nblk;
    const int blocks = (nwalks + WARPS - 1) / WARPS;
    if (H < 4 || nwalks > MAX_WALKS || blocks > sms * per_sm) return VERIS_ERR_UNSUPPORTED;
    if (cudaMemsetAsync(c.wprog, 0, (size_t)nwalks * sizeof(int), st) != cudaSuccess) return VERIS_ERR_LAUNCH;
    const FastIO<float> io0{state[0][0], state[0][1], state[0][2], state[0][3], state[0][4],
                            state[1][0], state[1][1], state[1][2], state[1][3], state[1][4], lp};
    const FastIO<float> io1{state[1][0], state[1][1], state[1][2], state[1][3], state[1][4],
                            state[0][0], state[0][1], state[0][2], state[0][3], state[0][4], lp};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(WARPS * 32);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, kern, d, lp, h, c, k, io0, io1, n, nstrips, nblk, H, status) != cudaSuccess) {
        cudaGetLastError();
        return VERIS_ERR_LAUNCH;
    }
    return VERIS_OK;
}

template <int V>
static int persistent_v(bool adapt, bool basal, bool turn, const Dims &d, int64_t lp, const HaloFill &h,
                        const FastConsts<float> &c, const FastScalars<float> &k, float *const state[2][5], int n,
                        int H, int *status, cudaStream_t st) {
    if (adapt)
        return basal ? (turn ? launch_persistent<true, true, V, true>(d, lp, h, c, k, state, n, H, status, st)
                             : launch_persistent<true, false, V, true>(d, lp, h, c, k, state, n, H, status, st))
                     : (turn ? launch_persistent<false, true, V, true>(d, lp, h, c, k, state, n, H, status, st)
                             : launch_persistent<false, false, V, true>(d, lp, h, c, k, state, n, H, status, st));
    return basal ? (turn ? launch_persistent<true, true, V, false>(d, lp, h, c, k, state, n, H, status, st)
                         : launch_persistent<true, false, V, false>(d, lp, h, c, k, state, n, H, status, st))
                 : (turn ? launch_persistent<false, true, V, false>(d, lp, h, c, k, state, n, H, status, st)
                         : launch_persistent<false, false, V, false>(d, lp, h, c, k, state, n, H, status, st));
}

// subcycles per launch of the float32 walk: 1, or all but the last (0 / 1)
static std::atomic<int> g_persistent{0};

}  // namespace walk

int evp_walk_subcycles(bool adapt, bool paired, const Dims &d, const HaloFill &h, const FastConsts<float> &c,
                       const FastScalars<float> &k,
                       float *const state[2][5], float *const outs[5], int64_t ldo, int n, bool basal, bool turn,
                       int rows, int variant, cudaStream_t st, bool paired_outs, int *status, float *const *rich) {
    const int64_t lp = internal_pitch(d.NY);
    if ((rows != 0 && (rows < 4 || rows > 4096)) || variant < 0 || variant >= walk::N_VARIANTS) return VERIS_ERR_ARG;
    if (rich && !(n == 1 && paired && paired_outs && !adapt && variant == 0)) return VERIS_ERR_ARG;
    int it0 = 0;
    if (paired && n >= 3 && status && walk::g_persistent.load(std::memory_order_relaxed)) {
        // subcycles 0 .. n-2 in one launch; the last below writes the caller's layout
        int stt;
        switch (variant) {
        case 1: stt = walk::persistent_v<1>(adapt, basal, turn, d, lp, h, c, k, state, n - 1, rows, status, st); break;
        case 2: stt = walk::persistent_v<2>(adapt, basal, turn, d, lp, h, c, k, state, n - 1, rows, status, st); break;
        case 3: stt = walk::persistent_v<3>(adapt, basal, turn, d, lp, h, c, k, state, n - 1, rows, status, st); break;
        default: stt = walk::persistent_v<0>(adapt, basal, turn, d, lp, h, c, k, state, n - 1, rows, status, st); break;
        }
        if (stt == VERIS_OK) it0 = n - 1;
        else if (stt != VERIS_ERR_UNSUPPORTED) return stt;
    }
    for (int it = it0; it < n; ++it) {
        const bool last = it == n - 1;
        const int b = it % 2;
        float *const *dst = last ? outs : state[(it + 1) % 2];
        FastIO<float> io{state[b][0], state[b][1], state[b][2], state[b][3], state[b][4],
                         dst[0], dst[1], dst[2], dst[3], dst[4], last ? ldo : lp};
        // paired: the state buffers hold (u, v, sigma1, sigma2) per point over
        // their four buffers; the last subcycle writes the caller's planar arrays
        int layout = paired ? ((last && !paired_outs) ? 2 : 1) : 0;
        if (rich) {   // checked above: one paired subcycle, paired outs, constant alpha, variant 0
            layout = 3;
            io.tDel = rich[0];
            io.tZeta = rich[1];
            io.tCd = rich[2];
        }
        int stt;
        switch (variant) {
        case 1: stt = walk::launch_v<1>(layout, adapt, basal, turn, d, lp, h, c, k, io, rows, st); break;
        case 2: stt = walk::launch_v<2>(layout, adapt, basal, turn, d, lp, h, c, k, io, rows, st); break;
        case 3: stt = walk::launch_v<3>(layout, adapt, basal, turn, d, lp, h, c, k, io, rows, st); break;
        default: stt = walk::launch_v<0>(layout, adapt, basal, turn, d, lp, h, c, k, io, rows, st); break;
        }
        if (stt != VERIS_OK) return stt;
    }
    return VERIS_OK;
}

}  // namespace veris

namespace veris {

// the walk's (u, v, sigma1, sigma2) layout (pitch lp) and planar sigma12 ->
// five planar arrays of pitch ldo
__global__ void unpack_walk_state_kernel(Dims d, int64_t lp, const float4 *q, const float *s12, float *u, float *v,
                                         float *s1, float *s2, float *s12o, int64_t ldo) {
    const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 8 + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    const int64_t o = (int64_t)i * lp + j, w = (int64_t)i * ldo + j;
    const float4 a = q[o];
    u[w] = a.x;
    v[w] = a.y;
    s1[w] = a.z;
    s2[w] = a.w;
    s12o[w] = s12[o];
}

int evp_walk_unpack(const Dims &d, const float *quad, const float *s12, float *const outs[5], int64_t ldo,
                    cudaStream_t st) {
    const int64_t lp = internal_pitch(d.NY);
    dim3 g((d.NY + 31) / 32, (d.NX + 7) / 8);
    unpack_walk_state_kernel<<<g, dim3(32, 8), 0, st>>>(d, lp, reinterpret_cast<const float4 *>(quad), s12,
                                                         outs[0], outs[1], outs[2], outs[3], outs[4], ldo);
    return launch_status();
}

}  // namespace veris

extern "C" int veris_evp_walk_persistent(int32_t on) {
    if (on != 0 && on != 1) return VERIS_ERR_ARG;
    veris::walk::g_persistent.store(on, std::memory_order_relaxed);
    return VERIS_OK;
}
