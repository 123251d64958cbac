// Batched ensemble of independent sea-ice domains of uneven sizes
// (veris/evp_solver.py:21-319 per member, float32 fast form).
//
// Every member keeps its own folded constants and ping-pong state in one
// caller-provided device workspace.  One launch advances ALL members by one
// subcycle: a persistent grid of CTAs pulls tile indices from a global work
// queue (one atomic per tile) over the concatenated tile lists of the members
// and runs the same shared-memory tile as the single-domain kernel
// (evp_tile.cuh), so each member's values are bit-identical to a
// single-domain run.  The queue counter is cleared once per call and each
// launch offsets its tickets by the tickets earlier launches drew (tiles +
// CTAs), so a call is a fixed sequence of a memset and n launches that a CUDA
// graph can capture.
//
// Workspace layout: [queue][member table][tile offsets per shape][members...]
// where each member holds the fast-form layout (constants + two states) and
// its float32 wind forcing (for refolding the momentum constant each step).
#include "evp_tile.cuh"
#include "evp_walk.cuh"

namespace veris {
namespace batch {

// shapes 0-3: shared-memory tiles (rows x columns); 4-8: register walks of
// 8, 16, 32, 64 or 128 rows over 28-column strips (one warp each; longer
// walks recompute fewer ring rows, shorter ones balance better)
constexpr int N_SHAPES = 9;
constexpr int FIRST_WALK = 4;
template <int S>
struct ShapeOf;
template <>
struct ShapeOf<0> { static constexpr int TI = 32, TJ = 32, MINB = 3; };
template <>
struct ShapeOf<1> { static constexpr int TI = 16, TJ = 32, MINB = 4; };
template <>
struct ShapeOf<2> { static constexpr int TI = 32, TJ = 16, MINB = 4; };
template <>
struct ShapeOf<3> { static constexpr int TI = 16, TJ = 16, MINB = 4; };

inline void shape_dims(int s, int *ti, int *tj) {
    static const int T[N_SHAPES][2] = {{32, 32}, {16, 32}, {32, 16}, {16, 16}, {8, 28}, {16, 28}, {32, 28},
                                       {64, 28}, {128, 28}};
    *ti = T[s][0];
    *tj = T[s][1];
}

struct Member {
    Dims d;
    int64_t lp;
    HaloFill h;
    FastConsts<float> c;
    float *state[2][5];
    float *WX, *WY;
    int *status;
};

// bytes of one member's region
static size_t member_bytes(const Dims &d) {
    FastConsts<float> c;
    float *st[2][5];
    int *status;
    const size_t fast = fast_layout<float>(d, nullptr, &c, st, &status);
    const size_t f2 = rup256((size_t)d.NX * internal_pitch(d.NY) * sizeof(float));
    return fast + 2 * f2;
}

static int dims_of(const VerisGrid &g, Dims *d) { return check_grid(&g, d); }

// offsets of the workspace parts; member m starts at members + moff[m]
static int layout(int n, const VerisGrid *grids, size_t *queue, size_t *table, size_t *tiles, size_t *members,
                  size_t *total, size_t *moff) {
    size_t off = 0;
    *queue = off;
    off += 256;
    *table = off;
    off += rup256((size_t)n * sizeof(Member));
    *tiles = off;
    off += rup256((size_t)N_SHAPES * (n + 1) * sizeof(int));
    *members = off;
    size_t mo = 0;
    for (int m = 0; m < n; ++m) {
        Dims d;
        const int st = dims_of(grids[m], &d);
        if (st != VERIS_OK) return st;
        if (moff) moff[m] = mo;
        mo += member_bytes(d);
    }
    off += mo;
    *total = off;
    return VERIS_OK;
}

static Member member_at(const VerisGrid &g, const VerisParams &p, char *base) {
    Member M;
    dims_of(g, &M.d);
    M.lp = internal_pitch(M.d.NY);
    M.h = halo_fill_of(p);
    const size_t fast = fast_layout<float>(M.d, base, &M.c, M.state, &M.status);
    const size_t f2 = rup256((size_t)M.d.NX * M.lp * sizeof(float));
    M.WX = reinterpret_cast<float *>(base + fast);
    M.WY = reinterpret_cast<float *>(base + fast + f2);
    return M;
}

template <int S, bool BASAL, bool TURN>
__global__ void __launch_bounds__(FAST_THREADS, ShapeOf<S>::MINB)
evp_batch_kernel(const Member *mem, const int *tile_start, int nmem, int ntiles, FastScalars<float> k, int buf,
                 unsigned *queue, unsigned base) {
    constexpr int TI = ShapeOf<S>::TI, TJ = ShapeOf<S>::TJ;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_t;
    for (;;) {
        if (threadIdx.x == 0) s_t = (int)(atomicAdd(queue, 1u) - base);
        __syncthreads();
        const int t = s_t;
        if (t >= ntiles) break;
        int lo = 0, hi = nmem - 1;   // last member whose first tile is <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(tile_start + mid) <= t) lo = mid;
            else hi = mid - 1;
        }
        const Member &m = mem[lo];
        const int lt = t - __ldg(tile_start + lo);
        const int ntx = (m.d.NY + TJ - 1) / TJ;
        FastIO<float> io;
        io.u = m.state[buf][0];
        io.v = m.state[buf][1];
        io.s1 = m.state[buf][2];
        io.s2 = m.state[buf][3];
        io.s12 = m.state[buf][4];
        io.uo = m.state[buf ^ 1][0];
        io.vo = m.state[buf ^ 1][1];
        io.s1o = m.state[buf ^ 1][2];
        io.s2o = m.state[buf ^ 1][3];
        io.s12o = m.state[buf ^ 1][4];
        io.ldo = m.lp;
        fast_tile<float, TI, TJ, BASAL, TURN>(smem_raw, m.d, m.lp, m.h, m.c, k, io, (lt / ntx) * TI,
                                              (lt % ntx) * TJ);
        __syncthreads();   // shared memory and s_t are reused by the next tile
    }
}

// the same work queue with one register walk per ticket, one ticket per warp
template <bool BASAL, bool TURN>
__global__ void __launch_bounds__(128, 4)
evp_batch_walk_kernel(const Member *mem, const int *walk_start, int nmem, int nwalks, FastScalars<float> k, int buf,
                      unsigned *queue, unsigned base, int H) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned tk = 0;
        if (lane == 0) tk = atomicAdd(queue, 1u);
        const int t = (int)(__shfl_sync(0xffffffffu, tk, 0) - base);
        if (t >= nwalks) break;
        int lo = 0, hi = nmem - 1;   // last member whose first walk is <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(walk_start + mid) <= t) lo = mid;
            else hi = mid - 1;
        }
        const Member &m = mem[lo];
        const int lt = t - __ldg(walk_start + lo);
        const int nstrips = (m.d.NY + walk::TW - 1) / walk::TW;
        FastIO<float> io;
        io.u = m.state[buf][0];
        io.v = m.state[buf][1];
        io.s1 = m.state[buf][2];
        io.s2 = m.state[buf][3];
        io.s12 = m.state[buf][4];
        io.uo = m.state[buf ^ 1][0];
        io.vo = m.state[buf ^ 1][1];
        io.s1o = m.state[buf ^ 1][2];
        io.s2o = m.state[buf ^ 1][3];
        io.s12o = m.state[buf ^ 1][4];
        io.ldo = m.lp;
        if ((__ldg(m.status + 1) & V_AREA2D) == 0)   // areas along j: held per lane
            walk::walk_strip<BASAL, TURN, 1, false, false, false, false, true>(
                m.d, m.lp, m.h, m.c, k, io, (lt / nstrips) * H, (lt % nstrips) * walk::TW, H, lane);
        else
            walk::walk_strip<BASAL, TURN, 1>(m.d, m.lp, m.h, m.c, k, io, (lt / nstrips) * H,
                                             (lt % nstrips) * walk::TW, H, lane);
    }
}

// cU = mU/dt u + WindForcingX, cV likewise, from the state in buffer buf
// (the fold fast_prep does once per step, for the steps after the first)
__global__ void refold_kernel(const Member *mem, int nmem, float rdt, int buf) {
    const Member &m = mem[blockIdx.y];
    const int64_t n = (int64_t)m.d.NX * m.lp;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        m.c.cU[q] = m.c.mU[q] * rdt * m.state[buf][0][q] + m.WX[q];
        m.c.cV[q] = m.c.mV[q] * rdt * m.state[buf][1][q] + m.WY[q];
    }
}

__global__ void forcing32_kernel(const double *WX, const double *WY, Dims d, int64_t lp, float *oX, float *oY) {
    const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 8 + threadIdx.y;
    if (i >= d.NX || j >= d.NY) return;
    oX[(int64_t)i * lp + j] = (float)WX[d.raw(i, j)];
    oY[(int64_t)i * lp + j] = (float)WY[d.raw(i, j)];
}

template <int S, bool B, bool R>
static int launch(const Member *mem, const int *ts, int nmem, int ntiles, const FastScalars<float> &k, int buf,
                  unsigned *queue, unsigned base, int blocks, cudaStream_t st) {
    auto kern = evp_batch_kernel<S, B, R>;
    const size_t sm = TileSmem<float, ShapeOf<S>::TI, ShapeOf<S>::TJ>::bytes();
    static std::atomic<bool> configured[MAX_DEVICES];
    if (!smem_configured(configured, kern, (int)sm)) return VERIS_ERR_LAUNCH;
    kern<<<blocks, FAST_THREADS, sm, st>>>(mem, ts, nmem, ntiles, k, buf, queue, base);
    return launch_status();
}

template <int S>
static int launch_s(bool basal, bool turn, const Member *mem, const int *ts, int nmem, int ntiles,
                    const FastScalars<float> &k, int buf, unsigned *queue, unsigned base, int blocks,
                    cudaStream_t st) {
    if (basal)
        return turn ? launch<S, true, true>(mem, ts, nmem, ntiles, k, buf, queue, base, blocks, st)
                    : launch<S, true, false>(mem, ts, nmem, ntiles, k, buf, queue, base, blocks, st);
    return turn ? launch<S, false, true>(mem, ts, nmem, ntiles, k, buf, queue, base, blocks, st)
                : launch<S, false, false>(mem, ts, nmem, ntiles, k, buf, queue, base, blocks, st);
}

template <bool B, bool R>
static int launch_walk(const Member *mem, const int *ts, int nmem, int ntiles, const FastScalars<float> &k, int buf,
                       unsigned *queue, unsigned base, int blocks, int H, cudaStream_t st) {
    evp_batch_walk_kernel<B, R><<<blocks, 128, 0, st>>>(mem, ts, nmem, ntiles, k, buf, queue, base, H);
    return launch_status();
}

static int launch_walk_s(bool basal, bool turn, const Member *mem, const int *ts, int nmem, int ntiles,
                         const FastScalars<float> &k, int buf, unsigned *queue, unsigned base, int blocks, int H,
                         cudaStream_t st) {
    if (basal)
        return turn ? launch_walk<true, true>(mem, ts, nmem, ntiles, k, buf, queue, base, blocks, H, st)
                    : launch_walk<true, false>(mem, ts, nmem, ntiles, k, buf, queue, base, blocks, H, st);
    return turn ? launch_walk<false, true>(mem, ts, nmem, ntiles, k, buf, queue, base, blocks, H, st)
                : launch_walk<false, false>(mem, ts, nmem, ntiles, k, buf, queue, base, blocks, H, st);
}

}  // namespace batch
}  // namespace veris

using namespace veris;
using namespace veris::batch;

extern "C" {

size_t veris_batch_workspace_bytes(int32_t n, const VerisGrid *grids) {
    if (n < 1 || !grids) return 0;
    size_t q, t, ts, m, total;
    if (layout(n, grids, &q, &t, &ts, &m, &total, nullptr) != VERIS_OK) return 0;
    return total;
}

int veris_batch_init(int32_t n, const VerisGrid *grids, const VerisParams *p, void *ws, size_t wsb) {
    VERIS_REQUIRE(n >= 1 && grids && p && ws, VERIS_ERR_ARG);
    size_t q, t, ts, mb, total;
    Member *host = static_cast<Member *>(malloc((size_t)n * sizeof(Member)));
    size_t *moff = static_cast<size_t *>(malloc((size_t)n * sizeof(size_t)));
    int *tiles = static_cast<int *>(malloc((size_t)N_SHAPES * (n + 1) * sizeof(int)));
    int st = (host && moff && tiles) ? layout(n, grids, &q, &t, &ts, &mb, &total, moff) : VERIS_ERR_ARG;
    if (st == VERIS_OK && wsb < total) st = VERIS_ERR_WORKSPACE;
    if (st == VERIS_OK) {
        char *base = static_cast<char *>(ws);
        for (int m = 0; m < n; ++m) host[m] = member_at(grids[m], *p, base + mb + moff[m]);
        for (int s = 0; s < N_SHAPES; ++s) {
            int ti, tj;
            shape_dims(s, &ti, &tj);
            int acc = 0;
            for (int m = 0; m < n; ++m) {
                tiles[s * (n + 1) + m] = acc;
                acc += ((host[m].d.NX + ti - 1) / ti) * ((host[m].d.NY + tj - 1) / tj);
            }
            tiles[s * (n + 1) + n] = acc;
        }
        if (cudaMemcpy(base + t, host, (size_t)n * sizeof(Member), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(base + ts, tiles, (size_t)N_SHAPES * (n + 1) * sizeof(int), cudaMemcpyHostToDevice) !=
                cudaSuccess ||
            cudaMemset(base + q, 0, 256) != cudaSuccess)
            st = VERIS_ERR_LAUNCH;
    }
    free(host);
    free(moff);
    free(tiles);
    return st;
}

int veris_batch_tiles(int32_t n, const VerisGrid *grids, int32_t shape) {
    if (n < 1 || !grids || shape < 0 || shape >= N_SHAPES) return -1;
    int ti, tj;
    shape_dims(shape, &ti, &tj);
    int acc = 0;
    for (int m = 0; m < n; ++m) {
        Dims d;
        if (check_grid(&grids[m], &d) != VERIS_OK) return -1;
        acc += ((d.NX + ti - 1) / ti) * ((d.NY + tj - 1) / tj);
    }
    return acc;
}

int veris_batch_prep_member_f32(int32_t n, const VerisGrid *grids, const VerisParams *p, void *ws, size_t wsb,
                                int32_t m, const VerisFieldsF64 *vs, veris_stream_t s) {
    VERIS_REQUIRE(n >= 1 && grids && p && ws && vs && m >= 0 && m < n, VERIS_ERR_ARG);
    VERIS_REQUIRE(fast_support(*p) == 0, VERIS_ERR_UNSUPPORTED);
    size_t q, t, ts, mb, total;
    size_t *moff = static_cast<size_t *>(malloc((size_t)n * sizeof(size_t)));
    VERIS_REQUIRE(moff, VERIS_ERR_ARG);
    int st = layout(n, grids, &q, &t, &ts, &mb, &total, moff);
    const size_t mo = moff[m];
    free(moff);
    if (st != VERIS_OK) return st;
    VERIS_REQUIRE(wsb >= total, VERIS_ERR_WORKSPACE);
    const Member M = member_at(grids[m], *p, static_cast<char *>(ws) + mb + mo);
    const Fields<double> &f = *reinterpret_cast<const Fields<double> *>(vs);
    cudaStream_t cs = (cudaStream_t)s;
    if ((st = fast_prep<float>(M.d, *p, f, M.c, M.state[0], cs)) != VERIS_OK) return st;
    // the member's state checks into its status word 1: the walks take the
    // cell areas along j (per lane) when they vary along j only
    if (cudaMemsetAsync(M.status + 1, 0, sizeof(int), cs) != cudaSuccess) return VERIS_ERR_LAUNCH;
    if ((st = veris_evp_fast_check(&grids[m], p, vs, M.status + 1, s)) != VERIS_OK) return st;
    dim3 g2((M.d.NY + 31) / 32, (M.d.NX + 7) / 8);
    forcing32_kernel<<<g2, dim3(32, 8), 0, cs>>>(f.WindForcingX, f.WindForcingY, M.d, M.lp, M.WX, M.WY);
    return launch_status();
}

int veris_batch_evp_f32(int32_t n, const VerisGrid *grids, const VerisParams *p, void *ws, size_t wsb,
                        int32_t n_subcycles, int32_t start_buf, int32_t refold, int32_t shape,
                        int32_t blocks_per_sm, veris_stream_t s) {
    VERIS_REQUIRE(n >= 1 && grids && p && ws && n_subcycles >= 0 && (start_buf == 0 || start_buf == 1),
                  VERIS_ERR_ARG);
    VERIS_REQUIRE(shape >= 0 && shape < N_SHAPES && blocks_per_sm >= 0 && blocks_per_sm <= 16, VERIS_ERR_ARG);
    VERIS_REQUIRE(fast_support(*p) == 0, VERIS_ERR_UNSUPPORTED);
    size_t q, t, ts, mb, total;
    int st = layout(n, grids, &q, &t, &ts, &mb, &total, nullptr);
    if (st != VERIS_OK) return st;
    VERIS_REQUIRE(wsb >= total, VERIS_ERR_WORKSPACE);
    const int ntiles = veris_batch_tiles(n, grids, shape);
    VERIS_REQUIRE(ntiles > 0, VERIS_ERR_ARG);
    char *base = static_cast<char *>(ws);
    const Member *mem = reinterpret_cast<const Member *>(base + t);
    const int *tstart = reinterpret_cast<const int *>(base + ts) + shape * (n + 1);
    unsigned *queue = reinterpret_cast<unsigned *>(base + q);
    cudaStream_t cs = (cudaStream_t)s;
    if (refold) {
        int maxc = 0;
        for (int m = 0; m < n; ++m) {
            Dims d;
            check_grid(&grids[m], &d);
            maxc = max(maxc, (int)((int64_t)d.NX * internal_pitch(d.NY) / 256 + 1));
        }
        refold_kernel<<<dim3(min(maxc, 64), n), 256, 0, cs>>>(mem, n, (float)p->recip_deltatDyn, start_buf);
        if ((st = launch_status()) != VERIS_OK) return st;
    }
    if (n_subcycles == 0) return VERIS_OK;
    const int nsm = sm_count();
    VERIS_REQUIRE(nsm > 0, VERIS_ERR_LAUNCH);
    const bool walker = shape >= FIRST_WALK;
    const int bps = blocks_per_sm > 0 ? blocks_per_sm : (walker ? 4 : 2);
    // tile kernels draw one ticket per CTA, the walk kernel one per warp;
    // every drawer ends on one ticket past the last
    const int blocks = walker ? min(nsm * bps, (ntiles + 3) / 4) : min(nsm * bps, ntiles);
    const int drawers = walker ? blocks * 4 : blocks;
    if (cudaMemsetAsync(queue, 0, sizeof(unsigned), cs) != cudaSuccess) return VERIS_ERR_LAUNCH;
    const FastScalars<float> k = fast_scalars<float>(*p);
    const bool basal = p->basalDragK2 != 0.0, turn = p->sinWat != 0.0;
    int buf = start_buf;
    for (int it = 0; it < n_subcycles; ++it) {
        const unsigned b = (unsigned)it * (unsigned)(ntiles + drawers);
        if (walker) {
            int H, tj;
            shape_dims(shape, &H, &tj);
            st = launch_walk_s(basal, turn, mem, tstart, n, ntiles, k, buf, queue, b, blocks, H, cs);
            if (st != VERIS_OK) return st;
            buf ^= 1;
            continue;
        }
        switch (shape) {
        case 0: st = launch_s<0>(basal, turn, mem, tstart, n, ntiles, k, buf, queue, b, blocks, cs); break;
        case 1: st = launch_s<1>(basal, turn, mem, tstart, n, ntiles, k, buf, queue, b, blocks, cs); break;
        case 2: st = launch_s<2>(basal, turn, mem, tstart, n, ntiles, k, buf, queue, b, blocks, cs); break;
        default: st = launch_s<3>(basal, turn, mem, tstart, n, ntiles, k, buf, queue, b, blocks, cs); break;
        }
        if (st != VERIS_OK) return st;
        buf ^= 1;
    }
    return VERIS_OK;
}

int veris_batch_copy_state_f32(int32_t n, const VerisGrid *grids, const VerisParams *p, const void *ws,
                               size_t wsb, int32_t m, int32_t buf, float *uIce, float *vIce, float *sigma1,
                               float *sigma2, float *sigma12, veris_stream_t s) {
    VERIS_REQUIRE(n >= 1 && grids && p && ws && m >= 0 && m < n && (buf == 0 || buf == 1), VERIS_ERR_ARG);
    VERIS_REQUIRE(uIce && vIce && sigma1 && sigma2 && sigma12, VERIS_ERR_ARG);
    size_t q, t, ts, mb, total;
    size_t *moff = static_cast<size_t *>(malloc((size_t)n * sizeof(size_t)));
    VERIS_REQUIRE(moff, VERIS_ERR_ARG);
    int st = layout(n, grids, &q, &t, &ts, &mb, &total, moff);
    const size_t mo = moff[m];
    free(moff);
    if (st != VERIS_OK) return st;
    VERIS_REQUIRE(wsb >= total, VERIS_ERR_WORKSPACE);
    const Member M = member_at(grids[m], *p, static_cast<char *>(const_cast<void *>(ws)) + mb + mo);
    float *out[5] = {uIce, vIce, sigma1, sigma2, sigma12};
    for (int k = 0; k < 5; ++k)
        if (cudaMemcpy2DAsync(out[k], M.d.ld * sizeof(float), M.state[buf][k], M.lp * sizeof(float),
                              M.d.NY * sizeof(float), M.d.NX, cudaMemcpyDeviceToDevice, (cudaStream_t)s) !=
            cudaSuccess)
            return VERIS_ERR_LAUNCH;
    return VERIS_OK;
}

}  // extern "C"
