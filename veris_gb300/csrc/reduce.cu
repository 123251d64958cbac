// Deterministic float64 sum over the interior of a field (optionally
// weighted), for conservation diagnostics.  The reference's global_sum
// (veris/global_sum.py:1-4) is the identity on one process; this is the sum
// it would feed.  Fixed grid, fixed per-block tree, fixed final pass: the
// result is bitwise reproducible run to run.
#include "common.cuh"

namespace veris {

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 1024;

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <class T>
__device__ T block_sum(T v) {
    __shared__ T part[RED_THREADS / 32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) part[warp] = v;
    __syncthreads();
    T r = 0;
    if (warp == 0) {
        r = lane < RED_THREADS / 32 ? part[lane] : T(0);
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

__global__ void interior_partial_kernel(const double *A, const double *w, Dims d, int olx, int oly,
                                        double *partial) {
    const int64_t n = (int64_t)d.nx * d.ny;
    double acc = 0.0;
    for (int64_t k = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; k < n; k += (int64_t)RED_BLOCKS * RED_THREADS) {
        const int i = (int)(k / d.ny) + olx, j = (int)(k % d.ny) + oly;
        const int64_t o = d.raw(i, j);
        acc += w ? A[o] * w[o] : A[o];
    }
    const double s = block_sum(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void final_sum_kernel(const double *partial, double *result) {
    double acc = 0.0;
    for (int k = threadIdx.x; k < RED_BLOCKS; k += RED_THREADS) acc += partial[k];
    const double s = block_sum(acc);
    if (threadIdx.x == 0) *result = s;
}

// Conservation diagnostics: up to BUD_MAX weighted interior sums in one
// pass.  Block (b, q) sums rows b, b + BUD_BLOCKS, ... of field q times its
// weight (rows then columns: no index division); one block then adds each
// field's partials in index order and writes the sums into the step's slot
// of a ring, the slot being the device step counter modulo the ring length.
// Fixed grid, fixed trees: bitwise reproducible.
constexpr int BUD_MAX = 16;
constexpr int BUD_BLOCKS = 256;

struct BudgetArgs {
    const double *f[BUD_MAX];
    const double *w[BUD_MAX];
};

__global__ void budget_partial_kernel(BudgetArgs a, Dims d, int olx, int oly, double *partial) {
    const int q = blockIdx.y;
    const double *f = a.f[q], *w = a.w[q];
    double acc = 0.0;
    for (int i = blockIdx.x; i < d.nx; i += BUD_BLOCKS) {
        const int64_t row = d.raw(i + olx, oly);
        for (int j = threadIdx.x; j < d.ny; j += RED_THREADS)
            acc += w ? f[row + j] * w[row + j] : f[row + j];
    }
    const double s = block_sum(acc);
    if (threadIdx.x == 0) partial[q * BUD_BLOCKS + blockIdx.x] = s;
}

__global__ void budget_final_kernel(const double *partial, int n, int first, double *ring, int ring_steps,
                                    int32_t *counter, int advance) {
    __shared__ int slot;
    if (threadIdx.x == 0) slot = ((*counter % ring_steps) + ring_steps) % ring_steps;
    __syncthreads();
    for (int q = 0; q < n; ++q) {
        double acc = 0.0;
        for (int k = threadIdx.x; k < BUD_BLOCKS; k += RED_THREADS) acc += partial[q * BUD_BLOCKS + k];
        const double s = block_sum(acc);
        if (threadIdx.x == 0) ring[(int64_t)slot * BUD_MAX + first + q] = s;
    }
    if (advance && threadIdx.x == 0) *counter += 1;
}

// Non-finite detection over whole padded arrays (halos included): each
// thread folds its elements into one flag, one warp vote, one atomicOr per
// warp that saw a NaN or an infinity.  Sticky: the caller clears the word.
constexpr int FIN_THREADS = 256;
constexpr int FIN_MAX_ARRAYS = 8;

template <class T>
struct FiniteArgs {
    const T *a[FIN_MAX_ARRAYS];
};

template <class T>
__global__ void finite_check_kernel(FiniteArgs<T> args, Dims d, int32_t flag, int32_t *status) {
    const T *a = args.a[blockIdx.y];
    bool bad = false;
    for (int i = blockIdx.x; i < d.NX; i += gridDim.x)   // rows, then columns: no index division
        for (int j = threadIdx.x; j < d.NY; j += FIN_THREADS) bad |= !isfinite(a[d.raw(i, j)]);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, flag);
}

template <class T>
static int check_finite(const VerisGrid *g, const T *const *arrays, int32_t n, int32_t flag, int32_t *status,
                        veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(arrays && status && n >= 1 && n <= FIN_MAX_ARRAYS && flag != 0, VERIS_ERR_ARG);
    FiniteArgs<T> args{};
    for (int k = 0; k < n; ++k) {
        VERIS_REQUIRE(arrays[k], VERIS_ERR_ARG);
        args.a[k] = arrays[k];
    }
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return VERIS_ERR_LAUNCH;
    const int blocks = d.NX < sms * 4 ? d.NX : sms * 4;   // up to 4 CTAs per SM per array
    finite_check_kernel<T><<<dim3(blocks, n), FIN_THREADS, 0, (cudaStream_t)s>>>(args, d, flag, status);
    return launch_status();
}

}  // namespace veris

using namespace veris;

extern "C" {

size_t veris_reduce_workspace_bytes(const VerisGrid *g) {
    (void)g;
    return RED_BLOCKS * sizeof(double);
}

int veris_check_finite_f64(const VerisGrid *g, const double *const *arrays, int32_t n, int32_t flag,
                           int32_t *status_device, veris_stream_t s) {
    return check_finite<double>(g, arrays, n, flag, status_device, s);
}

int veris_check_finite_f32(const VerisGrid *g, const float *const *arrays, int32_t n, int32_t flag,
                           int32_t *status_device, veris_stream_t s) {
    return check_finite<float>(g, arrays, n, flag, status_device, s);
}

size_t veris_budget_workspace_bytes(void) { return (size_t)BUD_MAX * BUD_BLOCKS * sizeof(double); }

int veris_budget_sums_f64(const VerisGrid *g, const double *const *fields, const double *const *weights,
                          int32_t n, int32_t first, double *ring, int32_t ring_steps, int32_t *step_counter,
                          int32_t advance, void *ws, size_t ws_bytes, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(fields && ring && step_counter && ring_steps >= 1, VERIS_ERR_ARG);
    VERIS_REQUIRE(n >= 1 && first >= 0 && first + n <= BUD_MAX, VERIS_ERR_ARG);
    VERIS_REQUIRE(ws && ws_bytes >= veris_budget_workspace_bytes(), VERIS_ERR_WORKSPACE);
    BudgetArgs a{};
    for (int q = 0; q < n; ++q) {
        VERIS_REQUIRE(fields[q], VERIS_ERR_ARG);
        a.f[q] = fields[q];
        a.w[q] = weights ? weights[q] : nullptr;
    }
    cudaStream_t st = (cudaStream_t)s;
    double *partial = static_cast<double *>(ws);
    budget_partial_kernel<<<dim3(BUD_BLOCKS, n), RED_THREADS, 0, st>>>(a, d, g->olx, g->oly, partial);
    budget_final_kernel<<<1, RED_THREADS, 0, st>>>(partial, n, first, ring, ring_steps, step_counter,
                                                   advance ? 1 : 0);
    return launch_status();
}

int veris_global_sum_f64(const VerisGrid *g, const double *A, const double *w, double *result, void *ws,
                         size_t ws_bytes, veris_stream_t s) {
    Dims d;
    VERIS_CHECK_GRID(g, d);
    VERIS_REQUIRE(A && result, VERIS_ERR_ARG);
    VERIS_REQUIRE(ws && ws_bytes >= RED_BLOCKS * sizeof(double), VERIS_ERR_WORKSPACE);
    cudaStream_t st = (cudaStream_t)s;
    double *partial = static_cast<double *>(ws);
    interior_partial_kernel<<<RED_BLOCKS, RED_THREADS, 0, st>>>(A, w, d, g->olx, g->oly, partial);
    final_sum_kernel<<<1, RED_THREADS, 0, st>>>(partial, result);
    return launch_status();
}

}  // extern "C"
