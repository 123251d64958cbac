// C-ABI plumbing: grid checks, status strings, layout introspection,
// conversions.
#include <cstring>

#include "common.cuh"

namespace veris {

int check_grid(const VerisGrid *g, Dims *d) {
    if (!g) return VERIS_ERR_ARG;
    if (g->olx != 2 || g->oly != 2) return VERIS_ERR_SHAPE;
    if (g->nx < 4 || g->ny < 4) return VERIS_ERR_SHAPE;
    const int NX = g->nx + 2 * g->olx, NY = g->ny + 2 * g->oly;
    if (g->ld < NY) return VERIS_ERR_SHAPE;
    if ((int64_t)NX * g->ld > ((int64_t)1 << 40)) return VERIS_ERR_SHAPE;
    d->NX = NX;
    d->NY = NY;
    d->nx = g->nx;
    d->ny = g->ny;
    d->ld = g->ld;
    return VERIS_OK;
}

int launch_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? VERIS_OK : VERIS_ERR_LAUNCH;
}

int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return dev >= 0 && dev < MAX_DEVICES ? dev : -1;
}

int sm_count() {
    static std::atomic<int> cached[MAX_DEVICES];
    const int dev = current_device();
    if (dev < 0) return 0;
    int n = cached[dev].load(std::memory_order_relaxed);
    if (n == 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            return 0;
        }
        cached[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

template <class S, class D>
__global__ void convert_kernel(const S *__restrict__ src, D *__restrict__ dst, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        dst[k] = (D)src[k];
}

template <class S, class D>
static int convert(const S *src, D *dst, int64_t n, veris_stream_t s) {
    VERIS_REQUIRE(n >= 0, VERIS_ERR_ARG);
    if (n == 0) return VERIS_OK;
    VERIS_REQUIRE(src && dst, VERIS_ERR_ARG);
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    convert_kernel<S, D><<<blocks, 256, 0, (cudaStream_t)s>>>(src, dst, n);
    return launch_status();
}

}  // namespace veris

using namespace veris;

static const char *kFieldNames[] = {
#define VERIS_NAME(name) #name,
    VERIS_FIELDS(VERIS_NAME)
#undef VERIS_NAME
};

extern "C" {

size_t veris_params_size(void) { return sizeof(VerisParams); }

size_t veris_fields_count(void) { return sizeof(kFieldNames) / sizeof(kFieldNames[0]); }

const char *veris_field_name(size_t index) {
    return index < veris_fields_count() ? kFieldNames[index] : nullptr;
}

const char *veris_status_string(int status) {
    switch (status) {
        case VERIS_OK: return "ok";
        case VERIS_ERR_SHAPE: return "bad grid shape, halo width or pitch";
        case VERIS_ERR_ALIGN: return "misaligned pointer or pitch";
        case VERIS_ERR_NAN: return "non-finite value detected";
        case VERIS_ERR_TIMEOUT: return "device-side wait timed out";
        case VERIS_ERR_LAUNCH: return "CUDA launch or API call failed";
        case VERIS_ERR_ARG: return "invalid argument";
        case VERIS_ERR_UNSUPPORTED: return "settings not supported by this entry point";
        case VERIS_ERR_WORKSPACE: return "workspace missing or too small";
        case VERIS_ERR_TOO_LARGE: return "grid larger than the fixed scratch of the allocation-free entry point";
        default: return "unknown status";
    }
}

int veris_device_ok(void) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return (prop.major == 10 && prop.minor == 3) ? 1 : 0;
}

int veris_convert_f64_to_f32(const double *src, float *dst, int64_t n, veris_stream_t s) {
    return convert<double, float>(src, dst, n, s);
}

int veris_convert_f32_to_f64(const float *src, double *dst, int64_t n, veris_stream_t s) {
    return convert<float, double>(src, dst, n, s);
}

}  // extern "C"
