// Shared device-side definitions: typed field tables, wrapped indexing and
// launch checks for the sea-ice kernels.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <stdint.h>

#include "veris_gb300.h"

namespace veris {

// The field table of the C ABI, typed by the arithmetic type.  Its layout is
// that of VerisFieldsF64 / VerisFieldsF32 (one pointer per state variable).
template <class T>
struct Fields {
#define VERIS_DECL_T(name) const T *name;
    VERIS_FIELDS(VERIS_DECL_T)
#undef VERIS_DECL_T
};
static_assert(sizeof(Fields<double>) == sizeof(VerisFieldsF64), "field table layout");
static_assert(sizeof(Fields<float>) == sizeof(VerisFieldsF32), "field table layout");

// Extent and pitch of the padded 2-D arrays.  wx()/wy() map an index at
// most one period outside [0, n) back inside, which is the reference's roll
// for stencils reaching a few cells; wxa()/wya() wrap any index, for tiles
// or walks whose ring reaches past the far edge of a small grid.
struct Dims {
    int NX, NY;   // padded sizes
    int nx, ny;   // interior sizes
    int64_t ld;   // pitch (elements)
    __host__ __device__ __forceinline__ int wx(int i) const {
        return i < 0 ? i + NX : (i >= NX ? i - NX : i);
    }
    __host__ __device__ __forceinline__ int wy(int j) const {
        return j < 0 ? j + NY : (j >= NY ? j - NY : j);
    }
    __host__ __device__ __forceinline__ int wxa(int i) const {
        while (i < 0) i += NX;
        while (i >= NX) i -= NX;
        return i;
    }
    __host__ __device__ __forceinline__ int wya(int j) const {
        while (j < 0) j += NY;
        while (j >= NY) j -= NY;
        return j;
    }
    // for tiles: indices in [-2, n + 33]; one period suffices when n > 33
    __host__ __device__ __forceinline__ int wxt(int i) const { return NX > 33 ? wx(i) : wxa(i); }
    __host__ __device__ __forceinline__ int wyt(int j) const { return NY > 33 ? wy(j) : wya(j); }
    __host__ __device__ __forceinline__ int64_t at(int i, int j) const {
        return (int64_t)wx(i) * ld + wy(j);
    }
    __host__ __device__ __forceinline__ int64_t raw(int i, int j) const {
        return (int64_t)i * ld + j;
    }
};

// read-only load through the non-coherent path
template <class T>
__device__ __forceinline__ T ldg(const T *p, int64_t k) {
    return __ldg(p + k);
}

template <class T>
__device__ __forceinline__ T sq(T x) { return x * x; }

template <class T>
__device__ __forceinline__ T sgn(T x) {
    return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0));
}

// The halo-fill image writes: a value computed at padded point (i, j) is
// also the value of its periodic images inside the halos that the fill
// refreshes.  x_fill: halo columns are images with period nx; y_fill: rows
// with period ny.  A point inside a refreshed halo does not write itself.
struct HaloFill {
    bool x_fill, y_fill;
    int olx, oly;
};

__host__ __device__ __forceinline__ bool in_xhalo(const Dims &d, int olx, int i) {
    return i < olx || i >= d.NX - olx;
}
__host__ __device__ __forceinline__ bool in_yhalo(const Dims &d, int oly, int j) {
    return j < oly || j >= d.NY - oly;
}

template <class T>
__device__ __forceinline__ void store_filled_ld(T *out, int64_t ld, const Dims &d, const HaloFill &h, int i,
                                                int j, T val) {
    const bool hx = h.x_fill && in_xhalo(d, h.olx, i);
    const bool hy = h.y_fill && in_yhalo(d, h.oly, j);
    if (hx || hy) return;
    out[(int64_t)i * ld + j] = val;
    // image columns inside the x halo
    int ix[2] = {i, -1};
    if (h.x_fill) {
        if (i + d.nx < d.NX && in_xhalo(d, h.olx, i + d.nx)) ix[1] = i + d.nx;
        else if (i - d.nx >= 0 && in_xhalo(d, h.olx, i - d.nx)) ix[1] = i - d.nx;
    }
    int jy[2] = {j, -1};
    if (h.y_fill) {
        if (j + d.ny < d.NY && in_yhalo(d, h.oly, j + d.ny)) jy[1] = j + d.ny;
        else if (j - d.ny >= 0 && in_yhalo(d, h.oly, j - d.ny)) jy[1] = j - d.ny;
    }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            if (a == 0 && b == 0) continue;
            if (ix[a] < 0 || jy[b] < 0) continue;
            out[(int64_t)ix[a] * ld + jy[b]] = val;
        }
}

template <class T>
__device__ __forceinline__ void store_filled(T *out, const Dims &d, const HaloFill &h, int i, int j, T val) {
    store_filled_ld(out, d.ld, d, h, i, j, val);
}

// The same store for a point of the register walk's four-value state
// (u, v, sigma1, sigma2): the own slot gets all four values unless the point
// lies in a refreshed halo, where it gets only its own stresses (its u, v are
// images); the image slots inside the refreshed halos get (u, v) only.
__device__ __forceinline__ void store_filled_quad(float4 *out, int64_t ld, const Dims &d, const HaloFill &h, int i,
                                                  int j, float4 val) {
    float2 *half = reinterpret_cast<float2 *>(out);
    const bool hx = h.x_fill && in_xhalo(d, h.olx, i);
    const bool hy = h.y_fill && in_yhalo(d, h.oly, j);
    const int64_t o = (int64_t)i * ld + j;
    if (hx || hy) {
        half[2 * o + 1] = make_float2(val.z, val.w);
        return;
    }
    out[o] = val;
    int ix[2] = {i, -1};
    if (h.x_fill) {
        if (i + d.nx < d.NX && in_xhalo(d, h.olx, i + d.nx)) ix[1] = i + d.nx;
        else if (i - d.nx >= 0 && in_xhalo(d, h.olx, i - d.nx)) ix[1] = i - d.nx;
    }
    int jy[2] = {j, -1};
    if (h.y_fill) {
        if (j + d.ny < d.NY && in_yhalo(d, h.oly, j + d.ny)) jy[1] = j + d.ny;
        else if (j - d.ny >= 0 && in_yhalo(d, h.oly, j - d.ny)) jy[1] = j - d.ny;
    }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            if (a == 0 && b == 0) continue;
            if (ix[a] < 0 || jy[b] < 0) continue;
            half[2 * ((int64_t)ix[a] * ld + jy[b])] = make_float2(val.x, val.y);
        }
}

inline HaloFill halo_fill_of(const VerisParams &p) {
    HaloFill h;
    h.olx = 2;
    h.oly = 2;
    if (p.veros_fill) {
        h.x_fill = p.enable_cyclic_x != 0;
        h.y_fill = false;
    } else {
        h.x_fill = true;
        h.y_fill = true;
    }
    return h;
}

int check_grid(const VerisGrid *g, Dims *d);
int launch_status();

// One-time host-side configuration per device (kernel attributes, SM
// counts): each call site keeps its own flags indexed by the current device,
// so a process driving several GPUs configures every one of them.
constexpr int MAX_DEVICES = 64;
int current_device();   // -1 when unavailable or beyond MAX_DEVICES
int sm_count();         // SMs of the current device (0 when unavailable)

// raises kern's dynamic shared-memory limit to `bytes` once per device
template <class K>
inline bool smem_configured(std::atomic<bool> (&done)[MAX_DEVICES], K kern, int bytes) {
    const int dev = current_device();
    if (dev < 0) return false;
    if (!done[dev].load(std::memory_order_acquire)) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        done[dev].store(true, std::memory_order_release);
    }
    return true;
}

}  // namespace veris

#define VERIS_CHECK_GRID(g, d)                        \
    do {                                              \
        int _st = veris::check_grid((g), &(d));       \
        if (_st != VERIS_OK) return _st;              \
    } while (0)

#define VERIS_REQUIRE(cond, code)  \
    do {                           \
        if (!(cond)) return (code); \
    } while (0)
