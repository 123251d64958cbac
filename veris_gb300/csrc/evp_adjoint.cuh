// Shared declarations of the EVP adjoint (evp_adjoint.cu, evp_adjoint_gather.cu).
#pragma once
#include "evp_fast.cuh"

namespace veris {

namespace adj {

template <class T>
struct Adj {
    // adjoints of the folded constants (internal pitch), accumulated over subcycles
    T *Ph, *mfC, *bfac, *mU, *cU, *AW, *uOc, *mV, *cV, *AS, *vOc;
    double *dragN, *dragS;   // d/d waterIceDrag, d/d waterIceDrag_south
    double *dragC;           // float64 gather passes: per-cell sum over subcycles of dL/dcDrag cDrag
};

// dragN, dragS += the per-cell sums dragC times rhoSea / (rhoSea drag) of
// each hemisphere (the float64 gather passes' water-drag gradients)
int reduce_drag(const Dims &d, int64_t lp, const uint32_t *flags, const double *dragC, double wN, double wS,
                double *dragN, double *dragS, cudaStream_t st);

// One subcycle of the adjoint sweep in gather passes (evp_adjoint_gather.cu).
// Its tape entries: the velocities before and after it (element stride sst:
// 1 planar, 4 in the float32 register walk's (u, v, sigma1, sigma2) layout)
// and the Delta, zeta and ocean-drag coefficient it computed (a tape holds
// them; for a float32 segment recomputed from a checkpoint the adjoint
// recomputes them first: NULL).
template <class T>
struct TapeG {
    const T *u, *v;          // slot k (pitch lp)
    const T *un, *vn;        // slot k + 1
    int64_t sst;
    const T *del, *zeta, *cd;
    __device__ __forceinline__ T U(int64_t o) const { return u[o * sst]; }
    __device__ __forceinline__ T V(int64_t o) const { return v[o * sst]; }
    __device__ __forceinline__ T UN(int64_t o) const { return un[o * sst]; }
    __device__ __forceinline__ T VN(int64_t o) const { return vn[o * sst]; }
};

// adjoints of the subcycle's outputs (pitch ldl; the image points of a
// filled halo included) and of its inputs (pitch lp, overwritten)
template <class T>
struct LamG {
    const T *lu, *lv, *ls1, *ls2, *ls12;
    int64_t ldl;
    T *ou, *ov, *os1, *os2, *os12;
};

// the passes' intermediate arrays, one internal field each (the last four:
// e12, Delta, zeta and cDrag recomputed for a tape that lacks them)
constexpr int N_SCRATCH = 30;

template <class T>
int adjoint_gather_subcycle(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c,
                            const FastScalars<T> &k, double rhoSea, const TapeG<T> &t, const LamG<T> &l,
                            const Adj<T> &a, T *const scratch[N_SCRATCH], bool basal, bool turn, cudaStream_t st);

// The sweep as a chain of subcycles, P4 of each fused with P1 of the one
// before it (no turning angle; instantiated for float32): `head` runs P1 of
// subcycle t first (the chain's first subcycle); then P2 and P3 of t; then,
// with t_prev and l_prev (subcycle t - 1: its tape entries, and the
// adjoints whose inputs are l's outputs), the fused P4 of t and P1 of t - 1,
// else P4 of t alone (the chain's last subcycle).
template <class T>
int adjoint_gather_chain(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<T> &c,
                         const FastScalars<T> &k, double rhoSea, const TapeG<T> &t, const LamG<T> &l,
                         const Adj<T> &a, T *const scratch[N_SCRATCH], bool basal, bool head,
                         const TapeG<T> *t_prev, const LamG<T> *l_prev, cudaStream_t st);

}  // namespace adj

}  // namespace veris
