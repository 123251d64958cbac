// Shared declarations of the EVP adjoint (evp_adjoint.cu, evp_adjoint64.cu).
#pragma once
#include "evp_fast.cuh"

namespace veris {

namespace adj {

template <class T>
struct Adj {
    // adjoints of the folded constants (internal pitch), accumulated over subcycles
    T *Ph, *mfC, *bfac, *mU, *cU, *AW, *uOc, *mV, *cV, *AS, *vOc;
    double *dragN, *dragS;   // d/d waterIceDrag, d/d waterIceDrag_south
};

// One float64 subcycle of the adjoint sweep in gather passes
// (evp_adjoint64.cu).  The subcycle's tape entries: the velocities before
// and after it, and the Delta, zeta and ocean-drag coefficient it computed.
struct Tape64 {
    const double *u, *v, *del, *zeta, *cd;   // slot k (pitch lp)
    const double *un, *vn;                   // u, v of slot k + 1
};

// adjoints of the subcycle's outputs (pitch ldl; the image points of a
// filled halo included) and of its inputs (pitch lp, overwritten)
struct Lam64 {
    const double *lu, *lv, *ls1, *ls2, *ls12;
    int64_t ldl;
    double *ou, *ov, *os1, *os2, *os12;
};

// the passes' intermediate arrays, one internal field each
constexpr int N_SCRATCH64 = 26;

int adjoint64_subcycle(const Dims &d, int64_t lp, const HaloFill &h, const FastConsts<double> &c,
                       const FastScalars<double> &k, double rhoSea, const Tape64 &t, const Lam64 &l,
                       const Adj<double> &a, double *const scratch[N_SCRATCH64], bool basal, bool turn,
                       cudaStream_t st);

}  // namespace adj

}  // namespace veris
