// Shared declarations of the Schwarz preconditioner's translation units:
// schwarz.cu (setup, the FP32-core FDM kernel, the coarse level and the
// prolongation) and schwarz_tc.cu (the tensor-core FDM kernel for lx = 8).
#pragma once

#include "common.cuh"

namespace ntg {
namespace sw {

// linear (Q1) basis at the GLL nodes, for the coarse level
struct CoarsePhi {
  float p[2][NTG_LXMAX];  // p[0][i] = (1 - xi_i) / 2, p[1][i] = (1 + xi_i) / 2
};

// device constants of the tensor-core FDM kernel
struct FdmTc {
  uint8_t* img = nullptr;  // the BF16 plane operator in both orientations, shared-memory image
  float* S = nullptr;      // reference eigenvectors S[p][f] (10 x 10)
  float* lam = nullptr;    // reference eigenvalues (10)
  int per_sm = 1;          // resident CTAs per SM
};

int fdm_tc_prepare(const double* Sref, const double* lamref, FdmTc* t);
void fdm_tc_free(FdmTc* t);
int fdm_tc_launch(const FdmTc& t, const float* r, float* ze, const float* esc, int Ex, int Ey, int Ez,
                  const Scalars* sc, float* corner, const CoarsePhi& ph, int* err, cudaStream_t s);

}  // namespace sw
}  // namespace ntg
