// Shared declarations of the Schwarz preconditioner's translation units:
// schwarz.cu (setup, the FP32-core FDM kernel, the coarse level and the
// prolongation on structured boxes), schwarz_tc.cu (the tensor-core FDM
// kernel for lx = 8) and schwarz_gen.cu (the face-neighbour tables, the
// prolongation and the coarse level on general hexahedral meshes).
#pragma once

#include <vector>

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

// General (unstructured, conforming) hexahedral meshes.  Element faces are
// numbered r-, r+, s-, s+, t-, t+ (0..5); a face's nodes by their two
// tangential indices, the lower axis fastest (p = s + lx t).
struct GenTopo {
  int lx = 0;
  int64_t nelv = 0, nu = 0;
  // ghost[(e * 6 + f) * lx^2 + p]: local index of the node one step inside
  // the element across face f from face node p, -1 on a boundary face
  int32_t* ghost = nullptr;
  // per global node (the plan's gather-scatter groups): the extended-result
  // indices (e lx_e^3 + a + lx_e b + lx_e^2 c, lx_e = lx + 2) that sum to it,
  // ascending; its local copies are the plan's perm[offs[g] .. offs[g+1])
  int64_t* soff = nullptr;
  int32_t* src = nullptr;
  const int32_t* perm = nullptr;
  const int64_t* offs = nullptr;
  std::vector<int64_t> gnum;  // host: global node (group) of every local node
  // coarse level: the Galerkin Q1 operator on the element vertices,
  // Dirichlet vertices removed, inverted densely
  int nv = 0;               // active vertices
  int coarse_ready = 0;
  int32_t* vid = nullptr;   // nelv x 8: active vertex of each element corner, -1 Dirichlet
  int32_t* voff = nullptr;  // nv + 1: each vertex's corner list in vsrc
  int32_t* vsrc = nullptr;  // e * 8 + v, ascending
  float* ainv = nullptr;    // nv x nv
  float* rc = nullptr;      // nv: restricted residual
  float* zc = nullptr;      // nv: coarse correction
};
constexpr int kGenCoarseMax = 8192;  // active vertices of the dense coarse level

int gen_create(ntg_plan* p, GenTopo** out);
void gen_free(GenTopo* g);
// (re)build the coarse level from the plan's mask and coefficients
int gen_coarse_setup(ntg_plan* p, GenTopo* g);
// rc = P^T r from the per-element corner sums, zc = A_c^-1 rc
int gen_coarse_launch(GenTopo* g, const float* corner, cudaStream_t s, const Scalars* sc);
// z = the assembled sum of the extended results (+ P zc, + dw r); dot: also
// (r, z) over global nodes into sc (FinRz{mode})
int gen_pull_launch(GenTopo* g, const float* ze, float* z, const float* r, const float* dw, const CoarsePhi& ph,
                    bool dot, double* part, int mode, Scalars* sc, cudaStream_t s);

int fdm_tc_prepare(const double* Sref, const double* lamref, FdmTc* t);
void fdm_tc_free(FdmTc* t);
int fdm_tc_launch(const FdmTc& t, const float* r, float* ze, const float* esc, int Ex, int Ey, int Ez,
                  const Scalars* sc, float* corner, const CoarsePhi& ph, int* err, cudaStream_t s);

}  // namespace sw
}  // namespace ntg
