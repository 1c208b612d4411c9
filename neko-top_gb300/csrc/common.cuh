// Shared definitions of the GB300 SEM library: error handling, the plan
// structure, device scalar block and deterministic reductions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/ntgb300.h"

#define NTG_LXMAX 12

namespace ntg {

void set_error(const char* fmt, ...);
void clear_error();

// Returns NTG_ERR_CUDA (and records the message) if a CUDA call failed.
#define NTG_CUDA_TRY(call)                                                             \
  do {                                                                                 \
    cudaError_t _e = (call);                                                           \
    if (_e != cudaSuccess) {                                                           \
      ::ntg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
      return NTG_ERR_CUDA;                                                             \
    }                                                                                  \
  } while (0)

#define NTG_CHECK_ARG(cond, msg)            \
  do {                                      \
    if (!(cond)) {                          \
      ::ntg::set_error("%s", msg);          \
      return NTG_ERR_INVALID;               \
    }                                       \
  } while (0)

#define NTG_TRY(expr)              \
  do {                             \
    int _s = (expr);               \
    if (_s != NTG_OK) return _s;   \
  } while (0)

template <typename T>
int dev_alloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return NTG_OK;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
  if (e != cudaSuccess) {
    set_error("cudaMalloc of %zu bytes failed: %s", sizeof(T) * count, cudaGetErrorString(e));
    *p = nullptr;
    return NTG_ERR_ALLOC;
  }
  return NTG_OK;
}
template <typename T>
void dev_free(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

// Partial-sum slots of the deterministic two-level reductions: each block
// writes its partial to part[blockIdx.x]; the last block to finish (found
// with an atomic ticket) sums part[0..gridDim.x) in index order.
constexpr int kRedSlots = 4096;   // max blocks of a reducing kernel
constexpr int kRedLanes = 32;     // up to 32 simultaneous sums per kernel

// Device-resident solver scalars (one block per solve, FP64).
struct Scalars {
  double rz;       // (r, z) of the current iteration
  double rz_new;
  double pap;      // (p, Ap)
  double alpha, beta;
  double rr;       // (r, r) mult-weighted
  double tol2;     // squared stopping threshold
  double ff;       // (f, f)
  double rtol, abstol;
  double pap_prev; // (p_{k-1}, A p_{k-1}) of the flexible CG
  double gamma;    // flexible-CG orthogonalisation coefficient
  double rr0;      // (r0, r0) at the start of the solve
  double rmax;     // reliable updates: largest ||r|| since the last FP64 residual
  double delta;    // reliable updates: replace the residual when ||r|| < delta * rmax
  double red[8];   // scratch results of generic reductions
  int ru_mode;     // 1 = FP32 iteration with FP64 reliable updates
  int need_ru;     // 1 = residual replacement due, 2 = FP32 residual converged (confirm in FP64)
  int ext_pc;      // 1 = preconditioner applied by separate kernels: (r, z) and beta come from k_rz
  int pad2;
  int iter;        // iterations performed
  int done;        // 1 = converged or stopped: later kernels are no-ops
  int status;      // NTG_OK / NTG_MAXITER / NTG_BREAKDOWN / NTG_NONFINITE
  int max_iter;
  unsigned ticket; // last-block ticket of the reducing kernels
  unsigned pad;
};

}  // namespace ntg

// The plan: mesh, coef_t, gs_t, Jacobi.
struct ntg_plan {
  int lx = 0;
  int64_t nelv = 0, n = 0, nu = 0, nshared = 0, nshared_idx = 0;
  cudaStream_t stream = 0;
  double D[NTG_LXMAX * NTG_LXMAX];
  double wq[NTG_LXMAX];
  float Df[NTG_LXMAX * NTG_LXMAX];
  // geometry (FP64 + FP32 copies)
  double* g[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  float* gf[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double* B = nullptr;
  double* mult = nullptr;
  float* multf = nullptr;
  // gather-scatter: full map (perm sorted by global id, offsets) and the
  // shared-node subset the hot kernels use
  int32_t* perm = nullptr;
  int64_t* offs = nullptr;
  int32_t* sh_idx = nullptr;  // local indices of nodes with > 1 copy, grouped
  int32_t* sh_off = nullptr;  // nshared + 1 offsets into sh_idx
  // the same groups split by multiplicity (2, 4, 8, other), each class
  // ordered by its first local index (gs_classes.cu)
  int gs_classes = 1;           // 1: class kernel (default); 0: one thread per group
  int64_t ncls[4] = {0, 0, 0, 0};
  int2* gs2 = nullptr;
  int4* gs4 = nullptr;
  int4* gs8 = nullptr;          // two int4 per group
  int32_t* gsx_idx = nullptr;
  int32_t* gsx_off = nullptr;
  // coefficients
  int h1_const = 1;
  double h1c = 1.0;
  double* h1 = nullptr;   // n (when !h1_const)
  float* h1f = nullptr;
  int ifh2 = 0;
  double* hB = nullptr;   // h2*B (when ifh2)
  float* hBf = nullptr;
  // Dirichlet mask (0-based)
  int32_t* mask = nullptr;
  int64_t nmask = 0;
  uint8_t* maskrow = nullptr;  // n / lx (lx <= 8): bit i of byte t set when node i of row t is masked (built on first use)
  // Jacobi
  double* dinv = nullptr;
  float* dinvf = nullptr;
  int jacobi_ready = 0;
  // FP32 Ax path: 1 = bulk-copy pipelined kernel for lx = 8 (default)
  int use_tma = 1;
  int* dev_err = nullptr;        // set by kernels whose bounded waits ran out
  // reductions
  double* red_part = nullptr;    // kRedSlots * kRedLanes
  ntg::Scalars* scal = nullptr;  // generic scalars for standalone dots
  double* host_red = nullptr;    // pinned
  // derivative operators (deriv.cu): 9 metric cofactors and 1/jac
  // (10 x n), and 1 / gs(B)
  double* met = nullptr;
  double* binv = nullptr;
  double* dscr = nullptr;  // their scratch (plan_scratch)
  int64_t dscr_n = 0;
};

namespace ntg {
// Every kernel launch of the library bumps this counter (read through
// ntg_launch_count); it is how callers count the library's launches.
void count_launch();
#define NTG_COUNT_LAUNCH() ::ntg::count_launch()

// Optional per-kernel device timers (CUDA events on the launching stream),
// off by default; enabled with ntg_timer_enable.
enum TimerId {
  TM_AX64 = 0, TM_AX32 = 1, TM_GS64 = 2, TM_GS32 = 3, TM_UPD64 = 4, TM_UPD32 = 5, TM_DIR64 = 6,
  TM_DIR32 = 7, TM_PC32 = 8, TM_FDM = 9, TM_CRS = 10, TM_PULL = 11, TM_COUNT = 16
};
// z = M r with the Schwarz preconditioner (schwarz.cu); no-op once sc->done
// z = M r (FP32).  With mult non-null also (r, z)_mult into sc (FinRz{rz_mode}).
int schwarz_apply(ntg_schwarz* sw, float* z, const float* r, cudaStream_t s, Scalars* sc, const float* mult = nullptr,
                  double* part = nullptr, int rz_mode = 0);
void timer_start(int id, cudaStream_t s);
void timer_stop(int id, cudaStream_t s);

// launch helpers implemented in the .cu files
int ax_launch(ntg_plan* p, double* w, const double* u, Scalars* dot_scal, int dot_slot, cudaStream_t s);
int ax_launch_f32(ntg_plan* p, float* w, const float* u, Scalars* dot_scal, int dot_slot, cudaStream_t s);
int gs_launch(ntg_plan* p, double* u, int op, cudaStream_t s);
int gs_launch_f32(ntg_plan* p, float* u, int op, cudaStream_t s);
int mask_launch(ntg_plan* p, double* u, cudaStream_t s);
int mask_launch_f32(ntg_plan* p, float* u, cudaStream_t s);
// assembled masked operator w = mask(gs(A u)); optional fused (u, Au_local)
int op_apply(ntg_plan* p, double* w, const double* u, cudaStream_t s);
int op_apply_f32(ntg_plan* p, float* w, const float* u, cudaStream_t s);
// generic deterministic weighted dot: sum a*b*c (c may be null -> 1)
int wdot(ntg_plan* p, const double* a, const double* b, const double* c, int64_t n, double* host_out,
         cudaStream_t s);
int gs_add_guarded(ntg_plan* p, double* u, cudaStream_t s, const Scalars* sc);
int gs_add_guarded_f32(ntg_plan* p, float* u, cudaStream_t s, const Scalars* sc);
int mask_guarded(ntg_plan* p, double* u, cudaStream_t s, const Scalars* sc);
int mask_guarded_f32(ntg_plan* p, float* u, cudaStream_t s, const Scalars* sc);
int ensure_fp32(ntg_plan* p);
int build_gs_classes(ntg_plan* p);
template <typename T>
int gs_cls_launch(ntg_plan* p, T* u, int op, cudaStream_t s, const Scalars* sc);
int grid_for(int64_t work, int threads);
int jacobi_update(ntg_plan* p);
int ensure_maskrow(ntg_plan* p);
// the element counts of a Schwarz preconditioner built on a structured box
// (1), or 0 for one built on a general mesh
int schwarz_box(const ntg_schwarz* w, int* ex, int* ey, int* ez);
// restarted flexible GMRES (gmres.cu)
struct GmresWork;
struct GmresOpts {
  int restart = 30, fp32 = 0, max_iter = 1000, check_every = 4;
  double rtol = 1e-10, abstol = 0.0, delta = 1e-4;
};
int gmres_solve(ntg_plan* p, GmresWork*& g, Scalars* sc, ntg_schwarz* sw, const GmresOpts& o, double* x,
                const double* f, ntg_monitor* mon);
void gmres_free(GmresWork* g);
// GLL nodes, weights and differentiation matrix of lx points
void gll_basis(int lx, double* xi, double* w, double* D);
int num_sms();
}  // namespace ntg
