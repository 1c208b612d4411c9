// Gather-scatter (direct stiffness summation) as a sorted-index segmented
// reduction, and the Dirichlet mask.
//
// Replaces Neko's gs_t%op(u, n, GS_OP_*) (called at
// sources/adjoint/adjoint_pnpn.f90:725,755-757 and
// sources/mapping_functions/PDE_filter_mapping.f90:249) and
// bc_list_apply_scalar (sources/adjoint/adjoint_pnpn.f90:726).
//
// The plan keeps only the nodes with more than one local copy: sh_idx lists
// their local indices grouped by global id (stable sort order), sh_off the
// group offsets.  One thread reduces one group in a fixed order and writes
// the result back to every copy, so results are deterministic and nodes
// with a single copy are never touched.  HBM bound: per shared local DOF
// one value read + write and one int32 index.
#include "common.cuh"

namespace ntg {

template <typename T, int OP>
__global__ void k_gs_shared(T* __restrict__ u, const int32_t* __restrict__ idx, const int32_t* __restrict__ off,
                            int64_t nseg, const Scalars* sc) {
  if (sc && sc->done) return;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nseg; s += (int64_t)gridDim.x * blockDim.x) {
    const int a = off[s], b = off[s + 1];
    T acc = u[idx[a]];
    for (int q = a + 1; q < b; ++q) {
      T v = u[idx[q]];
      if (OP == NTG_GS_ADD) acc += v;
      else if (OP == NTG_GS_MUL) acc *= v;
      else if (OP == NTG_GS_MIN) acc = v < acc ? v : acc;
      else acc = v > acc ? v : acc;
    }
    for (int q = a; q < b; ++q) u[idx[q]] = acc;
  }
}

template <typename T>
__global__ void k_mask_zero(T* __restrict__ u, const int32_t* __restrict__ mask, int64_t m, const Scalars* sc) {
  if (sc && sc->done) return;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m; q += (int64_t)gridDim.x * blockDim.x)
    u[mask[q]] = T(0);
}

template <typename T>
static int gs_any(ntg_plan* p, T* u, int op, cudaStream_t s, const Scalars* sc) {
  if (p->nshared == 0) return NTG_OK;
  const int TPB = 256;
  const int G = grid_for(p->nshared, TPB);
  const int tid = sizeof(T) == 8 ? TM_GS64 : TM_GS32;
  timer_start(tid, s);
  struct Stop {
    int id;
    cudaStream_t s;
    ~Stop() { timer_stop(id, s); }
  } stop_{tid, s};
  if (p->gs_classes) return gs_cls_launch<T>(p, u, op, s, sc);
  switch (op) {
    case NTG_GS_ADD: { k_gs_shared<T, NTG_GS_ADD><<<G, TPB, 0, s>>>(u, p->sh_idx, p->sh_off, p->nshared, sc); NTG_COUNT_LAUNCH(); } break;
    case NTG_GS_MUL: { k_gs_shared<T, NTG_GS_MUL><<<G, TPB, 0, s>>>(u, p->sh_idx, p->sh_off, p->nshared, sc); NTG_COUNT_LAUNCH(); } break;
    case NTG_GS_MIN: { k_gs_shared<T, NTG_GS_MIN><<<G, TPB, 0, s>>>(u, p->sh_idx, p->sh_off, p->nshared, sc); NTG_COUNT_LAUNCH(); } break;
    case NTG_GS_MAX: { k_gs_shared<T, NTG_GS_MAX><<<G, TPB, 0, s>>>(u, p->sh_idx, p->sh_off, p->nshared, sc); NTG_COUNT_LAUNCH(); } break;
    default: set_error("gs_op: unknown op %d", op); return NTG_ERR_INVALID;
  }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

int gs_launch(ntg_plan* p, double* u, int op, cudaStream_t s) { return gs_any<double>(p, u, op, s, nullptr); }
int gs_launch_f32(ntg_plan* p, float* u, int op, cudaStream_t s) { return gs_any<float>(p, u, op, s, nullptr); }
int gs_add_guarded(ntg_plan* p, double* u, cudaStream_t s, const Scalars* sc) {
  return gs_any<double>(p, u, NTG_GS_ADD, s, sc);
}
int gs_add_guarded_f32(ntg_plan* p, float* u, cudaStream_t s, const Scalars* sc) {
  return gs_any<float>(p, u, NTG_GS_ADD, s, sc);
}

template <typename T>
static int mask_any(ntg_plan* p, T* u, cudaStream_t s, const Scalars* sc) {
  if (p->nmask == 0) return NTG_OK;
  { k_mask_zero<T><<<grid_for(p->nmask, 256), 256, 0, s>>>(u, p->mask, p->nmask, sc); NTG_COUNT_LAUNCH(); }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}
int mask_launch(ntg_plan* p, double* u, cudaStream_t s) { return mask_any<double>(p, u, s, nullptr); }
int mask_launch_f32(ntg_plan* p, float* u, cudaStream_t s) { return mask_any<float>(p, u, s, nullptr); }
int mask_guarded(ntg_plan* p, double* u, cudaStream_t s, const Scalars* sc) { return mask_any<double>(p, u, s, sc); }
int mask_guarded_f32(ntg_plan* p, float* u, cudaStream_t s, const Scalars* sc) { return mask_any<float>(p, u, s, sc); }

int op_apply(ntg_plan* p, double* w, const double* u, cudaStream_t s) {
  NTG_TRY(ax_launch(p, w, u, nullptr, 0, s));
  NTG_TRY(gs_launch(p, w, NTG_GS_ADD, s));
  return mask_launch(p, w, s);
}
int op_apply_f32(ntg_plan* p, float* w, const float* u, cudaStream_t s) {
  NTG_TRY(ax_launch_f32(p, w, u, nullptr, 0, s));
  NTG_TRY(gs_launch_f32(p, w, NTG_GS_ADD, s));
  return mask_launch_f32(p, w, s);
}

}  // namespace ntg

using namespace ntg;

extern "C" int ntg_gs_op(ntg_plan* plan, double* u_d, int op) {
  clear_error();
  NTG_CHECK_ARG(plan && u_d, "ntg_gs_op: null argument");
  return gs_launch(plan, u_d, op, plan->stream);
}
extern "C" int ntg_gs_op_f32(ntg_plan* plan, float* u_d, int op) {
  clear_error();
  NTG_CHECK_ARG(plan && u_d, "ntg_gs_op_f32: null argument");
  return gs_launch_f32(plan, u_d, op, plan->stream);
}
extern "C" int ntg_bc_apply_scalar(ntg_plan* plan, double* x_d) {
  clear_error();
  NTG_CHECK_ARG(plan && x_d, "ntg_bc_apply_scalar: null argument");
  return mask_launch(plan, x_d, plan->stream);
}

// the same for an FP32 field (the FP32 iteration of the mixed solvers)
extern "C" int ntg_bc_apply_scalar_f32(ntg_plan* plan, float* x_d) {
  clear_error();
  NTG_CHECK_ARG(plan && x_d, "ntg_bc_apply_scalar_f32: null argument");
  return mask_launch_f32(plan, x_d, plan->stream);
}
