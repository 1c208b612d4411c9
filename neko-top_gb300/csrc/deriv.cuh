// Shared pieces of the FP64 element-tile derivative kernels (deriv.cu,
// pnpn.cu): the D matrix and GLL weights as a kernel parameter, the block
// shape (elements per block for NT element tiles of shared memory), the
// reference-direction derivatives of a tile, and the launch helpers.
#pragma once
#include <type_traits>

#include "common.cuh"

namespace ntg {
namespace dv {

template <int LX>
struct DMat {
  double d[LX * LX];
  double w[LX];  // GLL weights
};

template <int LX, int NT>
struct Shape {
  static constexpr int LX2 = LX * LX, LX3 = LX2 * LX;
  static constexpr int EPB0 = 256 / LX2 < 1 ? 1 : 256 / LX2;
  static constexpr int EPBS = 45056 / (NT * LX3 * 8) < 1 ? 1 : 45056 / (NT * LX3 * 8);
  static constexpr int EPB = EPB0 < EPBS ? EPB0 : EPBS;
  static constexpr int NW = EPB * LX2, THREADS = (NW + 31) / 32 * 32;
};

// reference derivatives at (i, j, k) of the tile s (s[c * LX2 + b * LX + a])
template <int LX>
__device__ __forceinline__ void rgrad(const double* s, const DMat<LX>& M, int i, int j, int k, double& ur, double& us,
                                      double& ut) {
  constexpr int LX2 = LX * LX;
  ur = us = ut = 0.0;
#pragma unroll
  for (int l = 0; l < LX; ++l) {
    ur = fma(M.d[i * LX + l], s[k * LX2 + j * LX + l], ur);
    us = fma(M.d[j * LX + l], s[k * LX2 + l * LX + i], us);
    ut = fma(M.d[k * LX + l], s[l * LX2 + j * LX + i], ut);
  }
}

template <int LX>
DMat<LX> dmat(const ntg_plan* p) {
  DMat<LX> M;
  for (int q = 0; q < LX * LX; ++q) M.d[q] = p->D[q];
  for (int q = 0; q < LX; ++q) M.w[q] = p->wq[q];
  return M;
}

template <int NT, typename F>
int dispatch(int lx, F&& f) {
  switch (lx) {
    case 2: return f(std::integral_constant<int, 2>{});
    case 3: return f(std::integral_constant<int, 3>{});
    case 4: return f(std::integral_constant<int, 4>{});
    case 5: return f(std::integral_constant<int, 5>{});
    case 6: return f(std::integral_constant<int, 6>{});
    case 7: return f(std::integral_constant<int, 7>{});
    case 8: return f(std::integral_constant<int, 8>{});
    case 9: return f(std::integral_constant<int, 9>{});
    case 10: return f(std::integral_constant<int, 10>{});
    default: set_error("derivative operators: lx=%d not compiled (2..10)", lx); return NTG_ERR_UNSUPPORTED;
  }
}

template <int LX, int NT>
int grid_of(const ntg_plan* p) {
  constexpr int EPB = Shape<LX, NT>::EPB;
  const int64_t g = (p->nelv + EPB - 1) / EPB, cap = (int64_t)num_sms() * 32;
  return (int)(g < cap ? g : cap);
}

}  // namespace dv

inline int need_metrics(const ntg_plan* p) {
  if (!p->met) {
    set_error("derivative operators: call ntg_metrics_set(plan, x, y, z) first");
    return NTG_ERR_INVALID;
  }
  return NTG_OK;
}

// w = B curl u, unassembled (deriv.cu)
int bcurl(ntg_plan* p, double* w0, double* w1, double* w2, const double* ux, const double* uy, const double* uz);
// w = Binv gs(B curl u) (deriv.cu)
int curl_avg(ntg_plan* p, double* w0, double* w1, double* w2, const double* ux, const double* uy, const double* uz);

// n-double device scratch owned by the plan (grown on demand, freed with it)
double* plan_scratch(ntg_plan* p, int64_t count);

}  // namespace ntg
