// Profiler regions: Neko's profiler_start_region(name[, colour]) /
// profiler_end_region (used on the path at
// sources/adjoint/adjoint_pnpn.f90:715,733,746,783 and
// sources/mapping_functions/PDE_filter_mapping.f90:254,341) as NVTX ranges,
// so nsys / ncu show the same regions ('Pressure residual', 'Pressure
// solve', 'Velocity residual', 'Velocity solve', 'filter solve') around the
// library's kernels.  NVTX v3 is header-only: without a profiler attached
// the calls cost a few nanoseconds and record nothing.
#include <nvtx3/nvToolsExt.h>

#include "common.cuh"

namespace {
// a small fixed palette indexed by the caller's colour id (Neko passes ids
// such as 3, 4, 18, 19); id <= 0 gives an uncoloured range
constexpr uint32_t kPalette[8] = {0xff1f77b4u, 0xffff7f0eu, 0xff2ca02cu, 0xffd62728u,
                                  0xff9467bdu, 0xff8c564bu, 0xffe377c2u, 0xff17becfu};
}  // namespace

extern "C" {

int ntg_profiler_start_region(const char* name, int colour) {
  ntg::clear_error();
  NTG_CHECK_ARG(name, "ntg_profiler_start_region: null name");
  if (colour <= 0) {
    nvtxRangePushA(name);
    return NTG_OK;
  }
  nvtxEventAttributes_t a = {};
  a.version = NVTX_VERSION;
  a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
  a.colorType = NVTX_COLOR_ARGB;
  a.color = kPalette[colour % 8];
  a.messageType = NVTX_MESSAGE_TYPE_ASCII;
  a.message.ascii = name;
  nvtxRangePushEx(&a);
  return NTG_OK;
}

int ntg_profiler_end_region(void) {
  ntg::clear_error();
  nvtxRangePop();
  return NTG_OK;
}

}  // extern "C"
