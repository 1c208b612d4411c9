// Gather-scatter by multiplicity class.
//
// The shared-node groups of the plan (sh_idx / sh_off, grouped by global id
// with the copies in ascending local order) are split into classes by their
// number of copies -- 2 (face nodes), 4 (edge nodes), 8 (corner nodes) and
// any other count -- and each class is ordered by the local index of its
// first copy, so a warp walks neighbouring faces of neighbouring elements.
// The 2-, 4- and 8-copy classes store their local indices as int2 / int4 /
// 2 x int4, so one vector load fetches all indices of a group; every thread
// handles 4 groups with all loads issued before the sums (the segmented
// reduction is latency bound otherwise).  Copies are summed in ascending
// local order, as before, so the results are bit-identical to the
// one-thread-per-group kernel and to the oracle.
#include <cub/cub.cuh>

#include "common.cuh"

namespace ntg {

constexpr int kGsThreads = 256;
constexpr int kGsItems = 4;
constexpr int kGsPerBlock = kGsThreads * kGsItems;

__global__ void k_gs_keys(const int32_t* __restrict__ idx, const int32_t* __restrict__ off, int64_t nseg,
                          uint64_t* __restrict__ key, int32_t* __restrict__ seg, unsigned long long* __restrict__ hist) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nseg; s += (int64_t)gridDim.x * blockDim.x) {
    const int c = off[s + 1] - off[s];
    const uint64_t cls = c == 2 ? 0 : (c == 4 ? 1 : (c == 8 ? 2 : 3));
    key[s] = (cls << 32) | (uint32_t)idx[off[s]];
    seg[s] = (int32_t)s;
    atomicAdd(&hist[cls], 1ull);
  }
}

__global__ void k_gs_fill(const uint64_t* __restrict__ key, const int32_t* __restrict__ seg, int64_t nseg,
                          const int32_t* __restrict__ idx, const int32_t* __restrict__ off, int64_t s2, int64_t s4,
                          int64_t s8, int2* __restrict__ g2, int4* __restrict__ g4, int4* __restrict__ g8,
                          int32_t* __restrict__ xcnt) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nseg; t += (int64_t)gridDim.x * blockDim.x) {
    const int cls = (int)(key[t] >> 32);
    const int64_t s = seg[t];
    const int a = off[s];
    if (cls == 0) {
      g2[t] = make_int2(idx[a], idx[a + 1]);
    } else if (cls == 1) {
      g4[t - s2] = make_int4(idx[a], idx[a + 1], idx[a + 2], idx[a + 3]);
    } else if (cls == 2) {
      const int64_t q = t - s4;
      g8[2 * q] = make_int4(idx[a], idx[a + 1], idx[a + 2], idx[a + 3]);
      g8[2 * q + 1] = make_int4(idx[a + 4], idx[a + 5], idx[a + 6], idx[a + 7]);
    } else {
      xcnt[t - s8] = off[s + 1] - a;
    }
  }
}

__global__ void k_gs_fill_x(const int32_t* __restrict__ seg, int64_t s8, int64_t nx, const int32_t* __restrict__ idx,
                            const int32_t* __restrict__ off, const int32_t* __restrict__ xoff,
                            int32_t* __restrict__ xidx) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nx; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = seg[s8 + q];
    const int a = off[s], c = off[s + 1] - a;
    for (int k = 0; k < c; ++k) xidx[xoff[q] + k] = idx[a + k];
  }
}

template <typename T, int OP>
__device__ __forceinline__ T gs_comb(T acc, T v) {
  if (OP == NTG_GS_ADD) return acc + v;
  if (OP == NTG_GS_MUL) return acc * v;
  if (OP == NTG_GS_MIN) return v < acc ? v : acc;
  return v > acc ? v : acc;
}

template <typename T, int OP>
__global__ void __launch_bounds__(kGsThreads)
    k_gs_cls(T* __restrict__ u, const int2* __restrict__ g2, int64_t n2, const int4* __restrict__ g4, int64_t n4,
             const int4* __restrict__ g8, int64_t n8, const int32_t* __restrict__ xidx,
             const int32_t* __restrict__ xoff, int64_t nx, int b2, int b4, int b8, const Scalars* sc) {
  if (sc && sc->done) return;
  int blk = blockIdx.x;
  if (blk < b2) {
    const int64_t base = (int64_t)blk * kGsPerBlock + threadIdx.x;
    int2 id[kGsItems];
    T a[kGsItems], b[kGsItems];
#pragma unroll
    for (int q = 0; q < kGsItems; ++q) {
      const int64_t t = base + q * kGsThreads;
      id[q] = t < n2 ? g2[t] : make_int2(-1, -1);
    }
#pragma unroll
    for (int q = 0; q < kGsItems; ++q)
      if (id[q].x >= 0) {
        a[q] = u[id[q].x];
        b[q] = u[id[q].y];
      }
#pragma unroll
    for (int q = 0; q < kGsItems; ++q)
      if (id[q].x >= 0) {
        const T s = gs_comb<T, OP>(a[q], b[q]);
        u[id[q].x] = s;
        u[id[q].y] = s;
      }
    return;
  }
  blk -= b2;
  if (blk < b4) {
    const int64_t base = (int64_t)blk * kGsPerBlock + threadIdx.x;
    int4 id[kGsItems];
    T v[kGsItems][4];
#pragma unroll
    for (int q = 0; q < kGsItems; ++q) {
      const int64_t t = base + q * kGsThreads;
      id[q] = t < n4 ? g4[t] : make_int4(-1, -1, -1, -1);
    }
#pragma unroll
    for (int q = 0; q < kGsItems; ++q)
      if (id[q].x >= 0) {
        v[q][0] = u[id[q].x]; v[q][1] = u[id[q].y]; v[q][2] = u[id[q].z]; v[q][3] = u[id[q].w];
      }
#pragma unroll
    for (int q = 0; q < kGsItems; ++q)
      if (id[q].x >= 0) {
        T s = gs_comb<T, OP>(v[q][0], v[q][1]);
        s = gs_comb<T, OP>(s, v[q][2]);
        s = gs_comb<T, OP>(s, v[q][3]);
        u[id[q].x] = s; u[id[q].y] = s; u[id[q].z] = s; u[id[q].w] = s;
      }
    return;
  }
  blk -= b4;
  if (blk < b8) {
    const int64_t base = (int64_t)blk * kGsPerBlock + threadIdx.x;
#pragma unroll
    for (int q = 0; q < kGsItems; ++q) {
      const int64_t t = base + q * kGsThreads;
      if (t >= n8) break;
      const int4 lo = g8[2 * t], hi = g8[2 * t + 1];
      const int ix[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
      T v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = u[ix[k]];
      T s = v[0];
#pragma unroll
      for (int k = 1; k < 8; ++k) s = gs_comb<T, OP>(s, v[k]);
#pragma unroll
      for (int k = 0; k < 8; ++k) u[ix[k]] = s;
    }
    return;
  }
  blk -= b8;
  // any other multiplicity: one thread per group
  for (int64_t q = (int64_t)blk * kGsThreads + threadIdx.x; q < nx; q += (int64_t)(gridDim.x - b2 - b4 - b8) * kGsThreads) {
    const int a = xoff[q], c = xoff[q + 1] - a;
    T s = u[xidx[a]];
    for (int k = 1; k < c; ++k) s = gs_comb<T, OP>(s, u[xidx[a + k]]);
    for (int k = 0; k < c; ++k) u[xidx[a + k]] = s;
  }
}

// Builds the class arrays from sh_idx / sh_off (called once per plan).
int build_gs_classes(ntg_plan* p) {
  const int64_t nseg = p->nshared;
  p->ncls[0] = p->ncls[1] = p->ncls[2] = p->ncls[3] = 0;
  if (nseg == 0) return NTG_OK;
  cudaStream_t s = p->stream;
  int st = NTG_OK;
  uint64_t *key = nullptr, *key_s = nullptr;
  int32_t *seg = nullptr, *seg_s = nullptr, *xcnt = nullptr;
  unsigned long long* hist = nullptr;
  void* tmp = nullptr;
  size_t tb = 0, tb2 = 0;
  unsigned long long h[4] = {0, 0, 0, 0};
  const int T = 256;
  int64_t s2 = 0, s4 = 0, s8 = 0, nx = 0;
  do {
    if ((st = dev_alloc(&key, nseg)) || (st = dev_alloc(&key_s, nseg)) || (st = dev_alloc(&seg, nseg)) ||
        (st = dev_alloc(&seg_s, nseg)) || (st = dev_alloc(&hist, 4)))
      break;
    cudaMemsetAsync(hist, 0, 4 * sizeof(unsigned long long), s);
    { k_gs_keys<<<grid_for(nseg, T), T, 0, s>>>(p->sh_idx, p->sh_off, nseg, key, seg, hist); NTG_COUNT_LAUNCH(); }
    cub::DeviceRadixSort::SortPairs(nullptr, tb, key, key_s, seg, seg_s, nseg, 0, 34, s);
    if (cudaMalloc(&tmp, tb) != cudaSuccess) { st = NTG_ERR_ALLOC; set_error("gs classes: tmp alloc"); break; }
    cub::DeviceRadixSort::SortPairs(tmp, tb, key, key_s, seg, seg_s, nseg, 0, 34, s);
    if (cudaMemcpyAsync(h, hist, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      st = NTG_ERR_CUDA; set_error("gs classes: histogram"); break;
    }
    s2 = (int64_t)h[0];
    s4 = s2 + (int64_t)h[1];
    s8 = s4 + (int64_t)h[2];
    nx = (int64_t)h[3];
    if ((st = dev_alloc(&p->gs2, h[0] ? h[0] : 1)) || (st = dev_alloc(&p->gs4, h[1] ? h[1] : 1)) ||
        (st = dev_alloc(&p->gs8, h[2] ? 2 * h[2] : 1)) || (st = dev_alloc(&xcnt, nx + 1)) ||
        (st = dev_alloc(&p->gsx_off, nx + 1)))
      break;
    { k_gs_fill<<<grid_for(nseg, T), T, 0, s>>>(key_s, seg_s, nseg, p->sh_idx, p->sh_off, s2, s4, s8, p->gs2, p->gs4, p->gs8, xcnt); NTG_COUNT_LAUNCH(); }
    int32_t total = 0;
    if (nx > 0) {
      cudaMemsetAsync(xcnt + nx, 0, sizeof(int32_t), s);
      cub::DeviceScan::ExclusiveSum(nullptr, tb2, xcnt, p->gsx_off, nx + 1, s);
      if (tb2 > tb) {
        cudaFree(tmp);
        tmp = nullptr;
        if (cudaMalloc(&tmp, tb2) != cudaSuccess) { st = NTG_ERR_ALLOC; set_error("gs classes: tmp alloc"); break; }
        tb = tb2;
      }
      cub::DeviceScan::ExclusiveSum(tmp, tb, xcnt, p->gsx_off, nx + 1, s);
      cudaMemcpyAsync(&total, p->gsx_off + nx, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
    }
    if ((st = dev_alloc(&p->gsx_idx, total > 0 ? total : 1))) break;
    if (nx > 0) { k_gs_fill_x<<<grid_for(nx, T), T, 0, s>>>(seg_s, s8, nx, p->sh_idx, p->sh_off, p->gsx_off, p->gsx_idx); NTG_COUNT_LAUNCH(); }
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
      st = NTG_ERR_CUDA;
      set_error("gs classes: build kernels failed");
      break;
    }
    p->ncls[0] = (int64_t)h[0];
    p->ncls[1] = (int64_t)h[1];
    p->ncls[2] = (int64_t)h[2];
    p->ncls[3] = nx;
  } while (0);
  if (tmp) cudaFree(tmp);
  dev_free(key); dev_free(key_s); dev_free(seg); dev_free(seg_s); dev_free(hist); dev_free(xcnt);
  return st;
}

template <typename T, int OP>
static void launch_cls(ntg_plan* p, T* u, cudaStream_t s, const Scalars* sc) {
  const int b2 = (int)((p->ncls[0] + kGsPerBlock - 1) / kGsPerBlock);
  const int b4 = (int)((p->ncls[1] + kGsPerBlock - 1) / kGsPerBlock);
  const int b8 = (int)((p->ncls[2] + kGsPerBlock - 1) / kGsPerBlock);
  int bx = (int)((p->ncls[3] + kGsThreads - 1) / kGsThreads);
  if (bx > num_sms() * 4) bx = num_sms() * 4;
  const int grid = b2 + b4 + b8 + bx;
  if (grid == 0) return;
  { k_gs_cls<T, OP><<<grid, kGsThreads, 0, s>>>(u, p->gs2, p->ncls[0], p->gs4, p->ncls[1], p->gs8, p->ncls[2], p->gsx_idx, p->gsx_off, p->ncls[3], b2, b4, b8, sc); NTG_COUNT_LAUNCH(); }
}

template <typename T>
int gs_cls_launch(ntg_plan* p, T* u, int op, cudaStream_t s, const Scalars* sc) {
  switch (op) {
    case NTG_GS_ADD: launch_cls<T, NTG_GS_ADD>(p, u, s, sc); break;
    case NTG_GS_MUL: launch_cls<T, NTG_GS_MUL>(p, u, s, sc); break;
    case NTG_GS_MIN: launch_cls<T, NTG_GS_MIN>(p, u, s, sc); break;
    case NTG_GS_MAX: launch_cls<T, NTG_GS_MAX>(p, u, s, sc); break;
    default: set_error("gs_op: unknown op %d", op); return NTG_ERR_INVALID;
  }
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}
template int gs_cls_launch<double>(ntg_plan*, double*, int, cudaStream_t, const Scalars*);
template int gs_cls_launch<float>(ntg_plan*, float*, int, cudaStream_t, const Scalars*);

}  // namespace ntg
