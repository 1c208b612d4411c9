// Neko's binary mesh format (.nmsh), read and written on the host, and the
// GLL node coordinates of straight-sided elements from their vertices.
//
// Layout (little-endian, no padding), as the reference's mesh files hold
// it (data/debugging_pipe.nmsh, examples/power_iterations/ext_cyl.nmsh) and
// its cases name it ("mesh_file", examples/brinkman_term/brinkman_term.case:4):
//   int32 nelv, int32 gdim
//   nelv x { int32 el_idx; nv x { int32 v_idx; float64 x, y, z } }
//                                    nv = 8 (gdim 3) or 4 (gdim 2)
//   int32 nzones, nzones x int32[9] { e, f, p_e, p_f, pt_ids[4], type }
//   int32 ncurves, ncurves x { int32 e; float64 data[12][5]; int32 type[12] }
// Vertices are stored in the cyclic order of each layer (0 1 2 3 around the
// bottom face, then the top): tensor corner v = i + 2 j + 4 k is stored at
// position (0, 1, 3, 2, 4, 5, 7, 6)[v].  Faces in zones are 1-based in the
// tensor frame: r-, r+, s-, s+, t-, t+.  The API below passes vertices in
// tensor order and zone / curve records as stored (labeled zones, type 7,
// carry their label in p_f).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace {

constexpr int kStored[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // stored position of tensor corner v (self-inverse)

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

bool read_all(FILE* f, void* p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }
bool write_all(FILE* f, const void* p, size_t bytes) { return fwrite(p, 1, bytes, f) == bytes; }

// the host is little-endian (x86-64, aarch64): records are read as stored
template <typename T>
T get(const uint8_t* p) {
  T v;
  memcpy(&v, p, sizeof(T));
  return v;
}

int scan(const char* path, int32_t* nelv, int32_t* gdim, int32_t* nzones, int32_t* ncurves, long* zone_off) {
  File fh;
  fh.f = fopen(path, "rb");
  if (!fh.f) {
    ntg::set_error("nmsh: cannot open %s", path);
    return NTG_ERR_INVALID;
  }
  int32_t h[2];
  if (!read_all(fh.f, h, sizeof(h)) || h[0] < 0 || (h[1] != 2 && h[1] != 3)) {
    ntg::set_error("nmsh: %s has no valid header", path);
    return NTG_ERR_INVALID;
  }
  const int nv = h[1] == 3 ? 8 : 4;
  const long rec = 4 + nv * 28;
  const long zo = 8 + (long)h[0] * rec;
  int32_t nz = 0, nc = 0;
  if (fseek(fh.f, zo, SEEK_SET) || !read_all(fh.f, &nz, 4) || nz < 0 ||
      fseek(fh.f, zo + 4 + (long)nz * 36, SEEK_SET) || !read_all(fh.f, &nc, 4) || nc < 0) {
    ntg::set_error("nmsh: %s is truncated", path);
    return NTG_ERR_INVALID;
  }
  const long end = zo + 8 + (long)nz * 36 + (long)nc * 532;
  if (fseek(fh.f, 0, SEEK_END) || ftell(fh.f) != end) {
    ntg::set_error("nmsh: %s has %ld bytes, the records need %ld", path, ftell(fh.f), end);
    return NTG_ERR_INVALID;
  }
  *nelv = h[0];
  *gdim = h[1];
  *nzones = nz;
  *ncurves = nc;
  if (zone_off) *zone_off = zo;
  return NTG_OK;
}

struct GllNodes {
  double xi[NTG_LXMAX];
};

}  // namespace

using namespace ntg;

// GLL node coordinates of straight-sided hexahedra: trilinear in the eight
// tensor-ordered vertices (xyz: nelv x 8 x 3), nodes x fastest
__global__ void k_nodes_from_vertices(const double* __restrict__ xyz, int64_t nelv, int lx, GllNodes bs,
                                      double* __restrict__ x, double* __restrict__ y, double* __restrict__ z) {
  const int lx3 = lx * lx * lx;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nelv * lx3;
       l += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = l / lx3;
    const int q = (int)(l - e * lx3), i = q % lx, j = (q / lx) % lx, k = q / (lx * lx);
    const double xi[3] = {bs.xi[i], bs.xi[j], bs.xi[k]};
    double o[3] = {0.0, 0.0, 0.0};
    for (int v = 0; v < 8; ++v) {
      const double w = 0.125 * ((v & 1) ? 1.0 + xi[0] : 1.0 - xi[0]) * (((v >> 1) & 1) ? 1.0 + xi[1] : 1.0 - xi[1]) *
                       ((v >> 2) ? 1.0 + xi[2] : 1.0 - xi[2]);
      for (int d = 0; d < 3; ++d) o[d] += w * xyz[(e * 8 + v) * 3 + d];
    }
    x[l] = o[0];
    y[l] = o[1];
    z[l] = o[2];
  }
}

extern "C" {

int ntg_nmsh_info(const char* path, int32_t* nelv, int32_t* gdim, int32_t* nzones, int32_t* ncurves) {
  clear_error();
  NTG_CHECK_ARG(path && nelv && gdim && nzones && ncurves, "ntg_nmsh_info: null argument");
  return scan(path, nelv, gdim, nzones, ncurves, nullptr);
}

int ntg_nmsh_read(const char* path, int32_t* el_idx, int32_t* v_idx, double* xyz, int32_t* zones, int32_t* curve_el,
                  double* curve_data, int32_t* curve_type) {
  clear_error();
  NTG_CHECK_ARG(path && el_idx && v_idx && xyz, "ntg_nmsh_read: null argument");
  int32_t ne = 0, gd = 0, nz = 0, nc = 0;
  long zo = 0;
  NTG_TRY(scan(path, &ne, &gd, &nz, &nc, &zo));
  NTG_CHECK_ARG(nz == 0 || zones, "ntg_nmsh_read: the file has zones: zones must not be null");
  NTG_CHECK_ARG(nc == 0 || (curve_el && curve_data && curve_type), "ntg_nmsh_read: the file has curves");
  File fh;
  fh.f = fopen(path, "rb");
  if (!fh.f) {
    set_error("nmsh: cannot open %s", path);
    return NTG_ERR_INVALID;
  }
  const int nv = gd == 3 ? 8 : 4;
  const size_t rec = 4 + (size_t)nv * 28;
  std::vector<uint8_t> buf((size_t)ne * rec);
  if (fseek(fh.f, 8, SEEK_SET) || !read_all(fh.f, buf.data(), buf.size())) {
    set_error("nmsh: %s: element records", path);
    return NTG_ERR_INVALID;
  }
  for (int64_t e = 0; e < ne; ++e) {
    const uint8_t* r = buf.data() + e * rec;
    el_idx[e] = get<int32_t>(r);
    for (int v = 0; v < nv; ++v) {
      const uint8_t* q = r + 4 + (size_t)kStored[v] * 28;
      v_idx[e * nv + v] = get<int32_t>(q);
      for (int d = 0; d < 3; ++d) xyz[(e * nv + v) * 3 + d] = get<double>(q + 4 + 8 * d);
    }
  }
  if (nz > 0 && (fseek(fh.f, zo + 4, SEEK_SET) || !read_all(fh.f, zones, (size_t)nz * 36))) {
    set_error("nmsh: %s: zones", path);
    return NTG_ERR_INVALID;
  }
  if (nc > 0) {
    std::vector<uint8_t> cb((size_t)nc * 532);
    if (fseek(fh.f, zo + 8 + (long)nz * 36, SEEK_SET) || !read_all(fh.f, cb.data(), cb.size())) {
      set_error("nmsh: %s: curves", path);
      return NTG_ERR_INVALID;
    }
    for (int64_t c = 0; c < nc; ++c) {
      const uint8_t* r = cb.data() + c * 532;
      curve_el[c] = get<int32_t>(r);
      memcpy(curve_data + c * 60, r + 4, 480);
      memcpy(curve_type + c * 12, r + 484, 48);
    }
  }
  return NTG_OK;
}

int ntg_nmsh_write(const char* path, int32_t nelv, int32_t gdim, const int32_t* el_idx, const int32_t* v_idx,
                   const double* xyz, int32_t nzones, const int32_t* zones, int32_t ncurves, const int32_t* curve_el,
                   const double* curve_data, const int32_t* curve_type) {
  clear_error();
  NTG_CHECK_ARG(path && el_idx && v_idx && xyz && nelv >= 0 && (gdim == 2 || gdim == 3) && nzones >= 0 &&
                    ncurves >= 0,
                "ntg_nmsh_write: bad argument");
  NTG_CHECK_ARG(nzones == 0 || zones, "ntg_nmsh_write: zones null");
  NTG_CHECK_ARG(ncurves == 0 || (curve_el && curve_data && curve_type), "ntg_nmsh_write: curves null");
  File fh;
  fh.f = fopen(path, "wb");
  if (!fh.f) {
    set_error("nmsh: cannot create %s", path);
    return NTG_ERR_INVALID;
  }
  const int nv = gdim == 3 ? 8 : 4;
  const size_t rec = 4 + (size_t)nv * 28;
  std::vector<uint8_t> buf(8 + (size_t)nelv * rec);
  memcpy(buf.data(), &nelv, 4);
  memcpy(buf.data() + 4, &gdim, 4);
  for (int64_t e = 0; e < nelv; ++e) {
    uint8_t* r = buf.data() + 8 + e * rec;
    memcpy(r, el_idx + e, 4);
    for (int v = 0; v < nv; ++v) {
      uint8_t* q = r + 4 + (size_t)kStored[v] * 28;
      memcpy(q, v_idx + e * nv + v, 4);
      memcpy(q + 4, xyz + (e * nv + v) * 3, 24);
    }
  }
  bool ok = write_all(fh.f, buf.data(), buf.size()) && write_all(fh.f, &nzones, 4) &&
            (nzones == 0 || write_all(fh.f, zones, (size_t)nzones * 36)) && write_all(fh.f, &ncurves, 4);
  for (int64_t c = 0; ok && c < ncurves; ++c)
    ok = write_all(fh.f, curve_el + c, 4) && write_all(fh.f, curve_data + c * 60, 480) &&
         write_all(fh.f, curve_type + c * 12, 48);
  if (!ok || fflush(fh.f)) {
    set_error("nmsh: write to %s failed", path);
    return NTG_ERR_INVALID;
  }
  return NTG_OK;
}

int ntg_nodes_from_vertices(int64_t nelv, int lx, const double* xyz_d, double* x_d, double* y_d, double* z_d,
                            void* stream) {
  clear_error();
  NTG_CHECK_ARG(nelv > 0 && lx >= 2 && lx <= NTG_LXMAX && xyz_d && x_d && y_d && z_d,
                "ntg_nodes_from_vertices: bad argument");
  GllNodes bs{};
  double w[NTG_LXMAX], D[NTG_LXMAX * NTG_LXMAX];
  gll_basis(lx, bs.xi, w, D);
  bs.xi[0] = -1.0;
  bs.xi[lx - 1] = 1.0;
  const cudaStream_t s = (cudaStream_t)stream;
  k_nodes_from_vertices<<<grid_for(nelv * lx * lx * lx, 256), 256, 0, s>>>(xyz_d, nelv, lx, bs, x_d, y_d, z_d);
  NTG_COUNT_LAUNCH();
  NTG_CUDA_TRY(cudaGetLastError());
  return NTG_OK;
}

}  // extern "C"
