// Field files in the Nek5000 binary format that Neko's fld_file_t writes and
// reads (the reference's field output: fld_file_output_t,
// sources/topology_optimization/topopt_design.f90:283-286 and
// steady_state_problem.f90:228-244), with the `.nek5000` index file that
// visualisation tools open.  Host code: fields come from device or host
// arrays.
//
// Layout, all in the writer's native byte order:
//   132-byte ASCII header
//     "#std" wdsize lx ly lz nelt nelgt time istep fid0 nfiles rdcode,
//     blank padded ('#std', 1x, i1, 3(1x, i2), 2(1x, i10), 1x, e20.13, 1x,
//     i9, 2(1x, i6), 1x, rdcode)
//   float32 6.54321 (byte-order mark)
//   int32 x nelt: 1-based global element numbers
//   per field in rdcode order (X coordinates, U velocity, P pressure,
//   T temperature, S + two digits scalars), per element, lx^3 values per
//   component (vectors: x block, y block, z block of the element), as
//   float32 (wdsize 4) or float64 (wdsize 8)
//   per field again, per element, float32 min and max of each component
//   (the 3-D metadata block).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace {

struct Src {
  const double* p;
  int on_device;
};

int fetch(std::vector<double>& h, const double* p, size_t n, int on_device) {
  h.resize(n);
  if (on_device) {
    if (cudaMemcpy(h.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
      ntg::set_error("fld: device copy failed");
      return NTG_ERR_CUDA;
    }
  } else {
    memcpy(h.data(), p, n * sizeof(double));
  }
  return NTG_OK;
}

int put(std::vector<double>& dst, const double* p, size_t n, int on_device) {
  if (on_device) {
    if (cudaMemcpy((void*)p, dst.data(), n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
      ntg::set_error("fld: device copy failed");
      return NTG_ERR_CUDA;
    }
  } else {
    memcpy((void*)p, dst.data(), n * sizeof(double));
  }
  return NTG_OK;
}

struct Field {
  char code;                       // X U P T S
  std::vector<const double*> comp;  // 1 or 3 (or one per scalar for S)
};

}  // namespace

extern "C" {

int ntg_fld_write(const char* path, int lx, int64_t nelv, const int64_t* glb_el, double time, int tstep, int wdsize,
                  int on_device, const double* x, const double* y, const double* z, const double* u,
                  const double* v, const double* w, const double* p, const double* t, const double* const* s,
                  int nscal) {
  ntg::clear_error();
  NTG_CHECK_ARG(path && lx >= 2 && lx <= 99 && nelv > 0 && (wdsize == 4 || wdsize == 8) && nscal >= 0 &&
                    nscal <= 99 && (nscal == 0 || s),
                "ntg_fld_write: bad argument");
  NTG_CHECK_ARG(!(x || y || z) || (x && y && z), "ntg_fld_write: coordinates need x, y and z");
  NTG_CHECK_ARG(!(u || v || w) || (u && v && w), "ntg_fld_write: velocity needs u, v and w");
  NTG_CHECK_ARG(nelv < 2147483647, "ntg_fld_write: nelv must fit int32");
  const size_t l3 = (size_t)lx * lx * lx, n = l3 * (size_t)nelv;
  std::vector<Field> fields;
  std::string rdcode;
  if (x) fields.push_back({'X', {x, y, z}}), rdcode += "X";
  if (u) fields.push_back({'U', {u, v, w}}), rdcode += "U";
  if (p) fields.push_back({'P', {p}}), rdcode += "P";
  if (t) fields.push_back({'T', {t}}), rdcode += "T";
  if (nscal) {
    Field f{'S', {}};
    for (int q = 0; q < nscal; ++q) {
      NTG_CHECK_ARG(s[q], "ntg_fld_write: null scalar field");
      f.comp.push_back(s[q]);
    }
    fields.push_back(f);
    char b[8];
    snprintf(b, sizeof b, "S%02d", nscal);
    rdcode += b;
  }
  NTG_CHECK_ARG(!fields.empty(), "ntg_fld_write: no field given");
  char hdr[160];
  snprintf(hdr, sizeof hdr, "#std %1d %2d %2d %2d %10lld %10lld %20.13E %9d %6d %6d %s", wdsize, lx, lx, lx,
           (long long)nelv, (long long)nelv, time, tstep, 0, 1, rdcode.c_str());
  std::string h(hdr);
  h.resize(132, ' ');
  FILE* fp = fopen(path, "wb");
  if (!fp) {
    ntg::set_error("ntg_fld_write: cannot open %s", path);
    return NTG_ERR_INVALID;
  }
  int st = NTG_OK;
  const float mark = 6.54321f;
  fwrite(h.data(), 1, 132, fp);
  fwrite(&mark, 4, 1, fp);
  std::vector<int32_t> el(nelv);
  for (int64_t e = 0; e < nelv; ++e) el[e] = (int32_t)(glb_el ? glb_el[e] : e + 1);
  fwrite(el.data(), 4, (size_t)nelv, fp);
  // data, then the per-element min/max block
  std::vector<std::vector<double>> host;
  for (const Field& f : fields)
    for (const double* c : f.comp) {
      host.emplace_back();
      if (!st) st = fetch(host.back(), c, n, on_device);
    }
  if (!st) {
    size_t k = 0;
    std::vector<float> b32(l3);
    for (const Field& f : fields) {
      const size_t nc = f.comp.size();
      const bool vec = f.code == 'X' || f.code == 'U';
      // vectors interleave the components per element; scalars S come
      // one field after another
      if (vec) {
        for (int64_t e = 0; e < nelv; ++e)
          for (size_t c = 0; c < nc; ++c) {
            const double* src = host[k + c].data() + e * l3;
            if (wdsize == 8) fwrite(src, 8, l3, fp);
            else {
              for (size_t q = 0; q < l3; ++q) b32[q] = (float)src[q];
              fwrite(b32.data(), 4, l3, fp);
            }
          }
      } else {
        for (size_t c = 0; c < nc; ++c)
          for (int64_t e = 0; e < nelv; ++e) {
            const double* src = host[k + c].data() + e * l3;
            if (wdsize == 8) fwrite(src, 8, l3, fp);
            else {
              for (size_t q = 0; q < l3; ++q) b32[q] = (float)src[q];
              fwrite(b32.data(), 4, l3, fp);
            }
          }
      }
      k += nc;
    }
    k = 0;
    for (const Field& f : fields) {
      const size_t nc = f.comp.size();
      const bool vec = f.code == 'X' || f.code == 'U';
      auto mm = [&](size_t c, int64_t e) {
        const double* src = host[k + c].data() + e * l3;
        double lo = src[0], hi = src[0];
        for (size_t q = 1; q < l3; ++q) lo = src[q] < lo ? src[q] : lo, hi = src[q] > hi ? src[q] : hi;
        const float b[2] = {(float)lo, (float)hi};
        fwrite(b, 4, 2, fp);
      };
      if (vec) {
        for (int64_t e = 0; e < nelv; ++e)
          for (size_t c = 0; c < nc; ++c) mm(c, e);
      } else {
        for (size_t c = 0; c < nc; ++c)
          for (int64_t e = 0; e < nelv; ++e) mm(c, e);
      }
      k += nc;
    }
  }
  if (ferror(fp)) {
    ntg::set_error("ntg_fld_write: write error on %s", path);
    st = NTG_ERR_INVALID;
  }
  fclose(fp);
  return st;
}

int ntg_fld_write_index(const char* path, const char* name, int first, int count) {
  ntg::clear_error();
  NTG_CHECK_ARG(path && name && count >= 0, "ntg_fld_write_index: bad argument");
  FILE* fp = fopen(path, "w");
  if (!fp) {
    ntg::set_error("ntg_fld_write_index: cannot open %s", path);
    return NTG_ERR_INVALID;
  }
  fprintf(fp, "filetemplate: %s%%01d.f%%05d\nfirsttimestep: %d\nnumtimesteps: %d\n", name, first, count);
  fclose(fp);
  return NTG_OK;
}

// Header of a field file: lx, element count, word size, time, step and the
// rdcode (NUL-terminated, up to cap - 1 characters).
int ntg_fld_info(const char* path, int* lx, int64_t* nelv, int* wdsize, double* time, int* tstep, char* rdcode,
                 int cap) {
  ntg::clear_error();
  NTG_CHECK_ARG(path, "ntg_fld_info: null path");
  FILE* fp = fopen(path, "rb");
  if (!fp) {
    ntg::set_error("ntg_fld_info: cannot open %s", path);
    return NTG_ERR_INVALID;
  }
  char h[133] = {0};
  float mark = 0.0f;
  const bool ok = fread(h, 1, 132, fp) == 132 && fread(&mark, 4, 1, fp) == 1;
  fclose(fp);
  int wd = 0, l1 = 0, l2 = 0, l3 = 0, step = 0, fid = 0, nf = 0;
  long long ne = 0, ng = 0;
  double tm = 0.0;
  char code[64] = {0};
  if (!ok || strncmp(h, "#std", 4) != 0 ||
      sscanf(h + 4, "%d %d %d %d %lld %lld %lf %d %d %d %63s", &wd, &l1, &l2, &l3, &ne, &ng, &tm, &step, &fid, &nf,
             code) < 10) {
    ntg::set_error("ntg_fld_info: %s is not a #std field file", path);
    return NTG_ERR_INVALID;
  }
  if (mark != 6.54321f) {
    ntg::set_error("ntg_fld_info: %s has the other byte order", path);
    return NTG_ERR_UNSUPPORTED;
  }
  if (lx) *lx = l1;
  if (nelv) *nelv = ne;
  if (wdsize) *wdsize = wd;
  if (time) *time = tm;
  if (tstep) *tstep = step;
  if (rdcode && cap > 0) {
    strncpy(rdcode, code, (size_t)cap - 1);
    rdcode[cap - 1] = 0;
  }
  return NTG_OK;
}

// Read the fields a file holds into the given arrays (NULL skips a field;
// element order as stored, element numbers to glb_el when given).
int ntg_fld_read(const char* path, int on_device, int64_t* glb_el, double* x, double* y, double* z, double* u,
                 double* v, double* w, double* p, double* t, double* const* s, int nscal) {
  int lx = 0, wd = 0, step = 0;
  int64_t nelv = 0;
  double tm = 0.0;
  char code[64];
  NTG_TRY(ntg_fld_info(path, &lx, &nelv, &wd, &tm, &step, code, sizeof code));
  FILE* fp = fopen(path, "rb");
  if (!fp) {
    ntg::set_error("ntg_fld_read: cannot open %s", path);
    return NTG_ERR_INVALID;
  }
  const size_t l3 = (size_t)lx * lx * lx, n = l3 * (size_t)nelv;
  int st = NTG_OK;
  fseek(fp, 136, SEEK_SET);
  std::vector<int32_t> el(nelv);
  if (fread(el.data(), 4, (size_t)nelv, fp) != (size_t)nelv) st = NTG_ERR_INVALID;
  if (!st && glb_el)
    for (int64_t e = 0; e < nelv; ++e) glb_el[e] = el[e];
  std::vector<double> buf(n);
  std::vector<double> rd(l3);
  std::vector<float> r32(l3);
  auto read_block = [&](double* dst) -> bool {
    if (wd == 8) {
      if (fread(rd.data(), 8, l3, fp) != l3) return false;
    } else {
      if (fread(r32.data(), 4, l3, fp) != l3) return false;
      for (size_t q = 0; q < l3; ++q) rd[q] = r32[q];
    }
    if (dst) memcpy(dst, rd.data(), l3 * sizeof(double));
    return true;
  };
  for (const char* c = code; *c && !st; ++c) {
    if (*c == 'X' || *c == 'U') {
      double* out[3] = {*c == 'X' ? x : u, *c == 'X' ? y : v, *c == 'X' ? z : w};
      std::vector<std::vector<double>> hv(3, std::vector<double>(n));
      for (int64_t e = 0; e < nelv && !st; ++e)
        for (int q = 0; q < 3 && !st; ++q)
          if (!read_block(hv[q].data() + e * l3)) st = NTG_ERR_INVALID;
      for (int q = 0; q < 3 && !st; ++q)
        if (out[q]) st = put(hv[q], out[q], n, on_device);
    } else if (*c == 'P' || *c == 'T') {
      double* out = *c == 'P' ? p : t;
      for (int64_t e = 0; e < nelv && !st; ++e)
        if (!read_block(buf.data() + e * l3)) st = NTG_ERR_INVALID;
      if (!st && out) st = put(buf, out, n, on_device);
    } else if (*c == 'S') {
      const int ns = (c[1] - '0') * 10 + (c[2] - '0');
      c += 2;
      for (int q = 0; q < ns && !st; ++q) {
        for (int64_t e = 0; e < nelv && !st; ++e)
          if (!read_block(buf.data() + e * l3)) st = NTG_ERR_INVALID;
        if (!st && s && q < nscal && s[q]) st = put(buf, s[q], n, on_device);
      }
    }
  }
  if (st == NTG_ERR_INVALID) ntg::set_error("ntg_fld_read: %s is truncated", path);
  fclose(fp);
  return st;
}

}  // extern "C"
