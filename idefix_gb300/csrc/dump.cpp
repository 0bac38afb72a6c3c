// Restart dumps in the reference's file format (Dump::Write / Dump::Read,
// output/dump.cpp:30-985; reader pytools/dump_io.py), so that a run can be
// checkpointed here and resumed by the reference or the other way round.
//
// File layout (serial, one block):
//   128-byte header "Idefix <version> Dump Data little endian", NUL padded
//   then fields, each: name (16 bytes, NUL padded), int32 type (0 double,
//   1 float, 2 int32, 3 bool), int32 ndim, int32 dims[ndim], raw data
//   (first index fastest)
//   fields: x1 xl1 xr1 x2 xl2 xr2 x3 xl3 xr3 (cell centres / left / right
//   edges of the active cells), then the registered fields in name order
//   (the reference keeps them in a std::map): Vc-PRS Vc-RHO Vc-VX1 .. Vc-VXd
//   (active cells), Vs-BX1s .. Vs-BXds (active faces, one more along the
//   field's direction), dt, time, vtkFileNumber; then "eof" (one double).
// The cell-centred field is not stored (it is rebuilt from the faces), as in
// the reference for COMPONENTS == DIMENSIONS (fluid.hpp:605-625).
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "../../include/idefix_gb300.h"

namespace {

constexpr int kHeader = 128;
constexpr int kName = 16;
constexpr int kDouble = 0, kInt = 2;

struct Layout {
  int dims, ng;
  int n[3], nt[3], ntv[3];
  long long ncell, nface;
  double xbeg[3], xend[3];
};

bool layout_of(const idfx_gpu_config* cfg, Layout& L) {
  if (!cfg || (cfg->dims != 2 && cfg->dims != 3)) return false;
  L.dims = cfg->dims;
  L.ng = (cfg->order == IDFX_PPM) ? 3 : 2;
  for (int d = 0; d < 3; d++) {
    const bool act = d < L.dims;
    L.n[d] = act ? cfg->n[d] : 1;
    if (L.n[d] < 1) return false;
    L.nt[d] = L.n[d] + (act ? 2 * L.ng : 0);
    L.ntv[d] = L.nt[d] + (act ? 1 : 0);
    L.xbeg[d] = act ? cfg->xbeg[d] : 0.0;
    L.xend[d] = act ? cfg->xend[d] : 1.0;
  }
  L.ncell = (long long)L.nt[0] * L.nt[1] * L.nt[2];
  L.nface = (long long)L.ntv[0] * L.ntv[1] * L.ntv[2];
  return true;
}

// variable index of the reference layout (RHO, VX1..VXd, PRS, BX1..BXd)
int var_index(const Layout& L, const std::string& s) {
  if (s == "RHO") return 0;
  if (s == "VX1") return 1;
  if (s == "VX2") return 2;
  if (s == "VX3") return L.dims == 3 ? 3 : -1;
  if (s == "PRS") return L.dims + 1;
  return -1;
}

bool write_field(FILE* f, const char* name, int type, const std::vector<int>& dims, const void* data,
                 size_t elem) {
  char nm[kName];
  std::memset(nm, 0, sizeof(nm));
  std::snprintf(nm, sizeof(nm), "%s", name);
  const int ndim = (int)dims.size();
  size_t ntot = 1;
  for (int d : dims) ntot *= (size_t)d;
  return std::fwrite(nm, 1, kName, f) == (size_t)kName && std::fwrite(&type, 4, 1, f) == 1 &&
         std::fwrite(&ndim, 4, 1, f) == 1 && std::fwrite(dims.data(), 4, ndim, f) == (size_t)ndim &&
         std::fwrite(data, elem, ntot, f) == ntot;
}

// the active block of one ghosted 3-D array as a contiguous (i fastest) copy;
// ext[d] = extra points along d (faces), stride dims st[] of the ghosted array
void gather(const Layout& L, const double* src, const int* cnt, const int* st, std::vector<double>& out) {
  out.resize((size_t)cnt[0] * cnt[1] * cnt[2]);
  size_t q = 0;
  for (int k = 0; k < cnt[2]; k++)
    for (int j = 0; j < cnt[1]; j++)
      for (int i = 0; i < cnt[0]; i++) {
        const int kk = (L.dims == 3 ? L.ng : 0) + k, jj = L.ng + j, ii = L.ng + i;
        out[q++] = src[((long long)kk * st[1] + jj) * st[0] + ii];
      }
}

void scatter(const Layout& L, double* dst, const int* cnt, const int* st, const std::vector<double>& in) {
  size_t q = 0;
  for (int k = 0; k < cnt[2]; k++)
    for (int j = 0; j < cnt[1]; j++)
      for (int i = 0; i < cnt[0]; i++) {
        const int kk = (L.dims == 3 ? L.ng : 0) + k, jj = L.ng + j, ii = L.ng + i;
        dst[((long long)kk * st[1] + jj) * st[0] + ii] = in[q++];
      }
}

struct Reader {
  FILE* f;
  bool field(std::string& name, int& type, std::vector<int>& dims) {
    char nm[kName + 1];
    std::memset(nm, 0, sizeof(nm));
    if (std::fread(nm, 1, kName, f) != (size_t)kName) return false;
    name = std::string(nm);
    int ndim = 0;
    if (std::fread(&type, 4, 1, f) != 1 || std::fread(&ndim, 4, 1, f) != 1) return false;
    if (ndim < 0 || ndim > 8) return false;
    dims.resize(ndim);
    return std::fread(dims.data(), 4, ndim, f) == (size_t)ndim;
  }
  static size_t elem(int type) { return type == 0 ? 8 : type == 1 ? 4 : type == 2 ? 4 : 1; }
  bool data(void* dst, int type, const std::vector<int>& dims) {
    size_t n = 1;
    for (int d : dims) n *= (size_t)d;
    return std::fread(dst, elem(type), n, f) == n;
  }
  bool skip(int type, const std::vector<int>& dims) {
    size_t n = 1;
    for (int d : dims) n *= (size_t)d;
    return std::fseek(f, (long)(n * elem(type)), SEEK_CUR) == 0;
  }
};

}  // namespace

extern "C" {

int idfx_dump_write(const char* path, const idfx_gpu_config* cfg, const double* Vc, const double* Vs, double t,
                    double dt, int vtk_file_number) {
  Layout L;
  if (!path || !Vc || !Vs || !layout_of(cfg, L)) return IDFX_ERR_STATE;
  FILE* f = std::fopen(path, "wb");
  if (!f) return IDFX_ERR_STATE;
  bool ok = true;
  char header[kHeader];
  std::memset(header, 0, sizeof(header));
  std::snprintf(header, sizeof(header), "Idefix %s Dump Data %s endian", "2.2.02", "little");
  ok = ok && std::fwrite(header, 1, kHeader, f) == (size_t)kHeader;
  // coordinates of the active cells (gridHost.cpp:80-86)
  for (int d = 0; d < 3 && ok; d++) {
    const double dx = (L.xend[d] - L.xbeg[d]) / (L.n[d]);
    std::vector<double> x(L.n[d]), xl(L.n[d]), xr(L.n[d]);
    for (int i = 0; i < L.n[d]; i++) {
      x[i] = L.xbeg[d] + (i + 0.5) * dx;
      xl[i] = L.xbeg[d] + i * dx;
      xr[i] = L.xbeg[d] + (i + 1) * dx;
    }
    char nm[kName];
    std::snprintf(nm, sizeof(nm), "x%d", d + 1);
    ok = ok && write_field(f, nm, kDouble, {L.n[d]}, x.data(), 8);
    std::snprintf(nm, sizeof(nm), "xl%d", d + 1);
    ok = ok && write_field(f, nm, kDouble, {L.n[d]}, xl.data(), 8);
    std::snprintf(nm, sizeof(nm), "xr%d", d + 1);
    ok = ok && write_field(f, nm, kDouble, {L.n[d]}, xr.data(), 8);
  }
  // registered fields in name order
  std::map<std::string, std::function<bool()>> fields;
  const int cst[2] = {L.nt[0], L.nt[1]};
  const int fst[2] = {L.ntv[0], L.ntv[1]};
  const char* vnames[] = {"RHO", "VX1", "VX2", "VX3", "PRS"};
  for (const char* vn : vnames) {
    const int v = var_index(L, vn);
    if (v < 0) continue;
    fields[std::string("Vc-") + vn] = [&, v, vn]() {
      std::vector<double> buf;
      gather(L, Vc + (size_t)v * L.ncell, L.n, cst, buf);
      return write_field(f, (std::string("Vc-") + vn).c_str(), kDouble, {L.n[0], L.n[1], L.n[2]}, buf.data(), 8);
    };
  }
  for (int d = 0; d < L.dims; d++) {
    const std::string nm = "Vs-BX" + std::to_string(d + 1) + "s";
    fields[nm] = [&, d, nm]() {
      int cnt[3] = {L.n[0], L.n[1], L.n[2]};
      cnt[d] += 1;
      std::vector<double> buf;
      gather(L, Vs + (size_t)d * L.nface, cnt, fst, buf);
      return write_field(f, nm.c_str(), kDouble, {cnt[0], cnt[1], cnt[2]}, buf.data(), 8);
    };
  }
  fields["time"] = [&]() { return write_field(f, "time", kDouble, {1}, &t, 8); };
  fields["dt"] = [&]() { return write_field(f, "dt", kDouble, {1}, &dt, 8); };
  fields["vtkFileNumber"] = [&]() { return write_field(f, "vtkFileNumber", kInt, {1}, &vtk_file_number, 4); };
  for (auto& kv : fields) ok = ok && kv.second();
  const double zero = 0.0;
  ok = ok && write_field(f, "eof", kDouble, {1}, &zero, 8);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? IDFX_OK : IDFX_ERR_STATE;
}

int idfx_dump_read(const char* path, const idfx_gpu_config* cfg, double* Vc, double* Vs, double* t, double* dt) {
  Layout L;
  if (!path || !Vc || !Vs || !layout_of(cfg, L)) return IDFX_ERR_STATE;
  FILE* f = std::fopen(path, "rb");
  if (!f) return IDFX_ERR_STATE;
  Reader R{f};
  int rc = IDFX_OK;
  char header[kHeader + 1];
  std::memset(header, 0, sizeof(header));
  if (std::fread(header, 1, kHeader, f) != (size_t)kHeader) rc = IDFX_ERR_STATE;
  if (!rc && std::strstr(header, "big endian")) rc = IDFX_ERR_CONFIG;  // the library writes little-endian
  if (!rc && std::strncmp(header, "Idefix ", 7) != 0) rc = IDFX_ERR_CONFIG;
  std::string name;
  int type = 0;
  std::vector<int> dims;
  // coordinates: the block size must match (Dump::Read, dump.cpp:676-693)
  for (int d = 0; d < 3 && !rc; d++)
    for (int s = 0; s < 3 && !rc; s++) {
      if (!R.field(name, type, dims) || dims.size() != 1) {
        rc = IDFX_ERR_STATE;
        break;
      }
      if (s == 0 && dims[0] != L.n[d]) rc = IDFX_ERR_CONFIG;
      if (!rc && !R.skip(type, dims)) rc = IDFX_ERR_STATE;
    }
  const int cst[2] = {L.nt[0], L.nt[1]};
  const int fst[2] = {L.ntv[0], L.ntv[1]};
  bool got_t = false, got_dt = false;
  while (!rc) {
    if (!R.field(name, type, dims)) {
      rc = IDFX_ERR_STATE;
      break;
    }
    if (name == "eof") break;
    if (name.rfind("Vc-", 0) == 0 && var_index(L, name.substr(3)) >= 0) {
      const int v = var_index(L, name.substr(3));
      if (type != kDouble || dims.size() != 3 || dims[0] != L.n[0] || dims[1] != L.n[1] || dims[2] != L.n[2]) {
        rc = IDFX_ERR_CONFIG;
        break;
      }
      std::vector<double> buf((size_t)L.n[0] * L.n[1] * L.n[2]);
      if (!R.data(buf.data(), type, dims)) rc = IDFX_ERR_STATE;
      else scatter(L, Vc + (size_t)v * L.ncell, L.n, cst, buf);
    } else if (name.size() == 7 && name.rfind("Vs-BX", 0) == 0 && name[6] == 's' && name[5] >= '1' &&
               name[5] < '1' + L.dims) {
      const int d = name[5] - '1';
      int cnt[3] = {L.n[0], L.n[1], L.n[2]};
      cnt[d] += 1;
      if (type != kDouble || dims.size() != 3 || dims[0] != cnt[0] || dims[1] != cnt[1] || dims[2] != cnt[2]) {
        rc = IDFX_ERR_CONFIG;
        break;
      }
      std::vector<double> buf((size_t)cnt[0] * cnt[1] * cnt[2]);
      if (!R.data(buf.data(), type, dims)) rc = IDFX_ERR_STATE;
      else scatter(L, Vs + (size_t)d * L.nface, cnt, fst, buf);
    } else if ((name == "time" || name == "dt") && type == kDouble && dims.size() == 1 && dims[0] == 1) {
      double v = 0.0;
      if (!R.data(&v, type, dims)) rc = IDFX_ERR_STATE;
      if (name == "time") {
        if (t) *t = v;
        got_t = true;
      } else {
        if (dt) *dt = v;
        got_dt = true;
      }
    } else if (!R.skip(type, dims)) {  // fields of other modules (dump.cpp:755-758)
      rc = IDFX_ERR_STATE;
    }
  }
  std::fclose(f);
  if (!rc && !(got_t && got_dt)) rc = IDFX_ERR_CONFIG;
  return rc;
}

}  // extern "C"
