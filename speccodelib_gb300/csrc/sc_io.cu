// Fortran unformatted field I/O: the files the reference's output3d /
// input3d write and read (output.f90:103-132, input.f90:106-136), so a state
// can move between the reference's solvers and a handle.
//
// `write(10) ux` on a sequential unformatted unit (gfortran) produces one
// record: a 4-byte little-endian length marker, the array's bytes in memory
// order, the marker again.  A record longer than the largest subrecord
// (2147483639 bytes by default) is split into subrecords, each with its own
// leading and trailing markers; a leading marker is negative when more
// subrecords follow, a trailing marker negative when one precedes.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/specns.h"

namespace sc {
int set_last_error(int code, const char* msg);   // sc_runtime.cu
}

namespace {

constexpr long long kMaxSubrecord = 2147483639LL;

int iofail(const std::string& msg) { return sc::set_last_error(SC_ERR_IO, msg.c_str()); }

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

int write_record(const char* path, const void* data, long long nbytes, long long max_sub) {
  if (!path || (!data && nbytes > 0) || nbytes < 0) return sc::set_last_error(SC_ERR_INVALID, "bad record arguments");
  if (max_sub <= 0) max_sub = kMaxSubrecord;
  if (max_sub > kMaxSubrecord) return sc::set_last_error(SC_ERR_INVALID, "subrecords are at most 2147483639 bytes");
  File fh;
  fh.f = std::fopen(path, "wb");
  if (!fh.f) return iofail(std::string("cannot open for writing: ") + path);
  const char* p = static_cast<const char*>(data);
  long long left = nbytes;
  bool first = true;
  do {
    const long long len = left < max_sub ? left : max_sub;
    const bool more = left > len;
    const int32_t lead = (int32_t)(more ? -len : len);
    const int32_t trail = (int32_t)(first ? len : -len);
    if (std::fwrite(&lead, 4, 1, fh.f) != 1 || (len > 0 && std::fwrite(p, 1, (size_t)len, fh.f) != (size_t)len) ||
        std::fwrite(&trail, 4, 1, fh.f) != 1)
      return iofail(std::string("write failed: ") + path);
    p += len;
    left -= len;
    first = false;
  } while (left > 0);
  if (std::fclose(fh.f) != 0) {
    fh.f = nullptr;
    return iofail(std::string("close failed: ") + path);
  }
  fh.f = nullptr;
  return SC_OK;
}

int read_record(const char* path, void* data, long long nbytes) {
  if (!path || (!data && nbytes > 0) || nbytes < 0) return sc::set_last_error(SC_ERR_INVALID, "bad record arguments");
  File fh;
  fh.f = std::fopen(path, "rb");
  if (!fh.f) return iofail(std::string("cannot open for reading: ") + path);
  char* p = static_cast<char*>(data);
  long long got = 0;
  bool first = true;
  for (;;) {
    int32_t lead = 0, trail = 0;
    if (std::fread(&lead, 4, 1, fh.f) != 1) return iofail(std::string("truncated record marker: ") + path);
    const long long len = lead < 0 ? -(long long)lead : (long long)lead;
    if (got + len > nbytes) return iofail(std::string("record longer than the field: ") + path);
    if (len > 0 && std::fread(p + got, 1, (size_t)len, fh.f) != (size_t)len)
      return iofail(std::string("truncated record: ") + path);
    if (std::fread(&trail, 4, 1, fh.f) != 1) return iofail(std::string("truncated record marker: ") + path);
    const long long tlen = trail < 0 ? -(long long)trail : (long long)trail;
    if (tlen != len || (trail < 0) == first) return iofail(std::string("inconsistent record markers: ") + path);
    got += len;
    first = false;
    if (lead >= 0) break;
  }
  if (got != nbytes) return iofail(std::string("record shorter than the field: ") + path);
  return SC_OK;
}

std::string field_path(const char* dir, const char* comp, int idump) {
  // './out/ux'//fnm//'.dat' with fnm the left-adjusted integer (output.f90:117-120)
  std::string d = dir && dir[0] ? dir : ".";
  if (d.back() != '/') d += '/';
  return d + comp + std::to_string(idump) + ".dat";
}

// n complex values stored in precision `from` as precision `to` (SC_FP32:
// two floats each, SC_FP64: two doubles each).
std::vector<char> convert_values(const std::vector<char>& in, size_t n, int from, int to) {
  if (from == to) return in;
  std::vector<char> out(n * (to == SC_FP32 ? 8 : 16));
  if (to == SC_FP32) {
    const double* s = reinterpret_cast<const double*>(in.data());
    float* d = reinterpret_cast<float*>(out.data());
    for (size_t i = 0; i < 2 * n; ++i) d[i] = (float)s[i];
  } else {
    const float* s = reinterpret_cast<const float*>(in.data());
    double* d = reinterpret_cast<double*>(out.data());
    for (size_t i = 0; i < 2 * n; ++i) d[i] = (double)s[i];
  }
  return out;
}

}  // namespace

extern "C" {

int sc_fortran_record_write(const char* path, const void* data, long long nbytes, long long max_subrecord) {
  return write_record(path, data, nbytes, max_subrecord);
}

int sc_fortran_record_read(const char* path, void* data, long long nbytes) {
  return read_record(path, data, nbytes);
}

int sc_output3d(sc_handle* h, const char* dir, int idump, int file_precision) {
  sc_params p{};
  if (!h || sc_get_params(h, &p) != SC_OK) return sc::set_last_error(SC_ERR_INVALID, "null handle");
  if (file_precision != SC_FP32 && file_precision != SC_FP64)
    return sc::set_last_error(SC_ERR_INVALID, "file precision must be SC_FP32 or SC_FP64");
  const size_t n = (size_t)(p.nx / 2 + 1) * p.ny * p.nz;
  const size_t hb = p.precision == SC_FP32 ? 8 : 16;
  std::vector<char> v[3];
  for (auto& a : v) a.resize(n * hb);
  if (int r = sc_get_state(h, v[0].data(), v[1].data(), v[2].data())) return r;
  const char* names[3] = {"ux", "uy", "uz"};
  for (int c = 0; c < 3; ++c) {
    std::vector<char> out;
    const void* src = v[c].data();
    if (file_precision != p.precision) {
      out.resize(n * (file_precision == SC_FP32 ? 8 : 16));
      if (file_precision == SC_FP32) {
        const double* s = reinterpret_cast<const double*>(v[c].data());
        float* d = reinterpret_cast<float*>(out.data());
        for (size_t i = 0; i < 2 * n; ++i) d[i] = (float)s[i];
      } else {
        const float* s = reinterpret_cast<const float*>(v[c].data());
        double* d = reinterpret_cast<double*>(out.data());
        for (size_t i = 0; i < 2 * n; ++i) d[i] = (double)s[i];
      }
      src = out.data();
    }
    const long long nb = (long long)n * (file_precision == SC_FP32 ? 8 : 16);
    if (int r = write_record(field_path(dir, names[c], idump).c_str(), src, nb, 0)) return r;
  }
  return SC_OK;
}

int sc_input3d(sc_handle* h, const char* dir, int idump, int file_precision) {
  sc_params p{};
  if (!h || sc_get_params(h, &p) != SC_OK) return sc::set_last_error(SC_ERR_INVALID, "null handle");
  if (file_precision != SC_FP32 && file_precision != SC_FP64)
    return sc::set_last_error(SC_ERR_INVALID, "file precision must be SC_FP32 or SC_FP64");
  const size_t n = (size_t)(p.nx / 2 + 1) * p.ny * p.nz;
  const size_t fbytes = file_precision == SC_FP32 ? 8 : 16, hb = p.precision == SC_FP32 ? 8 : 16;
  const char* names[3] = {"ux", "uy", "uz"};
  std::vector<char> v[3];
  for (int c = 0; c < 3; ++c) {
    std::vector<char> in(n * fbytes);
    if (int r = read_record(field_path(dir, names[c], idump).c_str(), in.data(), (long long)(n * fbytes)))
      return r;
    if (fbytes == hb) {
      v[c].swap(in);
    } else {
      v[c].resize(n * hb);
      if (hb == 8) {
        const double* s = reinterpret_cast<const double*>(in.data());
        float* d = reinterpret_cast<float*>(v[c].data());
        for (size_t i = 0; i < 2 * n; ++i) d[i] = (float)s[i];
      } else {
        const float* s = reinterpret_cast<const float*>(in.data());
        double* d = reinterpret_cast<double*>(v[c].data());
        for (size_t i = 0; i < 2 * n; ++i) d[i] = (double)s[i];
      }
    }
  }
  return sc_set_state(h, v[0].data(), v[1].data(), v[2].data());
}

// outputphi(phi,idump,lx1,ly,lz), outputphi.f90:1-20: <dir>/phi<idump>.dat,
// one record of complex(sp) (nx/2+1, ny, nz).
int sc_outputphi(sc_handle* h, const char* dir, int idump, int file_precision) {
  sc_params p{};
  if (!h || sc_get_params(h, &p) != SC_OK) return sc::set_last_error(SC_ERR_INVALID, "null handle");
  if (file_precision != SC_FP32 && file_precision != SC_FP64)
    return sc::set_last_error(SC_ERR_INVALID, "file precision must be SC_FP32 or SC_FP64");
  const size_t n = (size_t)(p.nx / 2 + 1) * p.ny * p.nz;
  std::vector<char> v(n * (p.precision == SC_FP32 ? 8 : 16));
  if (int r = sc_get_scalar(h, v.data())) return r;
  const std::vector<char> out = convert_values(v, n, p.precision, file_precision);
  return write_record(field_path(dir, "phi", idump).c_str(), out.data(), (long long)out.size(), 0);
}

// inputphi(phi,idump,lx1,ly,lz), inputphi.f90:1-22: loads the scalar as
// sc_set_scalar does.
int sc_inputphi(sc_handle* h, const char* dir, int idump, int file_precision) {
  sc_params p{};
  if (!h || sc_get_params(h, &p) != SC_OK) return sc::set_last_error(SC_ERR_INVALID, "null handle");
  if (file_precision != SC_FP32 && file_precision != SC_FP64)
    return sc::set_last_error(SC_ERR_INVALID, "file precision must be SC_FP32 or SC_FP64");
  const size_t n = (size_t)(p.nx / 2 + 1) * p.ny * p.nz;
  std::vector<char> in(n * (file_precision == SC_FP32 ? 8 : 16));
  if (int r = read_record(field_path(dir, "phi", idump).c_str(), in.data(), (long long)in.size())) return r;
  const std::vector<char> v = convert_values(in, n, file_precision, p.precision);
  return sc_set_scalar(h, v.data());
}

}  // extern "C"
