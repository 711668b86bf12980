// Restart files of the reference, host side (no device code).
//
//  * Fortran sequential unformatted records as gfortran writes them: every
//    record is framed by 4-byte little-endian length markers before and after
//    its payload.  A record longer than kSubMax bytes is split into
//    subrecords; the leading marker of a subrecord is negated when another
//    subrecord of the same record follows, the trailing marker is negated
//    when one precedes it.
//  * vel.out  (io.f90:1212-1217, read initial.f90:226-239): one record of the
//    11 fields u, v, w, RHSx, RHSy, RHSz, Cs_opt2, F_LM, F_MM, F_QN, F_NN,
//    each (ld, ny, 1:nz) in FP64.
//  * grid.out (io.f90:1220-1224): one record nproc, Nx, Ny, Nz (int32) and
//    L_x, L_y, L_z (FP64).
//  * total_time.dat (io.f90:1260-1264, read io.f90:73-96): list-directed text
//    "jt_total total_time total_time_dim dt cfl".
//  * tavg.out (time_average.f90:665-716, read :114-150): total_time, then the
//    25 sums u .. vortz (no pressure), each (nx, ny, 1:nz).
//  * ic_interp (initial.f90:242-380): trilinear regrid of u, v, w from a
//    checkpoint of another grid.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace lesgo {
namespace fio {

constexpr int64_t kSubMax = 2147483639;   // gfortran's largest subrecord

struct IoError {
  std::string msg;
};

static void put_i32(FILE* f, int32_t v) {
  unsigned char b[4];
  for (int i = 0; i < 4; ++i) b[i] = (unsigned char)(((uint32_t)v >> (8 * i)) & 0xFF);
  if (std::fwrite(b, 1, 4, f) != 4) throw IoError{"write failed"};
}
static bool get_i32(FILE* f, int32_t* v) {
  unsigned char b[4];
  if (std::fread(b, 1, 4, f) != 4) return false;
  uint32_t u = 0;
  for (int i = 0; i < 4; ++i) u |= (uint32_t)b[i] << (8 * i);
  std::memcpy(v, &u, 4);
  return true;
}

// One record made of several contiguous byte ranges.
struct Part {
  const void* p;
  int64_t n;
};

static void write_record(FILE* f, const std::vector<Part>& parts) {
  int64_t total = 0;
  for (const Part& q : parts) total += q.n;
  size_t pi = 0;
  int64_t off = 0, left = total;
  bool first = true;
  do {
    const int64_t len = left > kSubMax ? kSubMax : left;
    const bool more = left > len;
    put_i32(f, (int32_t)(more ? -len : len));
    int64_t need = len;
    while (need > 0) {
      const int64_t avail = parts[pi].n - off;
      const int64_t take = avail < need ? avail : need;
      if (take > 0 && std::fwrite((const char*)parts[pi].p + off, 1, (size_t)take, f) != (size_t)take)
        throw IoError{"write failed"};
      off += take;
      need -= take;
      if (off == parts[pi].n) { ++pi; off = 0; }
    }
    put_i32(f, (int32_t)(first ? len : -len));
    first = false;
    left -= len;
  } while (left > 0);
}

// Bytes from the current position to the end of the file.
static int64_t bytes_left(FILE* f) {
  const long at = std::ftell(f);
  if (at < 0 || std::fseek(f, 0, SEEK_END) != 0) return INT64_MAX;
  const long end = std::ftell(f);
  std::fseek(f, at, SEEK_SET);
  return end < at ? 0 : (int64_t)(end - at);
}

static int32_t bswap32(int32_t v) {
  const uint32_t u = (uint32_t)v;
  return (int32_t)((u >> 24) | ((u >> 8) & 0xFF00u) | ((u << 8) & 0xFF0000u) | (u << 24));
}

// Read the next record; false at end of file.  A record whose length marker
// only makes sense byte-swapped was written big-endian (the reference's
// WRITE_ENDIAN=BIG build, convert='BIG_ENDIAN'): it is rejected by name
// rather than read as a huge length.
static bool read_record(FILE* f, std::vector<char>& out) {
  out.clear();
  bool first = true;
  for (;;) {
    int32_t lead;
    if (!get_i32(f, &lead)) {
      if (first) return false;
      throw IoError{"truncated record"};
    }
    const int64_t len = lead < 0 ? -(int64_t)lead : lead;
    const int64_t left = bytes_left(f);
    if (len + 4 > left) {
      const int32_t sw = bswap32(lead);
      const int64_t slen = sw < 0 ? -(int64_t)sw : sw;
      if (slen + 4 <= left) throw IoError{"big-endian checkpoint (WRITE_ENDIAN=BIG) not supported"};
      throw IoError{"truncated record"};
    }
    const size_t at = out.size();
    out.resize(at + (size_t)len);
    if (len > 0 && std::fread(out.data() + at, 1, (size_t)len, f) != (size_t)len) throw IoError{"truncated record"};
    int32_t trail;
    if (!get_i32(f, &trail)) throw IoError{"truncated record"};
    const int64_t tl = trail < 0 ? -(int64_t)trail : trail;
    if (tl != len || (trail < 0) == first) throw IoError{"bad record marker"};
    first = false;
    if (lead >= 0) return true;
  }
}

struct File {
  FILE* f = nullptr;
  File(const std::string& path, const char* mode) : f(std::fopen(path.c_str(), mode)) {}
  ~File() { if (f) std::fclose(f); }
  File(const File&) = delete;
  File& operator=(const File&) = delete;
};

static bool exists(const std::string& path) {
  File fl(path, "rb");
  return fl.f != nullptr;
}

struct GridOut {
  int32_t nproc, nx, ny, nz;
  double Lx, Ly, Lz;
};

static void write_grid(const std::string& path, const GridOut& g) {
  File fl(path, "wb");
  if (!fl.f) throw IoError{"cannot open " + path};
  int32_t iv[4] = {g.nproc, g.nx, g.ny, g.nz};
  double dv[3] = {g.Lx, g.Ly, g.Lz};
  write_record(fl.f, {{iv, 16}, {dv, 24}});
}

static GridOut read_grid(const std::string& path) {
  File fl(path, "rb");
  if (!fl.f) throw IoError{"cannot open " + path};
  std::vector<char> r;
  if (!read_record(fl.f, r) || r.size() != 40) throw IoError{path + ": not a grid.out record"};
  GridOut g;
  int32_t iv[4];
  std::memcpy(iv, r.data(), 16);
  std::memcpy(&g.Lx, r.data() + 16, 8);
  std::memcpy(&g.Ly, r.data() + 24, 8);
  std::memcpy(&g.Lz, r.data() + 32, 8);
  g.nproc = iv[0]; g.nx = iv[1]; g.ny = iv[2]; g.nz = iv[3];
  return g;
}

struct TimeDat {
  long long jt_total;
  double total_time, total_time_dim, dt, cfl;
};

static void write_time(const std::string& path, const TimeDat& t) {
  File fl(path, "w");
  if (!fl.f) throw IoError{"cannot open " + path};
  std::fprintf(fl.f, " %12lld %24.17E %24.17E %24.17E %24.17E\n", t.jt_total, t.total_time, t.total_time_dim, t.dt,
               t.cfl);
}

// List-directed read of five values (blanks, commas or newlines between).
static TimeDat read_time(const std::string& path) {
  File fl(path, "r");
  if (!fl.f) throw IoError{"cannot open " + path};
  std::string s;
  char buf[512];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, fl.f)) > 0) s.append(buf, n);
  for (char& c : s)
    if (c == ',' || c == '\n' || c == '\r' || c == '\t') c = ' ';
  // Fortran exponents may be written with D
  for (char& c : s)
    if (c == 'D' || c == 'd') c = 'E';
  TimeDat t{};
  const char* p = s.c_str();
  char* end;
  t.jt_total = std::strtoll(p, &end, 10);
  if (end == p) throw IoError{path + ": no jt_total"};
  double* dst[4] = {&t.total_time, &t.total_time_dim, &t.dt, &t.cfl};
  for (double* d : dst) {
    p = end;
    *d = std::strtod(p, &end);
    if (end == p) throw IoError{path + ": expected 5 values"};
  }
  return t;
}

// functions.f90:811-860: index of the interval holding val (1-based), 0 below
// the first node, N above the last.
static int binary_search(const std::vector<double>& a, double val) {
  const int N = (int)a.size();
  if (val < a[0]) return 0;
  if (val > a[N - 1]) return N;
  int low = 1, high = N;
  while (high - low > 1) {
    const int mid = (low + high) / 2;
    if (a[mid - 1] > val) high = mid;
    else if (a[mid - 1] < val) low = mid;
    else return mid;
  }
  return low;
}

// initial.f90:242-380 for one file grid (ld_f, ny_f, 1:nz_f) onto (ld, ny,
// 1:nz): bilinear in x-y with periodic wrap, linear in z between file levels,
// nearest file level above or below the file's range.  uv fields on
// z = (k - 1/2) dz, w on zw = (k - 1) dz.
struct Regrid {
  int nx_f, ny_f, nz_f, ld_f;
  double Lx_f, Ly_f, Lz_f;
  int nx, ny, nz, ld;
  double dx, dy, dz;

  void apply(const double* uf, const double* vf, const double* wf, double* u, double* v, double* w) const {
    const double dx_f = Lx_f / nx_f, dy_f = Ly_f / ny_f, dz_f = Lz_f / (nz_f - 1);
    std::vector<double> x_f(nx_f), y_f(ny_f), z_r(nz_f), zw_r(nz_f);
    for (int i = 0; i < nx_f; ++i) x_f[i] = i * Lx_f / nx_f;
    for (int j = 0; j < ny_f; ++j) y_f[j] = j * Ly_f / ny_f;
    for (int k = 0; k < nz_f; ++k) { zw_r[k] = k * dz_f; z_r[k] = zw_r[k] + 0.5 * dz_f; }
    const long long pf = (long long)ld_f * ny_f, pl = (long long)ld * ny;
    auto F = [&](const double* a, int i, int j, int k) { return a[(k - 1) * pf + (long long)(j - 1) * ld_f + (i - 1)]; };
    for (int i = 1; i <= nx; ++i) {
      const double xg = (i - 1) * dx;
      const double xx = xg - std::floor(xg / Lx_f) * Lx_f;
      const int i1 = binary_search(x_f, xx), i2 = i1 % nx_f + 1;
      const double bx = (xx - x_f[i1 - 1]) / dx_f, ax = 1.0 - bx;
      for (int j = 1; j <= ny; ++j) {
        const double yg = (j - 1) * dy;
        const double yy = yg - std::floor(yg / Ly_f) * Ly_f;
        const int j1 = binary_search(y_f, yy), j2 = j1 % ny_f + 1;
        const double by = (yy - y_f[j1 - 1]) / dy_f, ay = 1.0 - by;
        for (int k = 1; k <= nz; ++k) {
          const long long q = (k - 1) * pl + (long long)(j - 1) * ld + (i - 1);
          auto plane = [&](const double* a, int kk) {
            return ax * ay * F(a, i1, j1, kk) + bx * ay * F(a, i2, j1, kk) + ax * by * F(a, i1, j2, kk) +
                   bx * by * F(a, i2, j2, kk);
          };
          auto vol = [&](const double* a, int k1, double az, double bz) {
            return ax * ay * az * F(a, i1, j1, k1) + bx * ay * az * F(a, i2, j1, k1) +
                   ax * by * az * F(a, i1, j2, k1) + bx * by * az * F(a, i2, j2, k1) +
                   ax * ay * bz * F(a, i1, j1, k1 + 1) + bx * ay * bz * F(a, i2, j1, k1 + 1) +
                   ax * by * bz * F(a, i1, j2, k1 + 1) + bx * by * bz * F(a, i2, j2, k1 + 1);
          };
          const double z = (k - 0.5) * dz;
          int k1 = binary_search(z_r, z);
          if (k1 == nz_f) { u[q] = plane(uf, k1); v[q] = plane(vf, k1); }
          else if (k1 == 0) { u[q] = plane(uf, 1); v[q] = plane(vf, 1); }
          else {
            const double bz = (z - z_r[k1 - 1]) / dz_f, az = 1.0 - bz;
            u[q] = vol(uf, k1, az, bz);
            v[q] = vol(vf, k1, az, bz);
          }
          const double zw = (k - 1) * dz;
          k1 = binary_search(zw_r, zw);
          if (k1 == nz_f) w[q] = plane(wf, k1);
          else if (k1 == 0) w[q] = plane(wf, 1);
          else {
            const double bz = (zw - zw_r[k1 - 1]) / dz_f, az = 1.0 - bz;
            w[q] = vol(wf, k1, az, bz);
          }
        }
      }
    }
  }
};

}  // namespace fio
}  // namespace lesgo
