// The reference's binary and XSF output files, written and read on the host.
//
// Binary files.  The reference (gfortran with -fconvert=big-endian,
// Source/Makefile:86) writes a density, potential or wavefunction with one
// `write(unit) object` statement; the type-bound write(unformatted)
// procedures (Source/density.f90:41,128-160, Source/pot.f90:41,194-224,
// Source/wave.f90:37,893-921) issue child transfers, which add to the parent
// statement's record, so each file is one Fortran sequential record:
//   .den           n_std(3) int32, charge(nr) complex128, spin(nr, 3)
//                  complex128, allocated logical (int32 1)
//   .pot / .potex  n_std(3) int32, nc_pot(nr, 2, 2) complex128, allocated
//   .wvfn          n_std(3) int32, coeff(nbox, nk, nb, nspinor) complex128,
//                  nbands int32, kpts int32, allocated
// with nr the fine-grid points, nbox the standard-grid box, arrays
// column-major, and the grid triple the standard grid, not the fine one
// (current_basis%ngx..ngz).  The potential reader (Source/pot.f90:303-340)
// checks that triple against the run's standard grid.
// A record is framed by 4-byte big-endian length markers.  A record longer
// than gfortran's subrecord limit (2^31 - 9 bytes) is split into
// subrecords: the leading marker of a subrecord that is followed by another
// and the trailing marker of a subrecord that follows another are negated.
//
// XSF (Source/xsf.f90:67-128): CRYSTAL / PRIMVEC with the rows of cell in
// F20.10, a placeholder atom, and the grid values one per line in E20.10,
// in the flat order of the array (z fastest, as the reference writes it).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "derek_gpu.h"

namespace {

long long g_subrecord_limit = 2147483639LL;   // gfortran's default

uint32_t be32(uint32_t v) { return __builtin_bswap32(v); }
uint64_t be64(uint64_t v) { return __builtin_bswap64(v); }

// Sequential-record writer for one record of known total length.
class RecordWriter {
 public:
  RecordWriter(FILE *f, long long total) : f_(f), total_(total) {
    nsub_ = total <= 0 ? 1 : (total + g_subrecord_limit - 1) / g_subrecord_limit;
    start_sub();
  }
  bool ok() const { return ok_; }
  void bytes(const void *p, long long n) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    while (n > 0 && ok_) {
      const long long k = n < left_ ? n : left_;
      if (k > 0 && fwrite(c, 1, (size_t)k, f_) != (size_t)k) ok_ = false;
      c += k;
      n -= k;
      left_ -= k;
      if (left_ == 0 && sub_ + 1 < nsub_) {
        end_sub();
        ++sub_;
        start_sub();
      }
    }
  }
  void i32(int32_t v) {
    const uint32_t b = be32((uint32_t)v);
    bytes(&b, 4);
  }
  // n doubles, each byte-swapped to big-endian
  void f64(const double *p, long long n) {
    std::vector<uint64_t> buf(1 << 16);
    while (n > 0 && ok_) {
      const long long k = n < (long long)buf.size() ? n : (long long)buf.size();
      for (long long i = 0; i < k; ++i) {
        uint64_t u;
        std::memcpy(&u, p + i, 8);
        buf[i] = be64(u);
      }
      bytes(buf.data(), 8 * k);
      p += k;
      n -= k;
    }
  }
  void zeros64(long long n) {
    std::vector<uint64_t> buf(1 << 16, 0);
    while (n > 0 && ok_) {
      const long long k = n < (long long)buf.size() ? n : (long long)buf.size();
      bytes(buf.data(), 8 * k);
      n -= k;
    }
  }
  bool finish() {
    if (ok_ && left_ != 0) ok_ = false;   // the payload must fill the record
    if (ok_) end_sub();
    return ok_;
  }

 private:
  long long sub_len(long long s) const {
    if (total_ <= 0) return 0;
    const long long rest = total_ - s * g_subrecord_limit;
    return rest < g_subrecord_limit ? rest : g_subrecord_limit;
  }
  void marker(long long len, bool negate) {
    const int32_t m = (int32_t)(negate ? -len : len);
    const uint32_t b = be32((uint32_t)m);
    if (fwrite(&b, 1, 4, f_) != 4) ok_ = false;
  }
  void start_sub() {
    left_ = sub_len(sub_);
    marker(left_, sub_ + 1 < nsub_);
  }
  void end_sub() { marker(sub_len(sub_), sub_ > 0); }

  FILE *f_;
  long long total_, nsub_ = 1, sub_ = 0, left_ = 0;
  bool ok_ = true;
};

// Reads one sequential record (all its subrecords) into memory.
bool read_record(FILE *f, std::vector<unsigned char> &out) {
  out.clear();
  bool first = true;
  for (;;) {
    uint32_t b;
    if (fread(&b, 1, 4, f) != 4) return false;
    const int32_t lead = (int32_t)be32(b);
    const long long len = lead < 0 ? -(long long)lead : lead;
    const size_t at = out.size();
    out.resize(at + (size_t)len);
    if (len > 0 && fread(out.data() + at, 1, (size_t)len, f) != (size_t)len) return false;
    if (fread(&b, 1, 4, f) != 4) return false;
    const int32_t trail = (int32_t)be32(b);
    const long long tlen = trail < 0 ? -(long long)trail : trail;
    if (tlen != len || (trail < 0) != !first) return false;
    first = false;
    if (lead >= 0) return true;
  }
}

class RecordReader {
 public:
  explicit RecordReader(const std::vector<unsigned char> &r) : r_(r) {}
  bool i32(int32_t &v) {
    if (pos_ + 4 > r_.size()) return false;
    uint32_t b;
    std::memcpy(&b, r_.data() + pos_, 4);
    v = (int32_t)be32(b);
    pos_ += 4;
    return true;
  }
  bool f64(double *p, long long n) {
    if (pos_ + 8 * (size_t)n > r_.size()) return false;
    for (long long i = 0; i < n; ++i) {
      uint64_t u;
      std::memcpy(&u, r_.data() + pos_ + 8 * i, 8);
      u = be64(u);
      if (p) std::memcpy(p + i, &u, 8);
    }
    pos_ += 8 * (size_t)n;
    return true;
  }
  bool done() const { return pos_ == r_.size(); }

 private:
  const std::vector<unsigned char> &r_;
  size_t pos_ = 0;
};

bool read_grid(RecordReader &rr, const int n_std[3]) {
  for (int i = 0; i < 3; ++i) {
    int32_t g;
    if (!rr.i32(g) || g != n_std[i]) return false;
  }
  return true;
}

bool read_true(RecordReader &rr) {
  int32_t a;
  return rr.i32(a) && a != 0 && rr.done();
}

// E20.10 as gfortran writes it: 0.dddddddddd with an E+ee exponent (a
// three-digit exponent drops the E), right-justified in 20 columns
std::string fortran_e20_10(double x) {
  if (!std::isfinite(x)) return std::string(20, '*');
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.9e", x);   // d.ddddddddde+xx: 10 significant digits
  const char *p = buf;
  std::string sign;
  if (*p == '-') {
    sign = "-";
    ++p;
  }
  std::string digits;
  for (; *p && *p != 'e'; ++p)
    if (*p != '.') digits += *p;
  int e = std::atoi(p + 1);
  const bool zero = digits.find_first_not_of('0') == std::string::npos;
  if (!zero) ++e;   // 0.d1d2... scale
  else e = 0;
  char ex[16];
  if (std::abs(e) <= 99)
    std::snprintf(ex, sizeof ex, "E%c%02d", e < 0 ? '-' : '+', std::abs(e));
  else
    std::snprintf(ex, sizeof ex, "%c%03d", e < 0 ? '-' : '+', std::abs(e));
  std::string s = sign + "0." + digits + ex;
  if (s.size() < 20) s = std::string(20 - s.size(), ' ') + s;
  return s;
}

std::string fortran_f20_10(double x) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%20.10f", x);
  std::string s = buf;
  return s.size() > 20 ? std::string(20, '*') : s;
}

// Fw.d as gfortran writes it: right-justified, w asterisks when the number
// does not fit, NaN and Infinity spelled out.
std::string fortran_f(double x, int w, int d) {
  std::string s;
  if (std::isnan(x)) {
    s = "NaN";
  } else if (std::isinf(x)) {
    s = x > 0 ? "Infinity" : "-Infinity";
    if ((int)s.size() > w) s = x > 0 ? "Inf" : "-Inf";
  } else {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%*.*f", w, d, x);
    s = buf;
  }
  if ((int)s.size() > w) return std::string(w, '*');
  return std::string(w - s.size(), ' ') + s;
}

// The formatted grid tables of density_writef (Source/density.f90:165-211)
// and pot_writef (Source/pot.f90:228-287): the fine-grid size block, column
// titles, a rule, then one row per point, x outermost.  Records as gfortran
// writes them: list-directed lines start with one blank, trailing X editing
// writes nothing.  The reference's io_out_file_header banner (a logo and
// the write time) is replaced by this library's own comment lines.
void table_head(FILE *f, const char *kind, const int n_fine[3]) {
  std::fprintf(f, " # DEReK-GB300 %s FILE\n # values in atomic units\n", kind);
  std::fprintf(f, "  FFT FINE BASIS GRID  \n");
  const char *ax[3] = {"nx:", "ny:", "nz:"};
  for (int i = 0; i < 3; ++i) std::fprintf(f, "  %s %6d\n", ax[i], n_fine[i]);
  std::fprintf(f, "\n");
}

}  // namespace

extern "C" {

int derek_io_set_subrecord_limit(long long bytes) {
  if (bytes < 0 || bytes > 2147483639LL) return DEREK_ERR_BAD_ARG;
  g_subrecord_limit = bytes == 0 ? 2147483639LL : bytes;
  return DEREK_OK;
}

int derek_io_write_den(const char *path, const int n_std[3], long long nr, const double *charge,
                       const double *spin) {
  if (!path || !n_std || nr <= 0 || !charge) return DEREK_ERR_BAD_ARG;
  FILE *f = std::fopen(path, "wb");
  if (!f) return DEREK_ERR_BAD_ARG;
  const long long total = 12 + 16 * nr + 16 * 3 * nr + 4;
  RecordWriter w(f, total);
  for (int i = 0; i < 3; ++i) w.i32(n_std[i]);
  w.f64(charge, 2 * nr);
  if (spin)
    w.f64(spin, 2 * 3 * nr);
  else
    w.zeros64(2 * 3 * nr);
  w.i32(1);
  const bool ok = w.finish();
  return std::fclose(f) == 0 && ok ? DEREK_OK : DEREK_ERR_BAD_ARG;
}

int derek_io_read_den(const char *path, const int n_std[3], long long nr, double *charge, double *spin) {
  if (!path || !n_std || nr <= 0) return DEREK_ERR_BAD_ARG;
  FILE *f = std::fopen(path, "rb");
  if (!f) return DEREK_ERR_BAD_ARG;
  std::vector<unsigned char> rec;
  const bool got = read_record(f, rec);
  std::fclose(f);
  if (!got || (long long)rec.size() != 12 + 64 * nr + 4) return DEREK_ERR_BAD_ARG;
  RecordReader rr(rec);
  if (!read_grid(rr, n_std) || !rr.f64(charge, 2 * nr) || !rr.f64(spin, 2 * 3 * nr) || !read_true(rr))
    return DEREK_ERR_BAD_ARG;
  return DEREK_OK;
}

int derek_io_write_pot(const char *path, const int n_std[3], long long nr, const double *nc_pot) {
  if (!path || !n_std || nr <= 0 || !nc_pot) return DEREK_ERR_BAD_ARG;
  FILE *f = std::fopen(path, "wb");
  if (!f) return DEREK_ERR_BAD_ARG;
  RecordWriter w(f, 12 + 64 * nr + 4);
  for (int i = 0; i < 3; ++i) w.i32(n_std[i]);
  w.f64(nc_pot, 8 * nr);
  w.i32(1);
  const bool ok = w.finish();
  return std::fclose(f) == 0 && ok ? DEREK_OK : DEREK_ERR_BAD_ARG;
}

int derek_io_read_pot(const char *path, const int n_std[3], long long nr, double *nc_pot) {
  if (!path || !n_std || nr <= 0) return DEREK_ERR_BAD_ARG;
  FILE *f = std::fopen(path, "rb");
  if (!f) return DEREK_ERR_BAD_ARG;
  std::vector<unsigned char> rec;
  const bool got = read_record(f, rec);
  std::fclose(f);
  if (!got || (long long)rec.size() != 12 + 64 * nr + 4) return DEREK_ERR_BAD_ARG;
  RecordReader rr(rec);
  if (!read_grid(rr, n_std) || !rr.f64(nc_pot, 8 * nr) || !read_true(rr)) return DEREK_ERR_BAD_ARG;
  return DEREK_OK;
}

int derek_io_write_wvfn(const char *path, const int n_std[3], long long nbox, int nk, int nb, int nspinor,
                        const double *coeff) {
  if (!path || !n_std || nbox <= 0 || nk <= 0 || nb <= 0 || nspinor <= 0 || !coeff) return DEREK_ERR_BAD_ARG;
  FILE *f = std::fopen(path, "wb");
  if (!f) return DEREK_ERR_BAD_ARG;
  const long long n = nbox * nk * nb * nspinor;
  RecordWriter w(f, 12 + 16 * n + 12);
  for (int i = 0; i < 3; ++i) w.i32(n_std[i]);
  w.f64(coeff, 2 * n);
  w.i32(nb);
  w.i32(nk);
  w.i32(1);
  const bool ok = w.finish();
  return std::fclose(f) == 0 && ok ? DEREK_OK : DEREK_ERR_BAD_ARG;
}

int derek_io_read_wvfn(const char *path, const int n_std[3], long long nbox, int nk, int nb, int nspinor,
                       double *coeff) {
  if (!path || !n_std || nbox <= 0 || nk <= 0 || nb <= 0 || nspinor <= 0) return DEREK_ERR_BAD_ARG;
  FILE *f = std::fopen(path, "rb");
  if (!f) return DEREK_ERR_BAD_ARG;
  std::vector<unsigned char> rec;
  const bool got = read_record(f, rec);
  std::fclose(f);
  const long long n = nbox * nk * nb * nspinor;
  if (!got || (long long)rec.size() != 12 + 16 * n + 12) return DEREK_ERR_BAD_ARG;
  RecordReader rr(rec);
  int32_t rb = 0, rk = 0;
  if (!read_grid(rr, n_std) || !rr.f64(coeff, 2 * n) || !rr.i32(rb) || !rr.i32(rk) || rb != nb || rk != nk ||
      !read_true(rr))
    return DEREK_ERR_BAD_ARG;
  return DEREK_OK;
}

int derek_io_write_fden(const char *path, const int n_fine[3], const double *charge, const double *spin) {
  if (!path || !n_fine || !charge || n_fine[0] <= 0 || n_fine[1] <= 0 || n_fine[2] <= 0) return DEREK_ERR_BAD_ARG;
  FILE *f = std::fopen(path, "w");
  if (!f) return DEREK_ERR_BAD_ARG;
  table_head(f, "DENSITY", n_fine);
  // format(1x,3(a4,2x),5x,4(3x,A6,1x)) and format(1x,3(i4,2x),5x,4(f9.4,2x))
  std::fprintf(f, " %4s  %4s  %4s       %9s    %6s    %6s    %6s\n", "ix", "iy", "iz", "Charge", "Sx", "Sy", "Sz");
  std::fprintf(f, " %s\n", std::string(65, '-').c_str());
  const long long nr = (long long)n_fine[0] * n_fine[1] * n_fine[2];
  long long n = 0;
  for (int ix = 1; ix <= n_fine[0]; ++ix)
    for (int iy = 1; iy <= n_fine[1]; ++iy)
      for (int iz = 1; iz <= n_fine[2]; ++iz, ++n) {
        std::fprintf(f, " %4d  %4d  %4d       %s", ix, iy, iz, fortran_f(charge[n], 9, 4).c_str());
        for (int c = 0; c < 3; ++c)
          std::fprintf(f, "  %s", fortran_f(spin ? spin[c * nr + n] : 0.0, 9, 4).c_str());
        std::fprintf(f, "\n");
      }
  return std::fclose(f) == 0 ? DEREK_OK : DEREK_ERR_BAD_ARG;
}

int derek_io_write_fpot(const char *path, const int n_fine[3], const double *nc_pot) {
  if (!path || !n_fine || !nc_pot || n_fine[0] <= 0 || n_fine[1] <= 0 || n_fine[2] <= 0) return DEREK_ERR_BAD_ARG;
  FILE *f = std::fopen(path, "w");
  if (!f) return DEREK_ERR_BAD_ARG;
  table_head(f, "POTENTIAL", n_fine);
  // format(1x,3(a4,2x),5x,4(9x,A5,6x,4x)) and format(1x,3(i4,2x),5x,4(f9.4,2x,f9.4,4x));
  // columns (1,1), (1,2), (2,1), (2,2) of nc_pot(n, i, j) at n + nr (i + 2 j)
  std::fprintf(f, " %4s  %4s  %4s       ", "ix", "iy", "iz");
  const char *heads[4] = {"(1,1)", "(1,2)", "(2,1)", "(2,2)"};
  for (int c = 0; c < 4; ++c) std::fprintf(f, "%s%14s", c ? "          " : "", heads[c]);
  std::fprintf(f, "\n %s\n", std::string(115, '-').c_str());
  const long long nr = (long long)n_fine[0] * n_fine[1] * n_fine[2];
  const int comp[4] = {0, 2, 1, 3};   // (1,1), (1,2), (2,1), (2,2) as i + 2 j
  long long n = 0;
  for (int ix = 1; ix <= n_fine[0]; ++ix)
    for (int iy = 1; iy <= n_fine[1]; ++iy)
      for (int iz = 1; iz <= n_fine[2]; ++iz, ++n) {
        std::fprintf(f, " %4d  %4d  %4d       ", ix, iy, iz);
        for (int c = 0; c < 4; ++c) {
          const double *z = nc_pot + 2 * (comp[c] * nr + n);
          std::fprintf(f, "%s%s  %s", c ? "    " : "", fortran_f(z[0], 9, 4).c_str(), fortran_f(z[1], 9, 4).c_str());
        }
        std::fprintf(f, "\n");
      }
  return std::fclose(f) == 0 ? DEREK_OK : DEREK_ERR_BAD_ARG;
}

int derek_io_write_xsf(const char *path, const double cell[9], const int n_fine[3], const double *data) {
  if (!path || !cell || !n_fine || !data) return DEREK_ERR_BAD_ARG;
  FILE *f = std::fopen(path, "w");
  if (!f) return DEREK_ERR_BAD_ARG;
  auto cell_rows = [&]() {
    for (int i = 0; i < 3; ++i)   // cell(i, 1:3), cell column-major
      std::fprintf(f, "%s%s%s\n", fortran_f20_10(cell[i]).c_str(), fortran_f20_10(cell[i + 3]).c_str(),
                   fortran_f20_10(cell[i + 6]).c_str());
  };
  const std::string zero3 = fortran_f20_10(0.0) + fortran_f20_10(0.0) + fortran_f20_10(0.0);
  std::fprintf(f, "CRYSTAL\nPRIMVEC\n");
  cell_rows();
  std::fprintf(f, "PRIMCOORD\n%5d%5d\n%s\n", 1, 1, zero3.c_str());
  std::fprintf(f, "BEGIN_BLOCK_DATAGRID_3D\nDATAGRID_3D_UNKNOWN\nBEGIN_DATAGRID_3D\n");
  std::fprintf(f, "%5d%5d%5d\n%s\n", n_fine[0], n_fine[1], n_fine[2], zero3.c_str());
  cell_rows();
  const long long nr = (long long)n_fine[0] * n_fine[1] * n_fine[2];
  for (long long i = 0; i < nr; ++i) std::fprintf(f, "%s\n", fortran_e20_10(data[i]).c_str());
  std::fprintf(f, "END_DATAGRID_3D\nEND_BLOCK_DATAGRID_3D\n");
  return std::fclose(f) == 0 ? DEREK_OK : DEREK_ERR_BAD_ARG;
}

}  // extern "C"
