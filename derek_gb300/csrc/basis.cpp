// Host-side basis construction.  Compiled without floating-point contraction
// so that sphere membership is decided by the same roundings as a plain
// left-to-right evaluation of the reference's formulas.
#include "basis.h"

#include <cmath>

namespace derek {

static int smooth_round(int n, const int *primes, int np, int max_cycles) {
  for (int cycle = 0; cycle < max_cycles; ++cycle) {
    int m = n;
    bool changed = true;
    while (changed) {
      changed = false;
      for (int i = 0; i < np; ++i) {
        if (m % primes[i] == 0) {
          m /= primes[i];
          changed = true;
        }
      }
    }
    if (m == 1) return n;
    ++n;
  }
  return n;
}

int prime_fact_round(int n) {
  static const int primes[6] = {2, 3, 5, 7, 11, 13};
  return smooth_round(n, primes, 6, 100);
}

int smooth23_round(int n) {
  static const int primes[2] = {2, 3};
  return smooth_round(n, primes, 2, 1 << 20);
}

void lattice_lengths(const double c[9], double len[3]) {
  for (int j = 0; j < 3; ++j)
    len[j] = std::sqrt(c[3 * j] * c[3 * j] + c[3 * j + 1] * c[3 * j + 1] + c[3 * j + 2] * c[3 * j + 2]);
}

double cell_volume(const double c[9]) {
  // det of the matrix whose (i,j) entry is c[3*j+i]
  auto a = [&](int i, int j) { return c[3 * j + i]; };
  double d = a(0, 0) * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1)) -
             a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
             a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
  return std::fabs(d);
}

void inverse_cell(const double c[9], double inv[9]) {
  auto a = [&](int i, int j) { return c[3 * j + i]; };
  double det = a(0, 0) * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1)) -
               a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
               a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
  double m[3][3];  // cell^-1
  m[0][0] = (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1)) / det;
  m[0][1] = (a(0, 2) * a(2, 1) - a(0, 1) * a(2, 2)) / det;
  m[0][2] = (a(0, 1) * a(1, 2) - a(0, 2) * a(1, 1)) / det;
  m[1][0] = (a(1, 2) * a(2, 0) - a(1, 0) * a(2, 2)) / det;
  m[1][1] = (a(0, 0) * a(2, 2) - a(0, 2) * a(2, 0)) / det;
  m[1][2] = (a(0, 2) * a(1, 0) - a(0, 0) * a(1, 2)) / det;
  m[2][0] = (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0)) / det;
  m[2][1] = (a(0, 1) * a(2, 0) - a(0, 0) * a(2, 1)) / det;
  m[2][2] = (a(0, 0) * a(1, 1) - a(0, 1) * a(1, 0)) / det;
  const double two_pi = 6.283185307179586476925286766559;
  // inv_cell(i,j) = 2 pi * m[j][i]; column-major storage inv[3*j+i]
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) inv[3 * j + i] = two_pi * m[j][i];
}

void grid_sizes(const double cell[9], double ecut, double g_fine_scale, int policy,
                int n_std[3], int n_fine[3]) {
  const double pi = 3.141592653589793238462643383279502884;
  double len[3];
  lattice_lengths(cell, len);
  const double k_cut = std::sqrt(2.0 * ecut);
  for (int d = 0; d < 3; ++d) {
    n_std[d] = prime_fact_round((int)std::ceil(k_cut * len[d] / pi));
    int f = (int)std::ceil(g_fine_scale * k_cut * len[d] / pi);
    n_fine[d] = policy == 0 ? prime_fact_round(f) : smooth23_round(f);
  }
}

void build_sphere(const double inv[9], double ecut, const double k[3], const int n_std[3],
                  Sphere &out) {
  out = Sphere();
  int row = 0;
  const int lo0 = -(n_std[0] / 2), hi0 = n_std[0] - n_std[0] / 2 - 1;
  const int lo1 = -(n_std[1] / 2), hi1 = n_std[1] - n_std[1] / 2 - 1;
  const int lo2 = -(n_std[2] / 2), hi2 = n_std[2] - n_std[2] / 2 - 1;
  for (int mx = lo0; mx <= hi0; ++mx)
    for (int my = lo1; my <= hi1; ++my)
      for (int mz = lo2; mz <= hi2; ++mz, ++row) {
        const double q0 = (double)mx + k[0], q1 = (double)my + k[1], q2 = (double)mz + k[2];
        double g[3];
        for (int i = 0; i < 3; ++i) {
          double t = inv[i] * q0;       // inv_cell(i,1)
          t = t + inv[3 + i] * q1;      // inv_cell(i,2)
          t = t + inv[6 + i] * q2;      // inv_cell(i,3)
          g[i] = t;
        }
        double g2 = g[0] * g[0];
        g2 = g2 + g[1] * g[1];
        g2 = g2 + g[2] * g[2];
        const double kin = 0.5 * g2;
        if (kin <= ecut) {
          out.box_row.push_back(row);
          out.mx.push_back(mx);
          out.my.push_back(my);
          out.mz.push_back(mz);
          out.kinetic.push_back(kin);
        }
      }
}

bool radix_plan(int n, int radices[8], int *nstages) {
  int ns = 0;
  int m = n;
  static const int order[] = {8, 4, 2, 3, 5, 7, 11, 13};
  for (int r : order) {
    while (m % r == 0 && ns < 8) {
      // prefer radix 8/4 only while the remaining power of two allows it
      radices[ns++] = r;
      m /= r;
    }
  }
  *nstages = ns;
  return m == 1 && ns <= 8;
}

bool line_plan(int n, int *a, int *b) {
  int best_a = 0, best_span = 1 << 30, best_pow2 = 0;
  for (int x = 1; x <= 16; ++x) {
    if (n % x) continue;
    const int y = n / x;
    if (y > 16) continue;
    const int span = x > y ? x : y;
    const int pow2 = (x & (x - 1)) == 0 && x > 1;
    if (span < best_span || (span == best_span && pow2 > best_pow2)) {
      best_a = x;
      best_span = span;
      best_pow2 = pow2;
    }
  }
  if (!best_a) return false;
  *a = best_a;
  *b = n / best_a;
  return true;
}

void twiddles(int n, std::vector<double> &out) {
  out.resize(2 * (size_t)n);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int t = 0; t < n; ++t) {
    long double ang = -two_pi * (long double)t / (long double)n;
    out[2 * t] = (double)cosl(ang);
    out[2 * t + 1] = (double)sinl(ang);
  }
}

void build_vext(const double c[9], const int n[3], double nelec, int nwells, const double *wells,
                std::vector<double> &v) {
  const long nr = (long)n[0] * n[1] * n[2];
  v.assign(nr, 0.5 * nelec / (double)nr);
  for (int w = 0; w < nwells; ++w) {
    const double cx = wells[5 * w], cy = wells[5 * w + 1], cz = wells[5 * w + 2];
    const double depth = wells[5 * w + 3], width = wells[5 * w + 4];
    const double inv2w2 = 1.0 / (2.0 * width * width);
    for (int ix = 0; ix < n[0]; ++ix) {
      double dx = (double)(ix + 1) / n[0] - cx;
      dx -= std::nearbyint(dx);
      for (int iy = 0; iy < n[1]; ++iy) {
        double dy = (double)(iy + 1) / n[1] - cy;
        dy -= std::nearbyint(dy);
        for (int iz = 0; iz < n[2]; ++iz) {
          double dz = (double)(iz + 1) / n[2] - cz;
          dz -= std::nearbyint(dz);
          double r2 = 0.0;
          for (int i = 0; i < 3; ++i) {
            double ri = c[i] * dx + c[3 + i] * dy + c[6 + i] * dz;
            r2 += ri * ri;
          }
          v[((long)ix * n[1] + iy) * n[2] + iz] -= depth * std::exp(-r2 * inv2w2);
        }
      }
    }
  }
}

}  // namespace derek
