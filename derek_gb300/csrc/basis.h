// Host-side basis construction: FFT grid sizes, plane-wave spheres, FFT radix
// plans, twiddle tables and the external potential.
#pragma once

#include <cstdint>
#include <vector>

namespace derek {

// Source/basis.f90:257-309 (basis_prime_fact): smallest m >= n that is
// {2,3,5,7,11,13}-smooth, searching at most 100 increments.
int prime_fact_round(int n);
// Smallest m >= n that is {2,3}-smooth.
int smooth23_round(int n);

// Column norms of the column-major cell (Source/io.f90:1956-1966).
void lattice_lengths(const double cell[9], double len[3]);
// transpose(2 pi cell^-1) in the same column-major storage (Source/io.f90:1954).
void inverse_cell(const double cell[9], double inv[9]);
double cell_volume(const double cell[9]);

// Standard and fine grid sizes (Source/basis.f90:87-105); policy 0 rounds with
// basis_prime_fact, 1 to {2,3}-smooth sizes.  The standard box always uses
// the reference rule because it defines the G list.
void grid_sizes(const double cell[9], double ecut, double g_fine_scale, int policy,
                int n_std[3], int n_fine[3]);

// Plane-wave sphere of one k-point: ordered subsequence of the centred
// standard-box list (Source/basis.f90:125-135, x outer, z inner) with
// 1/2|k+G|^2 <= ecut.  G = inv_cell . (m + k) evaluated row by row in the
// order of Fortran's matmul without fused multiply-adds.
struct Sphere {
  std::vector<int32_t> box_row;   // 0-based row in the standard-box list
  std::vector<int32_t> mx, my, mz;
  std::vector<double> kinetic;    // 1/2 |k+G|^2
};
void build_sphere(const double inv_cell_cm[9], double ecut, const double kfrac[3],
                  const int n_std[3], Sphere &out);

// Radix factorisation of n for the Stockham kernels (radices 8,4,2,3,5,7,11,13).
// Returns false if n has another prime factor.
bool radix_plan(int n, int radices[8], int *nstages);

// Split n = a * b with a, b <= 16 for the four-step line kernels: the
// smallest max(a, b), ties broken toward a power-of-two a.
bool line_plan(int n, int *a, int *b);

// exp(-2 pi i t / n), t = 0..n-1, interleaved (re, im).
void twiddles(int n, std::vector<double> &out);

// Jellium constant 0.5 Ne / N (Source/pot.f90:133-134) minus Gaussian wells
// depth*exp(-|r-R|^2/(2 w^2)) with minimum-image distances, sampled at the
// reference's real grid frac = i/n, i = 1..n (Source/basis.f90:156-188).
void build_vext(const double cell_cm[9], const int n[3], double nelec, int nwells,
                const double *wells, std::vector<double> &v);

}  // namespace derek
