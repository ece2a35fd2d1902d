// Host-side construction of the spectral-transform tables (Gaussian grid, associated Legendre functions,
// FFT twiddles) and a host restatement of the scalar synthesis used by the seeded initialisers.
#pragma once
#include <complex>
#include <vector>

#include "lmw_internal.h"

namespace lmw {

using cplx = std::complex<double>;

// cpp/sphere.cpp:47-64, same arithmetic (bitwise identical nodes and weights)
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w);
// cpp/sphere.cpp:66-73, same arithmetic; out has nmax + 2 - m entries
void legendre_column(int m, int nmax, double mu, std::vector<double> &out);
// the recurrence coefficient of cpp/sphere.cpp:11
double legendre_eps(int n, int m);
// cpp/sphere.cpp:21-45 (radix-2, sign -1 forward, unnormalised)
void fft_host(std::vector<cplx> &a, int sign);

// Host tables in the engine's layouts. tri(m) = offset of wavenumber m in the packed triangle.
struct HostTables {
  int N = 0, M = 0, nlat = 0, nlon = 0, nh = 0, ntri = 0;
  std::vector<double> mu, w;
  std::vector<int> tri;
  // southern-half tables (latitudes jh = 0 .. nh-1), coefficient-major [tri][jh]
  std::vector<double> P, H;
  void build(int truncation);
  double Pj(int j, int m, int n) const;  // any latitude, through the hemispheric symmetry
  double Hj(int j, int m, int n) const;
  // scalar synthesis of a spectrum in the reference layout ((T+1)^2, index m*(T+1)+n) onto the grid
  void synthesize(const std::vector<cplx> &spec, std::vector<double> &grid) const;
  // U = u cos(lat), V = v cos(lat) from vorticity and divergence (cpp/sphere.cpp:179-206)
  void winds(const std::vector<cplx> &z, const std::vector<cplx> &d, double radius, std::vector<double> &U,
             std::vector<double> &V) const;
};

}  // namespace lmw
