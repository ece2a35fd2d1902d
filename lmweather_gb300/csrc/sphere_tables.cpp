// Host construction of the sphere tables. The Gauss-Legendre nodes and the normalised associated Legendre
// functions follow the reference's recurrences operation for operation (cpp/sphere.cpp:11,47-73,84-96), so
// the device tables hold exactly the reference's values. Compiled with -ffp-contract=off.
#include "sphere_tables.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace lmw {
namespace {
const double kPi = 3.14159265358979323846;
inline double eps_nm(int n, int m) { return std::sqrt(static_cast<double>(n * n - m * m) / static_cast<double>(4 * n * n - 1)); }
}  // namespace

void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
  x.assign(n, 0);
  w.assign(n, 0);
  for (int i = 0; i < (n + 1) / 2; i++) {
    double z = std::cos(kPi * (i + 0.75) / (n + 0.5)), pp = 1;
    for (int it = 0; it < 100; it++) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; j++) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
      double dz = p1 / pp;
      z -= dz;
      if (std::fabs(dz) < 1e-15) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2 / ((1 - z * z) * pp * pp);
  }
}

double legendre_eps(int n, int m) { return eps_nm(n, m); }

void legendre_column(int m, int nmax, double mu, std::vector<double> &out) {
  out.assign(static_cast<size_t>(nmax + 2 - m), 0.0);
  double c = std::sqrt(std::max(0.0, 1 - mu * mu)), p = 1 / std::sqrt(2.0);
  for (int k = 1; k <= m; k++) p *= std::sqrt((2.0 * k + 1) / (2.0 * k)) * c;
  out[0] = p;
  if (nmax + 1 >= m + 1) out[1] = std::sqrt(2.0 * m + 3) * mu * p;
  for (int n = m + 2; n <= nmax + 1; n++) out[n - m] = (mu * out[n - 1 - m] - eps_nm(n - 1, m) * out[n - 2 - m]) / eps_nm(n, m);
}

void fft_host(std::vector<cplx> &a, int sign) {
  const size_t n = a.size();
  for (size_t i = 1, j = 0; i < n; i++) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    double ang = 2 * kPi / static_cast<double>(len) * sign;
    cplx wl(std::cos(ang), std::sin(ang));
    for (size_t i = 0; i < n; i += len) {
      cplx w(1.0, 0.0);
      for (size_t k = 0; k < len / 2; k++) {
        if ((k & 15) == 0) w = cplx(std::cos(ang * static_cast<double>(k)), std::sin(ang * static_cast<double>(k)));
        cplx u = a[i + k], v = a[i + k + len / 2] * w;
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
        w *= wl;
      }
    }
  }
}

void HostTables::build(int truncation) {
  N = truncation;
  M = N + 1;
  nlon = 4;
  while (nlon < 3 * N + 1) nlon *= 2;  // cpp/sphere.cpp:77-79
  nlat = nlon / 2;
  nh = nlat / 2;
  ntri = M * (M + 1) / 2;
  gauss_legendre(nlat, mu, w);
  tri.assign(M + 1, 0);
  for (int m = 0, o = 0; m <= M; m++) {
    tri[m] = o;
    o += N - m + 1;
  }
  P.assign(static_cast<size_t>(ntri) * nh, 0.0);
  H.assign(static_cast<size_t>(ntri) * nh, 0.0);
  std::vector<double> col;
  for (int jh = 0; jh < nh; jh++)
    for (int m = 0; m <= N; m++) {
      legendre_column(m, N, mu[jh], col);
      for (int n = m; n <= N; n++) {
        size_t q = static_cast<size_t>(tri[m] + n - m);
        double plus = col[n + 1 - m], minus = (n > m) ? col[n - 1 - m] : 0.0;
        P[q * nh + jh] = col[n - m];
        H[q * nh + jh] = -n * eps_nm(n + 1, m) * plus + (n + 1) * eps_nm(n, m) * minus;  // cpp/sphere.cpp:91-94
      }
    }
}

// P_n^m(-mu) = (-1)^(n-m) P_n^m(mu), H_n^m(-mu) = -(-1)^(n-m) H_n^m(mu): exact in floating point, because the
// recurrence of cpp/sphere.cpp:66-73 only flips signs when mu does
double HostTables::Pj(int j, int m, int n) const {
  bool north = j >= nh;
  int jh = north ? nlat - 1 - j : j;
  double v = P[static_cast<size_t>(tri[m] + n - m) * nh + jh];
  return (north && ((n - m) & 1)) ? -v : v;
}
double HostTables::Hj(int j, int m, int n) const {
  bool north = j >= nh;
  int jh = north ? nlat - 1 - j : j;
  double v = H[static_cast<size_t>(tri[m] + n - m) * nh + jh];
  return (north && !((n - m) & 1)) ? -v : v;
}

// cpp/sphere.cpp:130-136,150-162
void HostTables::synthesize(const std::vector<cplx> &spec, std::vector<double> &grid) const {
  grid.assign(static_cast<size_t>(nlat) * nlon, 0.0);
  std::vector<cplx> a(nlon);
  for (int j = 0; j < nlat; j++) {
    std::fill(a.begin(), a.end(), cplx(0, 0));
    for (int m = 0; m <= N; m++) {
      cplx s = 0;
      for (int n = m; n <= N; n++) s += spec[static_cast<size_t>(m) * M + n] * Pj(j, m, n);
      if (m == 0) a[0] = cplx(s.real(), 0);
      else {
        a[m] = s;
        a[nlon - m] = std::conj(s);
      }
    }
    fft_host(a, +1);
    for (int k = 0; k < nlon; k++) grid[static_cast<size_t>(j) * nlon + k] = a[k].real();
  }
}

// cpp/sphere.cpp:179-206
void HostTables::winds(const std::vector<cplx> &z, const std::vector<cplx> &d, double radius, std::vector<double> &U,
                       std::vector<double> &V) const {
  const double a = radius;
  const cplx I(0, 1);
  std::vector<cplx> psi(z.size(), 0), chi(z.size(), 0);
  for (int m = 0; m <= N; m++)
    for (int n = std::max(m, 1); n <= N; n++) {
      double k = -a * a / (n * (n + 1.0));
      psi[static_cast<size_t>(m) * M + n] = z[static_cast<size_t>(m) * M + n] * k;
      chi[static_cast<size_t>(m) * M + n] = d[static_cast<size_t>(m) * M + n] * k;
    }
  U.assign(static_cast<size_t>(nlat) * nlon, 0.0);
  V.assign(U.size(), 0.0);
  std::vector<cplx> au(nlon), av(nlon);
  for (int j = 0; j < nlat; j++) {
    std::fill(au.begin(), au.end(), cplx(0, 0));
    std::fill(av.begin(), av.end(), cplx(0, 0));
    for (int m = 0; m <= N; m++) {
      cplx sp = 0, sc = 0, hp = 0, hc = 0;
      for (int n = m; n <= N; n++) {
        double P = Pj(j, m, n), H = Hj(j, m, n);
        size_t q = static_cast<size_t>(m) * M + n;
        sp += psi[q] * P;
        sc += chi[q] * P;
        hp += psi[q] * H;
        hc += chi[q] * H;
      }
      cplx fu = (I * static_cast<double>(m) * sc - hp) / a, fv = (I * static_cast<double>(m) * sp + hc) / a;
      if (m == 0) {
        au[0] = cplx(fu.real(), 0);
        av[0] = cplx(fv.real(), 0);
      } else {
        au[m] = fu;
        au[nlon - m] = std::conj(fu);
        av[m] = fv;
        av[nlon - m] = std::conj(fv);
      }
    }
    fft_host(au, +1);
    fft_host(av, +1);
    for (int k = 0; k < nlon; k++) {
      U[static_cast<size_t>(j) * nlon + k] = au[k].real();
      V[static_cast<size_t>(j) * nlon + k] = av[k].real();
    }
  }
}

}  // namespace lmw
