// The C++ classes of include/lmweather_gb300.hpp used as lmweather's own core classes are used: Williamson test
// case 2 stays steady, point probes agree with the grids, the run guard throws std::invalid_argument with the
// reference's text, the plane conserves mass, and bad arguments raise the reference's exception classes.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "lmweather_gb300.hpp"

namespace lg = lmweather_gb300;

static int failures = 0;
#define EXPECT(cond, what)                                   \
  do {                                                       \
    if (!(cond)) {                                           \
      std::printf("FAIL %s (line %d)\n", what, __LINE__);    \
      failures++;                                            \
    }                                                        \
  } while (0)

int main() {
  const double pi = 3.14159265358979323846;
  lg::SphereParams sp;
  lg::Sphere s(42, sp);
  const int nlat = s.nlat(), nlon = s.nlon();
  EXPECT(nlat == 64 && nlon == 128, "T42 grid is 128 x 64");
  // Williamson TC2 with an untilted axis: u = u0 cos(lat), geostrophic h
  const double u0 = 2 * pi * sp.radius / (12 * 86400.0), h0 = 2.94e4 / sp.gravity;
  std::vector<double> h(nlat * nlon), u(nlat * nlon), v(nlat * nlon, 0.0);
  for (int j = 0; j < nlat; j++)
    for (int k = 0; k < nlon; k++) {
      const double la = s.lat(j), t = std::sin(la);
      u[j * nlon + k] = u0 * std::cos(la);
      h[j * nlon + k] = h0 - (sp.radius * sp.omega * u0 + 0.5 * u0 * u0) * t * t / sp.gravity;
    }
  s.set_state_grid(h, u, v);
  const double e0 = s.energy(), m0 = s.mean_height();
  s.run(86400.0, 1800.0);
  EXPECT(s.height_error_l2() < 1e-10, "TC2 stays steady");
  EXPECT(std::fabs(s.energy() - e0) < 1e-9 * e0, "TC2 energy");
  EXPECT(std::fabs(s.mean_height() - m0) < 1e-12 * m0, "mass is conserved");
  EXPECT(std::fabs(s.time() - 86400.0) < 1e-6, "time advances");
  // point probes against the grids at grid points
  const std::vector<double> gh = s.grid_height(), gu = s.grid_u();
  double worst_h = 0, worst_u = 0;
  for (int j = 3; j < nlat; j += 17)
    for (int k = 5; k < nlon; k += 29) {
      worst_h = std::max(worst_h, std::fabs(s.height_at(s.lat(j), s.lon(k)) - gh[j * nlon + k]) / h0);
      worst_u = std::max(worst_u, std::fabs(s.wind_at(s.lat(j), s.lon(k), true) - gu[j * nlon + k]) / u0);
    }
  EXPECT(worst_h < 1e-12, "height_at matches grid_height");
  EXPECT(worst_u < 1e-11, "wind_at matches grid_u");
  EXPECT(std::fabs(s.mode_coefficient(0, 0, false) / std::sqrt(2.0) - s.mean_height()) < 1e-9, "mode (0,0) is the mean height");
  std::vector<double> ke, pe;
  s.spectrum(ke, pe);
  EXPECT(static_cast<int>(ke.size()) == 43 && ke[1] > 0, "spectrum");
  // the run guard and the reference's exception classes
  bool threw = false;
  try {
    s.run(86400.0, 1.0e5);
  } catch (const std::invalid_argument &e) {
    threw = std::string(e.what()).find("exceeds the RK4 stability limit") != std::string::npos;
  }
  EXPECT(threw, "run rejects an unstable dt with invalid_argument");
  threw = false;
  try {
    lg::Sphere bad(3, sp);
  } catch (const std::invalid_argument &) {
    threw = true;
  }
  EXPECT(threw, "truncation below 4 is invalid_argument");
  threw = false;
  try {
    s.tracer_at(0.1, 0.2);
  } catch (const std::runtime_error &) {
    threw = true;
  }
  EXPECT(threw, "tracer_at without a tracer is runtime_error");
  // the transform test hooks through the C ABI, restating the reference's T21 round trip: a seeded spectrum is
  // synthesised and analysed back to 1e-12; the divergence operator of the solid-body winds U = u cos(lat),
  // V = 0 is zero, and D(V, -U) is the vorticity 2 u0 sin(lat) / a, which is (n, m) = (1, 0) alone
  {
    lg::Sphere s21(21, sp);
    std::vector<lg::Sphere::cplx> spec(22 * 22, 0), back, div, vor;
    unsigned seed = 5;
    auto rnd = [&] {
      seed = seed * 1664525u + 1013904223u;
      return (seed >> 8) / 16777216.0 - 0.5;
    };
    for (int m = 0; m <= 21; m++)
      for (int n = m; n <= 21; n++) spec[m * 22 + n] = lg::Sphere::cplx(rnd(), m == 0 ? 0.0 : rnd());
    std::vector<double> g;
    s21.synthesize_scalar(spec, g);
    s21.analyze_scalar(g, back);
    double worst = 0;
    for (size_t i = 0; i < spec.size(); i++) worst = std::max(worst, std::abs(back[i] - spec[i]));
    EXPECT(worst < 1e-12, "T21 spectral round trip through the hooks");
    const int nl = s21.nlat(), nn = s21.nlon();
    std::vector<double> U(nl * nn), V(nl * nn, 0.0), mU(nl * nn);
    for (int j = 0; j < nl; j++)
      for (int k = 0; k < nn; k++) {
        U[j * nn + k] = 10 * std::cos(s21.lat(j)) * std::cos(s21.lat(j));
        mU[j * nn + k] = -U[j * nn + k];
      }
    s21.analyze_divergence(U, V, div);
    s21.analyze_divergence(V, mU, vor);
    double dmax = 0;
    for (const auto &c : div) dmax = std::max(dmax, std::abs(c));
    EXPECT(dmax < 1e-18, "solid-body winds have no divergence");
    // zeta = 2 u0 mu / a = (2 u0 / a) sqrt(2/3) P_1^0(mu) with P_1^0 = sqrt(3/2) mu
    EXPECT(std::fabs(vor[1].real() - 2 * 10 / sp.radius * std::sqrt(2.0 / 3.0)) < 1e-12 * 2 * 10 / sp.radius, "solid-body vorticity");
    double rest = 0;
    for (size_t i = 0; i < vor.size(); i++)
      if (i != 1) rest = std::max(rest, std::abs(vor[i]));
    EXPECT(rest < 1e-12 * 2 * 10 / sp.radius, "solid-body vorticity has one mode");
  }
  // plane: mass conservation and element accessors
  lg::PlaneParams pp;
  pp.nx = 64;
  pp.ny = 32;
  pp.lx = 3.2e5;
  pp.ly = 1.6e5;
  pp.f0 = 1e-4;
  pp.beta = 1.6e-11;
  lg::Plane p(pp);
  p.perturb(0.1, 7);
  const double d0 = p.mean_depth();
  p.run(3600.0, 60.0);
  EXPECT(std::fabs(p.mean_depth() - d0) < 1e-12 * d0, "plane mass");
  EXPECT(std::fabs(p.time() - 3600.0) < 1e-9, "plane time");
  double hsum = 0;
  for (int j = 0; j < pp.ny; j++)
    for (int i = 0; i < pp.nx; i++) hsum += p.h(i, j);
  EXPECT(std::fabs(hsum / (pp.nx * pp.ny) - p.mean_depth()) < 1e-9, "plane accessors read the device state");
  EXPECT(p.v(3, 0) == 0.0 && p.v(3, pp.ny) == 0.0, "walls stay at rest");
  // device probes agree with the element accessors: at a cell centre h_at is the cell's value
  EXPECT(p.h_at(p.x_center(5), p.y_center(9)) == p.h(5, 9), "h_at at a cell centre");
  EXPECT(p.u_at(5 * p.dx(), p.y_center(9)) == p.u(5, 9), "u_at at a west face");
  EXPECT(std::isfinite(p.zeta_at_corner(pp.nx, pp.ny)) && p.harmonic_energy(3) >= 0, "corner vorticity and harmonic energy");
  threw = false;
  try {
    p.zonal_crest(pp.nx / 2, 0);
  } catch (const std::invalid_argument &e) {
    threw = std::string(e.what()).find("zonal harmonic or row out of range") != std::string::npos;
  }
  EXPECT(threw, "zonal_crest out of range is invalid_argument with the reference's text");
  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
