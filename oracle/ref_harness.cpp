// C entry points over the reference numerical core, for pinning the oracle and generating golden fixtures.
//
// TEST INFRASTRUCTURE ONLY. oracle/Makefile compiles this file together with the reference's own
// cpp/sphere.cpp and cpp/plane.cpp, read in place from the reference checkout (never copied), into
// oracle/_ref/libref.so. The reference classes keep their spectral state private; the harness opens the
// class for reading (access control only: the layout the reference's translation units use is unchanged).
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#define private public
#include "plane.hpp"
#include "sphere.hpp"
#undef private

using lmweather::cplx;
using lmweather::Plane;
using lmweather::PlaneParams;
using lmweather::Sphere;
using lmweather::SphereParams;

namespace {
template <class F> int guarded(char *err, int len, F &&fn) {
  try {
    fn();
    return 0;
  } catch (const std::invalid_argument &e) {
    if (err && len > 0) std::snprintf(err, len, "%s", e.what());
    return 1;
  } catch (const std::exception &e) {
    if (err && len > 0) std::snprintf(err, len, "%s", e.what());
    return 2;
  }
}
size_t ngrid(const Sphere *s) { return static_cast<size_t>(s->nlat()) * s->nlon(); }
std::vector<double> grid_in(const Sphere *s, const double *p) { return std::vector<double>(p, p + ngrid(s)); }
void copy_out(const std::vector<double> &v, double *out) { std::memcpy(out, v.data(), v.size() * sizeof(double)); }
void spec_out(const std::vector<cplx> &v, double *out) { std::memcpy(out, v.data(), v.size() * sizeof(cplx)); }
}  // namespace

extern "C" {

int ref_fft(double *a, int n, int sign) {
  std::vector<cplx> v(reinterpret_cast<cplx *>(a), reinterpret_cast<cplx *>(a) + n);
  return guarded(nullptr, 0, [&] {
    lmweather::fft(v, sign);
    std::memcpy(a, v.data(), n * sizeof(cplx));
  });
}
void ref_gauss_legendre(int n, double *x, double *w) {
  std::vector<double> xv, wv;
  lmweather::gauss_legendre(n, xv, wv);
  copy_out(xv, x);
  copy_out(wv, w);
}
void ref_legendre_column(int m, int nmax, double mu, double *out) {
  std::vector<double> v;
  lmweather::legendre_column(m, nmax, mu, v);
  copy_out(v, out);
}

void *ref_sphere_new(int T, double radius, double omega, double gravity, double diffusion, char *err, int len) {
  Sphere *s = nullptr;
  SphereParams p;
  p.radius = radius; p.omega = omega; p.gravity = gravity; p.diffusion = diffusion;
  if (guarded(err, len, [&] { s = new Sphere(T, p); })) return nullptr;
  return s;
}
void ref_sphere_free(void *h) { delete static_cast<Sphere *>(h); }
int ref_sphere_nlat(void *h) { return static_cast<Sphere *>(h)->nlat(); }
int ref_sphere_nlon(void *h) { return static_cast<Sphere *>(h)->nlon(); }
double ref_sphere_time(void *h) { return static_cast<Sphere *>(h)->time(); }
void ref_sphere_mu_w(void *h, double *mu, double *w) {
  auto *s = static_cast<Sphere *>(h);
  copy_out(s->gauss_mu(), mu);
  copy_out(s->gauss_weights(), w);
}
void ref_sphere_set_axis_tilt(void *h, double alpha) { static_cast<Sphere *>(h)->set_axis_tilt(alpha); }
void ref_sphere_set_diffusion(void *h, double nu) { static_cast<Sphere *>(h)->set_diffusion(nu); }
void ref_sphere_set_advect_only(void *h, int on) { static_cast<Sphere *>(h)->set_advect_only(on != 0); }
int ref_sphere_set_state_grid(void *h, const double *hh, const double *u, const double *v, char *err, int len) {
  auto *s = static_cast<Sphere *>(h);
  return guarded(err, len, [&] { s->set_state_grid(grid_in(s, hh), grid_in(s, u), grid_in(s, v)); });
}
int ref_sphere_set_orography_grid(void *h, const double *hs, char *err, int len) {
  auto *s = static_cast<Sphere *>(h);
  return guarded(err, len, [&] { s->set_orography_grid(grid_in(s, hs)); });
}
int ref_sphere_set_tracer_grid(void *h, const double *q, char *err, int len) {
  auto *s = static_cast<Sphere *>(h);
  return guarded(err, len, [&] { s->set_tracer_grid(grid_in(s, q)); });
}
int ref_sphere_perturb(void *h, double amp, unsigned long long seed, int nmax, char *err, int len) {
  auto *s = static_cast<Sphere *>(h);
  return guarded(err, len, [&] { s->perturb(amp, seed, nmax); });
}
int ref_sphere_add_mode(void *h, int n, int m, double amp, double depth, char *err, int len) {
  auto *s = static_cast<Sphere *>(h);
  return guarded(err, len, [&] { s->add_mode(n, m, amp, depth); });
}
void ref_sphere_mark_reference(void *h) { static_cast<Sphere *>(h)->mark_reference(); }
void ref_sphere_get_state(void *h, double *z, double *d, double *f, double *q) {
  auto *s = static_cast<Sphere *>(h);
  spec_out(s->zeta_, z);
  spec_out(s->delta_, d);
  spec_out(s->phi_, f);
  if (q) {
    if (s->has_tracer_) spec_out(s->q_, q);
    else std::memset(q, 0, s->zeta_.size() * sizeof(cplx));
  }
}
void ref_sphere_set_state(void *h, const double *z, const double *d, const double *f, double t) {
  auto *s = static_cast<Sphere *>(h);
  size_t n = s->zeta_.size();
  std::memcpy(s->zeta_.data(), z, n * sizeof(cplx));
  std::memcpy(s->delta_.data(), d, n * sizeof(cplx));
  std::memcpy(s->phi_.data(), f, n * sizeof(cplx));
  s->t_ = t;
}
void ref_sphere_step(void *h, double dt) { static_cast<Sphere *>(h)->step(dt); }
int ref_sphere_run(void *h, double seconds, double dt, char *err, int len) {
  auto *s = static_cast<Sphere *>(h);
  return guarded(err, len, [&] { s->run(seconds, dt); });
}
double ref_sphere_stable_dt(void *h, double safety) {
  double r = 0;
  guarded(nullptr, 0, [&] { r = static_cast<Sphere *>(h)->stable_dt(safety); });
  return r;
}
// out: mean_height, kinetic, potential, energy, enstrophy, max_wind, error_l2, error_linf
void ref_sphere_diagnostics(void *h, double *out) {
  auto *s = static_cast<Sphere *>(h);
  out[0] = s->mean_height();
  out[1] = s->kinetic_energy();
  out[2] = s->potential_energy();
  out[3] = s->energy();
  out[4] = s->potential_enstrophy();
  out[5] = s->max_wind();
  out[6] = s->height_error_l2();
  out[7] = s->height_error_linf();
}
void ref_sphere_spectrum(void *h, double *ke, double *pe) {
  std::vector<double> k, p;
  static_cast<Sphere *>(h)->spectrum(k, p);
  copy_out(k, ke);
  copy_out(p, pe);
}
double ref_sphere_tracer_mean(void *h) { return static_cast<Sphere *>(h)->tracer_mean(); }
double ref_sphere_tracer_mass(void *h) { return static_cast<Sphere *>(h)->tracer_mass(); }
void ref_sphere_grids(void *h, double *hh, double *u, double *v, double *z) {
  auto *s = static_cast<Sphere *>(h);
  if (hh) copy_out(s->grid_height(), hh);
  if (u) copy_out(s->grid_u(), u);
  if (v) copy_out(s->grid_v(), v);
  if (z) copy_out(s->grid_vorticity(), z);
}
void ref_sphere_analyze_scalar(void *h, const double *grid, double *spec) {
  auto *s = static_cast<Sphere *>(h);
  std::vector<cplx> out;
  s->analyze_scalar(grid_in(s, grid), out);
  spec_out(out, spec);
}
void ref_sphere_synthesize_scalar(void *h, const double *spec, double *grid) {
  auto *s = static_cast<Sphere *>(h);
  size_t n = s->zeta_.size();
  std::vector<cplx> in(reinterpret_cast<const cplx *>(spec), reinterpret_cast<const cplx *>(spec) + n);
  std::vector<double> out;
  s->synthesize_scalar(in, out);
  copy_out(out, grid);
}
void ref_sphere_analyze_divergence(void *h, const double *A, const double *B, double *spec) {
  auto *s = static_cast<Sphere *>(h);
  std::vector<cplx> out;
  s->analyze_divergence(grid_in(s, A), grid_in(s, B), out);
  spec_out(out, spec);
}

void *ref_plane_new(int nx, int ny, double lx, double ly, double gravity, double depth, double f0, double beta,
                    double viscosity, double drag, int linear, char *err, int len) {
  PlaneParams p;
  p.nx = nx; p.ny = ny; p.lx = lx; p.ly = ly; p.gravity = gravity; p.depth = depth;
  p.f0 = f0; p.beta = beta; p.viscosity = viscosity; p.drag = drag; p.linear = linear != 0;
  Plane *pl = nullptr;
  if (guarded(err, len, [&] { pl = new Plane(p); })) return nullptr;
  return pl;
}
void ref_plane_free(void *h) { delete static_cast<Plane *>(h); }
double ref_plane_time(void *h) { return static_cast<Plane *>(h)->time(); }
void ref_plane_get(void *h, double *hh, double *u, double *v) {
  auto *p = static_cast<Plane *>(h);
  copy_out(p->h_, hh);
  copy_out(p->u_, u);
  copy_out(p->v_, v);
}
int ref_plane_set(void *h, const double *hh, const double *u, const double *v, char *err, int len) {
  auto *p = static_cast<Plane *>(h);
  size_t n = p->h_.size(), nv = p->v_.size();
  return guarded(err, len, [&] {
    p->set_h_from_grid(std::vector<double>(hh, hh + n));
    p->set_u_from_grid(std::vector<double>(u, u + n));
    p->set_v_from_grid(std::vector<double>(v, v + nv));
  });
}
void ref_plane_perturb(void *h, double amp, unsigned long long seed) { static_cast<Plane *>(h)->perturb(amp, seed); }
void ref_plane_step(void *h, double dt) { static_cast<Plane *>(h)->step(dt); }
int ref_plane_run(void *h, double seconds, double dt, char *err, int len) {
  auto *p = static_cast<Plane *>(h);
  return guarded(err, len, [&] { p->run(seconds, dt); });
}
double ref_plane_stable_dt(void *h, double safety) {
  double r = 0;
  guarded(nullptr, 0, [&] { r = static_cast<Plane *>(h)->stable_dt(safety); });
  return r;
}
// out: mean_depth, energy, max_speed, pv_anomaly_rms
void ref_plane_diagnostics(void *h, double *out) {
  auto *p = static_cast<Plane *>(h);
  out[0] = p->mean_depth();
  out[1] = p->energy();
  out[2] = p->max_speed();
  out[3] = p->potential_vorticity_anomaly_rms();
}

// the plane's point and harmonic diagnostics (cpp/plane.cpp:220-310); a status of 1 is std::invalid_argument
double ref_plane_probe(void *h, int kind, double x, double y) {
  auto *p = static_cast<Plane *>(h);
  return kind == 0 ? p->h_at(x, y) : kind == 1 ? p->u_at(x, y) : p->v_at(x, y);
}
double ref_plane_zeta_at_corner(void *h, int i, int j) { return static_cast<Plane *>(h)->zeta_at_corner(i, j); }
// which: 0 zonal_amplitude(m, j), 1 zonal_crest(m, j), 2 v_zonal_crest(m, j), 3 harmonic_energy(m)
int ref_plane_harmonic(void *h, int which, int m, int j, double *out, char *err, int len) {
  auto *p = static_cast<Plane *>(h);
  return guarded(err, len, [&] {
    *out = which == 0 ? p->zonal_amplitude(m, j) : which == 1 ? p->zonal_crest(m, j) : which == 2 ? p->v_zonal_crest(m, j) : p->harmonic_energy(m);
  });
}

}  // extern "C"
