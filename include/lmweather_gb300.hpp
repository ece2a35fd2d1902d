/* C++ classes over the C ABI with the method names and exception types of lmweather's numerical core
 * (lmweather::Sphere, cpp/sphere.hpp:27-121; lmweather::Plane, cpp/plane.hpp:20-68), so that code written
 * against those classes (the wx.* registrations of cpp/main.cpp) compiles against the GPU engine by changing the
 * namespace. Status LMW_INVALID_ARGUMENT becomes std::invalid_argument, every other failure std::runtime_error,
 * each with the engine's message (the reference's texts). Header-only; link with liblmw_gb300.so.
 *
 * State lives on the GPU. Calls are synchronous with respect to the caller, like the reference's methods.
 * Plane::h/u/v(i, j) read a host copy of the fields that the accessors refresh after every change. */
#ifndef LMWEATHER_GB300_HPP
#define LMWEATHER_GB300_HPP

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lmweather_gb300.h"

namespace lmweather_gb300 {

inline void check(int status) {
  if (status == LMW_OK) return;
  const char *msg = lmw_last_error();
  if (status == LMW_INVALID_ARGUMENT) throw std::invalid_argument(msg ? msg : "invalid argument");
  throw std::runtime_error(msg ? msg : "lmweather-gb300 failure");
}

// cpp/sphere.hpp:20-25
struct SphereParams {
  double radius = 6.37122e6;
  double omega = 7.292e-5;
  double gravity = 9.80616;
  double diffusion = 0;
};

class Sphere {
 public:
  Sphere(int truncation, const SphereParams &p) : p_(p) {
    check(lmw_sphere_create(truncation, p.radius, p.omega, p.gravity, p.diffusion, &s_));
    int members = 0;
    check(lmw_sphere_dims(s_, &N_, &nlat_, &nlon_, &members));
    mu_.resize(nlat_);
    w_.resize(nlat_);
    check(lmw_sphere_gauss(s_, mu_.data(), w_.data()));
  }
  ~Sphere() {
    if (s_) lmw_sphere_destroy(s_);
  }
  Sphere(const Sphere &) = delete;
  Sphere &operator=(const Sphere &) = delete;
  Sphere(Sphere &&o) noexcept { *this = std::move(o); }
  Sphere &operator=(Sphere &&o) noexcept {
    std::swap(s_, o.s_);
    std::swap(p_, o.p_);
    std::swap(N_, o.N_);
    std::swap(nlat_, o.nlat_);
    std::swap(nlon_, o.nlon_);
    std::swap(mu_, o.mu_);
    std::swap(w_, o.w_);
    std::swap(has_orography_, o.has_orography_);
    std::swap(hs_, o.hs_);
    std::swap(has_tracer_, o.has_tracer_);
    std::swap(advect_only_, o.advect_only_);
    return *this;
  }

  int truncation() const { return N_; }
  int nlat() const { return nlat_; }
  int nlon() const { return nlon_; }
  const SphereParams &params() const { return p_; }
  double time() const {
    double t = 0;
    check(lmw_sphere_time(s_, 0, &t));
    return t;
  }
  double lat(int j) const { return std::asin(mu_.at(j)); }
  double lon(int k) const { return 2 * 3.14159265358979323846 * k / nlon_; }

  void set_state_grid(const std::vector<double> &h, const std::vector<double> &u, const std::vector<double> &v) {
    if (h.size() != u.size() || h.size() != v.size()) throw std::invalid_argument("grid size mismatch");
    check(lmw_sphere_set_state_grid(s_, 0, h.data(), u.data(), v.data(), h.size()));
  }
  void set_axis_tilt(double alpha) { check(lmw_sphere_set_axis_tilt(s_, 0, alpha)); }
  void set_diffusion(double nu4) {
    check(lmw_sphere_set_diffusion(s_, nu4));
    p_.diffusion = nu4;
  }
  void mark_reference() { check(lmw_sphere_mark_reference(s_, 0)); }
  void add_mode(int n, int m, double amplitude, double mean_depth) { check(lmw_sphere_add_mode(s_, 0, n, m, amplitude, mean_depth)); }
  void perturb(double amplitude, uint64_t seed, int max_wave) { check(lmw_sphere_perturb(s_, 0, amplitude, seed, max_wave)); }

  void set_orography_grid(const std::vector<double> &hs) {
    check(lmw_sphere_set_orography_grid(s_, 0, hs.data(), hs.size()));
    hs_ = hs;
    has_orography_ = true;
  }
  bool has_orography() const { return has_orography_; }
  const std::vector<double> &grid_orography() const { return hs_; }

  void set_tracer_grid(const std::vector<double> &q) {
    check(lmw_sphere_set_tracer_grid(s_, 0, q.data(), q.size()));
    has_tracer_ = true;
  }
  bool has_tracer() const { return has_tracer_; }
  void set_advect_only(bool on) {
    check(lmw_sphere_set_advect_only(s_, on ? 1 : 0));
    advect_only_ = on;
  }
  bool advect_only() const { return advect_only_; }
  std::vector<double> grid_tracer() const {
    std::vector<double> g(static_cast<size_t>(nlat_) * nlon_);
    check(lmw_sphere_tracer_grid(s_, 0, g.data(), g.size()));
    return g;
  }
  double tracer_mean() const { return tracer_diag(0); }
  double tracer_mass() const { return tracer_diag(1); }
  double tracer_at(double lat, double lon) const { return probe(4, lat, lon); }
  double tracer_min() const {
    const std::vector<double> g = grid_tracer();
    return *std::min_element(g.begin(), g.end());
  }
  double tracer_max() const {
    const std::vector<double> g = grid_tracer();
    return *std::max_element(g.begin(), g.end());
  }
  double tracer_error_l2() const { return tracer_diag(2); }
  double tracer_error_linf() const { return tracer_diag(3); }

  void step(double dt) { check(lmw_sphere_step(s_, dt)); }
  void run(double seconds, double dt) { check(lmw_sphere_run(s_, seconds, dt)); }
  double stable_dt(double safety = 1.5) const {
    double dt = 0;
    check(lmw_sphere_stable_dt(s_, 0, safety, &dt));
    return dt;
  }

  double mean_height() const { return diag(0); }
  double kinetic_energy() const { return diag(1); }
  double potential_energy() const { return diag(2); }
  double energy() const { return diag(3); }
  double potential_enstrophy() const { return diag(4); }
  double max_wind() const { return diag(5); }
  double height_error_l2() const { return diag(6); }
  double height_error_linf() const { return diag(7); }
  void spectrum(std::vector<double> &ke, std::vector<double> &pe) const {
    ke.assign(N_ + 1, 0.0);
    pe.assign(N_ + 1, 0.0);
    check(lmw_sphere_spectrum(s_, 0, ke.data(), pe.data()));
  }
  double height_at(double lat, double lon) const { return probe(0, lat, lon); }
  double wind_at(double lat, double lon, bool zonal) const { return probe(zonal ? 1 : 2, lat, lon); }
  double vorticity_at(double lat, double lon) const { return probe(3, lat, lon); }
  double mode_coefficient(int n, int m, bool imag) const {
    double c = 0;
    check(lmw_sphere_mode_coefficient(s_, 0, n, m, imag ? 1 : 0, &c));
    return c;
  }
  double wave_crest(int m, double lat) const {
    double x = 0;
    check(lmw_sphere_wave_crest(s_, 0, m, lat, &x));
    return x;
  }

  std::vector<double> grid_height() const { return grid(0); }
  std::vector<double> grid_u() const { return grid(1); }
  std::vector<double> grid_v() const { return grid(2); }
  std::vector<double> grid_vorticity() const { return grid(3); }
  const std::vector<double> &gauss_weights() const { return w_; }
  const std::vector<double> &gauss_mu() const { return mu_; }

  // exposed for tests (cpp/sphere.hpp:96-99): spectra in the reference layout, (T+1)^2 values at m*(T+1)+n
  using cplx = std::complex<double>;
  void analyze_scalar(const std::vector<double> &grid, std::vector<cplx> &spec) const {
    spec.assign(static_cast<size_t>(N_ + 1) * (N_ + 1), cplx(0, 0));
    check(lmw_sphere_analyze_scalar(s_, grid.data(), grid.size(), reinterpret_cast<double *>(spec.data())));
  }
  void synthesize_scalar(const std::vector<cplx> &spec, std::vector<double> &grid) const {
    if (spec.size() != static_cast<size_t>(N_ + 1) * (N_ + 1)) throw std::invalid_argument("spectrum size mismatch");
    grid.assign(static_cast<size_t>(nlat_) * nlon_, 0.0);
    check(lmw_sphere_synthesize_scalar(s_, reinterpret_cast<const double *>(spec.data()), grid.data(), grid.size()));
  }
  void analyze_divergence(const std::vector<double> &A, const std::vector<double> &B, std::vector<cplx> &spec) const {
    if (A.size() != B.size()) throw std::invalid_argument("grid size mismatch");
    spec.assign(static_cast<size_t>(N_ + 1) * (N_ + 1), cplx(0, 0));
    check(lmw_sphere_analyze_divergence(s_, A.data(), B.data(), A.size(), reinterpret_cast<double *>(spec.data())));
  }

  // the engine handle, for the entry points beyond the reference's class (precision, ensembles, state I/O)
  lmw_sphere *handle() const { return s_; }

 private:
  lmw_sphere *s_ = nullptr;
  SphereParams p_;
  int N_ = 0, nlat_ = 0, nlon_ = 0;
  std::vector<double> mu_, w_, hs_;
  bool has_orography_ = false, has_tracer_ = false, advect_only_ = false;

  double diag(int i) const {
    double out[8];
    check(lmw_sphere_diagnostics(s_, 0, out));
    return out[i];
  }
  double tracer_diag(int i) const {
    double out[6];
    check(lmw_sphere_tracer_diagnostics(s_, 0, out));
    return out[i];
  }
  double probe(int which, double lat, double lon) const {
    double x = 0;
    check(lmw_sphere_probe(s_, 0, which, lat, lon, &x));
    return x;
  }
  std::vector<double> grid(int which) const {
    std::vector<double> g(static_cast<size_t>(nlat_) * nlon_);
    check(lmw_sphere_grid(s_, 0, which, g.data(), g.size()));
    return g;
  }
};

// cpp/plane.hpp:9-18
struct PlaneParams {
  int nx = 0, ny = 0;
  double lx = 0, ly = 0;
  double gravity = 9.81;
  double depth = 100;
  double f0 = 0, beta = 0;
  double viscosity = 0;
  double drag = 0;
  bool linear = false;
};

class Plane {
 public:
  explicit Plane(const PlaneParams &p) : p_(p) {
    check(lmw_plane_create(p.nx, p.ny, p.lx, p.ly, p.gravity, p.depth, p.f0, p.beta, p.viscosity, p.drag, p.linear ? 1 : 0, &h_));
    refresh();
  }
  ~Plane() {
    if (h_) lmw_plane_destroy(h_);
  }
  Plane(const Plane &) = delete;
  Plane &operator=(const Plane &) = delete;

  const PlaneParams &params() const { return p_; }
  // the reference lets callers edit the parameters in place; apply them with apply_params()
  PlaneParams &params() { return p_; }
  void apply_params() { check(lmw_plane_set_params(h_, p_.gravity, p_.depth, p_.f0, p_.beta, p_.viscosity, p_.drag, p_.linear ? 1 : 0)); }
  double time() const {
    double t = 0;
    check(lmw_plane_time(h_, &t));
    return t;
  }
  double dx() const { return p_.lx / p_.nx; }
  double dy() const { return p_.ly / p_.ny; }
  double x_center(int i) const { return (i + 0.5) * dx(); }
  double y_center(int j) const { return (j + 0.5) * dy(); }
  double h(int i, int j) const { return hh_[static_cast<size_t>(j) * p_.nx + i]; }
  double u(int i, int j) const { return uu_[static_cast<size_t>(j) * p_.nx + i]; }
  double v(int i, int j) const { return vv_[static_cast<size_t>(j) * p_.nx + i]; }

  void reset() {
    check(lmw_plane_reset(h_));
    refresh();
  }
  void perturb(double amplitude, uint64_t seed) {
    check(lmw_plane_perturb(h_, amplitude, seed));
    refresh();
  }
  void step(double dt) {
    check(lmw_plane_step(h_, dt));
    refresh();
  }
  void run(double seconds, double dt) {
    check(lmw_plane_run(h_, seconds, dt));
    refresh();
  }
  double stable_dt(double safety = 0.5) const {
    double dt = 0;
    check(lmw_plane_stable_dt(h_, safety, &dt));
    return dt;
  }
  double mean_depth() const { return diag(0); }
  double energy() const { return diag(1); }
  double max_speed() const { return diag(2); }
  double potential_vorticity_anomaly_rms() const { return diag(3); }
  void set_u_from_grid(const std::vector<double> &g) {
    check(lmw_plane_set_u(h_, g.data(), g.size()));
    refresh();
  }
  void set_h_from_grid(const std::vector<double> &g) {
    check(lmw_plane_set_h(h_, g.data(), g.size()));
    refresh();
  }
  void set_v_from_grid(const std::vector<double> &g) {
    check(lmw_plane_set_v(h_, g.data(), g.size()));
    refresh();
  }
  double coriolis(double y) const { return p_.f0 + p_.beta * (y - 0.5 * p_.ly); }
  // point and harmonic diagnostics (cpp/plane.hpp:49-59), computed on the device
  double h_at(double x, double y) const { return scalar(lmw_plane_probe, 0, x, y); }
  double u_at(double x, double y) const { return scalar(lmw_plane_probe, 1, x, y); }
  double v_at(double x, double y) const { return scalar(lmw_plane_probe, 2, x, y); }
  double zeta_at_corner(int i, int j) const { return scalar(lmw_plane_zeta_at_corner, i, j); }
  double zonal_amplitude(int m, int j) const { return scalar(lmw_plane_zonal_amplitude, m, j); }
  double zonal_crest(int m, int j) const { return scalar(lmw_plane_zonal_crest, m, j); }
  double v_zonal_crest(int m, int j) const { return scalar(lmw_plane_v_zonal_crest, m, j); }
  double harmonic_energy(int m) const { return scalar(lmw_plane_harmonic_energy, m); }

  lmw_plane *handle() const { return h_; }

 private:
  lmw_plane *h_ = nullptr;
  PlaneParams p_;
  std::vector<double> hh_, uu_, vv_;

  void refresh() {
    hh_.resize(static_cast<size_t>(p_.nx) * p_.ny);
    uu_.resize(static_cast<size_t>(p_.nx) * p_.ny);
    vv_.resize(static_cast<size_t>(p_.nx) * (p_.ny + 1));
    check(lmw_plane_get(h_, hh_.data(), uu_.data(), vv_.data()));
  }
  double diag(int i) const {
    double out[4];
    check(lmw_plane_diagnostics(h_, out));
    return out[i];
  }
  template <class F, class... A> double scalar(F fn, A... args) const {
    double out = 0;
    check(fn(h_, args..., &out));
    return out;
  }
};

}  // namespace lmweather_gb300

#endif
