// The C ABI (include/lmweather_gb300.h): exceptions become status codes, the message is kept per thread.
#include <cuda_profiler_api.h>

#include <cstdio>
#include <exception>
#include <new>
#include <string>

#include "../../include/lmweather_gb300.h"
#include "engine.h"
#include "sphere_tables.h"
#include "surrogate.h"
#include "tc_gemm.h"

struct lmw_sphere {
  lmw::SphereEngine *e;
};
struct lmw_plane {
  lmw::PlaneEngine *e;
};
struct lmw_ensemble {
  lmw::EnsembleEngine *e;
};
struct lmw_mlp {
  lmw::Mlp *m;
};
struct lmw_surrogate {
  lmw::Surrogate *s;
};

namespace lmw {
thread_local uint64_t g_launches = 0;

void cuda_check(cudaError_t e, const char *what, const char *file, int line) {
  if (e == cudaSuccess) return;
  char buf[512];
  std::snprintf(buf, sizeof buf, "CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e), what, file, line);
  throw DeviceError(buf);
}

std::string fmt_f(double x) {
  char b[512];
  std::snprintf(b, sizeof b, "%f", x);
  return b;
}
std::string fmt_g(double x) {
  char b[48];
  std::snprintf(b, sizeof b, "%.10g", x);
  return b;
}
void write_text(const std::string &path, const std::string &text, const char *who) {
  std::FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) throw RuntimeError(std::string(who) + ": cannot write " + path);
  const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
  if (std::fclose(f) != 0 || !ok) throw RuntimeError(std::string(who) + ": cannot write " + path);
}
}  // namespace lmw

namespace {
thread_local std::string g_err;

template <class F> int guard(F &&fn) {
  try {
    fn();
    g_err.clear();
    return LMW_OK;
  } catch (const lmw::DeviceError &e) {
    g_err = e.what();
    return LMW_DEVICE_ERROR;
  } catch (const std::invalid_argument &e) {
    g_err = e.what();
    return LMW_INVALID_ARGUMENT;
  } catch (const std::bad_alloc &) {
    g_err = "out of host memory";
    return LMW_RUNTIME_ERROR;
  } catch (const std::exception &e) {
    g_err = e.what();
    return LMW_RUNTIME_ERROR;
  }
}

void need(bool ok, const char *msg) {
  if (!ok) throw lmw::InvalidArgument(msg);
}
}  // namespace

int lmw::run_guarded(const std::function<void()> &fn) { return guard(fn); }

extern "C" {

const char *lmw_last_error(void) { return g_err.c_str(); }
const char *lmw_version(void) { return "lmweather-gb300 0.1.0"; }
uint64_t lmw_launch_count(void) { return lmw::g_launches; }
uint64_t lmw_alloc_count(void) { return lmw::alloc_counter().load(); }
int lmw_profiler_range(int on) {
  return guard([&] { LMW_CUDA(on ? cudaProfilerStart() : cudaProfilerStop()); });
}
int lmw_tc_gemm_selftest(const float *A, const float *B, float *D, int N, int K, int terms, int layout, int *kernel_status) {
  return guard([&] {
    need(A && B && D && kernel_status, "pointer is null");
    *kernel_status = lmw::tc_gemm_selftest(A, B, D, N, K, terms, layout);
  });
}
int lmw_conversion_selftest(const uint32_t *f, int nf, const uint64_t *x, int nx, int *mismatches) {
  return guard([&] {
    need(mismatches != nullptr && (nf == 0 || f != nullptr) && (nx == 0 || x != nullptr), "null buffer");
    lmw::conversion_selftest_run(f, nf, x, nx, mismatches);
  });
}
int lmw_division_selftest(const uint64_t *x, int nx, const double *divisors, int nd, long long *counts) {
  return guard([&] {
    need(counts != nullptr && (nx == 0 || x != nullptr) && (nd == 0 || divisors != nullptr), "null buffer");
    lmw::division_selftest_run(x, nx, divisors, nd, counts);
  });
}
int lmw_wait_selftest(int timeout_us, int *completed, int *ran_out) {
  return guard([&] {
    need(completed != nullptr && ran_out != nullptr, "null buffer");
    lmw::wait_selftest_run(timeout_us, completed, ran_out);
  });
}

// ------------------------------------------------------------------------------------------------ sphere
static int create_sphere(int truncation, double radius, double omega, double gravity, double diffusion, int precision, int members,
                         int max_truncation, int split_terms, lmw_sphere **out) {
  return guard([&] {
    need(out != nullptr, "output handle pointer is null");
    *out = nullptr;
    lmw::SphereConfig c;
    c.truncation = truncation;
    c.radius = radius;
    c.omega = omega;
    c.gravity = gravity;
    c.diffusion = diffusion;
    c.precision = precision;
    c.members = members;
    c.max_truncation = max_truncation;
    c.split_terms = split_terms;
    need(max_truncation >= 4 && max_truncation <= 341, "the truncation cap must be between 4 and 341");
    auto *h = new lmw_sphere{nullptr};
    try {
      h->e = new lmw::SphereEngine(c);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int lmw_sphere_create_ex(int truncation, double radius, double omega, double gravity, double diffusion, int precision, int members,
                         int max_truncation, lmw_sphere **out) {
  return create_sphere(truncation, radius, omega, gravity, diffusion, precision, members, max_truncation, 3, out);
}
int lmw_sphere_create_split(int truncation, double radius, double omega, double gravity, double diffusion, int members, int max_truncation,
                            int split_terms, lmw_sphere **out) {
  return create_sphere(truncation, radius, omega, gravity, diffusion, LMW_SPLIT_BF16, members, max_truncation, split_terms, out);
}
int lmw_sphere_create(int truncation, double radius, double omega, double gravity, double diffusion, lmw_sphere **out) {
  return lmw_sphere_create_ex(truncation, radius, omega, gravity, diffusion, LMW_FP64, 1, 170, out);
}
int lmw_sphere_destroy(lmw_sphere *s) {
  return guard([&] {
    if (!s) return;
    delete s->e;
    delete s;
  });
}

#define SPH(...)                                                 \
  guard([&] {                                                    \
    need(s != nullptr && s->e != nullptr, "null sphere handle"); \
    __VA_ARGS__;                                                 \
  })

int lmw_sphere_dims(const lmw_sphere *s, int *truncation, int *nlat, int *nlon, int *members) {
  return SPH({
    if (truncation) *truncation = s->e->N;
    if (nlat) *nlat = s->e->nlat;
    if (nlon) *nlon = s->e->nlon;
    if (members) *members = s->e->B;
  });
}
int lmw_sphere_gauss(const lmw_sphere *s, double *mu, double *w) {
  return SPH({
    std::vector<double> x, ww;
    lmw::gauss_legendre(s->e->nlat, x, ww);
    if (mu) std::copy(x.begin(), x.end(), mu);
    if (w) std::copy(ww.begin(), ww.end(), w);
  });
}
int lmw_sphere_analyze_scalar(lmw_sphere *s, const double *grid, size_t n, double *spec) {
  return SPH({
    need(grid && spec, "grid or spectrum pointer is null");
    s->e->analyze_scalar(grid, n, spec);
  });
}
int lmw_sphere_synthesize_scalar(lmw_sphere *s, const double *spec, double *grid, size_t n) {
  return SPH({
    need(grid && spec, "grid or spectrum pointer is null");
    s->e->synthesize_scalar(spec, grid, n);
  });
}
int lmw_sphere_analyze_divergence(lmw_sphere *s, const double *A, const double *B, size_t n, double *spec) {
  return SPH({
    need(A && B && spec, "grid or spectrum pointer is null");
    s->e->analyze_divergence(A, B, n, spec);
  });
}
int lmw_sphere_time(const lmw_sphere *s, int member, double *out) {
  return SPH({
    need(member >= 0 && member < s->e->B, "member index out of range");
    *out = s->e->t[member];
  });
}
int lmw_sphere_set_state_grid(lmw_sphere *s, int member, const double *h, const double *u, const double *v, size_t n) {
  return SPH({
    need(h && u && v, "grid pointer is null");
    s->e->set_state_grid(h, u, v, n, member);
  });
}
int lmw_sphere_set_axis_tilt(lmw_sphere *s, int member, double alpha) { return SPH(s->e->set_axis_tilt(alpha, member)); }
int lmw_sphere_set_omega(lmw_sphere *s, int member, double omega) { return SPH(s->e->set_omega(omega, member)); }
int lmw_sphere_set_diffusion(lmw_sphere *s, double nu4) { return SPH(s->e->set_diffusion(nu4)); }
int lmw_sphere_set_orography_grid(lmw_sphere *s, int member, const double *hs, size_t n) {
  return SPH({
    need(hs != nullptr, "grid pointer is null");
    s->e->set_orography(hs, n, member);
  });
}
int lmw_sphere_probe(lmw_sphere *s, int member, int which, double lat, double lon, double *out) {
  return SPH({
    need(out != nullptr, "null buffer");
    *out = s->e->probe(which, lat, lon, member);
  });
}
int lmw_sphere_mode_coefficient(lmw_sphere *s, int member, int n, int m, int imag, double *out) {
  return SPH({
    need(out != nullptr, "null buffer");
    *out = s->e->mode_coefficient(n, m, imag != 0, member);
  });
}
int lmw_sphere_wave_crest(lmw_sphere *s, int member, int m, double lat, double *out) {
  return SPH({
    need(out != nullptr, "null buffer");
    *out = s->e->wave_crest(m, lat, member);
  });
}
int lmw_sphere_set_tracer_grid(lmw_sphere *s, int member, const double *q, size_t n) {
  return SPH({
    need(q != nullptr, "grid pointer is null");
    s->e->set_tracer_grid(q, n, member);
  });
}
int lmw_sphere_set_advect_only(lmw_sphere *s, int on) { return SPH(s->e->set_advect_only(on != 0)); }
int lmw_sphere_tracer_state(lmw_sphere *s, int member, double *q) {
  return SPH({
    need(q != nullptr, "null buffer");
    s->e->tracer_state(q, member);
  });
}
int lmw_sphere_set_tracer_state(lmw_sphere *s, int member, const double *q) {
  return SPH({
    need(q != nullptr, "null buffer");
    s->e->set_tracer_state(q, member);
  });
}
int lmw_sphere_tracer_grid(lmw_sphere *s, int member, double *out, size_t n) {
  return SPH({
    need(out != nullptr, "null buffer");
    if (n != s->e->ngrid()) throw lmw::InvalidArgument("grid size mismatch");
    s->e->tracer_grid(out, member);
  });
}
int lmw_sphere_tracer_diagnostics(lmw_sphere *s, int member, double *out) {
  return SPH({
    need(out != nullptr, "null buffer");
    s->e->tracer_diagnostics(out, member);
  });
}
int lmw_sphere_add_mode(lmw_sphere *s, int member, int n, int m, double amplitude, double mean_depth) {
  return SPH(s->e->add_mode(n, m, amplitude, mean_depth, member));
}
int lmw_sphere_perturb(lmw_sphere *s, int member, double amplitude, uint64_t seed, int max_wave) {
  return SPH(s->e->perturb(amplitude, seed, max_wave, member));
}
int lmw_sphere_mark_reference(lmw_sphere *s, int member) { return SPH(s->e->mark_reference(member)); }
int lmw_sphere_turbulence(lmw_sphere *s, int member, uint64_t seed, double mean_height, double max_wind, int nforce) {
  return SPH(s->e->turbulence(seed, mean_height, max_wind, nforce, member));
}
int lmw_sphere_get_state(lmw_sphere *s, int member, double *zeta, double *delta, double *phi) {
  return SPH(s->e->get_state(zeta, delta, phi, member));
}
int lmw_sphere_set_state(lmw_sphere *s, int member, const double *zeta, const double *delta, const double *phi, double time) {
  return SPH({
    need(zeta && delta && phi, "state pointer is null");
    s->e->set_state(zeta, delta, phi, time, member);
  });
}
int lmw_sphere_step(lmw_sphere *s, double dt) { return SPH(s->e->step(dt)); }
int lmw_sphere_run(lmw_sphere *s, double seconds, double dt) { return SPH(s->e->run(seconds, dt)); }
int lmw_sphere_stable_dt(lmw_sphere *s, int member, double safety, double *out) {
  return SPH({
    need(member >= 0 && member < s->e->B, "member index out of range");
    *out = s->e->stable_dt(safety, member);
  });
}
int lmw_sphere_diagnostics(lmw_sphere *s, int member, double *out) { return SPH(s->e->diagnostics(out, member)); }
int lmw_sphere_grid(lmw_sphere *s, int member, int which, double *out, size_t n) {
  return SPH({
    need(n == s->e->ngrid(), "grid size mismatch");
    s->e->grid(which, out, member);
  });
}
int lmw_sphere_spectrum(lmw_sphere *s, int member, double *ke, double *pe) {
  return SPH({
    need(member >= 0 && member < s->e->B, "member index out of range");
    s->e->spectrum(ke, pe, member);
  });
}
int lmw_sphere_save_csv(lmw_sphere *s, int member, const char *path) {
  return SPH({
    need(path != nullptr, "Sphere.save_csv: no path");
    s->e->save_csv(path, member);
  });
}
int lmw_sphere_save_zonal_mean(lmw_sphere *s, int member, const char *path) {
  return SPH({
    need(path != nullptr, "Sphere.save_zonal_mean: no path");
    s->e->save_zonal_mean(path, member);
  });
}
int lmw_sphere_save_spectrum(lmw_sphere *s, int member, const char *path) {
  return SPH({
    need(path != nullptr, "Sphere.save_spectrum: no path");
    s->e->save_spectrum(path, member);
  });
}

int lmw_sphere_stream(const lmw_sphere *s, void **stream) { return SPH(*stream = static_cast<void *>(s->e->stream)); }
int lmw_sphere_kernel_times(lmw_sphere *s, double dt, int reps, double *ms) {
  return SPH({
    need(reps > 0, "reps must be positive");
    s->e->kernel_times(dt, reps, ms);
  });
}

// ------------------------------------------------------------------------------------------------ plane
int lmw_plane_create(int nx, int ny, double lx, double ly, double gravity, double depth, double f0, double beta, double viscosity,
                     double drag, int linear, lmw_plane **out) {
  return guard([&] {
    need(out != nullptr, "output handle pointer is null");
    *out = nullptr;
    lmw::PlaneConfig c;
    c.nx = nx;
    c.ny = ny;
    c.lx = lx;
    c.ly = ly;
    c.gravity = gravity;
    c.depth = depth;
    c.f0 = f0;
    c.beta = beta;
    c.viscosity = viscosity;
    c.drag = drag;
    c.linear = linear != 0;
    auto *h = new lmw_plane{nullptr};
    try {
      h->e = new lmw::PlaneEngine(c);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int lmw_plane_destroy(lmw_plane *p) {
  return guard([&] {
    if (!p) return;
    delete p->e;
    delete p;
  });
}

#define PLN(...)                                                \
  guard([&] {                                                   \
    need(p != nullptr && p->e != nullptr, "null plane handle"); \
    __VA_ARGS__;                                                \
  })

int lmw_plane_set_params(lmw_plane *p, double gravity, double depth, double f0, double beta, double viscosity, double drag, int linear) {
  return PLN({
    p->e->p.gravity = gravity;
    p->e->p.depth = depth;
    p->e->p.f0 = f0;
    p->e->p.beta = beta;
    p->e->p.viscosity = viscosity;
    p->e->p.drag = drag;
    p->e->p.linear = linear != 0;
  });
}
int lmw_plane_reset(lmw_plane *p) { return PLN(p->e->reset()); }
int lmw_plane_set_h(lmw_plane *p, const double *h, size_t n) {
  return PLN({
    need(h != nullptr, "grid pointer is null");
    p->e->set_h(h, n);
  });
}
int lmw_plane_set_u(lmw_plane *p, const double *u, size_t n) {
  return PLN({
    need(u != nullptr, "grid pointer is null");
    p->e->set_u(u, n);
  });
}
int lmw_plane_set_v(lmw_plane *p, const double *v, size_t n) {
  return PLN({
    need(v != nullptr, "grid pointer is null");
    p->e->set_v(v, n);
  });
}
int lmw_plane_get(lmw_plane *p, double *h, double *u, double *v) { return PLN(p->e->get(h, u, v)); }
int lmw_plane_perturb(lmw_plane *p, double amplitude, uint64_t seed) { return PLN(p->e->perturb(amplitude, seed)); }
int lmw_plane_jet(lmw_plane *p, double u0, double width, double noise_rms, uint64_t seed) {
  return PLN(p->e->jet(u0, width, noise_rms, seed));
}
int lmw_plane_step(lmw_plane *p, double dt) { return PLN(p->e->step(dt)); }
int lmw_plane_run(lmw_plane *p, double seconds, double dt) { return PLN(p->e->run(seconds, dt)); }
int lmw_plane_stable_dt(lmw_plane *p, double safety, double *out) { return PLN(*out = p->e->stable_dt(safety)); }
int lmw_plane_time(const lmw_plane *p, double *out) { return PLN(*out = p->e->t); }
int lmw_plane_diagnostics(lmw_plane *p, double *out) { return PLN(p->e->diagnostics(out)); }
int lmw_plane_probe(lmw_plane *p, int kind, double x, double y, double *out) { return PLN(*out = p->e->probe(kind, x, y)); }
int lmw_plane_zeta_at_corner(lmw_plane *p, int i, int j, double *out) { return PLN(*out = p->e->zeta_at_corner(i, j)); }
int lmw_plane_zonal_amplitude(lmw_plane *p, int m, int j, double *out) { return PLN(*out = p->e->zonal_amplitude(m, j)); }
int lmw_plane_zonal_crest(lmw_plane *p, int m, int j, double *out) { return PLN(*out = p->e->zonal_crest(m, j)); }
int lmw_plane_v_zonal_crest(lmw_plane *p, int m, int j, double *out) { return PLN(*out = p->e->v_zonal_crest(m, j)); }
int lmw_plane_harmonic_energy(lmw_plane *p, int m, double *out) { return PLN(*out = p->e->harmonic_energy(m)); }
int lmw_plane_save_csv(lmw_plane *p, const char *path) {
  return PLN({
    need(path != nullptr, "Plane.save_csv: no path");
    p->e->save_csv(path);
  });
}
int lmw_plane_save_row(lmw_plane *p, int j, const char *path) {
  return PLN({
    need(path != nullptr, "Plane.save_row: no path");
    p->e->save_row(j, path);
  });
}
int lmw_plane_save_column(lmw_plane *p, int i, const char *path) {
  return PLN({
    need(path != nullptr, "Plane.save_column: no path");
    p->e->save_column(i, path);
  });
}
int lmw_plane_step_noalloc(int nx, int ny, double lx, double ly, double gravity, double depth, double f0, double beta,
                           double viscosity, double drag, int linear, double *h, double *u, double *v, double dt, int steps,
                           void *stream) {
  return guard([&] {
    lmw::PlaneConfig c;
    c.nx = nx;
    c.ny = ny;
    c.lx = lx;
    c.ly = ly;
    c.gravity = gravity;
    c.depth = depth;
    c.f0 = f0;
    c.beta = beta;
    c.viscosity = viscosity;
    c.drag = drag;
    c.linear = linear != 0;
    lmw::plane_step_noalloc(c, h, u, v, dt, steps, static_cast<cudaStream_t>(stream));
  });
}
int lmw_plane_stream(const lmw_plane *p, void **stream) { return PLN(*stream = static_cast<void *>(p->e->stream)); }
int lmw_plane_kernel_time(lmw_plane *p, double dt, int reps, double *ms) {
  return PLN({
    need(reps > 0, "reps must be positive");
    *ms = p->e->kernel_time(dt, reps);
  });
}

// ------------------------------------------------------------------------------------------------ ensemble
int lmw_ensemble_create(int count, const int *truncation, const uint64_t *seed, const double *mean_height, const double *omega, double radius,
                        double gravity, double max_wind, int precision, int split_terms, lmw_ensemble **out) {
  return guard([&] {
    need(out != nullptr, "output handle pointer is null");
    *out = nullptr;
    need(count > 0 && truncation && seed && mean_height && omega, "member arrays are missing");
    std::vector<lmw::MemberSpec> specs(count);
    for (int i = 0; i < count; i++) {
      specs[i].truncation = truncation[i];
      specs[i].seed = seed[i];
      specs[i].mean_height = mean_height[i];
      specs[i].omega = omega[i];
    }
    auto *h = new lmw_ensemble{nullptr};
    try {
      h->e = new lmw::EnsembleEngine(specs, radius, gravity, max_wind, precision, split_terms);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int lmw_ensemble_destroy(lmw_ensemble *e) {
  return guard([&] {
    if (!e) return;
    delete e->e;
    delete e;
  });
}
#define ENS(...)                                                   \
  guard([&] {                                                      \
    need(e != nullptr && e->e != nullptr, "null ensemble handle"); \
    __VA_ARGS__;                                                   \
  })
int lmw_ensemble_run(lmw_ensemble *e, double seconds) { return ENS(e->e->run(seconds)); }
int lmw_ensemble_groups(lmw_ensemble *e, int *ngroups, int *truncations, int *counts, double *last_dt, int64_t *last_steps) {
  return ENS({
    const int G = static_cast<int>(e->e->groups.size());
    if (ngroups) *ngroups = G;
    for (int g = 0; g < G; g++) {
      if (truncations) truncations[g] = e->e->truncations[g];
      if (counts) counts[g] = e->e->groups[g]->B;
      if (last_dt) last_dt[g] = e->e->last_dt[g];
      if (last_steps) last_steps[g] = e->e->last_steps[g];
    }
  });
}
int lmw_ensemble_get_states(lmw_ensemble *e, double *zeta, double *delta, double *phi) {
  return guard([&] {
    need(e != nullptr && e->e != nullptr, "null ensemble handle");
    need(zeta != nullptr && delta != nullptr && phi != nullptr, "null buffer");
    e->e->get_states(zeta, delta, phi);
  });
}
int lmw_ensemble_set_states(lmw_ensemble *e, const double *zeta, const double *delta, const double *phi) {
  return guard([&] {
    need(e != nullptr && e->e != nullptr, "null ensemble handle");
    need(zeta != nullptr && delta != nullptr && phi != nullptr, "null buffer");
    e->e->set_states(zeta, delta, phi);
  });
}
int lmw_ensemble_member_state(lmw_ensemble *e, int member, double *zeta, double *delta, double *phi) {
  return ENS({
    int k = 0;
    e->e->engine_of(member, &k).get_state(zeta, delta, phi, k);
  });
}
int lmw_ensemble_member_set_state(lmw_ensemble *e, int member, const double *zeta, const double *delta, const double *phi) {
  return ENS({
    need(zeta && delta && phi, "state pointer is null");
    int k = 0;
    lmw::SphereEngine &s = e->e->engine_of(member, &k);
    s.set_state(zeta, delta, phi, s.t[k], k);
  });
}
int lmw_ensemble_member_diagnostics(lmw_ensemble *e, int member, double *out) {
  return ENS({
    int k = 0;
    e->e->engine_of(member, &k).diagnostics(out, k);
  });
}
int lmw_ensemble_stream(lmw_ensemble *e, int group, void **stream) {
  return ENS({
    need(group >= 0 && group < static_cast<int>(e->e->groups.size()), "group index out of range");
    *stream = static_cast<void *>(e->e->groups[group]->stream);
  });
}
int lmw_ensemble_kernel_times(lmw_ensemble *e, int group, int reps, double *ms) {
  return ENS({
    need(group >= 0 && group < static_cast<int>(e->e->groups.size()), "group index out of range");
    need(reps > 0, "reps must be positive");
    lmw::SphereEngine &g = *e->e->groups[group];
    const double dt = e->e->last_dt[group] > 0 ? e->e->last_dt[group] : 300.0;
    g.kernel_times(dt, reps, ms);
  });
}
int lmw_ensemble_member_grid(lmw_ensemble *e, int member, int which, double *out, size_t n) {
  return ENS({
    int k = 0;
    lmw::SphereEngine &s = e->e->engine_of(member, &k);
    need(n == s.ngrid(), "grid size mismatch");
    s.grid(which, out, k);
  });
}


// ------------------------------------------------------------------------------------------------ surrogate
int lmw_mlp_create(int in_dim, int hidden, int out_dim, int max_batch, uint64_t seed, double last_layer_scale, lmw_mlp **out) {
  return guard([&] {
    need(out != nullptr, "null output pointer");
    *out = nullptr;
    auto *h = new lmw_mlp{nullptr};
    try {
      h->m = new lmw::Mlp(in_dim, hidden, out_dim, max_batch, seed, last_layer_scale);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int lmw_mlp_destroy(lmw_mlp *m) {
  return guard([&] {
    if (!m) return;
    delete m->m;
    delete m;
  });
}
#define MLP(m, ...)                                           \
  guard([&] {                                                 \
    need((m) != nullptr && (m)->m != nullptr, "null network"); \
    __VA_ARGS__;                                              \
  })
int lmw_mlp_set_layer(lmw_mlp *m, int layer, const float *w, const float *b) {
  return MLP(m, need(w != nullptr, "null weights"); m->m->set_layer(layer, w, b));
}
int lmw_mlp_get_layer(lmw_mlp *m, int layer, float *w, float *b) {
  return MLP(m, need(w != nullptr, "null weights"); m->m->get_layer(layer, w, b));
}
int lmw_mlp_forward(lmw_mlp *m, const float *x, int batch, float *y) {
  return MLP(m, need(x != nullptr && y != nullptr, "null buffer"); m->m->upload_input(x, batch); m->m->forward(batch); m->m->check_status();
             m->m->download_output(y, batch));
}
int lmw_mlp_backward(lmw_mlp *m, const float *x, const float *target, const float *mask, int batch, double *loss) {
  return MLP(m, need(x != nullptr && target != nullptr, "null buffer"); m->m->upload_input(x, batch); m->m->upload_target(target, mask, batch);
             m->m->take_loss(); m->m->forward(batch); m->m->backward(batch); const double l = m->m->take_loss(); if (loss) *loss = l);
}
int lmw_mlp_get_grad(lmw_mlp *m, int layer, float *gw, float *gb) {
  return MLP(m, need(gw != nullptr, "null gradient buffer"); m->m->get_grad(layer, gw, gb));
}
int lmw_mlp_adam(lmw_mlp *m, double lr, double beta1, double beta2, double eps) {
  return MLP(m, m->m->adam(lr, beta1, beta2, eps); m->m->check_status());
}
int lmw_mlp_time(lmw_mlp *m, int batch, int reps, double *train_ms, double *forward_ms) {
  return MLP(m, need(reps > 0, "reps must be positive"); const double a = m->m->time_train_step(batch, reps);
             const double f = m->m->time_forward(batch, reps); if (train_ms) *train_ms = a; if (forward_ms) *forward_ms = f);
}
int lmw_gemm_bf16(const float *a, const float *b, int M, int N, int K, float *c) {
  return guard([&] {
    need(a != nullptr && b != nullptr && c != nullptr, "null buffer");
    need(M > 0 && N > 0 && K > 0 && M % 128 == 0 && N % 128 == 0 && K % 64 == 0, "M, N must be multiples of 128 and K of 64");
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) throw lmw::DeviceError("no CUDA device");
    cudaStream_t s;
    LMW_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    lmw::DevBuf<__nv_bfloat16> A, B;
    lmw::DevBuf<float> C;
    lmw::DevBuf<int> err;
    A.alloc(static_cast<size_t>(M) * K);
    B.alloc(static_cast<size_t>(N) * K);
    C.alloc(static_cast<size_t>(M) * N);
    err.alloc(1);
    err.zero(s);
    lmw::to_blocked(a, M, K, M, K, A.p, s);
    lmw::to_blocked(b, N, K, N, K, B.p, s);
    lmw::mlp_gemm_f32(A.p, B.p, M, N, K, C.p, N, nullptr, err.p, s);
    int e = 0;
    LMW_CUDA(cudaMemcpyAsync(c, C.p, C.bytes(), cudaMemcpyDeviceToHost, s));
    LMW_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    LMW_CUDA(cudaStreamSynchronize(s));
    cudaStreamDestroy(s);
    if (e) throw lmw::RuntimeError("the tensor-core GEMM timed out waiting on its pipeline");
  });
}

int lmw_surrogate_create(int truncation, int hidden, uint64_t seed, double window_seconds, double dt, double radius, double omega, double gravity,
                         lmw_surrogate **out) {
  return guard([&] {
    need(out != nullptr, "null output pointer");
    *out = nullptr;
    auto *h = new lmw_surrogate{nullptr};
    try {
      h->s = new lmw::Surrogate(truncation, hidden, seed, window_seconds, dt, radius, omega, gravity);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}
int lmw_surrogate_destroy(lmw_surrogate *s) {
  return guard([&] {
    if (!s) return;
    delete s->s;
    delete s;
  });
}
#define SUR(s, ...)                                             \
  guard([&] {                                                   \
    need((s) != nullptr && (s)->s != nullptr, "null surrogate"); \
    __VA_ARGS__;                                                \
  })
int lmw_surrogate_dims(lmw_surrogate *s, int *dims) {
  return SUR(s, need(dims != nullptr, "null buffer"); dims[0] = s->s->nfeat; dims[1] = s->s->net->dim[0]; dims[2] = s->s->net->hidden);
}
int lmw_surrogate_generate(lmw_surrogate *s, int trajectories, int windows, uint64_t seed0, double hmin, double hmax, int precision,
                           double *seconds) {
  return SUR(s, need(precision >= 0 && precision <= 2, "precision must be 0 (FP64), 1 (FP32) or 2 (split BF16)");
             s->s->generate(trajectories, windows, seed0, hmin, hmax, precision, 1024); if (seconds) *seconds = s->s->gen_seconds);
}
int lmw_surrogate_generate_drifted(lmw_surrogate *s, int trajectories, int net_windows, uint64_t seed0, double hmin, double hmax, int precision,
                                   double *seconds) {
  return SUR(s, need(precision >= 0 && precision <= 2, "precision must be 0 (FP64), 1 (FP32) or 2 (split BF16)");
             s->s->generate_drifted(trajectories, net_windows, seed0, hmin, hmax, precision, 1024); if (seconds) *seconds = s->s->gen_seconds);
}
int lmw_surrogate_fit(lmw_surrogate *s, int epochs, int batch, double lr, double lr_min, double val_fraction, uint64_t shuffle_seed,
                      int loss_mode, double *stats) {
  return SUR(s, need(loss_mode == 0 || loss_mode == 1, "loss mode must be 0 or 1");
             if (s->s->loss_mode != loss_mode) s->s->have_norm = false; s->s->loss_mode = loss_mode;
             const lmw::SurrogateStats st = s->s->fit(epochs, batch, lr, lr_min, val_fraction, shuffle_seed); if (stats) {
    stats[0] = st.train_loss;
    stats[1] = st.val_err_mean;
    stats[2] = st.val_err_median;
    stats[3] = st.val_err_p90;
    stats[4] = st.val_err_max;
    stats[5] = st.val_persist_mean;
    stats[6] = st.val_untrained_mean;
    stats[7] = st.seconds;
    stats[8] = st.steps;
  });
}
int lmw_surrogate_evaluate(lmw_surrogate *s, int first, int count, double *err, double *persistence) {
  return SUR(s, need(err != nullptr && persistence != nullptr, "null buffer"); need(count > 0, "count must be positive"); std::vector<double> e, p;
             s->s->evaluate(first, first + count, e, p); std::copy(e.begin(), e.end(), err); std::copy(p.begin(), p.end(), persistence));
}
int lmw_surrogate_advance(lmw_surrogate *s, int count, double *states) {
  return SUR(s, need(states != nullptr, "null buffer"); need(count > 0, "count must be positive"); lmw::DevBuf<double> d;
             const size_t n = static_cast<size_t>(count) * s->s->nfeat; d.alloc(n);
             LMW_CUDA(cudaMemcpyAsync(d.p, states, n * sizeof(double), cudaMemcpyHostToDevice, s->s->stream));
             s->s->advance_states(d.p, count, nullptr);
             LMW_CUDA(cudaMemcpyAsync(states, d.p, n * sizeof(double), cudaMemcpyDeviceToHost, s->s->stream));
             LMW_CUDA(cudaStreamSynchronize(s->s->stream)); s->s->net->check_status());
}
int lmw_surrogate_rollout(lmw_surrogate *s, int members, uint64_t seed0, double hmin, double hmax, int windows, int check_every, double threshold,
                          int check_precision, int ref_windows, double *out, double *window_err, double *final_states) {
  return SUR(s, need(out != nullptr, "null buffer"); need(check_precision >= 0 && check_precision <= 2, "check precision must be 0, 1 or 2");
             s->s->rollout(members, seed0, hmin, hmax, windows, check_every, threshold, check_precision, ref_windows, out, window_err,
                           final_states));
}
int lmw_surrogate_time(lmw_surrogate *s, int batch, int reps, double *train_ms, double *forward_ms) {
  return SUR(s, need(reps > 0, "reps must be positive"); need(s->s->ntraj > 0, "no training data yet");
             const double a = s->s->net->time_train_step(batch, reps); const double f = s->s->net->time_forward(batch, reps);
             if (train_ms) *train_ms = a; if (forward_ms) *forward_ms = f);
}

}  // extern "C"

extern "C" {
int lmw_sphere_split_plan(lmw_sphere *s, int *out) {
  return guard([&] {
    need(s != nullptr && s->e != nullptr, "null sphere handle");
    need(out != nullptr, "null buffer");
    s->e->split_plan(out);
  });
}
int lmw_sphere_inject_split_error(lmw_sphere *s, int code) {
  return guard([&] {
    need(s != nullptr && s->e != nullptr, "null sphere handle");
    s->e->inject_split_error(code);
  });
}
int lmw_sphere_set_split_plan(lmw_sphere *s, const int *plan) {
  return guard([&] {
    need(s != nullptr && s->e != nullptr, "null sphere handle");
    need(plan != nullptr, "null buffer");
    s->e->set_split_plan(plan);
  });
}
int lmw_sphere_set_split_form(lmw_sphere *s, int linear_exact) {
  return guard([&] {
    need(s != nullptr && s->e != nullptr, "null sphere handle");
    s->e->set_split_form(linear_exact);
  });
}
int lmw_ensemble_set_split_form(lmw_ensemble *e, int linear_exact) {
  return guard([&] {
    need(e != nullptr && e->e != nullptr, "null ensemble handle");
    for (auto &g : e->e->groups) g->set_split_form(linear_exact);
  });
}
int lmw_ensemble_split_plan(lmw_ensemble *e, int group, int *out) {
  return guard([&] {
    need(e != nullptr && e->e != nullptr, "null ensemble handle");
    need(out != nullptr, "null buffer");
    need(group >= 0 && group < static_cast<int>(e->e->groups.size()), "group index out of range");
    e->e->groups[group]->split_plan(out);
  });
}
int lmw_surrogate_reset(lmw_surrogate *s, uint64_t seed) { return SUR(s, s->s->reset(seed)); }
int lmw_surrogate_set_augment(lmw_surrogate *s, int on) { return SUR(s, s->s->augment = on != 0); }
int lmw_surrogate_set_symmetry_average(lmw_surrogate *s, int maps) {
  return SUR(s, need(maps == 1 || (maps >= 2 && maps <= 64 && maps % 2 == 0), "the symmetry maps must be 1 or an even number up to 64");
             s->s->sym_average = maps);
}
int lmw_surrogate_set_kinetic_weight(lmw_surrogate *s, double weight) {
  return SUR(s, need(weight > 0 && weight <= 16, "the kinetic-energy weight must lie in (0, 16]"); need(!s->s->have_norm, "set the loss weights before the first fit");
             s->s->ke_weight = weight);
}
int lmw_surrogate_set_takeover(lmw_surrogate *s, int mode) {
  return SUR(s, need(mode == 0 || mode == 1, "the takeover mode must be 0 (member) or 1 (window)"); s->s->takeover_mode = mode);
}
int lmw_surrogate_set_averaging(lmw_surrogate *s, double decay) {
  return SUR(s, need(decay >= 0 && decay < 1, "the averaging decay must lie in [0, 1)"); s->s->ema = decay);
}
int lmw_surrogate_set_clip(lmw_surrogate *s, double ratio) {
  return SUR(s, need(ratio >= 0, "the clipping ratio must not be negative"); s->s->clip_ratio = ratio);
}
int lmw_surrogate_history(lmw_surrogate *s, int max, double *loss, double *grad_norm, int *count) {
  return SUR(s, need(count != nullptr, "null buffer"); const int n = static_cast<int>(s->s->hist_loss.size()); *count = n;
             for (int i = 0; i < n && i < max; i++) {
               if (loss) loss[i] = s->s->hist_loss[i];
               if (grad_norm) grad_norm[i] = s->s->hist_gnorm[i];
             });
}
}  // extern "C"
