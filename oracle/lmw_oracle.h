/* CPU oracle for the lmweather shallow-water time stepping.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference numerical core
 * (lmweather cpp/sphere.cpp and cpp/plane.cpp), written operation for operation in the reference's
 * order of evaluation so that, built with -ffp-contract=off, it reproduces the reference bit for bit.
 * It is pinned against the reference itself (oracle/_ref, compiled from the reference sources by
 * oracle/Makefile) and against the golden fixtures in tests/golden/. Only tests/, the smoke check
 * and bench.py's CPU-baseline leg may load it. The product library never links it.
 *
 * Spectral layout: (T+1)^2 complex values per field, index m*(T+1)+n with n >= m, stored as
 * interleaved (re, im) doubles. Grids: row-major [nlat][nlon], latitudes south to north.
 * Plane: h, u are [ny][nx]; v is [ny+1][nx] with rows 0 and ny on the walls.
 */
#ifndef LMW_ORACLE_H
#define LMW_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ free functions */
/* in-place radix-2 complex FFT of n interleaved complex values; returns 0, or 1 if n is not a power of two */
int or_fft(double *a, int n, int sign);
void or_gauss_legendre(int n, double *x, double *w);
/* out has nmax + 2 - m entries */
void or_legendre_column(int m, int nmax, double mu, double *out);

/* ------------------------------------------------------------------ sphere */
typedef struct or_sphere or_sphere;
/* returns NULL (and writes err) outside 4..max_truncation; max_truncation 170 mirrors the reference, larger lifts the cap */
or_sphere *or_sphere_new(int T, double radius, double omega, double gravity, double diffusion, int max_truncation);
void or_sphere_free(or_sphere *s);
int or_sphere_nlat(const or_sphere *s);
int or_sphere_nlon(const or_sphere *s);
double or_sphere_time(const or_sphere *s);
const double *or_sphere_mu(const or_sphere *s);
const double *or_sphere_w(const or_sphere *s);
void or_sphere_set_diffusion(or_sphere *s, double nu4);
void or_sphere_set_axis_tilt(or_sphere *s, double alpha);
int or_sphere_set_state_grid(or_sphere *s, const double *h, const double *u, const double *v);
void or_sphere_set_orography_grid(or_sphere *s, const double *hs);
void or_sphere_set_tracer_grid(or_sphere *s, const double *q);
void or_sphere_set_advect_only(or_sphere *s, int on);
void or_sphere_mark_reference(or_sphere *s);
int or_sphere_add_mode(or_sphere *s, int n, int m, double amplitude, double mean_depth);
int or_sphere_perturb(or_sphere *s, double amplitude, uint64_t seed, int max_wave);
/* spectral state in/out; q may be NULL */
void or_sphere_get_state(const or_sphere *s, double *zeta, double *delta, double *phi, double *q);
void or_sphere_set_state(or_sphere *s, const double *zeta, const double *delta, const double *phi, double t);
void or_sphere_step(or_sphere *s, double dt);
/* 0 ok, 1 invalid_argument, 2 runtime_error; the message goes to err (the reference's text) */
int or_sphere_run(or_sphere *s, double seconds, double dt, char *err, int errlen);
double or_sphere_stable_dt(const or_sphere *s, double safety, int *status);
double or_sphere_mean_height(const or_sphere *s);
double or_sphere_kinetic_energy(const or_sphere *s);
double or_sphere_potential_energy(const or_sphere *s);
double or_sphere_energy(const or_sphere *s);
double or_sphere_potential_enstrophy(const or_sphere *s);
double or_sphere_max_wind(const or_sphere *s);
double or_sphere_height_error_l2(const or_sphere *s);
double or_sphere_height_error_linf(const or_sphere *s);
double or_sphere_tracer_mean(const or_sphere *s);
double or_sphere_tracer_mass(const or_sphere *s);
double or_sphere_tracer_error_l2(const or_sphere *s);
void or_sphere_spectrum(const or_sphere *s, double *ke, double *pe);
void or_sphere_grid_height(const or_sphere *s, double *g);
void or_sphere_grid_u(const or_sphere *s, double *g);
void or_sphere_grid_v(const or_sphere *s, double *g);
void or_sphere_grid_vorticity(const or_sphere *s, double *g);
void or_sphere_grid_tracer(const or_sphere *s, double *g);
void or_sphere_analyze_scalar(const or_sphere *s, const double *grid, double *spec);
void or_sphere_synthesize_scalar(const or_sphere *s, const double *spec, double *grid);
void or_sphere_analyze_divergence(const or_sphere *s, const double *A, const double *B, double *spec);
/* seeded balanced turbulence (grids h, u, v) for the benchmark configurations */
void or_sphere_turbulence_grids(const or_sphere *s, uint64_t seed, double mean_height, double max_wind, int nforce,
                                double *h, double *u, double *v);

/* ------------------------------------------------------------------ plane */
typedef struct or_plane or_plane;
or_plane *or_plane_new(int nx, int ny, double lx, double ly, double gravity, double depth, double f0, double beta,
                       double viscosity, double drag, int linear);
void or_plane_free(or_plane *p);
void or_plane_reset(or_plane *p);
double or_plane_time(const or_plane *p);
void or_plane_get(const or_plane *p, double *h, double *u, double *v);
void or_plane_set(or_plane *p, const double *h, const double *u, const double *v);
void or_plane_perturb(or_plane *p, double amplitude, uint64_t seed);
void or_plane_step(or_plane *p, double dt);
int or_plane_run(or_plane *p, double seconds, double dt, char *err, int errlen);
double or_plane_stable_dt(const or_plane *p, double safety, int *status);
double or_plane_mean_depth(const or_plane *p);
double or_plane_energy(const or_plane *p);
double or_plane_max_speed(const or_plane *p);
double or_plane_pv_anomaly_rms(const or_plane *p);
double or_plane_zeta_at_corner(const or_plane *p, int i, int j);
/* kind: 0 h, 1 u, 2 v */
double or_plane_probe(const or_plane *p, int kind, double x, double y);
void or_plane_row_harmonic(const or_plane *p, int kind, int m, int j, double shift, double *re, double *im);
/* these four return 1 (invalid_argument) when the harmonic or the row is out of range */
int or_plane_zonal_amplitude(const or_plane *p, int m, int j, double *out);
int or_plane_zonal_crest(const or_plane *p, int m, int j, double *out);
int or_plane_v_zonal_crest(const or_plane *p, int m, int j, double *out);
int or_plane_harmonic_energy(const or_plane *p, int m, double *out);
/* geostrophic zonal jet plus white height noise (grids h, u; v = 0) */
void or_plane_jet_grids(const or_plane *p, double u0, double width, double noise_rms, uint64_t seed, double *h, double *u);

#ifdef __cplusplus
}
#endif
#endif
