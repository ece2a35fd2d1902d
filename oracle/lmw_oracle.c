/* CPU oracle for the lmweather shallow-water time stepping (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference numerical core. Every function below names the reference
 * function and lines it follows (paths inside the lmweather project). Expressions keep the reference's
 * order of evaluation, and complex products are spelled out the way std::complex<double> evaluates them
 * ((a+ib)(c+id) = (ac-bd) + i(ad+bc); complex times real scales both parts), so that a build with
 * -ffp-contract=off reproduces the reference bit for bit. Parity is pinned by tests that compare this
 * file with the reference compiled from its own sources (oracle/_ref) and with tests/golden/.
 *
 * The product library never links this file; only tests/, the smoke check and bench.py's CPU-baseline
 * leg load it.
 */
#include "lmw_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static const double kPi = 3.14159265358979323846;

typedef struct { double re, im; } cx;
static inline cx cmk(double re, double im) { cx r; r.re = re; r.im = im; return r; }
static inline cx cmul(cx a, cx b) { return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cx cscale(cx a, double s) { return cmk(a.re * s, a.im * s); }
static inline cx cadd(cx a, cx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cx csub(cx a, cx b) { return cmk(a.re - b.re, a.im - b.im); }
static inline cx cdivr(cx a, double s) { return cmk(a.re / s, a.im / s); }
/* std::complex<double>(0, 1) * static_cast<double>(m) */
static inline cx cim(int m) { return cmk(0.0 * (double)m, 1.0 * (double)m); }

/* cpp/sphere.cpp:11 */
static inline double eps_nm(int n, int m) { return sqrt((double)(n * n - m * m) / (double)(4 * n * n - 1)); }

/* cpp/sphere.cpp:13-18 (identical in cpp/plane.cpp:12-17) */
static uint64_t splitmix(uint64_t *x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
/* Irwin-Hall normal: cpp/sphere.cpp:316-320, cpp/plane.cpp:37-41 */
static double irwin_hall(uint64_t *st) {
  double s = 0;
  for (int i = 0; i < 12; i++) s += (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
  return s - 6.0;
}

/* ================================================================== free functions */

/* cpp/sphere.cpp:21-45 */
int or_fft(double *a, int n, int sign) {
  if (n < 2 || (n & (n - 1))) return 1;
  cx *c = (cx *)a;
  for (int i = 1, j = 0; i < n; i++) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) { cx t = c[i]; c[i] = c[j]; c[j] = t; }
  }
  for (int len = 2; len <= n; len <<= 1) {
    double ang = 2 * kPi / (double)len * (double)sign;
    cx wl = cmk(cos(ang), sin(ang));
    for (int i = 0; i < n; i += len) {
      cx w = cmk(1.0, 0.0);
      for (int k = 0; k < len / 2; k++) {
        if ((k & 15) == 0) w = cmk(cos(ang * (double)k), sin(ang * (double)k));
        cx u = c[i + k], v = cmul(c[i + k + len / 2], w);
        c[i + k] = cadd(u, v);
        c[i + k + len / 2] = csub(u, v);
        w = cmul(w, wl);
      }
    }
  }
  return 0;
}

/* cpp/sphere.cpp:47-64 */
void or_gauss_legendre(int n, double *x, double *w) {
  for (int i = 0; i < n; i++) { x[i] = 0; w[i] = 0; }
  for (int i = 0; i < (n + 1) / 2; i++) {
    double z = cos(kPi * (i + 0.75) / (n + 0.5)), pp = 1;
    for (int it = 0; it < 100; it++) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; j++) { double p3 = p2; p2 = p1; p1 = ((2.0 * j - 1) * z * p2 - (j - 1.0) * p3) / j; }
      pp = n * (z * p1 - p2) / (z * z - 1);
      double dz = p1 / pp;
      z -= dz;
      if (fabs(dz) < 1e-15) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2 / ((1 - z * z) * pp * pp);
  }
}

/* cpp/sphere.cpp:66-73 */
void or_legendre_column(int m, int nmax, double mu, double *out) {
  int len = nmax + 2 - m;
  for (int i = 0; i < len; i++) out[i] = 0.0;
  double omm = 1 - mu * mu;
  double c = sqrt(omm > 0.0 ? omm : 0.0), p = 1 / sqrt(2.0);
  for (int k = 1; k <= m; k++) p *= sqrt((2.0 * k + 1) / (2.0 * k)) * c;
  out[0] = p;
  if (nmax + 1 >= m + 1) out[1] = sqrt(2.0 * m + 3) * mu * p;
  for (int n = m + 2; n <= nmax + 1; n++) out[n - m] = (mu * out[n - 1 - m] - eps_nm(n - 1, m) * out[n - 2 - m]) / eps_nm(n, m);
}

/* ================================================================== sphere */

struct or_sphere {
  int N, nlat, nlon, ntri;
  double radius, omega, gravity, diffusion;
  double t;
  double *mu, *w;
  double *P, *H;          /* [j][tri(m) + n - m] */
  int *tri;               /* offset of wavenumber m inside one latitude's triangle */
  cx *zeta, *delta, *phi, *q;
  int has_tracer, advect_only, has_orography;
  double *ref_phi, *ref_q, *f_grid, *hs_grid;
  /* scratch */
  cx *row;                /* nlon */
};

static inline size_t sidx(const or_sphere *s, int m, int n) { return (size_t)m * (s->N + 1) + n; }
static inline double Ptab(const or_sphere *s, int j, int m, int n) { return s->P[(size_t)j * s->ntri + s->tri[m] + (n - m)]; }
static inline double Htab(const or_sphere *s, int j, int m, int n) { return s->H[(size_t)j * s->ntri + s->tri[m] + (n - m)]; }
static size_t nspec(const or_sphere *s) { return (size_t)(s->N + 1) * (s->N + 1); }
static size_t ngrid(const or_sphere *s) { return (size_t)s->nlat * s->nlon; }
static cx *cx_zeros(size_t n) { return (cx *)calloc(n ? n : 1, sizeof(cx)); }
static double *d_zeros(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

static double lon_of(const or_sphere *s, int k) { return 2 * kPi * k / s->nlon; } /* cpp/sphere.cpp:121 */

/* cpp/sphere.cpp:111-118 */
void or_sphere_set_axis_tilt(or_sphere *s, double alpha) {
  for (int j = 0; j < s->nlat; j++)
    for (int k = 0; k < s->nlon; k++) {
      double lam = lon_of(s, k), c = sqrt(1 - s->mu[j] * s->mu[j]);
      s->f_grid[(size_t)j * s->nlon + k] = 2 * s->omega * (-cos(lam) * c * sin(alpha) + s->mu[j] * cos(alpha));
    }
}

/* cpp/sphere.cpp:75-103 */
or_sphere *or_sphere_new(int N, double radius, double omega, double gravity, double diffusion, int max_truncation) {
  if (N < 4 || N > max_truncation) return NULL;
  or_sphere *s = (or_sphere *)calloc(1, sizeof(or_sphere));
  s->N = N;
  s->radius = radius; s->omega = omega; s->gravity = gravity; s->diffusion = diffusion;
  s->nlon = 4;
  while (s->nlon < 3 * N + 1) s->nlon *= 2;
  s->nlat = s->nlon / 2;
  s->ntri = (N + 1) * (N + 2) / 2;
  s->mu = d_zeros(s->nlat);
  s->w = d_zeros(s->nlat);
  or_gauss_legendre(s->nlat, s->mu, s->w);
  s->tri = (int *)calloc(N + 2, sizeof(int));
  for (int m = 0, o = 0; m <= N; m++) { s->tri[m] = o; o += N - m + 1; }
  s->P = d_zeros((size_t)s->nlat * s->ntri);
  s->H = d_zeros((size_t)s->nlat * s->ntri);
  double *col = d_zeros(N + 2);
  for (int j = 0; j < s->nlat; j++)
    for (int m = 0; m <= N; m++) {
      or_legendre_column(m, N, s->mu[j], col);
      double *Pr = s->P + (size_t)j * s->ntri + s->tri[m];
      double *Hr = s->H + (size_t)j * s->ntri + s->tri[m];
      for (int n = m; n <= N; n++) Pr[n - m] = col[n - m];
      for (int n = m; n <= N; n++) {
        double plus = col[n + 1 - m], minus = (n > m) ? col[n - 1 - m] : 0.0;
        Hr[n - m] = -n * eps_nm(n + 1, m) * plus + (n + 1) * eps_nm(n, m) * minus;
      }
    }
  free(col);
  s->zeta = cx_zeros(nspec(s));
  s->delta = cx_zeros(nspec(s));
  s->phi = cx_zeros(nspec(s));
  s->q = NULL;
  s->hs_grid = d_zeros(ngrid(s));
  s->f_grid = d_zeros(ngrid(s));
  s->ref_phi = d_zeros(ngrid(s));
  s->ref_q = d_zeros(ngrid(s));
  s->row = cx_zeros(s->nlon);
  or_sphere_set_axis_tilt(s, 0);
  return s;
}

void or_sphere_free(or_sphere *s) {
  if (!s) return;
  free(s->mu); free(s->w); free(s->P); free(s->H); free(s->tri);
  free(s->zeta); free(s->delta); free(s->phi); free(s->q);
  free(s->ref_phi); free(s->ref_q); free(s->f_grid); free(s->hs_grid); free(s->row);
  free(s);
}
int or_sphere_nlat(const or_sphere *s) { return s->nlat; }
int or_sphere_nlon(const or_sphere *s) { return s->nlon; }
double or_sphere_time(const or_sphere *s) { return s->t; }
const double *or_sphere_mu(const or_sphere *s) { return s->mu; }
const double *or_sphere_w(const or_sphere *s) { return s->w; }
void or_sphere_set_diffusion(or_sphere *s, double nu4) { s->diffusion = nu4; }
void or_sphere_set_advect_only(or_sphere *s, int on) { s->advect_only = on; }

/* cpp/sphere.cpp:123-129 (fm has N+1 entries) */
static void fourier_forward(const or_sphere *s, const double *row, cx *fm) {
  cx *a = s->row;
  for (int k = 0; k < s->nlon; k++) a[k] = cmk(row[k], 0.0);
  or_fft((double *)a, s->nlon, -1);
  for (int m = 0; m <= s->N; m++) fm[m] = cdivr(a[m], (double)s->nlon);
}
/* cpp/sphere.cpp:130-136 */
static void fourier_backward(const or_sphere *s, const cx *fm, double *row) {
  cx *a = s->row;
  for (int k = 0; k < s->nlon; k++) a[k] = cmk(0, 0);
  a[0] = cmk(fm[0].re, 0);
  for (int m = 1; m <= s->N; m++) { a[m] = fm[m]; a[s->nlon - m] = cmk(fm[m].re, -fm[m].im); }
  or_fft((double *)a, s->nlon, +1);
  for (int k = 0; k < s->nlon; k++) row[k] = a[k].re;
}

/* cpp/sphere.cpp:138-149 */
static void analyze_scalar(const or_sphere *s, const double *grid, cx *spec) {
  memset(spec, 0, nspec(s) * sizeof(cx));
  cx *fm = cx_zeros(s->N + 1);
  for (int j = 0; j < s->nlat; j++) {
    fourier_forward(s, grid + (size_t)j * s->nlon, fm);
    for (int m = 0; m <= s->N; m++) {
      cx f = cscale(fm[m], s->w[j]);
      for (int n = m; n <= s->N; n++) spec[sidx(s, m, n)] = cadd(spec[sidx(s, m, n)], cscale(f, Ptab(s, j, m, n)));
    }
  }
  free(fm);
}
/* cpp/sphere.cpp:150-162 */
static void synthesize_scalar(const or_sphere *s, const cx *spec, double *grid) {
  cx *fm = cx_zeros(s->N + 1);
  for (int j = 0; j < s->nlat; j++) {
    for (int m = 0; m <= s->N; m++) {
      cx acc = cmk(0, 0);
      for (int n = m; n <= s->N; n++) acc = cadd(acc, cscale(spec[sidx(s, m, n)], Ptab(s, j, m, n)));
      fm[m] = acc;
    }
    fourier_backward(s, fm, grid + (size_t)j * s->nlon);
  }
  free(fm);
}
/* cpp/sphere.cpp:164-177 */
static void analyze_divergence(const or_sphere *s, const double *A, const double *B, cx *spec) {
  memset(spec, 0, nspec(s) * sizeof(cx));
  cx *fa = cx_zeros(s->N + 1), *fb = cx_zeros(s->N + 1);
  for (int j = 0; j < s->nlat; j++) {
    fourier_forward(s, A + (size_t)j * s->nlon, fa);
    fourier_forward(s, B + (size_t)j * s->nlon, fb);
    double wj = s->w[j] / (1 - s->mu[j] * s->mu[j]) / s->radius;
    for (int m = 0; m <= s->N; m++) {
      cx ca = cscale(cmul(cim(m), fa[m]), wj), cb = cscale(fb[m], wj);
      for (int n = m; n <= s->N; n++) {
        cx t = csub(cscale(ca, Ptab(s, j, m, n)), cscale(cb, Htab(s, j, m, n)));
        spec[sidx(s, m, n)] = cadd(spec[sidx(s, m, n)], t);
      }
    }
  }
  free(fa); free(fb);
}
/* cpp/sphere.cpp:179-206 */
static void winds_spectral_to_grid(const or_sphere *s, const cx *z, const cx *d, double *U, double *V) {
  const double a = s->radius;
  cx *psi = cx_zeros(nspec(s)), *chi = cx_zeros(nspec(s));
  for (int m = 0; m <= s->N; m++)
    for (int n = (m > 1 ? m : 1); n <= s->N; n++) {
      double k = -a * a / (n * (n + 1.0));
      psi[sidx(s, m, n)] = cscale(z[sidx(s, m, n)], k);
      chi[sidx(s, m, n)] = cscale(d[sidx(s, m, n)], k);
    }
  cx *fu = cx_zeros(s->N + 1), *fv = cx_zeros(s->N + 1);
  for (int j = 0; j < s->nlat; j++) {
    for (int m = 0; m <= s->N; m++) {
      cx sp = cmk(0, 0), sc = cmk(0, 0), hp = cmk(0, 0), hc = cmk(0, 0);
      for (int n = m; n <= s->N; n++) {
        double P = Ptab(s, j, m, n), H = Htab(s, j, m, n);
        size_t q = sidx(s, m, n);
        sp = cadd(sp, cscale(psi[q], P)); sc = cadd(sc, cscale(chi[q], P));
        hp = cadd(hp, cscale(psi[q], H)); hc = cadd(hc, cscale(chi[q], H));
      }
      fu[m] = cdivr(csub(cmul(cim(m), sc), hp), a);
      fv[m] = cdivr(cadd(cmul(cim(m), sp), hc), a);
    }
    fourier_backward(s, fu, U + (size_t)j * s->nlon);
    fourier_backward(s, fv, V + (size_t)j * s->nlon);
  }
  free(psi); free(chi); free(fu); free(fv);
}
/* cpp/sphere.cpp:208-215 */
static void analyze_vort_div(const or_sphere *s, const double *U, const double *V, cx *z, cx *d) {
  size_t n = ngrid(s);
  double *mU = d_zeros(n);
  for (size_t i = 0; i < n; i++) mU[i] = -U[i];
  analyze_divergence(s, V, mU, z);
  analyze_divergence(s, U, V, d);
  z[0] = cmk(0, 0);
  d[0] = cmk(0, 0);
  free(mU);
}

/* cpp/sphere.cpp:236-239 */
void or_sphere_mark_reference(or_sphere *s) {
  synthesize_scalar(s, s->phi, s->ref_phi);
  if (s->has_tracer) synthesize_scalar(s, s->q, s->ref_q);
}
/* cpp/sphere.cpp:217-234 */
int or_sphere_set_state_grid(or_sphere *s, const double *h, const double *u, const double *v) {
  size_t n = ngrid(s);
  double *U = d_zeros(n), *V = d_zeros(n), *ph = d_zeros(n);
  for (int j = 0; j < s->nlat; j++) {
    double c = sqrt(1 - s->mu[j] * s->mu[j]);
    for (int k = 0; k < s->nlon; k++) {
      size_t i = (size_t)j * s->nlon + k;
      U[i] = u[i] * c;
      V[i] = v[i] * c;
      ph[i] = s->gravity * h[i];
    }
  }
  analyze_vort_div(s, U, V, s->zeta, s->delta);
  analyze_scalar(s, ph, s->phi);
  s->t = 0;
  or_sphere_mark_reference(s);
  free(U); free(V); free(ph);
  return 0;
}
/* cpp/sphere.cpp:105-109 */
void or_sphere_set_orography_grid(or_sphere *s, const double *hs) {
  memcpy(s->hs_grid, hs, ngrid(s) * sizeof(double));
  s->has_orography = 1;
}
/* cpp/sphere.cpp:241-246 */
void or_sphere_set_tracer_grid(or_sphere *s, const double *q) {
  if (!s->q) s->q = cx_zeros(nspec(s));
  analyze_scalar(s, q, s->q);
  s->has_tracer = 1;
  synthesize_scalar(s, s->q, s->ref_q);
}

/* cpp/sphere.cpp:301-311 */
int or_sphere_add_mode(or_sphere *s, int n, int m, double amplitude, double mean_depth) {
  if (m < 0 || n < (m > 1 ? m : 1) || n > s->N) return 1;
  memset(s->zeta, 0, nspec(s) * sizeof(cx));
  memset(s->delta, 0, nspec(s) * sizeof(cx));
  memset(s->phi, 0, nspec(s) * sizeof(cx));
  s->phi[0] = cmk(s->gravity * mean_depth * sqrt(2.0), 0.0);
  s->phi[sidx(s, m, n)] = cadd(s->phi[sidx(s, m, n)], cmk(s->gravity * amplitude * (m == 0 ? 1.0 : 0.5), 0.0));
  s->t = 0;
  or_sphere_mark_reference(s);
  return 0;
}

/* cpp/sphere.cpp:313-336 */
int or_sphere_perturb(or_sphere *s, double amplitude, uint64_t seed, int max_wave) {
  if (max_wave < 1 || max_wave > s->N) return 1;
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 12345;
  cx *add = cx_zeros(nspec(s));
  for (int m = 0; m <= max_wave; m++)
    for (int n = (m > 1 ? m : 1); n <= max_wave; n++) {
      double re = irwin_hall(&st), im = m == 0 ? 0.0 : irwin_hall(&st);
      add[sidx(s, m, n)] = cmk(re, im);
    }
  double *g = d_zeros(ngrid(s));
  synthesize_scalar(s, add, g);
  double ms = 0, wsum = 0;
  for (int j = 0; j < s->nlat; j++)
    for (int k = 0; k < s->nlon; k++) { double x = g[(size_t)j * s->nlon + k]; ms += s->w[j] * x * x; wsum += s->w[j]; }
  double rms = sqrt(ms / wsum);
  double scale = rms > 0 ? amplitude / rms * s->gravity : 0;
  for (size_t i = 0; i < nspec(s); i++) s->phi[i] = cadd(s->phi[i], cscale(add[i], scale));
  s->t = 0;
  or_sphere_mark_reference(s);
  free(add); free(g);
  return 0;
}

void or_sphere_get_state(const or_sphere *s, double *zeta, double *delta, double *phi, double *q) {
  size_t b = nspec(s) * sizeof(cx);
  if (zeta) memcpy(zeta, s->zeta, b);
  if (delta) memcpy(delta, s->delta, b);
  if (phi) memcpy(phi, s->phi, b);
  if (q) { if (s->q) memcpy(q, s->q, b); else memset(q, 0, b); }
}
void or_sphere_set_state(or_sphere *s, const double *zeta, const double *delta, const double *phi, double t) {
  size_t b = nspec(s) * sizeof(cx);
  memcpy(s->zeta, zeta, b);
  memcpy(s->delta, delta, b);
  memcpy(s->phi, phi, b);
  s->t = t;
}

/* cpp/sphere.cpp:250-263 */
static void tracer_tendency(const or_sphere *s, const cx *z, const cx *d, const cx *q, cx *dq) {
  size_t ng = ngrid(s);
  double *U = d_zeros(ng), *V = d_zeros(ng), *qg = d_zeros(ng), *dg = d_zeros(ng);
  double *A = d_zeros(ng), *B = d_zeros(ng), *C = d_zeros(ng);
  winds_spectral_to_grid(s, z, d, U, V);
  synthesize_scalar(s, q, qg);
  synthesize_scalar(s, d, dg);
  for (size_t i = 0; i < ng; i++) { A[i] = U[i] * qg[i]; B[i] = V[i] * qg[i]; C[i] = qg[i] * dg[i]; }
  cx *flux = cx_zeros(nspec(s)), *corr = cx_zeros(nspec(s));
  analyze_divergence(s, A, B, flux);
  analyze_scalar(s, C, corr);
  for (size_t i = 0; i < nspec(s); i++) dq[i] = csub(corr[i], flux[i]);
  free(U); free(V); free(qg); free(dg); free(A); free(B); free(C); free(flux); free(corr);
}

/* cpp/sphere.cpp:338-390 */
static void tendencies(const or_sphere *s, const cx *z, const cx *d, const cx *f, cx *dz, cx *dd, cx *df) {
  size_t ng = ngrid(s);
  const double a = s->radius;
  double *U = d_zeros(ng), *V = d_zeros(ng), *zg = d_zeros(ng), *pg = d_zeros(ng);
  winds_spectral_to_grid(s, z, d, U, V);
  synthesize_scalar(s, z, zg);
  synthesize_scalar(s, f, pg);
  double *A = d_zeros(ng), *B = d_zeros(ng), *UP = d_zeros(ng), *VP = d_zeros(ng), *PE = d_zeros(ng);
  for (int j = 0; j < s->nlat; j++) {
    double om = 1 - s->mu[j] * s->mu[j];
    for (int k = 0; k < s->nlon; k++) {
      size_t i = (size_t)j * s->nlon + k;
      double eta = zg[i] + s->f_grid[i];
      A[i] = U[i] * eta;
      B[i] = V[i] * eta;
      UP[i] = U[i] * pg[i];
      VP[i] = V[i] * pg[i];
      PE[i] = pg[i] + s->gravity * s->hs_grid[i] + (U[i] * U[i] + V[i] * V[i]) / (2 * om);
    }
  }
  memset(dz, 0, nspec(s) * sizeof(cx));
  memset(dd, 0, nspec(s) * sizeof(cx));
  memset(df, 0, nspec(s) * sizeof(cx));
  int M = s->N + 1;
  cx *fa = cx_zeros(M), *fb = cx_zeros(M), *fu = cx_zeros(M), *fv = cx_zeros(M), *fe = cx_zeros(M);
  for (int j = 0; j < s->nlat; j++) {
    size_t o = (size_t)j * s->nlon;
    fourier_forward(s, A + o, fa);
    fourier_forward(s, B + o, fb);
    fourier_forward(s, UP + o, fu);
    fourier_forward(s, VP + o, fv);
    fourier_forward(s, PE + o, fe);
    double wj = s->w[j], wd = s->w[j] / (1 - s->mu[j] * s->mu[j]) / a;
    for (int m = 0; m <= s->N; m++) {
      cx ima = cim(m);
      cx ca = cscale(cmul(ima, fa[m]), wd), cb = cscale(fb[m], wd), cu = cscale(cmul(ima, fu[m]), wd), cv = cscale(fv[m], wd);
      cx cb2 = cscale(cmul(ima, fb[m]), wd), ca2 = cscale(fa[m], wd);
      cx ce = cscale(fe[m], wj);
      for (int n = m; n <= s->N; n++) {
        double P = Ptab(s, j, m, n), H = Htab(s, j, m, n);
        size_t q = sidx(s, m, n);
        dz[q] = csub(dz[q], csub(cscale(ca, P), cscale(cb, H)));
        dd[q] = cadd(dd[q], cadd(cscale(cb2, P), cscale(ca2, H)));
        dd[q] = cadd(dd[q], cscale(cscale(ce, P), n * (n + 1.0) / (a * a)));
        df[q] = csub(df[q], csub(cscale(cu, P), cscale(cv, H)));
      }
    }
  }
  dz[0] = cmk(0, 0);
  dd[0] = cmk(0, 0);
  df[0] = cmk(0, 0);
  free(U); free(V); free(zg); free(pg); free(A); free(B); free(UP); free(VP); free(PE);
  free(fa); free(fb); free(fu); free(fv); free(fe);
}

/* cpp/sphere.cpp:392-405 */
static void sphere_filter(or_sphere *s, double dt) {
  if (s->diffusion <= 0) return;
  const double a2 = s->radius * s->radius;
  for (int m = 0; m <= s->N; m++)
    for (int n = (m > 1 ? m : 1); n <= s->N; n++) {
      double l = n * (n + 1.0);
      double kv = (l - 2) / a2, kp = l / a2;
      double fv = exp(-s->diffusion * kv * kv * dt), fp = exp(-s->diffusion * kp * kp * dt);
      size_t q = sidx(s, m, n);
      s->zeta[q] = cscale(s->zeta[q], fv);
      s->delta[q] = cscale(s->delta[q], fv);
      s->phi[q] = cscale(s->phi[q], fp);
      if (s->has_tracer) s->q[q] = cscale(s->q[q], fp);
    }
}

typedef struct { cx *z, *d, *f, *q; } sstate;
static void sstate_alloc(const or_sphere *s, sstate *x) {
  x->z = cx_zeros(nspec(s)); x->d = cx_zeros(nspec(s)); x->f = cx_zeros(nspec(s)); x->q = cx_zeros(nspec(s));
}
static void sstate_free(sstate *x) { free(x->z); free(x->d); free(x->f); free(x->q); }
/* the rhs lambda of cpp/sphere.cpp:411-415 */
static void rhs(const or_sphere *s, const sstate *x, sstate *k) {
  if (s->advect_only) {
    memset(k->z, 0, nspec(s) * sizeof(cx)); memset(k->d, 0, nspec(s) * sizeof(cx)); memset(k->f, 0, nspec(s) * sizeof(cx));
  } else {
    tendencies(s, x->z, x->d, x->f, k->z, k->d, k->f);
  }
  if (s->has_tracer) tracer_tendency(s, x->z, x->d, x->q, k->q);
}
/* the axpy/advance lambdas of cpp/sphere.cpp:416-422 */
static void advance(const or_sphere *s, const sstate *x, const sstate *k, double c, sstate *out) {
  for (size_t i = 0; i < nspec(s); i++) {
    out->z[i] = cadd(x->z[i], cscale(k->z[i], c));
    out->d[i] = cadd(x->d[i], cscale(k->d[i], c));
    out->f[i] = cadd(x->f[i], cscale(k->f[i], c));
    if (s->has_tracer) out->q[i] = cadd(x->q[i], cscale(k->q[i], c));
  }
}
/* combined RK4 update of cpp/sphere.cpp:428-433: x += dt/6 * (k1 + 2 k2 + 2 k3 + k4) */
static cx rk4_combine(cx x, cx k1, cx k2, cx k3, cx k4, double dt) {
  cx sum = cadd(cadd(cadd(k1, cscale(k2, 2.0)), cscale(k3, 2.0)), k4);
  return cadd(x, cscale(sum, dt / 6));
}

/* cpp/sphere.cpp:407-436 */
void or_sphere_step(or_sphere *s, double dt) {
  sstate s0, k1, k2, k3, k4, tmp;
  s0.z = s->zeta; s0.d = s->delta; s0.f = s->phi; s0.q = s->q;
  sstate_alloc(s, &k1); sstate_alloc(s, &k2); sstate_alloc(s, &k3); sstate_alloc(s, &k4); sstate_alloc(s, &tmp);
  rhs(s, &s0, &k1);
  advance(s, &s0, &k1, 0.5 * dt, &tmp);
  rhs(s, &tmp, &k2);
  advance(s, &s0, &k2, 0.5 * dt, &tmp);
  rhs(s, &tmp, &k3);
  advance(s, &s0, &k3, dt, &tmp);
  rhs(s, &tmp, &k4);
  for (size_t i = 0; i < nspec(s); i++) {
    s->zeta[i] = rk4_combine(s->zeta[i], k1.z[i], k2.z[i], k3.z[i], k4.z[i], dt);
    s->delta[i] = rk4_combine(s->delta[i], k1.d[i], k2.d[i], k3.d[i], k4.d[i], dt);
    s->phi[i] = rk4_combine(s->phi[i], k1.f[i], k2.f[i], k3.f[i], k4.f[i], dt);
    if (s->has_tracer) s->q[i] = rk4_combine(s->q[i], k1.q[i], k2.q[i], k3.q[i], k4.q[i], dt);
  }
  sphere_filter(s, dt);
  s->t += dt;
  sstate_free(&k1); sstate_free(&k2); sstate_free(&k3); sstate_free(&k4); sstate_free(&tmp);
}

/* cpp/sphere.cpp:486-508 */
void or_sphere_grid_height(const or_sphere *s, double *g) {
  synthesize_scalar(s, s->phi, g);
  for (size_t i = 0; i < ngrid(s); i++) g[i] /= s->gravity;
}
void or_sphere_grid_vorticity(const or_sphere *s, double *g) { synthesize_scalar(s, s->zeta, g); }
void or_sphere_grid_u(const or_sphere *s, double *g) {
  double *V = d_zeros(ngrid(s));
  winds_spectral_to_grid(s, s->zeta, s->delta, g, V);
  for (int j = 0; j < s->nlat; j++) {
    double c = sqrt(1 - s->mu[j] * s->mu[j]);
    for (int k = 0; k < s->nlon; k++) g[(size_t)j * s->nlon + k] /= c;
  }
  free(V);
}
void or_sphere_grid_v(const or_sphere *s, double *g) {
  double *U = d_zeros(ngrid(s));
  winds_spectral_to_grid(s, s->zeta, s->delta, U, g);
  for (int j = 0; j < s->nlat; j++) {
    double c = sqrt(1 - s->mu[j] * s->mu[j]);
    for (int k = 0; k < s->nlon; k++) g[(size_t)j * s->nlon + k] /= c;
  }
  free(U);
}
void or_sphere_grid_tracer(const or_sphere *s, double *g) {
  if (s->q) synthesize_scalar(s, s->q, g); else memset(g, 0, ngrid(s) * sizeof(double));
}

/* cpp/sphere.cpp:438-447 */
double or_sphere_stable_dt(const or_sphere *s, double safety, int *status) {
  size_t ng = ngrid(s);
  double *h = d_zeros(ng), *u = d_zeros(ng), *v = d_zeros(ng);
  or_sphere_grid_height(s, h);
  or_sphere_grid_u(s, u);
  or_sphere_grid_v(s, v);
  double hmax = 0, wmax = 0;
  for (size_t i = 0; i < ng; i++) {
    hmax = fmax(hmax, h[i]);
    double sp = hypot(u[i], v[i]);
    wmax = wmax < sp ? sp : wmax;
  }
  free(h); free(u); free(v);
  if (status) *status = 0;
  if (!(hmax > 0)) { if (status) *status = 2; return 0; }
  double omega = s->advect_only ? (s->N / s->radius) * wmax
                                : (s->N / s->radius) * (sqrt(s->gravity * hmax) + wmax) + 2 * s->omega;
  if (!(omega > 0)) return 1e9;
  return safety / omega;
}

/* cpp/sphere.cpp:449-455 */
static int check_finite(const or_sphere *s) {
  double sum = 0;
  for (size_t i = 0; i < nspec(s); i++)
    sum += hypot(s->zeta[i].re, s->zeta[i].im) + hypot(s->delta[i].re, s->delta[i].im) + hypot(s->phi[i].re, s->phi[i].im);
  if (s->has_tracer) for (size_t i = 0; i < nspec(s); i++) sum += hypot(s->q[i].re, s->q[i].im);
  return isfinite(sum) ? 0 : 2;
}

/* cpp/sphere.cpp:457-484 */
int or_sphere_run(or_sphere *s, double seconds, double dt, char *err, int errlen) {
  int st = 0;
  if (!(seconds >= 0)) { snprintf(err, errlen, "run: seconds must not be negative"); return 1; }
  if (s->advect_only && !s->has_tracer) { snprintf(err, errlen, "advect_only: set a tracer first (Sphere.tracer)"); return 1; }
  if (seconds == 0) return 0;
  if (!(dt > 0)) {
    dt = or_sphere_stable_dt(s, 1.5, &st);
    if (st) { snprintf(err, errlen, "the height field must be positive to step the model"); return 2; }
  }
  const double limit = or_sphere_stable_dt(s, 2.0 * sqrt(2.0), &st);
  if (st) { snprintf(err, errlen, "the height field must be positive to step the model"); return 2; }
  if (!(dt <= limit)) {
    snprintf(err, errlen, "run: dt = %f s exceeds the RK4 stability limit of about %f s for the present state: use a smaller dt", dt, limit);
    return 1;
  }
  int64_t n = (int64_t)ceil(seconds / dt - 1e-9);
  if (n < 1) n = 1;
  if (n > 50000000) { snprintf(err, errlen, "run: more than 5e7 steps; use a larger dt"); return 1; }
  double h = seconds / (double)n;
  for (int64_t i = 0; i < n; i++) {
    or_sphere_step(s, h);
    if ((i & 63) == 63) {
      if (check_finite(s)) { snprintf(err, errlen, "the integration blew up (not finite): use a smaller dt"); return 2; }
      const double now = or_sphere_stable_dt(s, 2.0 * sqrt(2.0), &st);
      if (st) { snprintf(err, errlen, "the height field must be positive to step the model"); return 2; }
      if (!(h <= now)) {
        snprintf(err, errlen, "run: dt = %f s exceeds the RK4 stability limit of about %f s reached at t = %f s (the flow accelerated): use a smaller dt", h, now, s->t);
        return 2;
      }
    }
  }
  if (check_finite(s)) { snprintf(err, errlen, "the integration blew up (not finite): use a smaller dt"); return 2; }
  return 0;
}

/* cpp/sphere.cpp:510 */
double or_sphere_mean_height(const or_sphere *s) { return s->phi[0].re / sqrt(2.0) / s->gravity; }

/* cpp/sphere.cpp:514-523 */
double or_sphere_kinetic_energy(const or_sphere *s) {
  size_t ng = ngrid(s);
  double *h = d_zeros(ng), *u = d_zeros(ng), *v = d_zeros(ng);
  or_sphere_grid_height(s, h); or_sphere_grid_u(s, u); or_sphere_grid_v(s, v);
  double sum = 0;
  for (int j = 0; j < s->nlat; j++) {
    double row = 0;
    for (int k = 0; k < s->nlon; k++) { size_t i = (size_t)j * s->nlon + k; row += 0.5 * h[i] * (u[i] * u[i] + v[i] * v[i]); }
    sum += s->w[j] * row / s->nlon;
  }
  free(h); free(u); free(v);
  return 0.5 * sum;
}
/* cpp/sphere.cpp:525-534 */
double or_sphere_potential_energy(const or_sphere *s) {
  size_t ng = ngrid(s);
  double *h = d_zeros(ng);
  or_sphere_grid_height(s, h);
  double sum = 0;
  for (int j = 0; j < s->nlat; j++) {
    double row = 0;
    for (int k = 0; k < s->nlon; k++) { size_t i = (size_t)j * s->nlon + k; row += 0.5 * s->gravity * h[i] * h[i] + s->gravity * h[i] * s->hs_grid[i]; }
    sum += s->w[j] * row / s->nlon;
  }
  free(h);
  return 0.5 * sum;
}
/* cpp/sphere.cpp:512 */
double or_sphere_energy(const or_sphere *s) { return or_sphere_kinetic_energy(s) + or_sphere_potential_energy(s); }

/* cpp/sphere.cpp:536-551 */
void or_sphere_spectrum(const or_sphere *s, double *ke, double *pe) {
  for (int n = 0; n <= s->N; n++) { ke[n] = 0; pe[n] = 0; }
  const double a2 = s->radius * s->radius, g2 = s->gravity * s->gravity;
  for (int m = 0; m <= s->N; m++) {
    double cm = m == 0 ? 1.0 : 2.0;
    for (int n = (m > 1 ? m : 1); n <= s->N; n++) {
      size_t q = sidx(s, m, n);
      double nz = s->zeta[q].re * s->zeta[q].re + s->zeta[q].im * s->zeta[q].im;
      double nd = s->delta[q].re * s->delta[q].re + s->delta[q].im * s->delta[q].im;
      double np = s->phi[q].re * s->phi[q].re + s->phi[q].im * s->phi[q].im;
      ke[n] += 0.25 * cm * a2 * (nz + nd) / (n * (n + 1.0));
      pe[n] += 0.25 * cm * s->gravity * np / g2;
    }
  }
}

/* cpp/sphere.cpp:553-562 */
double or_sphere_potential_enstrophy(const or_sphere *s) {
  size_t ng = ngrid(s);
  double *h = d_zeros(ng), *z = d_zeros(ng);
  or_sphere_grid_height(s, h); or_sphere_grid_vorticity(s, z);
  double sum = 0;
  for (int j = 0; j < s->nlat; j++) {
    double row = 0;
    for (int k = 0; k < s->nlon; k++) { size_t i = (size_t)j * s->nlon + k; double f = s->f_grid[i]; row += 0.5 * (z[i] + f) * (z[i] + f) / h[i]; }
    sum += s->w[j] * row / s->nlon;
  }
  free(h); free(z);
  return 0.5 * sum;
}

/* cpp/sphere.cpp:564-569 */
double or_sphere_max_wind(const or_sphere *s) {
  size_t ng = ngrid(s);
  double *u = d_zeros(ng), *v = d_zeros(ng);
  or_sphere_grid_u(s, u); or_sphere_grid_v(s, v);
  double m = 0;
  for (size_t i = 0; i < ng; i++) { double sp = hypot(u[i], v[i]); m = m < sp ? sp : m; }
  free(u); free(v);
  return m;
}

/* cpp/sphere.cpp:571-586 */
static void errors(const or_sphere *s, const double *ref, const double *h, double g, double *l2, double *linf) {
  double num = 0, den = 0, mn = 0, mr = 0;
  for (int j = 0; j < s->nlat; j++)
    for (int k = 0; k < s->nlon; k++) {
      size_t i = (size_t)j * s->nlon + k;
      double r = ref[i] / g, d = h[i] - r;
      num += s->w[j] * d * d;
      den += s->w[j] * r * r;
      mn = fmax(mn, fabs(d));
      mr = fmax(mr, fabs(r));
    }
  *l2 = sqrt(num / den);
  *linf = mn / mr;
}
double or_sphere_height_error_l2(const or_sphere *s) {
  double *h = d_zeros(ngrid(s)), a, b;
  or_sphere_grid_height(s, h);
  errors(s, s->ref_phi, h, s->gravity, &a, &b);
  free(h);
  return a;
}
double or_sphere_height_error_linf(const or_sphere *s) {
  double *h = d_zeros(ngrid(s)), a, b;
  or_sphere_grid_height(s, h);
  errors(s, s->ref_phi, h, s->gravity, &a, &b);
  free(h);
  return b;
}
/* cpp/sphere.cpp:271-284, 589 */
double or_sphere_tracer_mean(const or_sphere *s) { return s->q ? s->q[0].re / sqrt(2.0) : 0.0; }
double or_sphere_tracer_mass(const or_sphere *s) {
  size_t ng = ngrid(s);
  double *h = d_zeros(ng), *q = d_zeros(ng);
  or_sphere_grid_height(s, h); or_sphere_grid_tracer(s, q);
  double sum = 0;
  for (int j = 0; j < s->nlat; j++) {
    double row = 0;
    for (int k = 0; k < s->nlon; k++) { size_t i = (size_t)j * s->nlon + k; row += h[i] * q[i]; }
    sum += s->w[j] * row / s->nlon;
  }
  free(h); free(q);
  return 0.5 * sum;
}
double or_sphere_tracer_error_l2(const or_sphere *s) {
  double *q = d_zeros(ngrid(s)), a, b;
  or_sphere_grid_tracer(s, q);
  errors(s, s->ref_q, q, 1.0, &a, &b);
  free(q);
  return a;
}

void or_sphere_analyze_scalar(const or_sphere *s, const double *grid, double *spec) { analyze_scalar(s, grid, (cx *)spec); }
void or_sphere_synthesize_scalar(const or_sphere *s, const double *spec, double *grid) { synthesize_scalar(s, (const cx *)spec, grid); }
void or_sphere_analyze_divergence(const or_sphere *s, const double *A, const double *B, double *spec) { analyze_divergence(s, A, B, (cx *)spec); }

/* Seeded balanced turbulence: the reference has no such initialiser, so this generator is this project's
 * own definition (the benchmark recipe). Vorticity coefficients for 1 <= n <= nforce are complex Gaussian
 * (Irwin-Hall normals from splitmix64, imaginary part 0 at m = 0), rescaled per degree n so that the
 * kinetic-energy spectrum (the reference's formula, cpp/sphere.cpp:547) goes as n^-3, then globally so that
 * the largest grid wind equals max_wind. Divergence is zero. Height is mean_height + f psi / g with
 * f = 2 Omega mu (linear balance), less the area mean of f psi / g so that the mean height is mean_height. The
 * grids feed set_state_grid. */
void or_sphere_turbulence_grids(const or_sphere *s, uint64_t seed, double mean_height, double max_wind, int nforce,
                                double *h, double *u, double *v) {
  const double a = s->radius, a2 = a * a;
  size_t ns = nspec(s), ng = ngrid(s);
  cx *z = cx_zeros(ns), *zero = cx_zeros(ns), *psi = cx_zeros(ns);
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 424242;
  if (nforce > s->N) nforce = s->N;
  for (int n = 1; n <= nforce; n++) {
    for (int m = 0; m <= n; m++) {
      double re = irwin_hall(&st), im = m == 0 ? 0.0 : irwin_hall(&st);
      z[sidx(s, m, n)] = cmk(re, im);
    }
    double e = 0;
    for (int m = 0; m <= n; m++) {
      cx c = z[sidx(s, m, n)];
      e += 0.25 * (m == 0 ? 1.0 : 2.0) * a2 * (c.re * c.re + c.im * c.im) / (n * (n + 1.0));
    }
    double target = 1.0 / ((double)n * n * n);
    double sc = e > 0 ? sqrt(target / e) : 0.0;
    for (int m = 0; m <= n; m++) z[sidx(s, m, n)] = cscale(z[sidx(s, m, n)], sc);
  }
  double *U = d_zeros(ng), *V = d_zeros(ng);
  winds_spectral_to_grid(s, z, zero, U, V);
  double wmax = 0;
  for (int j = 0; j < s->nlat; j++) {
    double c = sqrt(1 - s->mu[j] * s->mu[j]);
    for (int k = 0; k < s->nlon; k++) {
      size_t i = (size_t)j * s->nlon + k;
      double sp = sqrt(U[i] * U[i] + V[i] * V[i]) / c;
      wmax = wmax < sp ? sp : wmax;
    }
  }
  double gsc = wmax > 0 ? max_wind / wmax : 0.0;
  for (size_t i = 0; i < ns; i++) z[i] = cscale(z[i], gsc);
  winds_spectral_to_grid(s, z, zero, U, V);
  for (int j = 0; j < s->nlat; j++) {
    double c = sqrt(1 - s->mu[j] * s->mu[j]);
    for (int k = 0; k < s->nlon; k++) {
      size_t i = (size_t)j * s->nlon + k;
      u[i] = U[i] / c;
      v[i] = V[i] / c;
    }
  }
  for (int m = 0; m <= s->N; m++)
    for (int n = (m > 1 ? m : 1); n <= s->N; n++) psi[sidx(s, m, n)] = cscale(z[sidx(s, m, n)], -a2 / (n * (n + 1.0)));
  synthesize_scalar(s, psi, h);
  for (int j = 0; j < s->nlat; j++) {
    double f = 2 * s->omega * s->mu[j];
    for (int k = 0; k < s->nlon; k++) {
      size_t i = (size_t)j * s->nlon + k;
      h[i] = f * h[i] / s->gravity;
    }
  }
  /* remove the area mean of the balanced part (Gaussian quadrature, as the reference's area means) so that the
     mean height is mean_height */
  double sum = 0;
  for (int j = 0; j < s->nlat; j++) {
    double row = 0;
    for (int k = 0; k < s->nlon; k++) row += h[(size_t)j * s->nlon + k];
    sum += s->w[j] * row / s->nlon;
  }
  const double hmean = 0.5 * sum;
  for (size_t i = 0; i < ng; i++) h[i] = mean_height + (h[i] - hmean);
  free(z); free(zero); free(psi); free(U); free(V);
}

/* ================================================================== plane */

struct or_plane {
  int nx, ny;
  double lx, ly, gravity, depth, f0, beta, viscosity, drag;
  int linear;
  double t;
  double *h, *u, *v;
};

static size_t pn(const or_plane *p) { return (size_t)p->nx * p->ny; }
static size_t pnv(const or_plane *p) { return (size_t)p->nx * (p->ny + 1); }
static double pdx(const or_plane *p) { return p->lx / p->nx; }
static double pdy(const or_plane *p) { return p->ly / p->ny; }
/* cpp/plane.hpp:67 */
static double coriolis(const or_plane *p, double y) { return p->f0 + p->beta * (y - 0.5 * p->ly); }

/* cpp/plane.cpp:20-32 (the argument checks live in the caller) */
or_plane *or_plane_new(int nx, int ny, double lx, double ly, double gravity, double depth, double f0, double beta,
                       double viscosity, double drag, int linear) {
  if (nx < 4 || ny < 4 || nx > 4000 || ny > 4000 || (int64_t)nx * ny > 8000000) return NULL;
  if (!(lx > 0 && ly > 0)) return NULL;
  or_plane *p = (or_plane *)calloc(1, sizeof(or_plane));
  p->nx = nx; p->ny = ny; p->lx = lx; p->ly = ly; p->gravity = gravity; p->depth = depth;
  p->f0 = f0; p->beta = beta; p->viscosity = viscosity; p->drag = drag; p->linear = linear;
  p->h = d_zeros(pn(p)); p->u = d_zeros(pn(p)); p->v = d_zeros(pnv(p));
  or_plane_reset(p);
  return p;
}
void or_plane_free(or_plane *p) { if (!p) return; free(p->h); free(p->u); free(p->v); free(p); }
void or_plane_reset(or_plane *p) {
  for (size_t i = 0; i < pn(p); i++) { p->h[i] = p->depth; p->u[i] = 0; }
  for (size_t i = 0; i < pnv(p); i++) p->v[i] = 0;
  p->t = 0;
}
double or_plane_time(const or_plane *p) { return p->t; }
void or_plane_get(const or_plane *p, double *h, double *u, double *v) {
  if (h) memcpy(h, p->h, pn(p) * sizeof(double));
  if (u) memcpy(u, p->u, pn(p) * sizeof(double));
  if (v) memcpy(v, p->v, pnv(p) * sizeof(double));
}
/* cpp/plane.cpp:312-318 */
void or_plane_set(or_plane *p, const double *h, const double *u, const double *v) {
  if (h) memcpy(p->h, h, pn(p) * sizeof(double));
  if (u) memcpy(p->u, u, pn(p) * sizeof(double));
  if (v) {
    memcpy(p->v, v, pnv(p) * sizeof(double));
    for (int i = 0; i < p->nx; i++) { p->v[i] = 0; p->v[(size_t)p->ny * p->nx + i] = 0; }
  }
}

/* cpp/plane.cpp:34-57 */
void or_plane_perturb(or_plane *p, double amplitude, uint64_t seed) {
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 777;
  size_t N = pn(p);
  double *n = d_zeros(N), *t = d_zeros(N);
  for (size_t i = 0; i < N; i++) n[i] = irwin_hall(&st);
  const int nx = p->nx, ny = p->ny;
  for (int pass = 0; pass < 3; pass++) {
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++)
        t[(size_t)j * nx + i] = 0.25 * n[(size_t)j * nx + (i + nx - 1) % nx] + 0.5 * n[(size_t)j * nx + i] + 0.25 * n[(size_t)j * nx + (i + 1) % nx];
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        int jm = j - 1 > 0 ? j - 1 : 0, jp = j + 1 < ny - 1 ? j + 1 : ny - 1;
        n[(size_t)j * nx + i] = 0.25 * t[(size_t)jm * nx + i] + 0.5 * t[(size_t)j * nx + i] + 0.25 * t[(size_t)jp * nx + i];
      }
  }
  double mean = 0, ms = 0;
  for (size_t i = 0; i < N; i++) mean += n[i];
  mean /= N;
  for (size_t i = 0; i < N; i++) { n[i] -= mean; ms += n[i] * n[i]; }
  double rms = sqrt(ms / N);
  double scale = rms > 0 ? amplitude / rms : 0;
  for (size_t i = 0; i < N; i++) p->h[i] += n[i] * scale;
  free(n); free(t);
}

/* cpp/plane.cpp:59-129 */
static void plane_tendency(const or_plane *p, const double *h, const double *u, const double *v, double *dh, double *du,
                           double *dv, double *B, double *eta) {
  const int nx = p->nx, ny = p->ny;
  const double dxx = pdx(p), dyy = pdy(p), g = p->gravity;
#define PH(i, j) h[(size_t)(j) * nx + (i)]
#define PU(i, j) u[(size_t)(j) * nx + (((i) % nx) + nx) % nx]
#define PV(i, j) v[(size_t)(j) * nx + (((i) % nx) + nx) % nx]
#define PB(i, j) B[(size_t)(j) * nx + (((i) % nx) + nx) % nx]
#define PE(i, j) eta[(size_t)(j) * nx + (((i) % nx) + nx) % nx]
  memset(dh, 0, pn(p) * sizeof(double));
  memset(du, 0, pn(p) * sizeof(double));
  memset(dv, 0, pnv(p) * sizeof(double));
  const int lin = p->linear;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      double k = 0;
      if (!lin) k = 0.5 * (0.5 * (PU(i, j) * PU(i, j) + PU(i + 1, j) * PU(i + 1, j)) + 0.5 * (PV(i, j) * PV(i, j) + PV(i, j + 1) * PV(i, j + 1)));
      B[(size_t)j * nx + i] = g * PH(i, j) + k;
    }
  for (int j = 0; j <= ny; j++) {
    double f = coriolis(p, j * dyy);
    for (int i = 0; i < nx; i++) {
      double zeta = 0;
      if (!lin) {
        double dvdx = (PV(i, j) - PV(i - 1, j)) / dxx;
        double uj = j < ny ? PU(i, j) : PU(i, ny - 1), ujm = j > 0 ? PU(i, j - 1) : PU(i, 0);
        zeta = dvdx - (uj - ujm) / dyy;
      }
      eta[(size_t)j * nx + i] = f + zeta;
    }
  }
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      double q = 0.5 * (PE(i, j) + PE(i, j + 1));
      double vbar = 0.25 * (PV(i - 1, j) + PV(i, j) + PV(i - 1, j + 1) + PV(i, j + 1));
      double r = q * vbar - (PB(i, j) - PB(i - 1, j)) / dxx - p->drag * PU(i, j);
      if (p->viscosity != 0) {
        double uy1 = j + 1 < ny ? PU(i, j + 1) : PU(i, j), uy0 = j > 0 ? PU(i, j - 1) : PU(i, j);
        r += p->viscosity * ((PU(i + 1, j) - 2 * PU(i, j) + PU(i - 1, j)) / (dxx * dxx) + (uy1 - 2 * PU(i, j) + uy0) / (dyy * dyy));
      }
      du[(size_t)j * nx + i] = r;
    }
  for (int j = 1; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      double q = 0.5 * (PE(i, j) + PE(i + 1, j));
      double ubar = 0.25 * (PU(i, j - 1) + PU(i + 1, j - 1) + PU(i, j) + PU(i + 1, j));
      double r = -q * ubar - (PB(i, j) - PB(i, j - 1)) / dyy - p->drag * PV(i, j);
      if (p->viscosity != 0) {
        double vy1 = j + 1 < ny ? PV(i, j + 1) : 0.0, vy0 = j - 1 > 0 ? PV(i, j - 1) : 0.0;
        r += p->viscosity * ((PV(i + 1, j) - 2 * PV(i, j) + PV(i - 1, j)) / (dxx * dxx) + (vy1 - 2 * PV(i, j) + vy0) / (dyy * dyy));
      }
      dv[(size_t)j * nx + i] = r;
    }
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      double hw = lin ? p->depth : 0.5 * (PH(i - 1 < 0 ? nx - 1 : i - 1, j) + PH(i % nx, j));
      double fe = (lin ? p->depth : 0.5 * (PH(i, j) + PH((i + 1) % nx, j))) * PU(i + 1, j);
      double fw = hw * PU(i, j);
      double fn = 0, fs = 0;
      if (j + 1 < ny) fn = (lin ? p->depth : 0.5 * (PH(i, j) + PH(i, j + 1))) * PV(i, j + 1);
      if (j > 0) fs = (lin ? p->depth : 0.5 * (PH(i, j - 1) + PH(i, j))) * PV(i, j);
      dh[(size_t)j * nx + i] = -((fe - fw) / dxx + (fn - fs) / dyy);
    }
#undef PH
#undef PU
#undef PV
#undef PB
#undef PE
}

/* cpp/plane.cpp:143-158 */
void or_plane_step(or_plane *p, double dt) {
  size_t N = pn(p), NV = pnv(p);
  double *B = d_zeros(N), *eta = d_zeros(NV);
  double *k[4][3], *ht = d_zeros(N), *ut = d_zeros(N), *vt = d_zeros(NV);
  for (int s = 0; s < 4; s++) { k[s][0] = d_zeros(N); k[s][1] = d_zeros(N); k[s][2] = d_zeros(NV); }
  plane_tendency(p, p->h, p->u, p->v, k[0][0], k[0][1], k[0][2], B, eta);
  const double cs[3] = {0.5 * dt, 0.5 * dt, dt};
  for (int s = 0; s < 3; s++) {
    double c = cs[s];
    for (size_t i = 0; i < N; i++) ht[i] = p->h[i] + c * k[s][0][i];
    for (size_t i = 0; i < N; i++) ut[i] = p->u[i] + c * k[s][1][i];
    for (size_t i = 0; i < NV; i++) vt[i] = p->v[i] + c * k[s][2][i];
    plane_tendency(p, ht, ut, vt, k[s + 1][0], k[s + 1][1], k[s + 1][2], B, eta);
  }
  for (size_t i = 0; i < N; i++) p->h[i] += dt / 6 * (k[0][0][i] + 2 * k[1][0][i] + 2 * k[2][0][i] + k[3][0][i]);
  for (size_t i = 0; i < N; i++) p->u[i] += dt / 6 * (k[0][1][i] + 2 * k[1][1][i] + 2 * k[2][1][i] + k[3][1][i]);
  for (size_t i = 0; i < NV; i++) p->v[i] += dt / 6 * (k[0][2][i] + 2 * k[1][2][i] + 2 * k[2][2][i] + k[3][2][i]);
  p->t += dt;
  for (int s = 0; s < 4; s++) { free(k[s][0]); free(k[s][1]); free(k[s][2]); }
  free(B); free(eta); free(ht); free(ut); free(vt);
}

/* cpp/plane.cpp:209-218 */
double or_plane_max_speed(const or_plane *p) {
  const int nx = p->nx, ny = p->ny;
  double m = 0;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      double uc = 0.5 * (p->u[(size_t)j * nx + i] + p->u[(size_t)j * nx + (i + 1) % nx]);
      double vc = 0.5 * (p->v[(size_t)j * nx + i] + p->v[(size_t)(j + 1) * nx + i]);
      double sp = hypot(uc, vc);
      m = m < sp ? sp : m;
    }
  return m;
}

/* cpp/plane.cpp:131-141 */
double or_plane_stable_dt(const or_plane *p, double safety, int *status) {
  double hmax = p->linear ? p->depth : 0, umax = p->linear ? 0 : or_plane_max_speed(p);
  if (!p->linear) for (size_t i = 0; i < pn(p); i++) hmax = hmax < p->h[i] ? p->h[i] : hmax;
  if (status) *status = 0;
  if (!(hmax > 0)) { if (status) *status = 2; return 0; }
  double c = sqrt(p->gravity * hmax) + umax;
  double dx = pdx(p), dy = pdy(p);
  double inv = c * sqrt(1.0 / (dx * dx) + 1.0 / (dy * dy));
  double visc = p->viscosity * (4.0 / (dx * dx) + 4.0 / (dy * dy));
  return safety * 2.0 / (inv + visc + fabs(p->f0) + fabs(p->beta) * p->ly);
}

/* cpp/plane.cpp:160-189 */
int or_plane_run(or_plane *p, double seconds, double dt, char *err, int errlen) {
  int st = 0;
  if (!(seconds >= 0)) { snprintf(err, errlen, "run: seconds must not be negative"); return 1; }
  if (seconds == 0) return 0;
  if (!(dt > 0)) {
    dt = or_plane_stable_dt(p, 0.5, &st);
    if (st) { snprintf(err, errlen, "the depth must be positive to step the model"); return 2; }
  }
  const double limit = or_plane_stable_dt(p, sqrt(0.5), &st);
  if (st) { snprintf(err, errlen, "the depth must be positive to step the model"); return 2; }
  if (!(dt <= limit)) {
    snprintf(err, errlen, "run: dt = %f s exceeds the RK4 stability limit of about %f s for the present state: use a smaller dt", dt, limit);
    return 1;
  }
  int64_t n = (int64_t)ceil(seconds / dt - 1e-9);
  if (n < 1) n = 1;
  if (n > 200000000) { snprintf(err, errlen, "run: too many steps; use a larger dt"); return 1; }
  double hstep = seconds / (double)n;
  for (int64_t i = 0; i < n; i++) {
    or_plane_step(p, hstep);
    if ((i & 63) == 63 || i + 1 == n) {
      double s = 0;
      for (size_t k = 0; k < pn(p); k++) s += p->h[k];
      for (size_t k = 0; k < pn(p); k++) s += p->u[k];
      for (size_t k = 0; k < pnv(p); k++) s += p->v[k];
      if (!isfinite(s)) { snprintf(err, errlen, "the integration blew up (not finite): use a smaller dt"); return 2; }
      const double now = or_plane_stable_dt(p, sqrt(0.5), &st);
      if (st) { snprintf(err, errlen, "the depth must be positive to step the model"); return 2; }
      if (!(hstep <= now)) {
        snprintf(err, errlen, "run: dt = %f s exceeds the RK4 stability limit of about %f s reached at t = %f s (the flow accelerated): use a smaller dt", hstep, now, p->t);
        return 2;
      }
    }
  }
  return 0;
}

/* cpp/plane.cpp:191-195 */
double or_plane_mean_depth(const or_plane *p) {
  double s = 0;
  for (size_t i = 0; i < pn(p); i++) s += p->h[i];
  return s / pn(p);
}
/* cpp/plane.cpp:197-207 */
double or_plane_energy(const or_plane *p) {
  const int nx = p->nx, ny = p->ny;
  double s = 0;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      double uc = 0.5 * (p->u[(size_t)j * nx + i] + p->u[(size_t)j * nx + (i + 1) % nx]);
      double vc = 0.5 * (p->v[(size_t)j * nx + i] + p->v[(size_t)(j + 1) * nx + i]);
      double hh = p->h[(size_t)j * nx + i];
      s += 0.5 * hh * (uc * uc + vc * vc) + 0.5 * p->gravity * hh * hh;
    }
  return s / pn(p);
}
/* cpp/plane.cpp:220-243 */
double or_plane_pv_anomaly_rms(const or_plane *p) {
  const int nx = p->nx, ny = p->ny;
  const double dx = pdx(p), dy = pdy(p);
  double s = 0;
  size_t cnt = 0;
  for (int j = 1; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      int im = (i + nx - 1) % nx;
      double hav = 0.25 * (p->h[(size_t)(j - 1) * nx + im] + p->h[(size_t)(j - 1) * nx + i] + p->h[(size_t)j * nx + im] + p->h[(size_t)j * nx + i]);
      double dvdx = (p->v[(size_t)j * nx + i % nx] - p->v[(size_t)j * nx + im]) / dx;
      double uj = j < ny ? p->u[(size_t)j * nx + i % nx] : p->u[(size_t)(ny - 1) * nx + i % nx];
      double ujm = j > 0 ? p->u[(size_t)(j - 1) * nx + i % nx] : p->u[i % nx];
      double z = dvdx - (uj - ujm) / dy;
      double q = z - p->f0 * (hav - p->depth) / p->depth;
      s += q * q;
      cnt++;
    }
  return sqrt(s / (double)cnt);
}

/* cpp/plane.cpp:220-226: relative vorticity at corner (i, j), i in 0..nx, j in 0..ny (free slip at the walls) */
double or_plane_zeta_at_corner(const or_plane *p, int i, int j) {
  const int nx = p->nx, ny = p->ny;
  int im = (i + nx - 1) % nx;
  double dvdx = (p->v[(size_t)j * nx + i % nx] - p->v[(size_t)j * nx + im]) / pdx(p);
  double uj = j < ny ? p->u[(size_t)j * nx + i % nx] : p->u[(size_t)(ny - 1) * nx + i % nx];
  double ujm = j > 0 ? p->u[(size_t)(j - 1) * nx + i % nx] : p->u[i % nx];
  return dvdx - (uj - ujm) / pdy(p);
}

/* cpp/plane.cpp:245-264: bilinear interpolation on the points of field `kind` (0 h at cell centres, 1 u at west
 * faces, 2 v at south faces), periodic in x and clamped in y */
double or_plane_probe(const or_plane *p, int kind, double x, double y) {
  double dxx = p->lx / p->nx, dyy = p->ly / p->ny;
  double xs = kind == 1 ? 0.0 : 0.5, ys = kind == 2 ? 0.0 : 0.5;
  double fx = x / dxx - xs, fy = y / dyy - ys;
  int rows = kind == 2 ? p->ny + 1 : p->ny;
  double fl = floor(fx);
  int i0 = (int)fl, j0 = (int)floor(fy);
  double ax = fx - fl, ay = fy - floor(fy);
  const double *f = kind == 0 ? p->h : kind == 1 ? p->u : p->v;
  double g[2][2];
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) {
      int i = (((i0 + a) % p->nx) + p->nx) % p->nx;
      int j = j0 + b;
      j = j < 0 ? 0 : (j > rows - 1 ? rows - 1 : j);
      g[a][b] = f[(size_t)j * p->nx + i];
    }
  return (1 - ax) * ((1 - ay) * g[0][0] + ay * g[0][1]) + ax * ((1 - ay) * g[1][0] + ay * g[1][1]);
}

/* cpp/plane.cpp:266-270: c_m = (1/nx) sum_i row_i exp(-2 pi i m (i + shift) / nx) of row j of field `kind`
 * (0 h, 1 u, 2 v); exp(i theta) = cos(theta) + i sin(theta) */
void or_plane_row_harmonic(const or_plane *p, int kind, int m, int j, double shift, double *re, double *im) {
  const int nx = p->nx;
  const double *row = (kind == 0 ? p->h : kind == 1 ? p->u : p->v) + (size_t)j * nx;
  double cr = 0, ci = 0;
  for (int i = 0; i < nx; i++) {
    double th = -2 * kPi * m * (i + shift) / nx;
    cr += row[i] * cos(th);
    ci += row[i] * sin(th);
  }
  *re = cr / (double)nx;
  *im = ci / (double)nx;
}

/* cpp/plane.cpp:271-277; returns 0, or 1 when m or j is out of range */
int or_plane_zonal_amplitude(const or_plane *p, int m, int j, double *out) {
  if (m < 1 || m >= p->nx / 2 || j < 0 || j >= p->ny) return 1;
  double re, im;
  or_plane_row_harmonic(p, 0, m, j, 0.5, &re, &im);
  *out = 2 * hypot(re, im);
  return 0;
}

/* crest position of a harmonic: cpp/plane.cpp:284-289 and 305-309 */
static double crest_of(const or_plane *p, int m, double re, double im) {
  double ph = atan2(im, re);
  double x = -ph / (2 * kPi * m) * p->lx;
  double per = p->lx / m;
  x = fmod(x, per);
  return x < 0 ? x + per : x;
}

/* cpp/plane.cpp:278-290 */
int or_plane_zonal_crest(const or_plane *p, int m, int j, double *out) {
  if (m < 1 || m >= p->nx / 2 || j < 0 || j >= p->ny) return 1;
  double re, im;
  or_plane_row_harmonic(p, 0, m, j, 0.5, &re, &im);
  *out = crest_of(p, m, re, im);
  return 0;
}

/* cpp/plane.cpp:300-310 (v rows 1..ny-1) */
int or_plane_v_zonal_crest(const or_plane *p, int m, int j, double *out) {
  if (m < 1 || m >= p->nx / 2 || j < 1 || j >= p->ny) return 1;
  double re, im;
  or_plane_row_harmonic(p, 2, m, j, 0.5, &re, &im);
  *out = crest_of(p, m, re, im);
  return 0;
}

/* cpp/plane.cpp:291-299: (sum over u rows of |c_m|^2 + sum over interior v rows of |c_m|^2) / ny */
int or_plane_harmonic_energy(const or_plane *p, int m, double *out) {
  if (m < 1 || m >= p->nx / 2) return 1;
  double s = 0, re, im;
  for (int j = 0; j < p->ny; j++) {
    or_plane_row_harmonic(p, 1, m, j, 0.0, &re, &im);
    s += re * re + im * im;
  }
  for (int j = 1; j < p->ny; j++) {
    or_plane_row_harmonic(p, 2, m, j, 0.5, &re, &im);
    s += re * re + im * im;
  }
  *out = s / p->ny;
  return 0;
}

/* Zonal jet in geostrophic balance plus white height noise: the reference has no such initialiser, so this
 * is this project's own definition (the benchmark recipe). u = u0 sech^2((y - ly/2) / width) at the u points
 * (cell-centre rows). h(y) integrates g dh/dy = -f u by the trapezoid rule between cell centres, shifted so the
 * balanced part has mean depth H; the noise is one unsmoothed Irwin-Hall normal per cell (row-major,
 * splitmix64 seeded as in cpp/plane.cpp:35), made zero-mean and scaled to noise_rms. */
void or_plane_jet_grids(const or_plane *p, double u0, double width, double noise_rms, uint64_t seed, double *h, double *u) {
  const int nx = p->nx, ny = p->ny;
  const double dy = pdy(p);
  double *prof = d_zeros(ny), *hy = d_zeros(ny);
  for (int j = 0; j < ny; j++) {
    double y = (j + 0.5) * dy;
    double c = cosh((y - 0.5 * p->ly) / width);
    prof[j] = u0 / (c * c);
  }
  hy[0] = 0;
  for (int j = 1; j < ny; j++) {
    double fa = coriolis(p, (j - 0.5) * dy) * prof[j - 1], fb = coriolis(p, (j + 0.5) * dy) * prof[j];
    hy[j] = hy[j - 1] - dy / p->gravity * 0.5 * (fa + fb);
  }
  double mean = 0;
  for (int j = 0; j < ny; j++) mean += hy[j];
  mean /= ny;
  size_t N = pn(p);
  double *noise = d_zeros(N);
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 777;
  for (size_t i = 0; i < N; i++) noise[i] = irwin_hall(&st);
  double nm = 0, ms = 0;
  for (size_t i = 0; i < N; i++) nm += noise[i];
  nm /= N;
  for (size_t i = 0; i < N; i++) { noise[i] -= nm; ms += noise[i] * noise[i]; }
  double rms = sqrt(ms / N);
  double sc = rms > 0 ? noise_rms / rms : 0;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      size_t k = (size_t)j * nx + i;
      h[k] = p->depth + (hy[j] - mean) + noise[k] * sc;
      u[k] = prof[j];
    }
  free(prof); free(hy); free(noise);
}
