/* lmweather-gb300: C ABI of the GB300 (sm_103a) shallow-water engine.
 *
 * The entry points replace the numerical core that lmweather's wx.* operator surface binds
 * (lmweather cpp/main.cpp:62-494 calls lmweather::Sphere, cpp/sphere.hpp:27-121, and lmweather::Plane,
 * cpp/plane.hpp:20-68). Each declaration names the reference member it replaces. Plain pointers and sizes
 * only; state lives on the GPU, owned by the handle, with one CUDA stream per handle.
 *
 * Errors: every function returns LMW_OK (0) or an error class that mirrors the reference's exceptions:
 * LMW_INVALID_ARGUMENT (std::invalid_argument), LMW_RUNTIME_ERROR (std::runtime_error) or LMW_DEVICE_ERROR
 * (a CUDA failure). lmw_last_error() returns the calling thread's last message, using the reference's texts.
 *
 * Layouts (host buffers, the reference's own): grids are row-major [nlat][nlon], latitudes south to north;
 * spectra are (T+1)^2 complex values per field at index m*(T+1)+n (n >= m), stored as interleaved
 * (re, im) doubles; plane h and u are [ny][nx], v is [ny+1][nx] with rows 0 and ny on the walls.
 */
#ifndef LMWEATHER_GB300_H
#define LMWEATHER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { LMW_OK = 0, LMW_INVALID_ARGUMENT = 1, LMW_RUNTIME_ERROR = 2, LMW_DEVICE_ERROR = 3 };
/* precision modes of the sphere engine */
enum { LMW_FP64 = 0, LMW_FP32 = 1, LMW_SPLIT_BF16 = 2 };
/* grid fields for lmw_sphere_grid */
enum { LMW_GRID_HEIGHT = 0, LMW_GRID_U = 1, LMW_GRID_V = 2, LMW_GRID_VORTICITY = 3 };

typedef struct lmw_sphere lmw_sphere;
typedef struct lmw_plane lmw_plane;

/* message of the calling thread's last failed call ("" after success) */
const char *lmw_last_error(void);
/* "lmweather-gb300 <version>" */
const char *lmw_version(void);
/* number of this library's kernel launches issued by the calling thread so far */
uint64_t lmw_launch_count(void);
/* number of device (cudaMalloc) and pinned host (cudaMallocHost) allocations this library has made so far, over
 * all threads. No reference counterpart (accounting hook: lets a caller check that an entry point allocates
 * nothing). */
uint64_t lmw_alloc_count(void);
/* on != 0: cudaProfilerStart(), else cudaProfilerStop() -- the region a profiler started with
 * --profile-from-start off captures. No reference counterpart (measurement hook). */
int lmw_profiler_range(int on);

/* The engine's split-BF16 tensor-core GEMM (tcgen05, FP32 accumulation in tensor memory) on one problem from
 * host arrays: D (128 x N) = A (128 x K) * B (N x K)^T with A and B split on the device into `terms` = 1 (BF16),
 * 3 (hi/lo) or 6 (hi/mid/lo) BF16 products. N and K multiples of 16, N <= 256. `layout` selects the shared-memory
 * descriptor stride convention (0, the engine's). kernel_status receives the kernel's error code (0: every wait
 * on the tensor cores completed). Validation hook; no reference counterpart. */
int lmw_tc_gemm_selftest(const float *A, const float *B, float *D, int N, int K, int terms, int layout, int *kernel_status);

/* The engine's integer-pipe IEEE conversions (binary32 <-> binary64, used where GB300's narrow FP64 pipe would
 * otherwise convert) against the hardware conversions on nf float and nx double bit patterns; mismatches[0] and
 * [1] receive the differing counts (0 and 0 expected). Validation hook; no reference counterpart. */
int lmw_conversion_selftest(const uint32_t *f, int nf, const uint64_t *x, int nx, int *mismatches);

/* The plane stencil's division by a fixed grid spacing (two-term reciprocal and an exact acceptance test, three
 * FP64 operations, falling back to the IEEE division when the test fails) against the IEEE division, on every pair
 * of nx double bit patterns and nd divisors (normal numbers with normal reciprocals). counts (2 entries) receives:
 * [0] the pairs whose quotients differ in any bit (0 expected), [1] the pairs the fast path answered without
 * falling back. Validation hook; no reference counterpart. */
int lmw_division_selftest(const uint64_t *x, int nx, const double *divisors, int nd, long long *counts);

/* The tensor-core kernels' bounded mbarrier wait, exercised: one wait on a phase that completes and one on a phase
 * that nothing completes, which must give up after timeout_us (1 us .. 1 s) and say so; *completed and *ran_out
 * receive 1 when both behave. The context stays usable. Failure-detection hook; no reference counterpart. */
int lmw_wait_selftest(int timeout_us, int *completed, int *ran_out);

/* ---------------------------------------------------------------------------------------- sphere */

/* Sphere::Sphere(int truncation, const SphereParams &) (cpp/sphere.hpp:29, cpp/sphere.cpp:75-103).
 * Truncation 4..170 as the reference (invalid_argument "truncation must be between 4 and 170"). */
int lmw_sphere_create(int truncation, double radius, double omega, double gravity, double diffusion, lmw_sphere **out);
/* Engine options beyond the reference: precision mode (LMW_FP64 .. LMW_SPLIT_BF16), an ensemble of `members`
 * states sharing the truncation (stepped together), and a truncation cap up to 341. */
int lmw_sphere_create_ex(int truncation, double radius, double omega, double gravity, double diffusion, int precision,
                         int members, int max_truncation, lmw_sphere **out);
/* Split-precision engine with an explicit number of BF16 products per Legendre term: 3 (hi/lo pieces, about 16
 * significant bits) or 6 (hi/mid/lo, FP32 level). lmw_sphere_create_ex with LMW_SPLIT_BF16 uses 3. */
int lmw_sphere_create_split(int truncation, double radius, double omega, double gravity, double diffusion, int members, int max_truncation,
                            int split_terms, lmw_sphere **out);
int lmw_sphere_destroy(lmw_sphere *s);
/* Sphere::truncation/nlat/nlon (cpp/sphere.hpp:30-32) and the member count */
int lmw_sphere_dims(const lmw_sphere *s, int *truncation, int *nlat, int *nlon, int *members);
/* Sphere::gauss_mu / gauss_weights (cpp/sphere.hpp:93-94): nlat values each */
int lmw_sphere_gauss(const lmw_sphere *s, double *mu, double *w);
/* The reference's transform test hooks (cpp/sphere.hpp:96-99), in FP64 on the device. Grids are nlat*nlon
 * values ([lat][lon], latitude ascending); spectra are the reference layout, (T+1)^2 complex values interleaved
 * re/im at index m*(T+1)+n (entries with n < m are zero). n must be nlat*nlon ("grid size mismatch").
 * Sphere::analyze_scalar (cpp/sphere.cpp:138-149): spec_nm = sum_j w_j F_m(grid)_j P_nm(mu_j) */
int lmw_sphere_analyze_scalar(lmw_sphere *s, const double *grid, size_t n, double *spec);
/* Sphere::synthesize_scalar (cpp/sphere.cpp:150-162): the grid of a spectrum */
int lmw_sphere_synthesize_scalar(lmw_sphere *s, const double *spec, double *grid, size_t n);
/* Sphere::analyze_divergence (cpp/sphere.cpp:164-177): spec_nm = sum_j w_j/((1-mu_j^2) a) (i m A_m P_nm - B_m H_nm) */
int lmw_sphere_analyze_divergence(lmw_sphere *s, const double *A, const double *B, size_t n, double *spec);
/* Sphere::time (cpp/sphere.hpp:34) of one member */
int lmw_sphere_time(const lmw_sphere *s, int member, double *out);
/* Sphere::set_state_grid (cpp/sphere.hpp:39, cpp/sphere.cpp:217-234); n = nlat*nlon values per grid */
int lmw_sphere_set_state_grid(lmw_sphere *s, int member, const double *h, const double *u, const double *v, size_t n);
/* Sphere::set_axis_tilt (cpp/sphere.hpp:40, cpp/sphere.cpp:111-118) */
int lmw_sphere_set_axis_tilt(lmw_sphere *s, int member, double alpha);
/* per-member rotation rate (ensembles scale Omega per member); untilted axis */
int lmw_sphere_set_omega(lmw_sphere *s, int member, double omega);
/* Sphere::set_diffusion (cpp/sphere.hpp:41) */
int lmw_sphere_set_diffusion(lmw_sphere *s, double nu4);
/* Sphere::set_orography_grid (cpp/sphere.hpp:47, cpp/sphere.cpp:105-109) */
int lmw_sphere_set_orography_grid(lmw_sphere *s, int member, const double *hs, size_t n);
/* exact point values from the spectral state (Sphere::height_at, wind_at, vorticity_at, tracer_at,
 * cpp/sphere.cpp:287-299, 592-637): which 0 height (m), 1 zonal wind u, 2 meridional wind v (m/s), 3 vorticity,
 * 4 tracer; lat, lon in radians */
int lmw_sphere_probe(lmw_sphere *s, int member, int which, double lat, double lon, double *out);
/* Sphere::mode_coefficient (cpp/sphere.cpp:639-643) and Sphere::wave_crest (cpp/sphere.cpp:645-652) */
int lmw_sphere_mode_coefficient(lmw_sphere *s, int member, int n, int m, int imag, double *out);
int lmw_sphere_wave_crest(lmw_sphere *s, int member, int m, double lat, double *out);
/* Sphere::set_tracer_grid (cpp/sphere.cpp:264-270): a passive tracer q from its grid (nlat*nlon, analysed as
 * analyze_scalar does); the grid's synthesis becomes the reference of the tracer errors. FP64 precision only. The
 * tracer is advected with the flow, dq = A(q delta) - D(U q, V q) (cpp/sphere.cpp:250-263), filtered like Phi. */
int lmw_sphere_set_tracer_grid(lmw_sphere *s, int member, const double *q, size_t n);
/* Sphere::set_advect_only (cpp/sphere.hpp:45): the flow is frozen (its tendencies are zero, the filter still
 * applies) and only the tracer moves; run() then needs a tracer ("advect_only: set a tracer first") */
int lmw_sphere_set_advect_only(lmw_sphere *s, int on);
/* the tracer's spectrum in the reference layout ((T+1)^2 complex), its grid (Sphere::grid_tracer,
 * cpp/sphere.cpp:283) and diagnostics: out[0] tracer_mean, out[1] tracer_mass (area mean of h q), out[2] l2 and
 * out[3] linf error against the grid it was set from, out[4] tracer_min, out[5] tracer_max of the grid
 * (cpp/sphere.cpp:271-286, 571-590; out has 6 entries); runtime_error without a tracer */
int lmw_sphere_tracer_state(lmw_sphere *s, int member, double *q);
int lmw_sphere_set_tracer_state(lmw_sphere *s, int member, const double *q);
int lmw_sphere_tracer_grid(lmw_sphere *s, int member, double *out, size_t n);
int lmw_sphere_tracer_diagnostics(lmw_sphere *s, int member, double *out);
/* Sphere::add_mode (cpp/sphere.hpp:43, cpp/sphere.cpp:301-311) */
int lmw_sphere_add_mode(lmw_sphere *s, int member, int n, int m, double amplitude, double mean_depth);
/* Sphere::perturb (cpp/sphere.hpp:44, cpp/sphere.cpp:313-336) */
int lmw_sphere_perturb(lmw_sphere *s, int member, double amplitude, uint64_t seed, int max_wave);
/* Sphere::mark_reference (cpp/sphere.hpp:42, cpp/sphere.cpp:236-239) */
int lmw_sphere_mark_reference(lmw_sphere *s, int member);
/* Seeded balanced turbulence (no reference counterpart: the benchmark initialiser): complex-Gaussian vorticity
 * for 1 <= n <= nforce with an n^-3 kinetic-energy spectrum scaled to max_wind, zero divergence and
 * h = mean_height + f psi / g, entered through set_state_grid */
int lmw_sphere_turbulence(lmw_sphere *s, int member, uint64_t seed, double mean_height, double max_wind, int nforce);
/* spectral state in the reference layout (the private zeta_, delta_, phi_ of cpp/sphere.hpp:111); any pointer may be NULL */
int lmw_sphere_get_state(lmw_sphere *s, int member, double *zeta, double *delta, double *phi);
int lmw_sphere_set_state(lmw_sphere *s, int member, const double *zeta, const double *delta, const double *phi, double time);
/* Sphere::step (cpp/sphere.hpp:67, cpp/sphere.cpp:407-436): one RK4 step of every member */
int lmw_sphere_step(lmw_sphere *s, double dt);
/* Sphere::run (cpp/sphere.hpp:68, cpp/sphere.cpp:457-484): equal steps, dt <= 0 picks a stable one, the
 * reference's stability and finiteness guards every 64 steps (over every member) */
int lmw_sphere_run(lmw_sphere *s, double seconds, double dt);
/* Sphere::stable_dt (cpp/sphere.hpp:69, cpp/sphere.cpp:438-447) */
int lmw_sphere_stable_dt(lmw_sphere *s, int member, double safety, double *out);
/* Sphere diagnostics (cpp/sphere.cpp:510-590): out[8] = mean_height, kinetic_energy, potential_energy, energy,
 * potential_enstrophy, max_wind, height_error_l2, height_error_linf */
int lmw_sphere_diagnostics(lmw_sphere *s, int member, double *out);
/* Sphere::grid_height/grid_u/grid_v/grid_vorticity (cpp/sphere.hpp:88-91, cpp/sphere.cpp:486-508) */
int lmw_sphere_grid(lmw_sphere *s, int member, int which, double *out, size_t n);
/* Sphere::spectrum (cpp/sphere.hpp:63, cpp/sphere.cpp:536-551): T+1 values each */
int lmw_sphere_spectrum(lmw_sphere *s, int member, double *ke, double *pe);
/* The wx layer's text files (cpp/main.cpp:328-335, 357-384), numbers as "%.10g": save_csv writes per grid
 * point "lon lat h u v vorticity tracer orography" (degrees; a blank line after each latitude row),
 * save_zonal_mean per latitude "lat mean_h mean_u", save_spectrum per degree n >= 1 "n ke pe". A file that cannot
 * be written is runtime_error "Sphere.save_csv: cannot write <path>" (and likewise). */
int lmw_sphere_save_csv(lmw_sphere *s, int member, const char *path);
int lmw_sphere_save_zonal_mean(lmw_sphere *s, int member, const char *path);
int lmw_sphere_save_spectrum(lmw_sphere *s, int member, const char *path);

/* the handle's CUDA stream (a cudaStream_t), for callers that order their own work or events after it */
int lmw_sphere_stream(const lmw_sphere *s, void **stream);
/* average device time (ms) per launch of each RK4-stage kernel class over `reps` launches (CUDA events on the
 * handle's stream): ms[0] Legendre synthesis, ms[1] FFTs + grid products, ms[2] Legendre analysis + RK4 update.
 * The spectral state is left unchanged. No reference counterpart (measurement hook). */
int lmw_sphere_kernel_times(lmw_sphere *s, double dt, int reps, double *ms);

/* ---------------------------------------------------------------------------------------- plane */

/* Plane::Plane(const PlaneParams &) (cpp/plane.hpp:22, cpp/plane.cpp:20-25) */
int lmw_plane_create(int nx, int ny, double lx, double ly, double gravity, double depth, double f0, double beta,
                     double viscosity, double drag, int linear, lmw_plane **out);
int lmw_plane_destroy(lmw_plane *p);
/* Plane::params() setters used by the wx builders (cpp/main.cpp:389-408): gravity, depth, f0, beta,
 * viscosity, drag, linear */
int lmw_plane_set_params(lmw_plane *p, double gravity, double depth, double f0, double beta, double viscosity, double drag,
                         int linear);
/* Plane::reset (cpp/plane.hpp:40, cpp/plane.cpp:27-32) */
int lmw_plane_reset(lmw_plane *p);
/* Plane::set_h_from_grid / set_u_from_grid / set_v_from_grid (cpp/plane.hpp:62-64, cpp/plane.cpp:312-318) */
int lmw_plane_set_h(lmw_plane *p, const double *h, size_t n);
int lmw_plane_set_u(lmw_plane *p, const double *u, size_t n);
int lmw_plane_set_v(lmw_plane *p, const double *v, size_t n);
/* Plane::h/u/v accessors (cpp/plane.hpp:33-38) for the whole fields; any pointer may be NULL */
int lmw_plane_get(lmw_plane *p, double *h, double *u, double *v);
/* Plane::perturb (cpp/plane.hpp:41, cpp/plane.cpp:34-57) */
int lmw_plane_perturb(lmw_plane *p, double amplitude, uint64_t seed);
/* Zonal jet in geostrophic balance plus white height noise (no reference counterpart: the benchmark
 * initialiser): u = u0 sech^2((y - ly/2)/width), h integrated from g dh/dy = -f u, noise of noise_rms */
int lmw_plane_jet(lmw_plane *p, double u0, double width, double noise_rms, uint64_t seed);
/* Plane::step (cpp/plane.hpp:42, cpp/plane.cpp:143-158) */
int lmw_plane_step(lmw_plane *p, double dt);
/* Plane::run (cpp/plane.hpp:43, cpp/plane.cpp:160-189) */
int lmw_plane_run(lmw_plane *p, double seconds, double dt);
/* Plane::stable_dt (cpp/plane.hpp:44, cpp/plane.cpp:131-141) */
int lmw_plane_stable_dt(lmw_plane *p, double safety, double *out);
/* Plane::time (cpp/plane.hpp:25) */
int lmw_plane_time(const lmw_plane *p, double *out);
/* Plane diagnostics (cpp/plane.cpp:191-243): out[4] = mean_depth, energy, max_speed, pv_anomaly_rms */
int lmw_plane_diagnostics(lmw_plane *p, double *out);
/* Plane::h_at / u_at / v_at (cpp/plane.hpp:49-51, cpp/plane.cpp:245-264): bilinear value of field `kind`
 * (0 h, 1 u, 2 v) at (x, y) metres, each field on its own points, periodic in x, rows clamped; computed on the
 * device (bitwise the reference's). A non-finite point is invalid_argument. */
int lmw_plane_probe(lmw_plane *p, int kind, double x, double y, double *out);
/* Plane::zeta_at_corner (cpp/plane.hpp:59, cpp/plane.cpp:220-226), corners i in 0..nx, j in 0..ny */
int lmw_plane_zeta_at_corner(lmw_plane *p, int i, int j, double *out);
/* Plane::zonal_amplitude / zonal_crest / v_zonal_crest / harmonic_energy (cpp/plane.hpp:52-58,
 * cpp/plane.cpp:266-310): zonal harmonics of rows, summed on the device; invalid_argument with the
 * reference's message when m or the row is out of range */
int lmw_plane_zonal_amplitude(lmw_plane *p, int m, int j, double *out);
int lmw_plane_zonal_crest(lmw_plane *p, int m, int j, double *out);
int lmw_plane_v_zonal_crest(lmw_plane *p, int m, int j, double *out);
int lmw_plane_harmonic_energy(lmw_plane *p, int m, double *out);
/* The wx layer's text files (cpp/main.cpp:464-494), numbers as "%.10g": save_csv per cell "x y h uc vc zeta"
 * (a blank line after each row), save_row "x h" along row j, save_column "y h" along column i; invalid_argument
 * for a row or column outside the grid, runtime_error "Plane.save_csv: cannot write <path>" (and likewise). */
int lmw_plane_save_csv(lmw_plane *p, const char *path);
int lmw_plane_save_row(lmw_plane *p, int j, const char *path);
int lmw_plane_save_column(lmw_plane *p, int i, const char *path);
/* the handle's CUDA stream (a cudaStream_t) */
int lmw_plane_stream(const lmw_plane *p, void **stream);

/* Allocation-free RK4 stepping of the plane, for callers that cannot allocate device memory: code that runs
 * inside a fixed memory budget taken up front, a real-time loop where cudaMalloc would stall on device-wide
 * synchronisation, or a host that hands out device memory only from its own pool. No counterpart in the
 * reference (whose Plane::step, cpp/plane.cpp:143-158, allocates its stage vectors on the host heap).
 *
 * h, u (nx*ny doubles) and v (nx*(ny+1) doubles) are caller-owned DEVICE pointers in the layouts above; they
 * are advanced in place by `steps` RK4 steps of size dt with the same kernels, and the same bits, as
 * lmw_plane_step. Rows 0 and ny of v are the channel walls: the call sets them to zero on `stream` before the
 * first step, as lmw_plane_set_v does for the handle. The parameters mean what they mean in lmw_plane_create. The call only enqueues work on
 * `stream` (a cudaStream_t; NULL is the default stream) and returns; the fields are ready when the stream
 * reaches that point. It calls no cudaMalloc, cudaFree or other allocating routine: the stage inputs and the
 * accumulator live in one fixed device array that every GPU loading this library reserves until the process
 * exits (about 19 MB). Grids above 262144 cells (nx*ny) are rejected with LMW_INVALID_ARGUMENT.
 *
 * The first call in a CUDA context looks up that array's device address in that context (once per context,
 * with it current; the array is loaded again at another address after cudaDeviceReset or in a second context
 * made on the same device, and such a context gets its own look-up); make that first call before any stream
 * capture. Every call shares the array and it keeps the last
 * call's contents (each step overwrites what it reads, so nothing needs clearing): calls whose work overlaps on
 * the GPU, on different streams or different threads, race on it and must be serialised by the caller. */
int lmw_plane_step_noalloc(int nx, int ny, double lx, double ly, double gravity, double depth, double f0, double beta,
                           double viscosity, double drag, int linear, double *h, double *u, double *v, double dt, int steps,
                           void *stream);
/* average device time (ms) of one RK4-stage kernel launch over `reps` launches; the state is left unchanged.
 * No reference counterpart (measurement hook). */
int lmw_plane_kernel_time(lmw_plane *p, double dt, int reps, double *ms);

/* ---------------------------------------------------------------------------------------- ensemble */

typedef struct lmw_ensemble lmw_ensemble;
/* An ensemble of spheres with mixed truncations (no single reference counterpart: each member is a
 * Sphere(T, SphereParams) of cpp/sphere.hpp:29 initialised by lmw_sphere_turbulence with nforce = T/2 and del^4
 * diffusion with a 1-day e-folding at n = T). Members of one truncation are stepped together as one batch;
 * precision and split_terms as in lmw_sphere_create_split. Arrays have `count` entries. */
int lmw_ensemble_create(int count, const int *truncation, const uint64_t *seed, const double *mean_height, const double *omega, double radius,
                        double gravity, double max_wind, int precision, int split_terms, lmw_ensemble **out);
int lmw_ensemble_destroy(lmw_ensemble *e);
/* Sphere::run(seconds, 0) for every member (cpp/sphere.cpp:457-484): each truncation group at its own stable step
 * (stable_dt(1.5), the smallest over the group), the guards every 64 steps over every member. */
int lmw_ensemble_run(lmw_ensemble *e, double seconds);
/* per truncation group: truncation, member count, and the step size and step count of the last run */
int lmw_ensemble_groups(lmw_ensemble *e, int *ngroups, int *truncations, int *counts, double *last_dt, int64_t *last_steps);
/* one member's spectral state (reference layout of its truncation), diagnostics (as lmw_sphere_diagnostics) and grids */
int lmw_ensemble_member_state(lmw_ensemble *e, int member, double *zeta, double *delta, double *phi);
int lmw_ensemble_member_set_state(lmw_ensemble *e, int member, const double *zeta, const double *delta, const double *phi);
/* every member's state at once (checkpoint and restart of a whole ensemble): each field holds the members in order,
 * member i in the reference layout ((T_i+1)^2 complex values, interleaved re/im) after the sum over j < i of
 * (T_j+1)^2 values. The layout conversion runs on the device; one host <-> device copy per run of consecutive
 * members of one truncation (pinned host memory copies fastest). set_states keeps each member's time. No reference
 * counterpart (the reference has no ensembles). */
int lmw_ensemble_get_states(lmw_ensemble *e, double *zeta, double *delta, double *phi);
int lmw_ensemble_set_states(lmw_ensemble *e, const double *zeta, const double *delta, const double *phi);
int lmw_ensemble_member_diagnostics(lmw_ensemble *e, int member, double *out);
int lmw_ensemble_member_grid(lmw_ensemble *e, int member, int which, double *out, size_t n);
/* the CUDA stream of a truncation group, and its stage-kernel times as lmw_sphere_kernel_times (measurement
 * hooks; the group's packed split operands are rebuilt before its next step) */
int lmw_ensemble_stream(lmw_ensemble *e, int group, void **stream);
/* the split path's launch plan as the engine's autotuner measured it at creation: out[0] latitude pairs per grid
 * CTA, out[1] FFT stages per shared-memory pass, out[2] synthesis and out[3] analysis pipeline stages, out[4] 1
 * when an analysis CTA handles both parities of m, out[5] the analysis CTA count (0: one per work item; else
 * persistent CTAs), out[6] 1 when the grid kernel writes the analysis operands (else the analysis gathers them
 * from an FP32 fold), out[7] the analysis kernel's register budget in CTAs per SM (2: 128 registers a thread, 3:
 * 80), out[8] the synthesis's latitude slices per (m, member tile) (1, 2 or 4), out[9] 0 for the analysis kernel
 * that alternates its MMAs and its epilogue, else the CTAs per SM (1 or 2) of the warp-specialised persistent
 * analysis (one warp streams operands, one issues MMAs into two tensor-memory accumulators, eight run the epilogue
 * of the previous item), out[10] 1 when the grid kernel is the one compiled for the transform length (lengths
 * 2^6 to 2^10; its FFT groups address shared memory with immediates), 0 for the any-length form, out[11] 0 for the
 * synthesis kernel that alternates its MMAs and its epilogue, else the CTAs per SM (1 or 2) of the warp-specialised
 * persistent synthesis (zeros when the engine is not in split precision; out has 12 entries). No reference
 * counterpart. */
int lmw_sphere_split_plan(lmw_sphere *s, int *out);
/* replaces the autotuned plan with `plan` (the 12 entries above), checked against the limits the autotuner's
 * candidates obey (invalid_argument otherwise); every plan computes the same arithmetic. Validation and tuning
 * hook; no reference counterpart. */
int lmw_sphere_set_split_plan(lmw_sphere *s, const int *plan);
/* The split path's treatment of the linear terms of the tendencies (cpp/sphere.cpp:338-390 computes every term
 * on the grid). linear_exact = 1 (the default): the terms that are linear in the state are added exactly in
 * spectral space by the analysis epilogue (in FP32, from the stage input rounded to FP32) -- n(n+1)/a^2 Phi in d delta, -Phi_mean delta in d Phi (the mean
 * height's gravity-wave term; D(U, V) = delta holds exactly for n <= T) and, for an untilted axis, the Coriolis
 * terms -D(fU, fV) and D(fV, -fU) with f = 2 Omega mu, which couple n - 1, n and n + 1 -- and only the nonlinear
 * products (U zeta, V zeta, U Phi', V Phi', E) go through the BF16 pieces. linear_exact = 0: every term through the
 * BF16 GEMMs (the plain split form). Mathematically the same tendencies; the forms differ in rounding only.
 * No reference counterpart (precision choice). */
int lmw_sphere_set_split_form(lmw_sphere *s, int linear_exact);
int lmw_ensemble_set_split_form(lmw_ensemble *e, int linear_exact);
/* writes `code` into a split-precision engine's error word, as a tensor-core wait that ran out does: the next step
 * or guard check fails with LMW_DEVICE_ERROR ("a wait on the tensor cores timed out ..."). Failure-detection
 * hook (the failure is made on the host); no reference counterpart. */
int lmw_sphere_inject_split_error(lmw_sphere *s, int code);
int lmw_ensemble_split_plan(lmw_ensemble *e, int group, int *out);
int lmw_ensemble_kernel_times(lmw_ensemble *e, int group, int reps, double *ms);

/* ---------------------------------------------------------------------------------------- learned surrogate */
/* No counterpart in the reference (it has no learned component). A residual MLP advances the packed spectral
 * state of a sphere by one window; plain RK4 (Sphere::run, cpp/sphere.cpp:457-484) generates its training data,
 * checks it and takes members over. Every GEMM of training and inference runs on tcgen05 with BF16 operands and
 * FP32 accumulation; weights are kept in FP32 for Adam. */

typedef struct lmw_mlp lmw_mlp;
/* four layers in_dim -> hidden -> hidden -> hidden -> out_dim, GELU after the first three; hidden and max_batch
 * multiples of 128; weights ~ N(0, 1/fan_in) (the last layer scaled by last_layer_scale), biases zero */
int lmw_mlp_create(int in_dim, int hidden, int out_dim, int max_batch, uint64_t seed, double last_layer_scale, lmw_mlp **out);
int lmw_mlp_destroy(lmw_mlp *m);
/* host row-major W [nout][nin] (logical sizes) and b [nout] of layer 0..3 */
int lmw_mlp_set_layer(lmw_mlp *m, int layer, const float *w, const float *b);
int lmw_mlp_get_layer(lmw_mlp *m, int layer, float *w, float *b);
/* y [batch][out_dim] = net(x [batch][in_dim]); batch a multiple of 128 */
int lmw_mlp_forward(lmw_mlp *m, const float *x, int batch, float *y);
/* forward, loss = 1/(2 batch) sum_f mask_f (y - target)^2 and the gradients of every layer; mask [out_dim] holds
 * per-output weights (0 masks an output; null: all 1) */
int lmw_mlp_backward(lmw_mlp *m, const float *x, const float *target, const float *mask, int batch, double *loss);
int lmw_mlp_get_grad(lmw_mlp *m, int layer, float *gw, float *gb);
/* one Adam step from the last gradients */
int lmw_mlp_adam(lmw_mlp *m, double lr, double beta1, double beta2, double eps);
/* device time (ms) of one training step (forward, backward, Adam) and of one forward pass at this batch; the
 * weights move (by a 1e-12 learning rate) */
int lmw_mlp_time(lmw_mlp *m, int batch, int reps, double *train_ms, double *forward_ms);
/* C [M][N] = bf16(A [M][K]) bf16(B [N][K])^T on the tensor cores (host buffers; M, N multiples of 128, K of 64) */
int lmw_gemm_bf16(const float *a, const float *b, int M, int N, int K, float *c);

typedef struct lmw_surrogate lmw_surrogate;
/* surrogate of a sphere of this truncation over windows of window_seconds, trained on RK4 runs with step dt;
 * hidden width as lmw_mlp_create; del^4 diffusion with a 1-day e-folding at n = T, as in the training runs */
int lmw_surrogate_create(int truncation, int hidden, uint64_t seed, double window_seconds, double dt, double radius, double omega, double gravity,
                         lmw_surrogate **out);
int lmw_surrogate_destroy(lmw_surrogate *s);
/* dims[0] = features (6 (T+1)(T+2)/2), dims[1] = padded features, dims[2] = hidden */
int lmw_surrogate_dims(lmw_surrogate *s, int *dims);
/* training data: `trajectories` members (seeds seed0 + i, balanced turbulence with nforce = T/2 and 30 m/s, mean
 * heights uniform in [hmin, hmax] from seed0) each run for `windows` windows by RK4 in `precision`; snapshots kept
 * on the device. seconds = wall time. */
int lmw_surrogate_generate(lmw_surrogate *s, int trajectories, int windows, uint64_t seed0, double hmin, double hmax, int precision,
                           double *seconds);
/* after a fit: `trajectories` more training trajectories (seeds seed0 + i, heights from seed0 as above) that start
 * where the network takes a state -- balanced turbulence advanced net_windows windows by the network -- and then
 * record the generated window count of RK4 in `precision`. They are placed before the existing trajectories; the
 * held-out validation trajectories of the first fit stay held out, and the normalisation stays. A following fit
 * continues from the current weights. No reference counterpart. */
int lmw_surrogate_generate_drifted(lmw_surrogate *s, int trajectories, int net_windows, uint64_t seed0, double hmin, double hmax, int precision,
                                   double *seconds);
/* Adam with a cosine learning rate from lr to lr_min over `epochs` epochs of the training trajectories (the last
 * val_fraction of the trajectories are held out). loss_mode 0: mean square of the per-n normalised increments;
 * 1: energy norm of the increment error (kinetic energy of the vorticity and divergence errors plus available
 * potential energy of the Phi errors). stats: [0] final training loss per step, [1] validation
 * per-window height error mean, [2] median, [3] 90th percentile, [4] max, [5] persistence error mean, [6] the
 * untrained network's error mean, [7] seconds, [8] optimiser steps */
int lmw_surrogate_fit(lmw_surrogate *s, int epochs, int batch, double lr, double lr_min, double val_fraction, uint64_t shuffle_seed,
                      int loss_mode, double *stats);
/* per-window relative L2 height errors of the network and of persistence on stored pairs [first, first + count) */
int lmw_surrogate_evaluate(lmw_surrogate *s, int first, int count, double *err, double *persistence);
/* one window of the network on host states [count][features] (packed spectral order of lmw_sphere_get_state's
 * packed layout: field, then m, then n, real and imaginary parts), in place */
int lmw_surrogate_advance(lmw_surrogate *s, int count, double *states);
/* hybrid rollout of `members` held-out members over `windows` windows; RK4 (check_precision) recomputes every
 * check_every-th window and takes members over whose relative L2 height error exceeds threshold. out[16]:
 * [0] hybrid s, [1] network s, [2] check s, [3] takeover s, [4] members taken over, [5] checks, [6] median
 * window error, [7] max, [8] fraction over threshold, [9] plain FP64 RK4 s for ref_windows windows, [10]
 * ref_windows, [11] hybrid member-sim-days/s, [12] plain RK4 member-sim-days/s, [13] network-only
 * member-sim-days/s, [14] mean window error, [15] 90th percentile. window_err (optional): [check][member],
 * -1 where the member was already taken over. final_states (optional): [member][features] after the last window.
 * Member j starts from balanced turbulence with seed seed0 + j and a mean height drawn from a 64-bit Mersenne
 * Twister seeded with seed0 (uniform in [hmin, hmax]). */
int lmw_surrogate_rollout(lmw_surrogate *s, int members, uint64_t seed0, double hmin, double hmax, int windows, int check_every, double threshold,
                          int check_precision, int ref_windows, double *out, double *window_err, double *final_states);
/* a fresh network (weights from seed) and optimiser; the training data stay */
int lmw_surrogate_reset(lmw_surrogate *s, uint64_t seed);
/* adaptive gradient clipping of training: the global gradient norm is held to at most ratio times its running
 * mean (default 2; 0 switches clipping off) */
int lmw_surrogate_set_clip(lmw_surrogate *s, double ratio);
/* on != 0 (the default): each training pair entering a batch is first mapped by a random symmetry of the untilted
 * equations, the same for the state and its successor -- a rotation about the polar axis (coefficient (m, n) times
 * e^{i m a}) and, for half of the pairs, the reflection mu -> -mu (Phi and delta times (-1)^(n-m), zeta times
 * -(-1)^(n-m)). No reference counterpart. */
int lmw_surrogate_set_augment(lmw_surrogate *s, int on);
/* decay in (0, 1): the trained network is the exponential moving average (this decay per step) of the weights over
 * the second half of lmw_surrogate_fit's steps (the default, 0.9995); 0: the last weights. No reference
 * counterpart. */
int lmw_surrogate_set_averaging(lmw_surrogate *s, double decay);
/* weight of the kinetic-energy part of the energy-norm training loss against the available potential energy
 * (default 1, the energy norm; below 1 leans the fit toward the height field). Set before the first fit. No
 * reference counterpart. */
int lmw_surrogate_set_kinetic_weight(lmw_surrogate *s, double weight);
/* what lmw_surrogate_rollout does with a member whose checked window exceeds the threshold: mode 0 (the default)
 * -- RK4 takes the member over for the rest of the rollout; mode 1 -- RK4's result (plain FP64) replaces that
 * window and the network keeps advancing the member (RK4 as the per-window fallback; out[4] of the rollout then
 * counts replaced member-windows). No reference counterpart. */
int lmw_surrogate_set_takeover(lmw_surrogate *s, int mode);
/* maps = 1: the network advances a state as it is. maps = 2k (the default 8): the network is applied to the state
 * under k rotations about the polar axis by multiples of 2 pi / k, each without and with the equatorial
 * reflection, each increment is mapped back, and the 2k increments are averaged (the exact dynamics commute with
 * these maps). Used by lmw_surrogate_advance, _rollout and the validation errors of _fit. No reference
 * counterpart. */
int lmw_surrogate_set_symmetry_average(lmw_surrogate *s, int maps);
/* per epoch of the last fit: mean training loss and mean global gradient norm per step (count = epochs; at most
 * max values written) */
int lmw_surrogate_history(lmw_surrogate *s, int max, double *loss, double *grad_norm, int *count);
/* device time (ms) of one training step and of one forward pass of the surrogate's network */
int lmw_surrogate_time(lmw_surrogate *s, int batch, int reps, double *train_ms, double *forward_ms);

#ifdef __cplusplus
}
#endif
#endif
