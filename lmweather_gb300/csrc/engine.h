// Engine objects behind the C ABI: device-resident state, one CUDA stream per object.
#pragma once
#include <memory>

#include "lmw_internal.h"

namespace lmw {

// ------------------------------------------------------------------------------------------------ plane
// Mirrors lmweather::PlaneParams (cpp/plane.hpp:9-18).
struct PlaneConfig {
  int nx = 0, ny = 0;
  double lx = 0, ly = 0;
  double gravity = 9.81, depth = 100, f0 = 0, beta = 0, viscosity = 0, drag = 0;
  bool linear = false;
};

class PlaneEngine {
 public:
  explicit PlaneEngine(const PlaneConfig &c);
  ~PlaneEngine();
  PlaneConfig p;
  double t = 0;

  size_t ncell() const { return static_cast<size_t>(p.nx) * p.ny; }
  size_t nvpt() const { return static_cast<size_t>(p.nx) * (p.ny + 1); }
  double dx() const { return p.lx / p.nx; }
  double dy() const { return p.ly / p.ny; }

  void reset();
  void set_h(const double *g, size_t n);
  void set_u(const double *g, size_t n);
  void set_v(const double *g, size_t n);
  void get(double *h, double *u, double *v);
  void perturb(double amplitude, uint64_t seed);
  void jet(double u0, double width, double noise_rms, uint64_t seed);
  void step(double dt);
  void run(double seconds, double dt);
  double stable_dt(double safety);
  // mean_depth, energy, max_speed, pv_anomaly_rms
  void diagnostics(double *out);
  // point and harmonic diagnostics of cpp/plane.cpp:220-310, computed on the device
  double probe(int kind, double x, double y);  // kind 0 h_at, 1 u_at, 2 v_at
  double zeta_at_corner(int i, int j);
  double zonal_amplitude(int m, int j);
  double zonal_crest(int m, int j);
  double v_zonal_crest(int m, int j);
  double harmonic_energy(int m);
  // the wx layer's text files (cpp/main.cpp:464-494)
  void save_csv(const std::string &path);
  void save_row(int j, const std::string &path);
  void save_column(int i, const std::string &path);
  // device pointers of the state (h, u, v), valid until the engine is destroyed
  void device_state(double **h, double **u, double **v) {
    *h = h0.p; *u = u0.p; *v = v0.p;
  }
  cudaStream_t stream = nullptr;
  // enqueue one RK4 step on the engine stream (no synchronisation)
  void enqueue_step(double dt);
  // average duration (ms) of one RK4-stage kernel launch over `reps` launches, timed with CUDA events on the
  // engine stream; the state is left unchanged
  double kernel_time(double dt, int reps);

 private:
  DevBuf<double> h0, u0, v0, ha, ua, va, hb, ub, vb, ah, au, av;
  DevBuf<double> part, diag;
  DevBuf<Reduce> dred;
  HostBuf<Reduce> hred;
  HostBuf<double> stage;
  int nblk_red = 0;
  cudaGraphExec_t graph = nullptr;
  double graph_dt = 0;
  int graph_steps = 0;
  void reduce(Reduce &r);
  double read_scalars(int n, double *out);
  void row_harmonic(int kind, int m, int j, double shift, double *re, double *im);
  void upload(double *dst, const double *src, size_t n);
  void launch_chunk(double dt, int steps);
};

// RK4 steps of caller-owned device fields with the scratch in a fixed device array (no allocation)
void plane_step_noalloc(const PlaneConfig &c, double *h, double *u, double *v, double dt, int steps, cudaStream_t stream);

// ------------------------------------------------------------------------------------------------ sphere
// Mirrors lmweather::SphereParams (cpp/sphere.hpp:20-25) plus the engine's precision mode.
enum Precision { kFP64 = 0, kFP32 = 1, kSplitBF16 = 2 };

struct SphereConfig {
  int truncation = 42;
  double radius = 6.37122e6, omega = 7.292e-5, gravity = 9.80616, diffusion = 0;
  int precision = kFP64;
  int members = 1;          // ensemble members sharing the truncation (batch dimension)
  int split_terms = 3;      // BF16 products per Legendre term in the split mode: 3 (hi/lo) or 6 (hi/mid/lo)
  int max_truncation = 341; // the reference caps at 170; the engine allows up to this
};

struct SphereTables;
struct SplitPlan;

class SphereEngine {
 public:
  explicit SphereEngine(const SphereConfig &c);
  ~SphereEngine();
  SphereConfig p;
  int N = 0, M = 0, nlat = 0, nlon = 0, nh = 0, ntri = 0, B = 1;
  std::vector<double> t;  // per member model time
  cudaStream_t stream = nullptr;

  size_t ngrid() const { return static_cast<size_t>(nlat) * nlon; }
  size_t nspec_ref() const { return static_cast<size_t>(M) * M; }  // the reference's (T+1)^2 layout

  void set_axis_tilt(double alpha, int member);
  void set_omega(double omega, int member);
  void set_diffusion(double nu4) { p.diffusion = nu4; filt_dt = -1; }
  void set_orography(const double *hs, size_t n, int member);
  void set_state_grid(const double *h, const double *u, const double *v, size_t n, int member);
  void set_state(const double *zeta, const double *delta, const double *phi, double time, int member);
  void get_state(double *zeta, double *delta, double *phi, int member);
  void add_mode(int n, int m, double amplitude, double mean_depth, int member);
  void perturb(double amplitude, uint64_t seed, int max_wave, int member);
  void turbulence(uint64_t seed, double mean_height, double max_wind, int nforce, int member);
  void mark_reference(int member);
  void step(double dt);
  void run(double seconds, double dt);
  double stable_dt(double safety, int member);
  double stable_dt_all(double safety);
  // a run split into guard-sized chunks, so that several engines can interleave their work on their streams
  struct RunPlan {
    int64_t n = 0, i = 0;
    double h = 0;
    bool guard_due = false;
  };
  RunPlan plan_run(double seconds, double dt);
  bool advance(RunPlan &rp);
  void guard(RunPlan &rp);
  // mean_height, kinetic, potential, energy, enstrophy, max_wind, error_l2, error_linf
  void diagnostics(double *out, int member);
  // which: 0 height, 1 u, 2 v, 3 vorticity
  void grid(int which, double *out, int member);
  void spectrum(double *ke, double *pe, int member);
  // every member's state in the reference layout, [field][member][(T+1)^2] complex, on the device:
  // x0 -> that buffer (asynchronous on the engine stream; returns its device pointer), and back
  double *states_to_ref();
  double *device_refstates();
  void states_from_ref();
  // the reference's transform test hooks (cpp/sphere.hpp:96-99), FP64 on the device: grids [nlat][nlon],
  // spectra in the reference layout ((T+1)^2 complex, interleaved)
  void analyze_scalar(const double *grid, size_t n, double *spec);
  void synthesize_scalar(const double *spec, double *grid, size_t n);
  void analyze_divergence(const double *A, const double *B, size_t n, double *spec);
  // the wx layer's text files (cpp/main.cpp:328-335, 357-384)
  void save_csv(const std::string &path, int member);
  void save_zonal_mean(const std::string &path, int member);
  void save_spectrum(const std::string &path, int member);
  // exact point values at (lat, lon) in radians from the spectral state (cpp/sphere.cpp:287-299, 592-637): which
  // 0 height, 1 zonal wind u, 2 meridional wind v, 3 vorticity, 4 tracer
  double probe(int which, double lat, double lon, int member);
  // cpp/sphere.cpp:639-652: h's spectral component (n, m), and the longitude of a crest of h's zonal harmonic m
  double mode_coefficient(int n, int m, bool imag, int member);
  double wave_crest(int m, double lat, int member);
  void enqueue_step(double dt);
  // passive tracer q (cpp/sphere.cpp:250-263, 264-300), FP64 precision only: set from a grid per member, advected
  // by the flow (or by a frozen flow in advect-only mode), filtered like Phi
  bool has_tracer = false, advect_only = false;
  void set_tracer_grid(const double *q, size_t n, int member);
  void set_advect_only(bool on);
  void tracer_grid(double *out, int member);
  void synth_tracer_grid(int member, double *dst_device);
  void tracer_state(double *q_ref_layout, int member);
  void set_tracer_state(const double *q_ref_layout, int member);
  // mean, mass (area mean of h q) and l2 / linf errors against the grid the tracer was set from
  void tracer_diagnostics(double *out, int member);
  // device pointer of the packed spectral state [member][field][tri] complex128 (FP64 state accumulation)
  double *device_state() { return x0.p; }
  // to be called after the state was written through device_state() (repacks the split operands)
  void state_written() { split_packed = false; }
  DevBuf<int> gflag;   // per member: bit 0 tilted Coriolis grid, bit 1 orography
  DevBuf<double> om2;  // per member: 2 Omega
  uint64_t launches_per_step() const { return launches_step; }
  // average duration (ms) per launch of each stage kernel class over `reps` launches (CUDA events on the
  // engine stream): out[0] synthesis, out[1] grid (FFTs + products), out[2] analysis + RK4 update. x0 unchanged.
  void kernel_times(double dt, int reps, double *out);
  // the split path's measured launch plan: latitude pairs per grid CTA, FFT stages per pass, synthesis and
  // analysis pipeline stages, both parities per analysis CTA, analysis CTA count (6 values; zeros without the split
  // path)
  void split_plan(int *out) const;
  // replaces the autotuned plan (same 7 entries as split_plan); checked against the shared-memory and
  // tensor-memory limits the autotuner's candidates obey
  void set_split_plan(const int *in);
  // 1 (default): the linear terms of the tendencies in spectral space (FP32), the nonlinear products through the BF16
  // pieces; 0: every term through the BF16 GEMMs
  void set_split_form(int linear_exact);
  // writes `code` into the split path's error word, as a tensor-core wait that ran out does (failure tests)
  void inject_split_error(int code);

 private:
  SphereTables *tab = nullptr;
  SplitPlan *split = nullptr;
  bool split_packed = false;
  void check_split_status();
  void ensure_packed();
  void autotune_split();
  // state (packed triangle, complex interleaved), stage input, accumulator; a second stage input (split form)
  DevBuf<double> x0, xs, acc, xs2;
  double2 *XS2() { return reinterpret_cast<double2 *>(xs2.p); }
  DevBuf<double> refstates;  // every member's state in the reference layout (allocated on first use)
  DevBuf<double> hookspec;   // one spectrum in the reference layout for the transform hooks (allocated on first use)
  void hook_analysis(const double *A, const double *B, size_t n, double *spec);

  // Fourier coefficients of the synthesised grids, folded analysis inputs
  DevBuf<double> four, fold;
  DevBuf<float> four32, fold32;
  DevBuf<double> fgrid, hsgrid, refgrid, filt, diagrows;
  DevBuf<double> tq0, tqs, tqacc, fourq, foldq, refq, tgrid;  // tracer state, stage input, accumulator; transforms
  void ensure_tracer();
  void tracer_stage(int stage, double dt, int part);
  std::vector<int> gflag_h;
  void upload_member_flags(int member);
  DevBuf<double> gridin;
  DevBuf<Reduce> dred;
  HostBuf<Reduce> hred;
  HostBuf<double> hstage;
  std::vector<double> omega_m;
  std::vector<char> has_orog;
  double filt_dt = -1;
  uint64_t launches_step = 0;
  // captured step chunks, keyed by (dt, steps); the guard-sized chunk and a run's remainder chunk both stay
  struct ChunkGraph {
    double dt;
    int steps;
    cudaGraphExec_t exec;
  };
  std::vector<ChunkGraph> graphs;
  void graphs_clear();
  void upload_filter(double dt);
  void launch_stage(int stage, double dt);
  void launch_chunk(double dt, int steps);
  void synth_grids(int member_first, int count);  // state x0 -> Fourier coefficients of U, V, zeta, phi
  void reduce_guard(Reduce &r, int member);
  void reduce_guard_all(bool exact = true);
  double limit_from(const Reduce &r, int b, double safety) const;
  void analyze_grids_to_state(int member);
  void to_packed(const double *ref_layout, double *packed);
  void from_packed(const double *packed, double *ref_layout);
};

// ------------------------------------------------------------------------------------------------ ensemble
struct MemberSpec {
  int truncation = 42;
  uint64_t seed = 1;
  double mean_height = 8000.0;
  double omega = 7.292e-5;
};

class EnsembleEngine {
 public:
  EnsembleEngine(const std::vector<MemberSpec> &specs, double radius, double gravity, double max_wind, int precision, int split_terms);
  std::vector<MemberSpec> members;
  std::vector<std::unique_ptr<SphereEngine>> groups;
  std::vector<int> truncations, group_of, index_in_group;
  std::vector<double> last_dt;
  std::vector<int64_t> last_steps;
  void run(double seconds);
  void check_member(int i) const;
  // every member's spectral state at once in the reference layout, members in order (member i at offset
  // sum_{j<i} (T_j+1)^2 complex values of each field); one host <-> device copy per run of consecutive members of a
  // truncation group
  void get_states(double *zeta, double *delta, double *phi);
  void set_states(const double *zeta, const double *delta, const double *phi);
  SphereEngine &engine_of(int i, int *k) {
    check_member(i);
    *k = index_in_group[i];
    return *groups[group_of[i]];
  }
};

}  // namespace lmw
