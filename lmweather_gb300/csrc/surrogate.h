// Learned surrogate of the spectral solver: a residual MLP that advances the packed spectral state of a sphere
// by one fixed window (6 hours at T42), trained on trajectories the solver generates, with every GEMM of its
// forward and backward passes on tcgen05 (BF16 operands, FP32 accumulation in tensor memory).
#pragma once
#include <cuda_bf16.h>

#include <memory>
#include <vector>

#include "engine.h"

namespace lmw {

// Four fully connected layers d0 -> h -> h -> h -> d4 with GELU after the first three. Feature dimensions are
// padded to multiples of 128 (padding stays exactly zero: zero inputs, zero weights, masked outputs); batches are
// multiples of 128. Every BF16 matrix lives in the blocked layout of the GEMM kernel (128-row blocks x 64-wide K
// chunks, each a contiguous 16 KB tile in the MMA's core-matrix order). FP32 master weights and Adam moments.
class Mlp {
 public:
  Mlp(int in_dim, int hidden, int out_dim, int max_batch, uint64_t seed, double last_layer_scale);
  ~Mlp();
  Mlp(const Mlp &) = delete;
  Mlp &operator=(const Mlp &) = delete;

  static constexpr int NL = 4;
  int din = 0, dout = 0, hidden = 0, max_batch = 0;
  int dim[NL + 1] = {0, 0, 0, 0, 0};  // padded layer widths
  int adam_t = 0;
  cudaStream_t stream = nullptr;

  struct Layer {
    int nin = 0, nout = 0;  // padded
    DevBuf<float> w, b, m, v, mb, vb, gw, gb;
    DevBuf<float> we, be;  // moving averages of w and b (allocated by ema_begin)
    DevBuf<__nv_bfloat16> wb, wt;  // blocked W [nout][nin] and W^T [nin][nout]
  };
  Layer L[NL];
  DevBuf<__nv_bfloat16> x0;              // input, blocked [batch][dim0]
  DevBuf<__nv_bfloat16> z[NL - 1], a[NL - 1];  // pre-activations and activations, blocked [batch][h]
  DevBuf<__nv_bfloat16> tact, tgrad;     // transposed activation / gradient, blocked [features][batch]
  DevBuf<__nv_bfloat16> dy, dz[2];       // output gradient [batch][dim4], hidden gradients [batch][h]
  DevBuf<float> y;                       // output, row-major [batch][dim4]
  DevBuf<float> target, mask;            // row-major [batch][dim4]; per output feature 1 or 0
  DevBuf<double> loss_acc, gnorm2, clip;
  DevBuf<float> gscale;
  DevBuf<int> err;

  // host row-major weights of the logical size [nout][nin] and biases [nout]
  void set_layer(int l, const float *w, const float *b);
  void get_layer(int l, float *w, float *b);
  void get_grad(int l, float *gw, float *gb);
  // host batch -> device (x [batch][din], target [batch][dout], mask [dout])
  void upload_input(const float *x, int batch);
  void upload_target(const float *t, const float *m, int batch);
  void download_output(float *y_host, int batch);

  void forward(int batch);                 // x0 -> y
  void backward(int batch);                // y, target, mask -> gradients; loss accumulated into loss_acc
  // clip_ratio > 0: the global gradient norm is clipped to clip_ratio times its running mean (on the device)
  void adam(double lr, double beta1, double beta2, double eps, double clip_ratio = 0.0);
  // moving average of the master weights, updated by every adam() step from ema_begin on (decay per step);
  // ema_apply() makes the average the network's weights and stops the averaging
  double ema_decay = 0;
  void ema_begin(double decay);
  void ema_apply();
  double take_grad_norm_sum();             // synchronises; the summed gradient norms since the last call
  double take_loss();                      // synchronises; returns and clears the accumulated loss
  void check_status();
  // average duration (ms) of one forward + backward + Adam step at this batch (CUDA events on the stream)
  double time_train_step(int batch, int reps);
  double time_forward(int batch, int reps);

 private:
  void publish(int l);  // FP32 master weights -> BF16 blocked copies
};

// GEMM of the blocked layout on tcgen05, exposed for its own test: C[M][N] = A[M][K] B[N][K]^T, FP32 row-major C
void mlp_gemm_f32(const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int N, int K, float *C, int ldc, const float *bias, int *err,
                  cudaStream_t s);
// host row-major [rows][cols] FP32 -> BF16 blocked (cols padded to a multiple of 64, rows to 128) and back
void to_blocked(const float *host, int rows, int cols, int rows_p, int cols_p, __nv_bfloat16 *dev, cudaStream_t s);

// A symmetry map of the untilted shallow-water equations on spectral states: rotation by 2 pi `turn` about the polar
// axis (coefficient (m, n) times e^{i m 2 pi turn}), then, with `reflect`, the equatorial reflection (Phi and delta
// times (-1)^(n-m), zeta times -(-1)^(n-m)). seed != 0: a random map per batch row instead.
struct SymMap {
  uint64_t seed = 0;
  float turn = 0.0f;
  int reflect = 0;
};

struct SurrogateStats {
  double train_loss = 0, val_err_mean = 0, val_err_median = 0, val_err_p90 = 0, val_err_max = 0, val_persist_mean = 0, val_untrained_mean = 0;
  double seconds = 0, steps = 0;
};

// The surrogate of one truncation: solver trajectories -> per-n normalisation -> training -> hybrid rollouts.
class Surrogate {
 public:
  Surrogate(int truncation, int hidden, uint64_t seed, double window_seconds, double dt, double radius, double omega, double gravity);
  ~Surrogate();
  int T = 42, ntri = 0, nfeat = 0, hidden = 4096;
  double window = 21600.0, dt = 900.0;
  double clip_ratio = 2.0;  // adaptive gradient clipping of training (0: off)
  // training pairs mapped by a random symmetry of the untilted equations (a rotation about the polar axis and,
  // for half of them, the equatorial reflection) each time they enter a batch
  bool augment = true;
  // decay of the moving average of the weights kept over the last half of a fit and used as the trained network
  // (0: the last weights)
  double ema = 0.9995;
  std::vector<double> hist_loss, hist_gnorm;  // per epoch of the last fit: mean loss and gradient norm per step
  SphereConfig cfg;
  std::unique_ptr<Mlp> net;
  cudaStream_t stream = nullptr;

  // dataset: snapshots [traj][nwin + 1][dp] (FP32) of solver runs from seeded balanced turbulence
  int ntraj = 0, nwin = 0;
  DevBuf<float> snaps;
  DevBuf<float> mu, sig, sigd, outmask, cw;
  DevBuf<int> fmq;  // per feature: m | (n - m) << 8 | field << 16
  // inference averages the network's increments over this many symmetry maps of the input (rotations about the
  // polar axis by multiples of 2 pi / (n / 2), each without and with the equatorial reflection), each increment
  // mapped back to the state's frame; 1: the plain network
  int sym_average = 8;
  DevBuf<float> incbuf;  // averaged increments of one batch [batch][dp]
  SymMap sym_map(int k) const;
  DevBuf<int> idx;
  DevBuf<double> errs;
  bool have_norm = false;
  double gen_seconds = 0;
  // training loss: 0 = mean square of the per-n normalised increments, 1 = energy norm of the increment error
  // (kinetic energy of the vorticity/divergence errors plus available potential energy of the Phi errors)
  int loss_mode = 1;
  // weight of the kinetic-energy part of the energy-norm loss against the available potential energy (1: the
  // energy norm itself; below 1 leans the fit toward the height field)
  double ke_weight = 1.0;
  // what a failed check does: 0 = RK4 takes the member over for the rest of the rollout; 1 = RK4's result
  // replaces that window of the member and the network keeps advancing it (RK4 as the per-window fallback)
  int takeover_mode = 0;

  void reset(uint64_t seed);  // a fresh network and optimiser (the data stay)
  void generate(int trajectories, int windows, uint64_t seed0, double hmin, double hmax, int precision, int batch_members);
  // more training trajectories that start where the network takes a state: seeded balanced turbulence advanced
  // net_windows windows by the network, then `windows` windows of RK4 recorded as generate() does. They go before
  // the existing trajectories, so the held-out validation trajectories stay the same (val_traj)
  void generate_drifted(int trajectories, int net_windows, uint64_t seed0, double hmin, double hmax, int precision, int batch_members);
  int val_traj = 0;  // held-out trajectories at the end of the data, fixed by the first fit
  void normalise(int ntrain_trajectories);
  SurrogateStats fit(int epochs, int batch, double lr, double lr_min, double val_fraction, uint64_t shuffle_seed);
  // per-window height errors of the current network on pairs [p0, p1): out[i] (network), pers[i] (persistence)
  void evaluate(int p0, int p1, std::vector<double> &err, std::vector<double> &pers);
  // one window of the network on device FP64 states [count][nfeat] in place; members with mode[b] != 0 are
  // left unchanged (mode may be null)
  void advance_states(double *states, int count, const int *mode);

  // hybrid rollout of `members` held-out members; out: see lmw_surrogate_rollout
  void rollout(int members, uint64_t seed0, double hmin, double hmax, int windows, int check_every, double threshold, int check_precision,
               int ref_windows, double *out, double *window_err, double *final_states);

 private:
  DevBuf<double> rs_state, rs_start;
  DevBuf<int> rs_mode;
};

}  // namespace lmw
