// Learned surrogate: BF16 MLP training and inference on tcgen05, solver-generated training data, hybrid rollouts
// in which plain RK4 checks the network and takes members over.
//
// GEMM layout. Every BF16 matrix X[R][K] (R a multiple of 128, K of 64) is stored blocked: tile (R/128, K/64)
// holds 128 rows x 64 columns in the MMA's K-major core-matrix order (core matrix = 8 rows x 8 columns, 128 B
// contiguous; 8 core matrices along K form an 8-row group of 1 KB), so every tile is one contiguous 16 KB run that
// one bulk asynchronous copy moves into shared memory and one no-swizzle descriptor addresses. C = A B^T with both
// operands K-major covers all three GEMMs of a layer: forward (X W^T), input gradient (dZ (W^T)^T) and weight
// gradient (dZ^T (X^T)^T); the transposed operands are written by small tile-transpose kernels and, for W^T, by
// the optimiser.
#include <cuda_bf16.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>

#include "surrogate.h"
#include "tc_common.cuh"

namespace lmw {

namespace {

using bf16 = __nv_bfloat16;
constexpr int BK = 64;
constexpr int TILE = 128 * BK;  // elements of one blocked tile (16 KB)

inline int pad128(int x) { return (x + 127) / 128 * 128; }

__host__ __device__ inline long boff(int r, int k, int K) {
  return (static_cast<long>(r >> 7) * (K >> 6) + (k >> 6)) * TILE + ((((r & 127) >> 3) << 3) + ((k & 63) >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

// GELU(z) = z Phi(z) with the normal CDF Phi(z) = (1 + erf(z / sqrt 2)) / 2; derivative Phi(z) + z phi(z)
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

enum Epi { EPI_F32 = 0, EPI_GELU = 1, EPI_DGELU = 2 };

struct GemmArgs {
  const bf16 *A, *B;
  int M, N, K;
  int epi;
  float *C;
  int ldc;
  const float *bias;
  bf16 *Z, *Act;    // EPI_GELU: pre-activation and activation, blocked [M][N]
  const bf16 *Zin;  // EPI_DGELU: pre-activation, blocked [M][N]
  bf16 *Dz;         // EPI_DGELU: gradient of the pre-activation, blocked [M][N]
  int *err;
};

// One 128 x BN output tile per CTA. Thread 0 streams (A, B) K chunks through S shared-memory stages with bulk
// copies; thread 32 issues the MMAs (4 per chunk, K = 16 each) into a 128 x BN FP32 accumulator in TMEM and frees
// each stage with tcgen05.commit; then all four warps read their 32 TMEM lanes back and apply the epilogue.
template <int BN, int S>
__global__ void __launch_bounds__(128, 1) mlp_gemm(GemmArgs g) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full[S], empty[S], done;
  __shared__ uint32_t tslot;
  __shared__ int fail, issued, consumed;
  constexpr int STAGE = (128 + BN) * BK * 2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n0 = blockIdx.x * BN, m0 = blockIdx.y * 128;
  const int nk = g.K / BK;
  if (warp == 0) tc::tmem_alloc(tc::su32(&tslot), BN);
  if (tid == 0) {
    for (int s = 0; s < S; s++) {
      tc::bar_init(tc::su32(&full[s]), 1);
      tc::bar_init(tc::su32(&empty[s]), 1);
    }
    tc::bar_init(tc::su32(&done), 1);
    tc::bar_init_fence();
    fail = 0;
    issued = 0;
    consumed = 0;
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  if (tid == 0) {
    const bf16 *a_src = g.A + static_cast<long>(m0 >> 7) * nk * TILE;
    for (int it = 0; it < nk; it++) {
      const int st = it % S;
      if (it >= S && !tc::wait(tc::su32(&empty[st]), ((it / S) - 1) & 1)) {
        fail = 1;
        atomicExch(g.err, 1);
        break;
      }
      const uint32_t bar = tc::su32(&full[st]);
      tc::expect_tx(bar, STAGE);
      uint8_t *base = smem + st * STAGE;
      tc::bulk_g2s(tc::su32(base), a_src + static_cast<long>(it) * TILE, TILE * 2, bar);
#pragma unroll
      for (int j = 0; j < BN / 128; j++)
        tc::bulk_g2s(tc::su32(base + (j + 1) * TILE * 2), g.B + (static_cast<long>((n0 >> 7) + j) * nk + it) * TILE, TILE * 2, bar);
      issued = it + 1;
    }
  } else if (tid == 32) {
    const uint32_t idesc = tc::idesc_m128(BN);
    bool ok = true;
    for (int it = 0; it < nk; it++) {
      const int st = it % S;
      if (!tc::wait(tc::su32(&full[st]), (it / S) & 1)) {
        fail = 1;
        atomicExch(g.err, 2);
        ok = false;
        break;
      }
      consumed = it + 1;
      tc::fence_after();
      const uint32_t base = tc::su32(smem + st * STAGE);
#pragma unroll
      for (int kk = 0; kk < 4; kk++)
        tc::mma(tmem, tc::chunk_desc(base + kk * 256), tc::chunk_desc(base + TILE * 2 + kk * 256), idesc, (it | kk) != 0 ? 1u : 0u);
      tc::commit(tc::su32(&empty[st]));
    }
    // completes `done` when every MMA issued so far has finished (after a failed wait too: the CTA drains its
    // own work before it frees tensor memory)
    tc::commit(tc::su32(&done));
  }
  __syncthreads();
  if (tid == 0) {
    if (!fail) {
      if (!tc::wait(tc::su32(&done), 0)) {
        fail = 1;
        atomicExch(g.err, 3);
      }
    } else {
      // a wait ran out: wait a bounded time for the MMAs in flight and for the bulk copies issued but not
      // consumed, so that none lands after the CTA has released its shared and tensor memory
      tc::wait_for(tc::su32(&done), 0, 200000000ull);
      for (int it = consumed; it < issued; it++) tc::wait_for(tc::su32(&full[it % S]), (it / S) & 1, 200000000ull);
    }
  }
  __syncthreads();
  tc::fence_after();
  if (!fail) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t lanebase = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    for (int cb = 0; cb < BN; cb += 32) {
      float v[32];
      tc::ld32(lanebase + cb, v);
      const int col = n0 + cb;
      if (g.epi == EPI_F32) {
        if (g.bias) {
#pragma unroll
          for (int i = 0; i < 32; i++) v[i] += g.bias[col + i];
        }
        float4 *dst = reinterpret_cast<float4 *>(g.C + static_cast<long>(row) * g.ldc + col);
#pragma unroll
        for (int q = 0; q < 8; q++) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      } else if (g.epi == EPI_GELU) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
          uint4 zz, aa;
          bf16 *zp = reinterpret_cast<bf16 *>(&zz), *ap = reinterpret_cast<bf16 *>(&aa);
#pragma unroll
          for (int j = 0; j < 8; j++) {
            const float z = v[8 * q + j] + g.bias[col + 8 * q + j];
            zp[j] = __float2bfloat16_rn(z);
            ap[j] = __float2bfloat16_rn(gelu(z));
          }
          const long o = boff(row, col + 8 * q, g.N);
          *reinterpret_cast<uint4 *>(g.Z + o) = zz;
          *reinterpret_cast<uint4 *>(g.Act + o) = aa;
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const long o = boff(row, col + 8 * q, g.N);
          const uint4 zz = *reinterpret_cast<const uint4 *>(g.Zin + o);
          const bf16 *zp = reinterpret_cast<const bf16 *>(&zz);
          uint4 dd;
          bf16 *dp = reinterpret_cast<bf16 *>(&dd);
#pragma unroll
          for (int j = 0; j < 8; j++) dp[j] = __float2bfloat16_rn(v[8 * q + j] * gelu_grad(__bfloat162float(zp[j])));
          *reinterpret_cast<uint4 *>(g.Dz + o) = dd;
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, BN);
}

constexpr int S256 = 4, S128 = 3;
constexpr size_t smem_bytes(int bn, int s) { return static_cast<size_t>(s) * (128 + bn) * BK * 2; }

void gemm_attrs() {
  int dev = 0;
  LMW_CUDA(cudaGetDevice(&dev));
  static bool done[64] = {false};
  if (dev < 0 || dev >= 64 || done[dev]) return;
  LMW_CUDA(cudaFuncSetAttribute(mlp_gemm<256, S256>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem_bytes(256, S256))));
  LMW_CUDA(cudaFuncSetAttribute(mlp_gemm<128, S128>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem_bytes(128, S128))));
  done[dev] = true;
}

void gemm(const GemmArgs &g, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.K <= 0 || g.M % 128 || g.N % 128 || g.K % BK) throw InvalidArgument("GEMM sizes must be multiples of 128 (M, N) and 64 (K)");
  gemm_attrs();
  const bool wide = g.N % 256 == 0 && (g.M / 128) * (g.N / 256) >= 148;
  if (wide) mlp_gemm<256, S256><<<dim3(g.N / 256, g.M / 128), 128, smem_bytes(256, S256), s>>>(g);
  else mlp_gemm<128, S128><<<dim3(g.N / 128, g.M / 128), 128, smem_bytes(128, S128), s>>>(g);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
}

// blocked [R][C] -> blocked [C][R], one 64 x 64 block per CTA
__global__ void transpose_blocked(const bf16 *__restrict__ in, bf16 *__restrict__ out, int R, int C) {
  __shared__ bf16 s[64][72];
  const int c0 = blockIdx.x * 64, r0 = blockIdx.y * 64;
  for (int e = threadIdx.x; e < 512; e += blockDim.x) {
    const int rr = e >> 3, cg = e & 7;
    const uint4 val = *reinterpret_cast<const uint4 *>(in + boff(r0 + rr, c0 + cg * 8, C));
    const bf16 *p = reinterpret_cast<const bf16 *>(&val);
#pragma unroll
    for (int j = 0; j < 8; j++) s[cg * 8 + j][rr] = p[j];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 512; e += blockDim.x) {
    const int cc = e >> 3, rg = e & 7;
    uint4 val;
    bf16 *p = reinterpret_cast<bf16 *>(&val);
#pragma unroll
    for (int j = 0; j < 8; j++) p[j] = s[cc][rg * 8 + j];
    *reinterpret_cast<uint4 *>(out + boff(c0 + cc, r0 + rg * 8, R)) = val;
  }
}

void transpose(const bf16 *in, bf16 *out, int R, int C, cudaStream_t s) {
  transpose_blocked<<<dim3(C / 64, R / 64), 256, 0, s>>>(in, out, R, C);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
}

// bias gradient: row sums of the transposed gradient (blocked [N][batch]), one warp per row reading 16-byte
// chunks; a fixed reduction order (deterministic)
__global__ void rowsum_blocked(const bf16 *__restrict__ gt, float *__restrict__ out, int N, int batch) {
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= N) return;
  float s = 0.0f;
  for (int k8 = lane * 8; k8 < batch; k8 += 256) {
    const uint4 v = *reinterpret_cast<const uint4 *>(gt + boff(row, k8, batch));
    const bf16 *p = reinterpret_cast<const bf16 *>(&v);
#pragma unroll
    for (int j = 0; j < 8; j++) s += __bfloat162float(p[j]);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[row] = s;
}

// loss 1/(2 batch) sum_f w_f (y - t)^2 with per-output weights w (0 masks an output) and its gradient
// dY = w (y - t) / batch (blocked BF16)
__global__ void loss_grad(const float *__restrict__ y, const float *__restrict__ t, const float *__restrict__ mask, bf16 *__restrict__ dy, int ld,
                          float inv_b, double *loss) {
  const int b = blockIdx.x;
  float acc = 0.0f;
  for (int f8 = threadIdx.x * 8; f8 < ld; f8 += blockDim.x * 8) {
    uint4 out;
    bf16 *p = reinterpret_cast<bf16 *>(&out);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const long i = static_cast<long>(b) * ld + f8 + j;
      const float e = y[i] - t[i], wgt = mask[f8 + j];
      acc += wgt * e * e;
      p[j] = __float2bfloat16_rn(wgt * e * inv_b);
    }
    *reinterpret_cast<uint4 *>(dy + boff(b, f8, ld)) = out;
  }
  __shared__ float red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); w++) s += red[w];
    atomicAdd(loss, 0.5 * static_cast<double>(s) * inv_b);
  }
}

struct AdamArgs {
  float *w, *m, *v;
  const float *g;
  bf16 *wb, *wt;
  int nout, nin;
  float lr, b1, b2, eps, c1, c2;
  int update;
  const float *scale;  // gradient scale from the clipping kernel (null: 1)
  float *ema;          // exponential moving average of the master weights (null: none), decay ema_decay
  float ema_decay;
};

// Adam on a 64 x 64 tile of W [nout][nin] (FP32 row-major), then the BF16 blocked copies W [nout][nin] and
// W^T [nin][nout] of the tile. update = 0 only publishes the master weights.
__global__ void adam_tile(AdamArgs a) {
  __shared__ bf16 s[64][72];
  const int k0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  for (int e = threadIdx.x; e < 4096; e += blockDim.x) {
    const int rr = e >> 6, cc = e & 63;
    const long i = static_cast<long>(n0 + rr) * a.nin + k0 + cc;
    float w = a.w[i];
    if (a.update) {
      const float g = a.g[i] * (a.scale ? *a.scale : 1.0f);
      const float m = a.b1 * a.m[i] + (1.0f - a.b1) * g;
      const float v = a.b2 * a.v[i] + (1.0f - a.b2) * g * g;
      w -= a.lr * (m * a.c1) / (sqrtf(v * a.c2) + a.eps);
      a.m[i] = m;
      a.v[i] = v;
      a.w[i] = w;
      if (a.ema) a.ema[i] = a.ema_decay * a.ema[i] + (1.0f - a.ema_decay) * w;
    }
    s[rr][cc] = __float2bfloat16_rn(w);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 512; e += blockDim.x) {
    const int rr = e >> 3, g8 = e & 7;
    uint4 val;
    bf16 *p = reinterpret_cast<bf16 *>(&val);
#pragma unroll
    for (int j = 0; j < 8; j++) p[j] = s[rr][g8 * 8 + j];
    *reinterpret_cast<uint4 *>(a.wb + boff(n0 + rr, k0 + g8 * 8, a.nin)) = val;
#pragma unroll
    for (int j = 0; j < 8; j++) p[j] = s[g8 * 8 + j][rr];
    *reinterpret_cast<uint4 *>(a.wt + boff(k0 + rr, n0 + g8 * 8, a.nout)) = val;
  }
}

__global__ void adam_vec(float *w, float *m, float *v, const float *g, int n, float lr, float b1, float b2, float eps, float c1, float c2,
                         const float *scale, float *ema, float ema_decay) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] * (scale ? *scale : 1.0f);
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  m[i] = mi;
  v[i] = vi;
  if (ema) ema[i] = ema_decay * ema[i] + (1.0f - ema_decay) * w[i];
}

// sum of squares of n values into *acc (double)
__global__ void sumsq(const float *__restrict__ x, long n, double *acc) {
  double s = 0;
  for (long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; i < n; i += static_cast<long>(gridDim.x) * blockDim.x) {
    const double v = x[i];
    s += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); w++) t += red[w];
    atomicAdd(acc, t);
  }
}

// adaptive clipping: the global gradient norm is held to at most `ratio` times its running mean (the first
// steps set the mean); clip[0] = scale for this step, clip[1] = running mean, clip[2] += this step's norm
__global__ void clip_scale(const double *gnorm2, float *scale, double *clip, float ratio) {
  const double norm = sqrt(*gnorm2);
  double mean = clip[1];
  if (!(mean > 0)) mean = norm;
  const double cap = ratio * mean;
  scale[0] = norm > cap && norm > 0 ? static_cast<float>(cap / norm) : 1.0f;
  clip[1] = 0.99 * mean + 0.01 * (norm < cap ? norm : cap);
  clip[2] += norm;
}

__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// W[i][k] ~ N(0, scale^2) on the logical block (Box-Muller on two counter-based uniforms), zero in the padding
__global__ void init_normal(float *w, int nout, int nin, int nout_l, int nin_l, float scale, uint64_t seed) {
  const long total = static_cast<long>(nout) * nin;
  for (long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; i < total; i += static_cast<long>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i / nin), c = static_cast<int>(i % nin);
    float val = 0.0f;
    if (r < nout_l && c < nin_l) {
      const uint64_t h = splitmix(seed ^ splitmix(static_cast<uint64_t>(i)));
      const float u1 = (static_cast<float>(h >> 40) + 0.5f) * (1.0f / 16777216.0f);
      const float u2 = static_cast<float>((h >> 16) & 0xFFFFFFull) * (1.0f / 16777216.0f);
      val = scale * sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    }
    w[i] = val;
  }
}

// row-major FP32 [rows][cols] (leading dimension ld) -> blocked BF16 [rows_p][cols_p], zero outside
__global__ void pack_blocked(const float *__restrict__ src, int rows, int cols, int ld, bf16 *__restrict__ dst, int rows_p, int cols_p) {
  const long chunks = static_cast<long>(rows_p) * (cols_p / 8);
  for (long e = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; e < chunks; e += static_cast<long>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(e / (cols_p / 8)), c8 = static_cast<int>(e % (cols_p / 8)) * 8;
    uint4 val;
    bf16 *p = reinterpret_cast<bf16 *>(&val);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int c = c8 + j;
      p[j] = __float2bfloat16_rn(r < rows && c < cols ? src[static_cast<long>(r) * ld + c] : 0.0f);
    }
    *reinterpret_cast<uint4 *>(dst + boff(r, c8, cols_p)) = val;
  }
}

int grid_for(long n, int threads) { return static_cast<int>(std::min<long>((n + threads - 1) / threads, 152L * 16)); }

}  // namespace

// ------------------------------------------------------------------------------------------------ Mlp
Mlp::Mlp(int in_dim, int hidden_, int out_dim, int max_batch_, uint64_t seed, double last_layer_scale)
    : din(in_dim), dout(out_dim), hidden(hidden_), max_batch(max_batch_) {
  if (in_dim < 1 || out_dim < 1) throw InvalidArgument("network dimensions must be positive");
  if (hidden_ < 128 || hidden_ % 128) throw InvalidArgument("the hidden width must be a positive multiple of 128");
  if (max_batch_ < 128 || max_batch_ % 128) throw InvalidArgument("the batch must be a positive multiple of 128");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) throw DeviceError("no CUDA device");
  dim[0] = pad128(in_dim);
  dim[1] = dim[2] = dim[3] = hidden_;
  dim[4] = pad128(out_dim);
  LMW_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  const int nin_l[NL] = {in_dim, hidden_, hidden_, hidden_};
  const int nout_l[NL] = {hidden_, hidden_, hidden_, out_dim};
  for (int l = 0; l < NL; l++) {
    Layer &Ly = L[l];
    Ly.nin = dim[l];
    Ly.nout = dim[l + 1];
    const size_t nw = static_cast<size_t>(Ly.nin) * Ly.nout;
    Ly.w.alloc(nw);
    Ly.m.alloc(nw);
    Ly.v.alloc(nw);
    Ly.gw.alloc(nw);
    Ly.b.alloc(Ly.nout);
    Ly.mb.alloc(Ly.nout);
    Ly.vb.alloc(Ly.nout);
    Ly.gb.alloc(Ly.nout);
    Ly.wb.alloc(nw);
    Ly.wt.alloc(nw);
    Ly.m.zero(stream);
    Ly.v.zero(stream);
    Ly.gw.zero(stream);
    Ly.b.zero(stream);
    Ly.mb.zero(stream);
    Ly.vb.zero(stream);
    Ly.gb.zero(stream);
    const double scale = (l == NL - 1 ? last_layer_scale : 1.0) / std::sqrt(static_cast<double>(nin_l[l]));
    init_normal<<<grid_for(static_cast<long>(nw), 256), 256, 0, stream>>>(Ly.w.p, Ly.nout, Ly.nin, nout_l[l], nin_l[l], static_cast<float>(scale),
                                                                         seed * 0x100000001B3ull + static_cast<uint64_t>(l) + 1);
    LMW_LAUNCH_CHECK();
    publish(l);
  }
  const int hmax = std::max(dim[0], hidden_), gmax = std::max(hidden_, dim[4]);
  x0.alloc(static_cast<size_t>(max_batch) * dim[0]);
  for (int i = 0; i < NL - 1; i++) {
    z[i].alloc(static_cast<size_t>(max_batch) * hidden_);
    a[i].alloc(static_cast<size_t>(max_batch) * hidden_);
  }
  tact.alloc(static_cast<size_t>(max_batch) * hmax);
  tgrad.alloc(static_cast<size_t>(max_batch) * gmax);
  dy.alloc(static_cast<size_t>(max_batch) * dim[4]);
  dz[0].alloc(static_cast<size_t>(max_batch) * hidden_);
  dz[1].alloc(static_cast<size_t>(max_batch) * hidden_);
  y.alloc(static_cast<size_t>(max_batch) * dim[4]);
  target.alloc(static_cast<size_t>(max_batch) * dim[4]);
  mask.alloc(dim[4]);
  x0.zero(stream);
  target.zero(stream);
  {
    std::vector<float> mk(dim[4], 0.0f);
    for (int i = 0; i < out_dim; i++) mk[i] = 1.0f;
    LMW_CUDA(cudaMemcpyAsync(mask.p, mk.data(), mk.size() * sizeof(float), cudaMemcpyHostToDevice, stream));
    LMW_CUDA(cudaStreamSynchronize(stream));
  }
  loss_acc.alloc(1);
  loss_acc.zero(stream);
  gnorm2.alloc(1);
  gscale.alloc(1);
  clip.alloc(3);
  clip.zero(stream);
  err.alloc(1);
  err.zero(stream);
  LMW_CUDA(cudaStreamSynchronize(stream));
}

Mlp::~Mlp() {
  if (stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
}

void Mlp::publish(int l) {
  Layer &Ly = L[l];
  AdamArgs a{Ly.w.p, Ly.m.p, Ly.v.p, Ly.gw.p, Ly.wb.p, Ly.wt.p, Ly.nout, Ly.nin, 0, 0, 0, 0, 0, 0, 0, nullptr};
  adam_tile<<<dim3(Ly.nin / 64, Ly.nout / 64), 256, 0, stream>>>(a);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
}

void Mlp::set_layer(int l, const float *w, const float *b) {
  if (l < 0 || l >= NL) throw InvalidArgument("layer index out of range");
  Layer &Ly = L[l];
  const int nin_l = l == 0 ? din : hidden, nout_l = l == NL - 1 ? dout : hidden;
  LMW_CUDA(cudaStreamSynchronize(stream));
  Ly.w.zero(stream);
  Ly.b.zero(stream);
  LMW_CUDA(cudaMemcpy2DAsync(Ly.w.p, Ly.nin * sizeof(float), w, nin_l * sizeof(float), nin_l * sizeof(float), nout_l, cudaMemcpyHostToDevice, stream));
  if (b) LMW_CUDA(cudaMemcpyAsync(Ly.b.p, b, nout_l * sizeof(float), cudaMemcpyHostToDevice, stream));
  publish(l);
  LMW_CUDA(cudaStreamSynchronize(stream));
}

void Mlp::get_layer(int l, float *w, float *b) {
  if (l < 0 || l >= NL) throw InvalidArgument("layer index out of range");
  Layer &Ly = L[l];
  const int nin_l = l == 0 ? din : hidden, nout_l = l == NL - 1 ? dout : hidden;
  LMW_CUDA(cudaMemcpy2DAsync(w, nin_l * sizeof(float), Ly.w.p, Ly.nin * sizeof(float), nin_l * sizeof(float), nout_l, cudaMemcpyDeviceToHost, stream));
  if (b) LMW_CUDA(cudaMemcpyAsync(b, Ly.b.p, nout_l * sizeof(float), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
}

void Mlp::get_grad(int l, float *gw, float *gb) {
  if (l < 0 || l >= NL) throw InvalidArgument("layer index out of range");
  Layer &Ly = L[l];
  const int nin_l = l == 0 ? din : hidden, nout_l = l == NL - 1 ? dout : hidden;
  LMW_CUDA(cudaMemcpy2DAsync(gw, nin_l * sizeof(float), Ly.gw.p, Ly.nin * sizeof(float), nin_l * sizeof(float), nout_l, cudaMemcpyDeviceToHost, stream));
  if (gb) LMW_CUDA(cudaMemcpyAsync(gb, Ly.gb.p, nout_l * sizeof(float), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
}

static void check_batch(int batch, int max_batch) {
  if (batch < 128 || batch % 128 || batch > max_batch) throw InvalidArgument("the batch must be a multiple of 128 and at most the network's batch");
}

void Mlp::upload_input(const float *x, int batch) {
  check_batch(batch, max_batch);
  DevBuf<float> tmp;
  tmp.alloc(static_cast<size_t>(batch) * din);
  LMW_CUDA(cudaMemcpyAsync(tmp.p, x, tmp.bytes(), cudaMemcpyHostToDevice, stream));
  pack_blocked<<<grid_for(static_cast<long>(batch) * dim[0] / 8, 256), 256, 0, stream>>>(tmp.p, batch, din, din, x0.p, batch, dim[0]);
  LMW_LAUNCH_CHECK();
  LMW_CUDA(cudaStreamSynchronize(stream));
}

void Mlp::upload_target(const float *t, const float *m, int batch) {
  check_batch(batch, max_batch);
  target.zero(stream);
  LMW_CUDA(cudaMemcpy2DAsync(target.p, dim[4] * sizeof(float), t, dout * sizeof(float), dout * sizeof(float), batch, cudaMemcpyHostToDevice, stream));
  if (m) {
    mask.zero(stream);
    LMW_CUDA(cudaMemcpyAsync(mask.p, m, dout * sizeof(float), cudaMemcpyHostToDevice, stream));
  }
  LMW_CUDA(cudaStreamSynchronize(stream));
}

void Mlp::download_output(float *yh, int batch) {
  check_batch(batch, max_batch);
  LMW_CUDA(cudaMemcpy2DAsync(yh, dout * sizeof(float), y.p, dim[4] * sizeof(float), dout * sizeof(float), batch, cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
}

void Mlp::forward(int batch) {
  check_batch(batch, max_batch);
  const int h = hidden;
  const bf16 *in = x0.p;
  int kin = dim[0];
  for (int l = 0; l < NL - 1; l++) {
    GemmArgs g{};
    g.A = in;
    g.B = L[l].wb.p;
    g.M = batch;
    g.N = h;
    g.K = kin;
    g.epi = EPI_GELU;
    g.bias = L[l].b.p;
    g.Z = z[l].p;
    g.Act = a[l].p;
    g.err = err.p;
    gemm(g, stream);
    in = a[l].p;
    kin = h;
  }
  GemmArgs g{};
  g.A = a[NL - 2].p;
  g.B = L[NL - 1].wb.p;
  g.M = batch;
  g.N = dim[4];
  g.K = h;
  g.epi = EPI_F32;
  g.C = y.p;
  g.ldc = dim[4];
  g.bias = L[NL - 1].b.p;
  g.err = err.p;
  gemm(g, stream);
}

void Mlp::backward(int batch) {
  check_batch(batch, max_batch);
  const int h = hidden;
  loss_grad<<<batch, 256, 0, stream>>>(y.p, target.p, mask.p, dy.p, dim[4], 1.0f / batch, loss_acc.p);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
  // gradient of the current layer's output (pre-activation for hidden layers), blocked [batch][width]
  const bf16 *gcur = dy.p;
  int wcur = dim[4];
  int zi = 0;
  for (int l = NL - 1; l >= 0; l--) {
    const bf16 *act = l == 0 ? x0.p : a[l - 1].p;
    const int win = dim[l];
    transpose(gcur, tgrad.p, batch, wcur, stream);
    transpose(act, tact.p, batch, win, stream);
    GemmArgs gw{};
    gw.A = tgrad.p;
    gw.B = tact.p;
    gw.M = wcur;
    gw.N = win;
    gw.K = batch;
    gw.epi = EPI_F32;
    gw.C = L[l].gw.p;
    gw.ldc = win;
    gw.err = err.p;
    gemm(gw, stream);
    rowsum_blocked<<<(wcur + 7) / 8, 256, 0, stream>>>(tgrad.p, L[l].gb.p, wcur, batch);
    LMW_LAUNCH_CHECK();
    g_launches += 1;
    if (l == 0) break;
    GemmArgs gd{};
    gd.A = gcur;
    gd.B = L[l].wt.p;
    gd.M = batch;
    gd.N = win;
    gd.K = wcur;
    gd.epi = EPI_DGELU;
    gd.Zin = z[l - 1].p;
    gd.Dz = dz[zi].p;
    gd.err = err.p;
    gemm(gd, stream);
    gcur = dz[zi].p;
    zi ^= 1;
    wcur = h;
  }
}

void Mlp::adam(double lr, double beta1, double beta2, double eps, double clip_ratio) {
  adam_t += 1;
  const float c1 = static_cast<float>(1.0 / (1.0 - std::pow(beta1, adam_t))), c2 = static_cast<float>(1.0 / (1.0 - std::pow(beta2, adam_t)));
  const float *scale = nullptr;
  if (clip_ratio > 0) {
    LMW_CUDA(cudaMemsetAsync(gnorm2.p, 0, sizeof(double), stream));
    for (int l = 0; l < NL; l++) {
      const long nw = static_cast<long>(L[l].nin) * L[l].nout;
      sumsq<<<grid_for(nw, 256), 256, 0, stream>>>(L[l].gw.p, nw, gnorm2.p);
      LMW_LAUNCH_CHECK();
      sumsq<<<grid_for(L[l].nout, 256), 256, 0, stream>>>(L[l].gb.p, L[l].nout, gnorm2.p);
      LMW_LAUNCH_CHECK();
    }
    clip_scale<<<1, 1, 0, stream>>>(gnorm2.p, gscale.p, clip.p, static_cast<float>(clip_ratio));
    LMW_LAUNCH_CHECK();
    g_launches += 2 * NL + 1;
    scale = gscale.p;
  }
  for (int l = 0; l < NL; l++) {
    Layer &Ly = L[l];
    const bool avg = ema_decay > 0 && Ly.we.p != nullptr;
    AdamArgs a{Ly.w.p, Ly.m.p, Ly.v.p, Ly.gw.p, Ly.wb.p, Ly.wt.p, Ly.nout, Ly.nin, static_cast<float>(lr), static_cast<float>(beta1), static_cast<float>(beta2),
               static_cast<float>(eps), c1, c2, 1, scale, avg ? Ly.we.p : nullptr, static_cast<float>(ema_decay)};
    adam_tile<<<dim3(Ly.nin / 64, Ly.nout / 64), 256, 0, stream>>>(a);
    LMW_LAUNCH_CHECK();
    adam_vec<<<(Ly.nout + 255) / 256, 256, 0, stream>>>(Ly.b.p, Ly.mb.p, Ly.vb.p, Ly.gb.p, Ly.nout, static_cast<float>(lr), static_cast<float>(beta1),
                                                       static_cast<float>(beta2), static_cast<float>(eps), c1, c2, scale, avg ? Ly.be.p : nullptr,
                                                       static_cast<float>(ema_decay));
    LMW_LAUNCH_CHECK();
    g_launches += 2;
  }
}

// averaged weights: the moving average starts at the present master weights; ema_apply makes the average the
// network's weights (master and BF16 copies)
void Mlp::ema_begin(double decay) {
  if (!(decay > 0 && decay < 1)) throw InvalidArgument("the averaging decay must lie in (0, 1)");
  ema_decay = decay;
  for (int l = 0; l < NL; l++) {
    Layer &Ly = L[l];
    if (!Ly.we.p) {
      Ly.we.alloc(Ly.w.n);
      Ly.be.alloc(Ly.b.n);
    }
    LMW_CUDA(cudaMemcpyAsync(Ly.we.p, Ly.w.p, Ly.w.bytes(), cudaMemcpyDeviceToDevice, stream));
    LMW_CUDA(cudaMemcpyAsync(Ly.be.p, Ly.b.p, Ly.b.bytes(), cudaMemcpyDeviceToDevice, stream));
  }
}

void Mlp::ema_apply() {
  if (!(ema_decay > 0)) return;
  for (int l = 0; l < NL; l++) {
    Layer &Ly = L[l];
    LMW_CUDA(cudaMemcpyAsync(Ly.w.p, Ly.we.p, Ly.w.bytes(), cudaMemcpyDeviceToDevice, stream));
    LMW_CUDA(cudaMemcpyAsync(Ly.b.p, Ly.be.p, Ly.b.bytes(), cudaMemcpyDeviceToDevice, stream));
    publish(l);
  }
  ema_decay = 0;
}

double Mlp::take_grad_norm_sum() {
  double v[3] = {0, 0, 0};
  LMW_CUDA(cudaMemcpyAsync(v, clip.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  const double zero = 0;
  LMW_CUDA(cudaMemcpyAsync(clip.p + 2, &zero, sizeof(double), cudaMemcpyHostToDevice, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  return v[2];
}

void Mlp::check_status() {
  int e = 0;
  LMW_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  if (e) {
    err.zero(stream);
    throw RuntimeError("a tensor-core GEMM of the network timed out waiting on its pipeline (code " + std::to_string(e) + ")");
  }
}

double Mlp::take_loss() {
  double v = 0;
  LMW_CUDA(cudaMemcpyAsync(&v, loss_acc.p, sizeof(double), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  loss_acc.zero(stream);
  check_status();
  return v;
}

double Mlp::time_train_step(int batch, int reps) {
  check_batch(batch, max_batch);
  cudaEvent_t e0, e1;
  LMW_CUDA(cudaEventCreate(&e0));
  LMW_CUDA(cudaEventCreate(&e1));
  // timing only: the moments and weights move, so save and restore nothing; callers time a scratch network
  forward(batch);
  backward(batch);
  LMW_CUDA(cudaEventRecord(e0, stream));
  for (int r = 0; r < reps; r++) {
    forward(batch);
    backward(batch);
    adam(1e-12, 0.9, 0.999, 1e-8, 2.0);
  }
  LMW_CUDA(cudaEventRecord(e1, stream));
  LMW_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  LMW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  loss_acc.zero(stream);
  check_status();
  return ms / reps;
}

double Mlp::time_forward(int batch, int reps) {
  check_batch(batch, max_batch);
  cudaEvent_t e0, e1;
  LMW_CUDA(cudaEventCreate(&e0));
  LMW_CUDA(cudaEventCreate(&e1));
  forward(batch);
  LMW_CUDA(cudaEventRecord(e0, stream));
  for (int r = 0; r < reps; r++) forward(batch);
  LMW_CUDA(cudaEventRecord(e1, stream));
  LMW_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  LMW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  check_status();
  return ms / reps;
}

void mlp_gemm_f32(const bf16 *A, const bf16 *B, int M, int N, int K, float *C, int ldc, const float *bias, int *errp, cudaStream_t s) {
  GemmArgs g{};
  g.A = A;
  g.B = B;
  g.M = M;
  g.N = N;
  g.K = K;
  g.epi = EPI_F32;
  g.C = C;
  g.ldc = ldc;
  g.bias = bias;
  g.err = errp;
  gemm(g, s);
}

void to_blocked(const float *host, int rows, int cols, int rows_p, int cols_p, bf16 *dev, cudaStream_t s) {
  DevBuf<float> tmp;
  tmp.alloc(static_cast<size_t>(rows) * cols);
  LMW_CUDA(cudaMemcpyAsync(tmp.p, host, tmp.bytes(), cudaMemcpyHostToDevice, s));
  pack_blocked<<<grid_for(static_cast<long>(rows_p) * cols_p / 8, 256), 256, 0, s>>>(tmp.p, rows, cols, cols, dev, rows_p, cols_p);
  LMW_LAUNCH_CHECK();
  LMW_CUDA(cudaStreamSynchronize(s));
}

// ------------------------------------------------------------------------------------------------ Surrogate
namespace {

// packed FP64 states [k][nfeat] -> FP32 snapshots of window w of trajectories traj0 ..
__global__ void snapshot(const double *__restrict__ st, int k, int nfeat, float *__restrict__ snaps, int traj0, int nwin1, int w, int dp) {
  const long total = static_cast<long>(k) * dp;
  for (long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; i < total; i += static_cast<long>(gridDim.x) * blockDim.x) {
    const int j = static_cast<int>(i / dp), f = static_cast<int>(i % dp);
    snaps[(static_cast<long>(traj0 + j) * nwin1 + w) * dp + f] = f < nfeat ? static_cast<float>(st[static_cast<long>(j) * nfeat + f]) : 0.0f;
  }
}

// per-feature sums over pairs [p0, p1): x, x^2 and (x' - x)^2, split over blockIdx.y
__global__ void pair_stats(const float *__restrict__ snaps, int nwin, int dp, long p0, long p1, double *__restrict__ out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= dp) return;
  const long per = (p1 - p0 + gridDim.y - 1) / gridDim.y;
  const long a = p0 + per * blockIdx.y, b = a + per < p1 ? a + per : p1;
  double s1 = 0, s2 = 0, d2 = 0;
  for (long p = a; p < b; p++) {
    const long traj = p / nwin, w = p % nwin;
    const float *xs = snaps + (traj * (nwin + 1) + w) * dp;
    const double x = xs[f], xn = xs[dp + f];
    s1 += x;
    s2 += x * x;
    d2 += (xn - x) * (xn - x);
  }
  double *o = out + (static_cast<long>(blockIdx.y) * dp + f) * 3;
  o[0] = s1;
  o[1] = s2;
  o[2] = d2;
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// the map of row b: a random one per row (24 random bits of angle, one of reflection) when map.seed != 0
__device__ __forceinline__ void sym_of_row(const SymMap &map, int b, float &t, bool &rf) {
  if (map.seed) {
    const uint64_t r = mix64(map.seed + 0x9E3779B97F4A7C15ULL * static_cast<uint64_t>(b + 1));
    t = static_cast<float>(r >> 40) * (1.0f / 16777216.0f);
    rf = (r >> 7) & 1;
  } else {
    t = map.turn;
    rf = map.reflect != 0;
  }
}

// coefficient (re, im) of a feature pair under the map: rotation by 2 pi t about the polar axis (sign < 0: the
// inverse rotation) then, with rf, the equatorial reflection. code = m | (n - m) << 8 | field << 16.
__device__ __forceinline__ void sym_apply(int code, float t, bool rf, float sign, float &re, float &im) {
  const int m = code & 255, nm = (code >> 8) & 255, q = code >> 16;
  float sn, cs;
  sincospif(2.0f * t * static_cast<float>(m), &sn, &cs);
  sn *= sign;
  const float sg = rf ? (((nm & 1) ? -1.0f : 1.0f) * (q == 0 ? -1.0f : 1.0f)) : 1.0f;
  const float xr = re, xi = im;
  re = sg * (xr * cs - xi * sn);
  im = sg * (xr * sn + xi * cs);
}

// batch of pairs -> normalised BF16 input (blocked) and normalised increments (row-major FP32). With fmq given
// and a map other than the identity, every pair is first mapped by a symmetry of the untilted shallow-water
// equations, the same for state and successor (the dynamics commute with it): a rotation about the polar axis
// (coefficient (m, n) times e^{i m a}) and, with the reflection mu -> -mu, Phi and delta coefficients times
// (-1)^(n-m) and zeta's times -(-1)^(n-m) (vorticity is odd under the reflection, as the Coriolis parameter is).
__global__ void gather_pairs(const float *__restrict__ snaps, const int *__restrict__ idx, int nwin, int dp, int nfeat, const float *__restrict__ mu,
                             const float *__restrict__ isig, const float *__restrict__ sigd, const float *__restrict__ outmask, bf16 *__restrict__ x0,
                             float *__restrict__ target, const int *__restrict__ fmq = nullptr, SymMap map = SymMap()) {
  const int b = blockIdx.x;
  const long p = idx[b];
  const long traj = p / nwin, w = p % nwin;
  const float *xs = snaps + (traj * (nwin + 1) + w) * dp, *xn = xs + dp;
  float turn = 0.0f;
  bool reflect = false;
  sym_of_row(map, b, turn, reflect);
  const bool mapped = fmq != nullptr && (map.seed != 0 || map.turn != 0.0f || map.reflect != 0);
  for (int f8 = threadIdx.x * 8; f8 < dp; f8 += blockDim.x * 8) {
    uint4 val;
    bf16 *pv = reinterpret_cast<bf16 *>(&val);
    float xv[8], dv[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int f = f8 + j;
      xv[j] = f < nfeat ? xs[f] : 0.0f;
      dv[j] = f < nfeat ? xn[f] - xs[f] : 0.0f;
    }
    if (mapped) {
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        const int f = f8 + j;
        if (f >= nfeat) break;
        sym_apply(fmq[f], turn, reflect, 1.0f, xv[j], xv[j + 1]);
        sym_apply(fmq[f], turn, reflect, 1.0f, dv[j], dv[j + 1]);
      }
    }
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int f = f8 + j;
      pv[j] = __float2bfloat16_rn(f < nfeat ? (xv[j] - mu[f]) * isig[f] : 0.0f);
      if (target) target[static_cast<long>(b) * dp + f] = outmask[f] > 0.0f ? dv[j] / sigd[f] : 0.0f;
    }
    *reinterpret_cast<uint4 *>(x0 + boff(b, f8, dp)) = val;
  }
}

__device__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); w++) s += red[w];
  return s;
}

// relative L2 height error of the network's prediction and of persistence, per pair (Phi coefficients weighted
// 1 for m = 0 and 2 for m > 0: the area mean of the squared grid field)
// inc: the predicted increments [count][dp] (un-normalised), or null for sigd * y
__global__ void pair_errors(const float *__restrict__ snaps, const int *__restrict__ idx, int nwin, int dp, const float *__restrict__ y,
                            const float *__restrict__ sigd, const float *__restrict__ outmask, const float *__restrict__ cw, int count,
                            double *__restrict__ err, double *__restrict__ pers, const float *__restrict__ inc = nullptr) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  if (b >= count) return;
  const long p = idx[b];
  const long traj = p / nwin, w = p % nwin;
  const float *xs = snaps + (traj * (nwin + 1) + w) * dp, *xn = xs + dp;
  double num = 0, den = 0, pn = 0;
  for (int f = threadIdx.x; f < dp; f += blockDim.x) {
    const double c = cw[f];
    if (c == 0.0) continue;
    const double x = xs[f], t = xn[f];
    const double pred = x + (outmask[f] > 0.0f ? (inc ? static_cast<double>(inc[static_cast<long>(b) * dp + f])
                                                       : static_cast<double>(sigd[f]) * y[static_cast<long>(b) * dp + f])
                                               : 0.0);
    num += c * (pred - t) * (pred - t);
    den += c * t * t;
    pn += c * (x - t) * (x - t);
  }
  num = block_sum(num, red);
  den = block_sum(den, red);
  pn = block_sum(pn, red);
  if (threadIdx.x == 0) {
    err[b] = sqrt(num / den);
    pers[b] = sqrt(pn / den);
  }
}

// FP64 states [count][nfeat] -> (mapped by `map` when fmq is given) normalised BF16 input rows (rows >= count zero)
__global__ void pack_states(const double *__restrict__ st, int count, int nfeat, int dp, const float *__restrict__ mu, const float *__restrict__ isig,
                            bf16 *__restrict__ x0, const int *__restrict__ fmq = nullptr, SymMap map = SymMap()) {
  const int b = blockIdx.x;
  float turn = 0.0f;
  bool reflect = false;
  sym_of_row(map, b, turn, reflect);
  for (int f8 = threadIdx.x * 8; f8 < dp; f8 += blockDim.x * 8) {
    uint4 val;
    bf16 *pv = reinterpret_cast<bf16 *>(&val);
    float xv[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int f = f8 + j;
      xv[j] = b < count && f < nfeat ? static_cast<float>(st[static_cast<long>(b) * nfeat + f]) : 0.0f;
    }
    if (fmq) {
#pragma unroll
      for (int j = 0; j < 8; j += 2)
        if (f8 + j < nfeat) sym_apply(fmq[f8 + j], turn, reflect, 1.0f, xv[j], xv[j + 1]);
    }
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int f = f8 + j;
      pv[j] = __float2bfloat16_rn(b < count && f < nfeat ? (xv[j] - mu[f]) * isig[f] : 0.0f);
    }
    *reinterpret_cast<uint4 *>(x0 + boff(b, f8, dp)) = val;
  }
}

// inc[b][f] (+)= weight * map^-1 (sigd * y) for rows b < count: the network's increment in the mapped frame taken
// back to the state's frame (first != 0 overwrites)
__global__ void accumulate_increment(const float *__restrict__ y, const float *__restrict__ sigd, const float *__restrict__ outmask, int count,
                                     int nfeat, int dp, const int *__restrict__ fmq, SymMap map, float weight, int first, float *__restrict__ inc) {
  const int b = blockIdx.x;
  if (b >= count) return;
  float turn = 0.0f;
  bool reflect = false;
  sym_of_row(map, b, turn, reflect);
  for (int f = threadIdx.x * 2; f < dp; f += blockDim.x * 2) {
    float re = 0.0f, im = 0.0f;
    if (f < nfeat) {
      re = outmask[f] > 0.0f ? sigd[f] * y[static_cast<long>(b) * dp + f] : 0.0f;
      im = outmask[f + 1] > 0.0f ? sigd[f + 1] * y[static_cast<long>(b) * dp + f + 1] : 0.0f;
      // the inverse map: the reflection is its own inverse and commutes with the rotations
      sym_apply(fmq[f], turn, false, -1.0f, re, im);
      if (reflect) sym_apply(fmq[f], 0.0f, true, 1.0f, re, im);
      if (outmask[f] <= 0.0f) re = 0.0f;
      if (outmask[f + 1] <= 0.0f) im = 0.0f;
    }
    float *o = inc + static_cast<long>(b) * dp + f;
    o[0] = first ? weight * re : o[0] + weight * re;
    o[1] = first ? weight * im : o[1] + weight * im;
  }
}

// x += inc for the members still on the network (mode 0)
__global__ void apply_increment(double *__restrict__ st, int count, int nfeat, int dp, const float *__restrict__ inc, const float *__restrict__ outmask,
                                const int *__restrict__ mode) {
  const long total = static_cast<long>(count) * nfeat;
  for (long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; i < total; i += static_cast<long>(gridDim.x) * blockDim.x) {
    const int b = static_cast<int>(i / nfeat), f = static_cast<int>(i % nfeat);
    if (mode && mode[b]) continue;
    if (outmask[f] > 0.0f) st[i] += static_cast<double>(inc[static_cast<long>(b) * dp + f]);
  }
}

// relative L2 height error between member amap[b] of a (b without a map) and member b of r
__global__ void state_errors(const double *__restrict__ a, const int *__restrict__ amap, const double *__restrict__ r, int nfeat,
                             const float *__restrict__ cw, double *__restrict__ err) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  const long ra = amap ? amap[b] : b;
  double num = 0, den = 0;
  for (int f = threadIdx.x; f < nfeat; f += blockDim.x) {
    const double c = cw[f];
    if (c == 0.0) continue;
    const double x = a[ra * nfeat + f], t = r[static_cast<long>(b) * nfeat + f];
    num += c * (x - t) * (x - t);
    den += c * t * t;
  }
  num = block_sum(num, red);
  den = block_sum(den, red);
  if (threadIdx.x == 0) err[b] = sqrt(num / den);
}

// dst[dmap[i]] = src[smap[i]] for whole members (nfeat doubles each); a null map is the identity
__global__ void copy_members(const double *__restrict__ src, const int *__restrict__ smap, double *__restrict__ dst, const int *__restrict__ dmap, int n,
                             int nfeat) {
  const long total = static_cast<long>(n) * nfeat;
  for (long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; i < total; i += static_cast<long>(gridDim.x) * blockDim.x) {
    const int k = static_cast<int>(i / nfeat), f = static_cast<int>(i % nfeat);
    const int s = smap ? smap[k] : k, d = dmap ? dmap[k] : k;
    dst[static_cast<long>(d) * nfeat + f] = src[static_cast<long>(s) * nfeat + f];
  }
}

void copy_members_launch(const double *src, const int *smap, double *dst, const int *dmap, int n, int nfeat, cudaStream_t s) {
  if (n <= 0) return;
  copy_members<<<grid_for(static_cast<long>(n) * nfeat, 256), 256, 0, s>>>(src, smap, dst, dmap, n, nfeat);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

Surrogate::Surrogate(int truncation, int hidden_, uint64_t seed, double window_seconds, double dt_, double radius, double omega, double gravity)
    : T(truncation), window(window_seconds), dt(dt_) {
  if (truncation < 4 || truncation > 170) throw InvalidArgument("truncation must be between 4 and 170");
  if (!(window_seconds > 0) || !(dt_ > 0)) throw InvalidArgument("the window and the step must be positive");
  ntri = (T + 1) * (T + 2) / 2;
  nfeat = 6 * ntri;
  cfg.truncation = T;
  cfg.radius = radius;
  cfg.omega = omega;
  cfg.gravity = gravity;
  // del^4 diffusion with a 1-day e-folding at n = T, as in the solver runs the network learns from
  cfg.diffusion = std::pow(radius, 4) / (86400.0 * std::pow(T * (T + 1.0), 2));
  cfg.precision = kFP64;
  cfg.max_truncation = 170;
  hidden = hidden_;
  net = std::make_unique<Mlp>(nfeat, hidden, nfeat, 1024, seed, 0.1);
  stream = net->stream;
  const int dp = net->dim[0];
  mu.alloc(dp);
  sig.alloc(dp);
  sigd.alloc(dp);
  outmask.alloc(dp);
  cw.alloc(dp);
  errs.alloc(2 * 1024);
  incbuf.alloc(static_cast<size_t>(net->max_batch) * dp);
  // per feature: m, n - m and field, for the symmetry maps of training pairs and of inference
  {
    std::vector<int> code(dp, 0);
    for (int q = 0; q < 3; q++)
      for (int m = 0, tri = 0; m <= T; m++)
        for (int n = m; n <= T; n++, tri++)
          for (int ri = 0; ri < 2; ri++) code[(q * ntri + tri) * 2 + ri] = m | ((n - m) << 8) | (q << 16);
    fmq.alloc(dp);
    LMW_CUDA(cudaMemcpyAsync(fmq.p, code.data(), dp * sizeof(int), cudaMemcpyHostToDevice, stream));
  }
  // Phi coefficient weights for the area-mean square of the height grid
  std::vector<float> c(dp, 0.0f);
  for (int m = 0, tri = 0; m <= T; m++)
    for (int n = m; n <= T; n++, tri++)
      for (int ri = 0; ri < 2; ri++) c[(2 * ntri + tri) * 2 + ri] = m == 0 ? 1.0f : 2.0f;
  LMW_CUDA(cudaMemcpyAsync(cw.p, c.data(), dp * sizeof(float), cudaMemcpyHostToDevice, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
}

Surrogate::~Surrogate() = default;

void Surrogate::reset(uint64_t seed) {
  net.reset();
  net = std::make_unique<Mlp>(nfeat, hidden, nfeat, 1024, seed, 0.1);
  stream = net->stream;
  have_norm = false;
  hist_loss.clear();
  hist_gnorm.clear();
}

void Surrogate::generate(int trajectories, int windows, uint64_t seed0, double hmin, double hmax, int precision, int batch_members) {
  if (trajectories < 2 || windows < 1) throw InvalidArgument("need at least two trajectories and one window");
  if (!(hmin > 0) || !(hmax >= hmin)) throw InvalidArgument("mean heights must be positive and ordered");
  const auto t0 = std::chrono::steady_clock::now();
  ntraj = trajectories;
  nwin = windows;
  have_norm = false;
  val_traj = 0;
  const int dp = net->dim[0];
  snaps.alloc(static_cast<size_t>(ntraj) * (nwin + 1) * dp);
  std::mt19937_64 rng(seed0);
  std::uniform_real_distribution<double> U(hmin, hmax);
  std::vector<double> H(ntraj);
  for (double &h : H) h = U(rng);
  const int bm = std::max(1, batch_members);
  for (int t0j = 0; t0j < ntraj; t0j += bm) {
    const int k = std::min(bm, ntraj - t0j);
    SphereConfig c = cfg;
    c.members = k;
    c.precision = precision;
    SphereEngine e(c);
    for (int j = 0; j < k; j++) e.turbulence(seed0 + static_cast<uint64_t>(t0j + j), H[t0j + j], 30.0, T / 2, j);
    for (int w = 0; w <= nwin; w++) {
      if (w > 0) e.run(window, dt);
      snapshot<<<grid_for(static_cast<long>(k) * dp, 256), 256, 0, e.stream>>>(e.device_state(), k, nfeat, snaps.p, t0j, nwin + 1, w, dp);
      LMW_LAUNCH_CHECK();
    }
    LMW_CUDA(cudaStreamSynchronize(e.stream));
  }
  gen_seconds = seconds_since(t0);
}

void Surrogate::generate_drifted(int trajectories, int net_windows, uint64_t seed0, double hmin, double hmax, int precision, int batch_members) {
  if (trajectories < 1 || net_windows < 1) throw InvalidArgument("need at least one trajectory and one network window");
  if (!(hmin > 0) || !(hmax >= hmin)) throw InvalidArgument("mean heights must be positive and ordered");
  if (!have_norm || ntraj < 2) throw InvalidArgument("fit the network on generated data before generating from its states");
  const auto t0 = std::chrono::steady_clock::now();
  const int dp = net->dim[0];
  const size_t per = static_cast<size_t>(nwin + 1) * dp;
  DevBuf<float> grown;
  grown.alloc((static_cast<size_t>(trajectories) + ntraj) * per);
  LMW_CUDA(cudaMemcpyAsync(grown.p + static_cast<size_t>(trajectories) * per, snaps.p, static_cast<size_t>(ntraj) * per * sizeof(float),
                           cudaMemcpyDeviceToDevice, stream));
  std::mt19937_64 rng(seed0);
  std::uniform_real_distribution<double> U(hmin, hmax);
  std::vector<double> H(trajectories);
  for (double &h : H) h = U(rng);
  const int bm = std::max(1, batch_members);
  const int total = trajectories + ntraj;
  for (int t0j = 0; t0j < trajectories; t0j += bm) {
    const int k = std::min(bm, trajectories - t0j);
    SphereConfig c = cfg;
    c.members = k;
    c.precision = precision;
    SphereEngine e(c);
    for (int j = 0; j < k; j++) e.turbulence(seed0 + static_cast<uint64_t>(t0j + j), H[t0j + j], 30.0, T / 2, j);
    LMW_CUDA(cudaStreamSynchronize(e.stream));
    for (int w = 0; w < net_windows; w++) advance_states(e.device_state(), k, nullptr);
    LMW_CUDA(cudaStreamSynchronize(stream));
    e.state_written();
    for (int w = 0; w <= nwin; w++) {
      if (w > 0) e.run(window, dt);
      snapshot<<<grid_for(static_cast<long>(k) * dp, 256), 256, 0, e.stream>>>(e.device_state(), k, nfeat, grown.p, t0j, nwin + 1, w, dp);
      LMW_LAUNCH_CHECK();
    }
    LMW_CUDA(cudaStreamSynchronize(e.stream));
  }
  snaps.swap(grown);
  ntraj = total;
  gen_seconds = seconds_since(t0);
}

// per-n normalisation from the training trajectories [0, ntrain): for each field and total wavenumber n, the mean
// and standard deviation of the live coefficients and the rms of their increments over one window
void Surrogate::normalise(int ntrain) {
  if (ntraj < 1) throw InvalidArgument("no training data: generate it first");
  if (ntrain < 1 || ntrain > ntraj) throw InvalidArgument("training trajectory count out of range");
  const int dp = net->dim[0];
  const long np = static_cast<long>(ntrain) * nwin;
  const int splits = 64;
  DevBuf<double> part;
  part.alloc(static_cast<size_t>(splits) * dp * 3);
  pair_stats<<<dim3((dp + 127) / 128, splits), 128, 0, stream>>>(snaps.p, nwin, dp, 0, np, part.p);
  LMW_LAUNCH_CHECK();
  std::vector<double> h(static_cast<size_t>(splits) * dp * 3);
  LMW_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  std::vector<double> s1(dp, 0), s2(dp, 0), d2(dp, 0);
  for (int s = 0; s < splits; s++)
    for (int f = 0; f < dp; f++) {
      s1[f] += h[(static_cast<size_t>(s) * dp + f) * 3];
      s2[f] += h[(static_cast<size_t>(s) * dp + f) * 3 + 1];
      d2[f] += h[(static_cast<size_t>(s) * dp + f) * 3 + 2];
    }
  // feature -> (field, m, n, part); dead features (imaginary parts at m = 0, the (0,0) vorticity and divergence)
  // are identically zero
  std::vector<int> fm(nfeat), fn(nfeat), fq(nfeat), fri(nfeat);
  for (int q = 0; q < 3; q++)
    for (int m = 0, tri = 0; m <= T; m++)
      for (int n = m; n <= T; n++, tri++)
        for (int ri = 0; ri < 2; ri++) {
          const int f = (q * ntri + tri) * 2 + ri;
          fm[f] = m;
          fn[f] = n;
          fq[f] = q;
          fri[f] = ri;
        }
  auto dead = [&](int f) { return (fm[f] == 0 && fri[f] == 1) || (fq[f] < 2 && fn[f] == 0); };
  const int G = 3 * (T + 1);
  std::vector<double> g1(G, 0), g2(G, 0), gd(G, 0), gc(G, 0);
  for (int f = 0; f < nfeat; f++) {
    if (dead(f)) continue;
    const int g = fq[f] * (T + 1) + fn[f];
    g1[g] += s1[f];
    g2[g] += s2[f];
    gd[g] += d2[f];
    gc[g] += static_cast<double>(np);
  }
  std::vector<float> hmu(dp, 0.0f), hisig(dp, 0.0f), hsigd(dp, 0.0f), hmask(dp, 0.0f), hloss(dp, 0.0f);
  // mean geopotential of the training states (Phi(0,0) = sqrt 2 * mean Phi for the orthonormal P(0,0))
  const double phibar = std::max(1.0, g1[2 * (T + 1)] / std::max(1.0, gc[2 * (T + 1)]) / std::sqrt(2.0));
  const double a2 = cfg.radius * cfg.radius;
  double lsum = 0;
  int lcount = 0;
  for (int f = 0; f < nfeat; f++) {
    if (dead(f)) continue;
    const int g = fq[f] * (T + 1) + fn[f];
    const double mean = g1[g] / gc[g];
    const double var = std::max(0.0, g2[g] / gc[g] - mean * mean);
    const double sd = std::sqrt(var);
    hmu[f] = static_cast<float>(mean);
    hisig[f] = sd > 0 ? static_cast<float>(1.0 / sd) : 0.0f;
    const double rd = std::sqrt(gd[g] / gc[g]);
    // the global mean of Phi is conserved exactly: its increment is not learned
    if (rd > 0 && !(fq[f] == 2 && fn[f] == 0)) {
      hsigd[f] = static_cast<float>(rd);
      hmask[f] = 1.0f;
      // energy-norm weight of an error in this coefficient's increment: kinetic energy
      // Phibar a^2 / (n (n + 1)) |zeta, delta|^2 and available potential energy |Phi|^2, both times 2 for m > 0
      const double cm = fm[f] == 0 ? 1.0 : 2.0;
      const double n = fn[f];
      const double e = fq[f] == 2 ? 1.0 : ke_weight * phibar * a2 / (n * (n + 1.0));
      hloss[f] = static_cast<float>(cm * e * rd * rd);
      lsum += hloss[f];
      lcount++;
    }
  }
  for (int f = 0; f < dp; f++) hloss[f] = lcount ? static_cast<float>(hloss[f] * lcount / lsum) : 0.0f;
  if (loss_mode == 0) hloss = hmask;
  LMW_CUDA(cudaMemcpyAsync(mu.p, hmu.data(), dp * sizeof(float), cudaMemcpyHostToDevice, stream));
  LMW_CUDA(cudaMemcpyAsync(sig.p, hisig.data(), dp * sizeof(float), cudaMemcpyHostToDevice, stream));
  LMW_CUDA(cudaMemcpyAsync(sigd.p, hsigd.data(), dp * sizeof(float), cudaMemcpyHostToDevice, stream));
  LMW_CUDA(cudaMemcpyAsync(outmask.p, hmask.data(), dp * sizeof(float), cudaMemcpyHostToDevice, stream));
  LMW_CUDA(cudaMemcpyAsync(net->mask.p, hloss.data(), dp * sizeof(float), cudaMemcpyHostToDevice, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  have_norm = true;
}

void Surrogate::evaluate(int p0, int p1, std::vector<double> &err, std::vector<double> &pers) {
  if (!have_norm) throw InvalidArgument("the network has no normalisation yet: fit it first");
  const long npairs = static_cast<long>(ntraj) * nwin;
  if (p0 < 0 || p1 > npairs || p1 <= p0) throw InvalidArgument("pair range out of range");
  const int dp = net->dim[0];
  const int mb = net->max_batch;
  err.assign(p1 - p0, 0.0);
  pers.assign(p1 - p0, 0.0);
  idx.alloc(mb);
  std::vector<int> ids(mb);
  std::vector<double> h(2 * mb);
  for (int s = p0; s < p1; s += mb) {
    const int cnt = std::min(mb, p1 - s);
    const int batch = (cnt + 127) / 128 * 128;
    for (int i = 0; i < batch; i++) ids[i] = s + std::min(i, cnt - 1);
    LMW_CUDA(cudaMemcpyAsync(idx.p, ids.data(), batch * sizeof(int), cudaMemcpyHostToDevice, stream));
    for (int k = 0; k < sym_average; k++) {
      const SymMap map = sym_map(k);
      gather_pairs<<<batch, 256, 0, stream>>>(snaps.p, idx.p, nwin, dp, nfeat, mu.p, sig.p, sigd.p, outmask.p, net->x0.p, nullptr, fmq.p, map);
      LMW_LAUNCH_CHECK();
      net->forward(batch);
      accumulate_increment<<<batch, 256, 0, stream>>>(net->y.p, sigd.p, outmask.p, cnt, nfeat, dp, fmq.p, map, 1.0f / sym_average, k == 0,
                                                      incbuf.p);
      LMW_LAUNCH_CHECK();
    }
    pair_errors<<<cnt, 256, 0, stream>>>(snaps.p, idx.p, nwin, dp, net->y.p, sigd.p, outmask.p, cw.p, cnt, errs.p, errs.p + mb, incbuf.p);
    LMW_LAUNCH_CHECK();
    LMW_CUDA(cudaMemcpyAsync(h.data(), errs.p, 2 * mb * sizeof(double), cudaMemcpyDeviceToHost, stream));
    LMW_CUDA(cudaStreamSynchronize(stream));
    for (int i = 0; i < cnt; i++) {
      err[s - p0 + i] = h[i];
      pers[s - p0 + i] = h[mb + i];
    }
  }
  net->check_status();
}

static double quantile(std::vector<double> v, double q) {
  if (v.empty()) return 0;
  std::sort(v.begin(), v.end());
  const size_t i = std::min(v.size() - 1, static_cast<size_t>(q * (v.size() - 1) + 0.5));
  return v[i];
}

SurrogateStats Surrogate::fit(int epochs, int batch, double lr, double lr_min, double val_fraction, uint64_t shuffle_seed) {
  if (ntraj < 2) throw InvalidArgument("no training data: generate it first");
  if (epochs < 0) throw InvalidArgument("epochs must not be negative");
  check_batch(batch, net->max_batch);
  if (!(val_fraction > 0 && val_fraction < 1)) throw InvalidArgument("the validation fraction must lie in (0, 1)");
  SurrogateStats st;
  // the held-out trajectories are fixed by the first fit (trajectories added later go before them)
  const int nval_traj = val_traj > 0 ? val_traj : std::max(1, static_cast<int>(std::lround(ntraj * val_fraction)));
  const int ntrain_traj = ntraj - nval_traj;
  if (ntrain_traj < 1) throw InvalidArgument("no training trajectories left after the validation split");
  if (!have_norm) normalise(ntrain_traj);
  val_traj = nval_traj;
  const int ntrain = ntrain_traj * nwin, p_val0 = ntrain, p_val1 = ntraj * nwin;
  if (ntrain < batch) throw InvalidArgument("fewer training pairs than one batch");
  std::vector<double> e, p;
  evaluate(p_val0, p_val1, e, p);
  st.val_untrained_mean = std::accumulate(e.begin(), e.end(), 0.0) / e.size();
  st.val_persist_mean = std::accumulate(p.begin(), p.end(), 0.0) / p.size();
  const int spe = ntrain / batch;
  const long total = static_cast<long>(epochs) * spe;
  // linear warm-up of the learning rate over the first 5 % of the steps (at most 1000)
  const long warmup = std::max<long>(1, std::min<long>(1000, total / 20));
  hist_loss.clear();
  hist_gnorm.clear();
  DevBuf<int> order;
  order.alloc(ntrain);
  std::vector<int> ids(ntrain);
  std::iota(ids.begin(), ids.end(), 0);
  const int dp = net->dim[0];
  const auto t0 = std::chrono::steady_clock::now();
  long step = 0;
  double last_loss = 0;
  for (int ep = 0; ep < epochs; ep++) {
    std::mt19937_64 rng(shuffle_seed + static_cast<uint64_t>(ep) * 7919u);
    std::shuffle(ids.begin(), ids.end(), rng);
    LMW_CUDA(cudaMemcpyAsync(order.p, ids.data(), ntrain * sizeof(int), cudaMemcpyHostToDevice, stream));
    for (int s = 0; s < spe; s++, step++) {
      // the trained network is the moving average of the weights over the second half of the steps
      if (ema > 0 && step == total / 2) net->ema_begin(ema);
      const double warm = std::min(1.0, static_cast<double>(step + 1) / static_cast<double>(warmup));
      const double lr_t =
          warm * (lr_min + 0.5 * (lr - lr_min) * (1.0 + std::cos(M_PI * static_cast<double>(step) / static_cast<double>(std::max<long>(1, total)))));
      SymMap aug;
      aug.seed = augment ? (shuffle_seed * 0x2545F4914F6CDD1DULL + static_cast<uint64_t>(step) + 1) | 1ULL : 0ULL;
      gather_pairs<<<batch, 256, 0, stream>>>(snaps.p, order.p + static_cast<long>(s) * batch, nwin, dp, nfeat, mu.p, sig.p, sigd.p, outmask.p, net->x0.p,
                                              net->target.p, fmq.p, aug);
      LMW_LAUNCH_CHECK();
      net->forward(batch);
      net->backward(batch);
      net->adam(lr_t, 0.9, 0.999, 1e-8, clip_ratio);
    }
    // the mean loss and gradient norm per step of this epoch (synchronises once per epoch)
    last_loss = net->take_loss() / spe;
    hist_loss.push_back(last_loss);
    hist_gnorm.push_back(net->take_grad_norm_sum() / spe);
    // keep the host's copy of the order alive until the stream has consumed it
    LMW_CUDA(cudaStreamSynchronize(stream));
  }
  net->ema_apply();
  LMW_CUDA(cudaStreamSynchronize(stream));
  st.seconds = seconds_since(t0);
  st.steps = static_cast<double>(total);
  st.train_loss = last_loss;
  evaluate(p_val0, p_val1, e, p);
  st.val_err_mean = std::accumulate(e.begin(), e.end(), 0.0) / e.size();
  st.val_err_median = quantile(e, 0.5);
  st.val_err_p90 = quantile(e, 0.9);
  st.val_err_max = *std::max_element(e.begin(), e.end());
  return st;
}

// the k-th of the sym_average maps of inference: rotations by multiples of 2 pi / (sym_average / 2), each without
// and with the reflection (a single map: the identity)
SymMap Surrogate::sym_map(int k) const {
  SymMap m;
  if (sym_average <= 1) return m;
  const int nrot = sym_average / 2;
  m.turn = static_cast<float>(k / 2) / static_cast<float>(nrot);
  m.reflect = k & 1;
  return m;
}

void Surrogate::advance_states(double *states, int count, const int *mode) {
  if (!have_norm) throw InvalidArgument("the network has no normalisation yet: fit it first");
  const int dp = net->dim[0], mb = net->max_batch;
  for (int s = 0; s < count; s += mb) {
    const int cnt = std::min(mb, count - s);
    const int batch = (cnt + 127) / 128 * 128;
    for (int k = 0; k < sym_average; k++) {
      const SymMap map = sym_map(k);
      pack_states<<<batch, 256, 0, stream>>>(states + static_cast<long>(s) * nfeat, cnt, nfeat, dp, mu.p, sig.p, net->x0.p, fmq.p, map);
      LMW_LAUNCH_CHECK();
      net->forward(batch);
      accumulate_increment<<<batch, 256, 0, stream>>>(net->y.p, sigd.p, outmask.p, cnt, nfeat, dp, fmq.p, map, 1.0f / sym_average, k == 0,
                                                      incbuf.p);
      LMW_LAUNCH_CHECK();
      g_launches += 2;
    }
    apply_increment<<<grid_for(static_cast<long>(cnt) * nfeat, 256), 256, 0, stream>>>(states + static_cast<long>(s) * nfeat, cnt, nfeat, dp, incbuf.p,
                                                                                      outmask.p, mode ? mode + s : nullptr);
    LMW_LAUNCH_CHECK();
    g_launches += 1;
  }
}

// Hybrid rollout. Every window the network advances the members it still owns; every check_every-th window plain
// RK4 recomputes that window from the same start states, the per-window height error of every network member is
// recorded, and a member whose error exceeds the threshold is taken over: its state becomes the RK4 state and
// (takeover_mode 0) RK4 advances it from then on (one batched FP64 engine for every member taken over so far), or
// (takeover_mode 1) the network keeps advancing it from the RK4 state (out[4] then counts the member-windows RK4
// replaced).
// out[0] hybrid seconds, [1] network seconds, [2] check seconds, [3] takeover seconds, [4] members taken over,
// [5] checks, [6] median window error, [7] max, [8] fraction of checked windows over the threshold,
// [9] plain RK4 seconds for ref windows (measured on the same members), [10] ref windows, [11] hybrid
// member-sim-days/s, [12] plain RK4 member-sim-days/s, [13] network-only member-sim-days/s, [14] mean window
// error, [15] 90th percentile. window_err (optional): [check][member], -1 for members already taken over.
// final_states (optional): the members' packed states after the last window, [member][nfeat].
void Surrogate::rollout(int members, uint64_t seed0, double hmin, double hmax, int windows, int check_every, double threshold, int check_precision,
                        int ref_windows, double *out, double *window_err, double *final_states) {
  if (members < 1 || windows < 1 || check_every < 1 || ref_windows < 1)
    throw InvalidArgument("members, windows, the check interval and the reference windows must be positive");
  if (!(hmin > 0) || !(hmax >= hmin)) throw InvalidArgument("mean heights must be positive and ordered");
  if (!have_norm) throw InvalidArgument("the network has no normalisation yet: fit it first");
  std::mt19937_64 rng(seed0);
  std::uniform_real_distribution<double> U(hmin, hmax);
  SphereConfig c = cfg;
  c.members = members;
  c.precision = kFP64;
  SphereEngine init(c);
  for (int j = 0; j < members; j++) init.turbulence(seed0 + static_cast<uint64_t>(j), U(rng), 30.0, T / 2, j);
  LMW_CUDA(cudaStreamSynchronize(init.stream));
  const size_t nst = static_cast<size_t>(members) * nfeat;
  rs_state.alloc(nst);
  rs_start.alloc(nst);
  rs_mode.alloc(members);
  rs_mode.zero(stream);
  LMW_CUDA(cudaMemcpyAsync(rs_state.p, init.device_state(), nst * sizeof(double), cudaMemcpyDeviceToDevice, stream));
  // the network's members are checked by one batched RK4 engine built once for all members: after takeovers its
  // first slots hold the network's members and the remaining slots repeat the first of them (the same RK4 step
  // for the members that count, no rebuild of the engine and its launch plan)
  std::vector<int> netids(members);
  std::iota(netids.begin(), netids.end(), 0);
  DevBuf<int> netids_d;
  netids_d.alloc(members);
  std::unique_ptr<SphereEngine> check;
  std::vector<int> slots(members);
  auto upload_slots = [&]() {
    for (int i = 0; i < members; i++) slots[i] = netids[i < static_cast<int>(netids.size()) ? i : 0];
    LMW_CUDA(cudaMemcpyAsync(netids_d.p, slots.data(), members * sizeof(int), cudaMemcpyHostToDevice, check->stream));
    LMW_CUDA(cudaStreamSynchronize(check->stream));
  };
  auto make_check = [&](int k) {
    SphereConfig cc = c;
    cc.members = k;
    cc.precision = check_precision;
    check = std::make_unique<SphereEngine>(cc);
    upload_slots();
  };
  struct Group {
    std::unique_ptr<SphereEngine> e;
    DevBuf<int> ids;
    std::vector<int> hids;
    int n = 0;
  };
  std::vector<std::unique_ptr<Group>> groups;
  std::vector<int> mode(members, 0);
  std::vector<double> checked;
  DevBuf<double> merr;
  merr.alloc(members);
  std::vector<double> herr(members);
  cudaEvent_t e0, e1;
  LMW_CUDA(cudaEventCreate(&e0));
  LMW_CUDA(cudaEventCreate(&e1));
  // one window of plain RK4 at the training step, or at the engine's own stable step where a state the network
  // produced has become too fast for it (the reference's stable_dt(1.5), cpp/sphere.cpp:438-447)
  const double rk4_limit = 2.0 * std::sqrt(2.0);
  auto rk4_window = [&](SphereEngine &e) {
    const double use = dt <= e.stable_dt_all(rk4_limit) ? dt : 0.0;
    e.run(window, use);
  };
  // warm the check engine's graphs and the network (not timed)
  LMW_CUDA(cudaStreamSynchronize(stream));
  make_check(members);
  copy_members_launch(rs_state.p, netids_d.p, check->device_state(), nullptr, members, nfeat, check->stream);
  check->state_written();
  check->run(window, dt);
  net->forward(std::min(net->max_batch, (members + 127) / 128 * 128));
  LMW_CUDA(cudaDeviceSynchronize());
  double t_net = 0, t_check = 0, t_take = 0;
  int taken = 0, nchecks = 0, over = 0;
  const auto t0 = std::chrono::steady_clock::now();
  for (int w = 0; w < windows; w++) {
    const bool is_check = (w % check_every) == check_every - 1;
    if (is_check) LMW_CUDA(cudaMemcpyAsync(rs_start.p, rs_state.p, nst * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    LMW_CUDA(cudaEventRecord(e0, stream));
    if (!netids.empty()) advance_states(rs_state.p, members, rs_mode.p);
    LMW_CUDA(cudaEventRecord(e1, stream));
    if (!groups.empty()) {
      const auto tg = std::chrono::steady_clock::now();
      for (auto &g : groups) rk4_window(*g->e);
      for (auto &g : groups) {
        LMW_CUDA(cudaStreamSynchronize(g->e->stream));
        copy_members_launch(g->e->device_state(), nullptr, rs_state.p, g->ids.p, g->n, nfeat, stream);
      }
      LMW_CUDA(cudaStreamSynchronize(stream));
      t_take += seconds_since(tg);
    }
    LMW_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    LMW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    t_net += ms * 1e-3;
    if (!is_check) continue;
    if (window_err)
      for (int b = 0; b < members; b++) window_err[static_cast<size_t>(nchecks) * members + b] = -1.0;
    nchecks++;
    if (netids.empty()) continue;
    const auto tc0 = std::chrono::steady_clock::now();
    const int k = static_cast<int>(netids.size());
    LMW_CUDA(cudaStreamSynchronize(stream));
    copy_members_launch(rs_start.p, netids_d.p, check->device_state(), nullptr, members, nfeat, check->stream);
    check->state_written();
    rk4_window(*check);
    state_errors<<<k, 256, 0, check->stream>>>(rs_state.p, netids_d.p, check->device_state(), nfeat, cw.p, merr.p);
    LMW_LAUNCH_CHECK();
    LMW_CUDA(cudaMemcpyAsync(herr.data(), merr.p, k * sizeof(double), cudaMemcpyDeviceToHost, check->stream));
    LMW_CUDA(cudaStreamSynchronize(check->stream));
    std::vector<int> fresh, rows, keep;
    for (int i = 0; i < k; i++) {
      const int b = netids[i];
      const double ev = herr[i];
      checked.push_back(ev);
      if (window_err) window_err[static_cast<size_t>(nchecks - 1) * members + b] = ev;
      if (!(ev <= threshold)) {
        over++;
        fresh.push_back(b);
        rows.push_back(i);
        mode[b] = 1;
      } else {
        keep.push_back(b);
      }
    }
    if (!fresh.empty()) {
      auto g = std::make_unique<Group>();
      g->n = static_cast<int>(fresh.size());
      g->ids.alloc(g->n);
      DevBuf<int> rows_d;
      rows_d.alloc(g->n);
      LMW_CUDA(cudaMemcpyAsync(g->ids.p, fresh.data(), g->n * sizeof(int), cudaMemcpyHostToDevice, check->stream));
      LMW_CUDA(cudaMemcpyAsync(rows_d.p, rows.data(), g->n * sizeof(int), cudaMemcpyHostToDevice, check->stream));
      SphereConfig gc = cfg;
      gc.members = g->n;
      gc.precision = kFP64;
      g->e = std::make_unique<SphereEngine>(gc);
      if (check_precision == kFP64) {
        copy_members_launch(check->device_state(), rows_d.p, g->e->device_state(), nullptr, g->n, nfeat, check->stream);
        LMW_CUDA(cudaStreamSynchronize(check->stream));
        g->e->state_written();
      } else {
        // the check ran in reduced precision: plain FP64 RK4 recomputes the window of the members it takes over
        copy_members_launch(rs_start.p, g->ids.p, g->e->device_state(), nullptr, g->n, nfeat, check->stream);
        LMW_CUDA(cudaStreamSynchronize(check->stream));
        g->e->state_written();
        rk4_window(*g->e);
        LMW_CUDA(cudaStreamSynchronize(g->e->stream));
      }
      copy_members_launch(g->e->device_state(), nullptr, rs_state.p, g->ids.p, g->n, nfeat, check->stream);
      LMW_CUDA(cudaStreamSynchronize(check->stream));
      taken += g->n;
      if (takeover_mode == 1) {
        // per-window fallback: the replaced window's members stay with the network
        for (int b : fresh) mode[b] = 0;
        t_check += seconds_since(tc0);
        continue;
      }
      // one FP64 engine advances every member taken over so far: the new members join the existing group (their
      // states and the group's copied into an engine of the combined count), so each window is one batched run
      if (groups.empty()) {
        g->hids = fresh;
        groups.push_back(std::move(g));
      } else {
        Group &old = *groups[0];
        auto mg = std::make_unique<Group>();
        mg->n = old.n + g->n;
        mg->hids = old.hids;
        mg->hids.insert(mg->hids.end(), fresh.begin(), fresh.end());
        mg->ids.alloc(mg->n);
        SphereConfig mc = cfg;
        mc.members = mg->n;
        mc.precision = kFP64;
        mg->e = std::make_unique<SphereEngine>(mc);
        LMW_CUDA(cudaMemcpyAsync(mg->ids.p, mg->hids.data(), mg->n * sizeof(int), cudaMemcpyHostToDevice, mg->e->stream));
        LMW_CUDA(cudaStreamSynchronize(old.e->stream));
        LMW_CUDA(cudaMemcpyAsync(mg->e->device_state(), old.e->device_state(), static_cast<size_t>(old.n) * nfeat * sizeof(double),
                                 cudaMemcpyDeviceToDevice, mg->e->stream));
        LMW_CUDA(cudaMemcpyAsync(mg->e->device_state() + static_cast<size_t>(old.n) * nfeat, g->e->device_state(),
                                 static_cast<size_t>(g->n) * nfeat * sizeof(double), cudaMemcpyDeviceToDevice, mg->e->stream));
        LMW_CUDA(cudaStreamSynchronize(mg->e->stream));
        mg->e->state_written();
        groups[0] = std::move(mg);
      }
      LMW_CUDA(cudaMemcpyAsync(rs_mode.p, mode.data(), members * sizeof(int), cudaMemcpyHostToDevice, stream));
      netids = keep;
      if (!netids.empty()) upload_slots();
    }
    t_check += seconds_since(tc0);
  }
  LMW_CUDA(cudaDeviceSynchronize());
  const double t_all = seconds_since(t0);
  if (final_states) LMW_CUDA(cudaMemcpy(final_states, rs_state.p, nst * sizeof(double), cudaMemcpyDeviceToHost));
  // plain RK4 on the same members (FP64), ref_windows windows after one untimed window
  double t_ref = 0;
  {
    SphereEngine ref(c);
    LMW_CUDA(cudaMemcpyAsync(ref.device_state(), init.device_state(), nst * sizeof(double), cudaMemcpyDeviceToDevice, ref.stream));
    ref.state_written();
    ref.run(window, dt);
    LMW_CUDA(cudaStreamSynchronize(ref.stream));
    const auto tr = std::chrono::steady_clock::now();
    ref.run(window * ref_windows, dt);
    LMW_CUDA(cudaStreamSynchronize(ref.stream));
    t_ref = seconds_since(tr);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  net->check_status();
  const double days = window / 86400.0;
  out[0] = t_all;
  out[1] = t_net;
  out[2] = t_check;
  out[3] = t_take;
  out[4] = taken;
  out[5] = nchecks;
  out[6] = quantile(checked, 0.5);
  out[7] = checked.empty() ? 0 : *std::max_element(checked.begin(), checked.end());
  out[8] = checked.empty() ? 0 : static_cast<double>(over) / checked.size();
  out[9] = t_ref;
  out[10] = ref_windows;
  out[11] = members * windows * days / t_all;
  out[12] = members * ref_windows * days / t_ref;
  out[13] = members * windows * days / std::max(t_net, 1e-12);
  out[14] = checked.empty() ? 0 : std::accumulate(checked.begin(), checked.end(), 0.0) / checked.size();
  out[15] = quantile(checked, 0.9);
}

}  // namespace lmw
