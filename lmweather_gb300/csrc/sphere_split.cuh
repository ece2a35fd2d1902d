// Split-precision Legendre transforms on the tensor cores (included by sphere.cu).
//
// Every Legendre sum of an RK4 stage is a small GEMM per zonal wavenumber m on tcgen05, with the operands split
// into BF16 pieces (hi/lo: 3 products per term; hi/mid/lo: 6) and FP32 accumulation in tensor memory:
//   synthesis  D[member x quantity][jh] = A[member x quantity][k] * T_m[jh][k]^T; k orders n with the even n - m
//              first and the odd second (two K segments, two accumulators: both mirror latitudes come out at
//              once); quantities psi, chi, zeta, Phi against the P table and psi, chi against the H table.
//   analysis   D[member x quantity][r] = A[member x quantity][jh] * T_{m,s}[r][jh]^T for n = m + s + 2r (one
//              parity s per CTA); A w_d, B w_d, U Phi w_d, (Phi + E) w at fold parity s against P and A w_d,
//              B w_d, V Phi w_d at parity 1 - s against H.
// Three launches per stage:
//   split_syn     per (m, member tile): H then P through a pipeline of bulk asynchronous copies (cp.async.bulk,
//                 the TMA engine) into shared memory, MMAs by one thread, accumulators read back with tcgen05.ld
//                 and combined into the Fourier coefficients of U, V, zeta and Phi at both mirror latitudes.
//   split_grid    per (block of latitude pairs, member): FP32 FFTs and products (the same arithmetic as
//                 sph_grid<float>), then the folded analysis inputs, stored m-major so that the analysis reads
//                 them with unit stride.
//   split_ana     per (m, parity, member tile): H then P as above; the epilogue forms the tendencies in FP32,
//                 applies the RK4 stage update to the FP64 state, and packs the next stage's synthesis operands.
// All operands live in global memory already in the MMA's canonical K-major core-matrix order, in 64-wide K
// chunks: element (row r, column k) of an R-row operand sits at
//   (k / 64) * R * 64 + ((r / 8) * 8 + (k % 64) / 8) * 64 + (r % 8) * 8 + k % 8
// so the chunk of every operand is one contiguous run of R * 128 bytes. Split pieces follow each other at a
// fixed element stride (the buffer size).
#pragma once
#include <cuda_bf16.h>

#include "sphere_common.cuh"
#include "sphere_tables.h"
#include "tc_common.cuh"

namespace lmw {

constexpr int SPLIT_NBT = 16;  // members per tile: 8 quantities x 16 members = 128 rows, the M of one MMA
constexpr int SPLIT_BK = 64;
constexpr int SPLIT_MAX_STAGES = 4;
constexpr int SPLIT_MARGIN = 16384;  // an M = 128 MMA reads 16 KB past an A base: every A base keeps 16 KB of allocation
constexpr int SPLIT_WS_THREADS = 320;  // warp-specialised kernels: producer warp, MMA warp, 8 epilogue warps
constexpr int SPLIT_WS_EPI = 256;      // epilogue threads (warps 2..9)
constexpr int SPLIT_THREADS = 128;
constexpr int SPLIT_ANA_THREADS = 256;  // analysis: 8 warps for the gather and the RK4 epilogue, warps 0-3 read TMEM
constexpr int SPLIT_NQ = 16;  // per (member, jh, m): U, V, zeta, Phi Fourier coefficients at the southern and northern latitude
constexpr int SPLIT_JB_MAX = 8;  // latitude pairs per grid CTA
// dynamic shared memory per CTA when two CTAs share an SM (228 KB per SM, 1 KB reserved per CTA, static barriers)
constexpr size_t SPLIT_HALF_SM = 115456;

struct SplitPlan {
  int pieces = 2, terms = 3;
  int nbt = 1, ntiles = 1, nh16 = 16, nh64 = 64, rAP = 8, rAH = 8, rSP = 8, rSH = 8, ra_max = 16;
  int bka = 32, nha = 64;  // analysis K (latitude) chunk width (32, or the padded latitude count below 32; 64-wide
                           // chunks measured slower at T85) and padded K
  int bks = 64;            // synthesis K (coefficient) chunk width: 32 up to T85 (less padding per m), 64 above
  std::vector<int> ke16, kps, ra16;  // kps[m]: synthesis K of m padded to the chunk width bks
  std::vector<long> tS_off, tA_off, aS_off, aSH_off;
  long tS_size = 0, tA_size = 0, aSP_size = 0, aSH_size = 0, aAP_size = 0, aAH_size = 0;
  DevBuf<__nv_bfloat16> tS_P, tS_H, tA_P, tA_H;   // tables (B operands), three pieces each
  DevBuf<__nv_bfloat16> aS_P, aS_H, aA_P, aA_H;   // per-stage operands (A)
  DevBuf<float> dsyn;                             // [member][jh][m][SPLIT_NQ]
  DevBuf<int> err;
  DevBuf<int> ke16_d, kps_d, ra16_d;
  DevBuf<long> tS_off_d, tA_off_d, aS_off_d, aSH_off_d;
  size_t smem_syn = 0, smem_ana = 0;
  int ns_syn = 2, ns_ana = 2;  // pipeline stages
  int jb = 1;                 // latitude pairs per grid CTA
  int syn_nh = 16, syn_split = 1;  // latitudes per synthesis CTA and slices of nh16
  int fgrp = 3;               // FFT stages per shared-memory pass
  int direct = 1;             // the grid kernel writes the analysis operands (else the FP32 fold, gathered)
  int ana_both = 0;           // analysis CTAs handle both parities of m
  int ana_grid = 0;           // analysis CTAs (0: one per work item)
  int ana_minb = 2;           // analysis register budget: CTAs per SM (2 or 3)
  int ana_ws = 0;             // 0: split_ana; 1 or 2: the warp-specialised persistent form with that many CTAs per SM
  int grid_fixed = 1;         // 1: the grid kernel compiled for the transform length (lengths 2^6..2^10); 0: any length
  int syn_ws = 0;             // 0: split_syn; 1 or 2: the warp-specialised persistent synthesis with that many CTAs per SM
  int nsm = 152;              // multiprocessors of the device (the persistent grid)
  int ra_pair = 32;           // largest ra16[2m] + ra16[2m + 1]
  // 1: the linear terms of the tendencies (gravity-wave terms of the mean height, the Laplacian of Phi, the
  // untilted Coriolis terms) added in spectral space, in FP32 from the FP32 stage input; only the nonlinear
  // products go through the BF16 pieces.
  // 0: every term through the BF16 GEMMs (the plain split form)
  int lin_exact = 1;
  DevBuf<float> lin32;        // per coefficient q: eps_{n+1} n/(n+1), eps_n (n+1)/n, m/(n(n+1)) (3 x ntri), FP32
  size_t syn_stage_bytes = 0, syn_min_bytes = 0, ana_min_bytes = 0, ana_both_min_bytes = 0, budget_bytes = 0;
  size_t ana_res_bytes_v[2] = {0, 0}, ana_stage_bytes_v[2] = {0, 0};  // per variant: [0] gathered A, [1] streamed A
};

struct SplitDev {
  int pieces, terms, nbt, ntiles, nh16, nh64, rAP, rAH, rSP, rSH, jb, fgrp, ana_cols_one, ana_cols_both, syn_nh, bka, nha, bks;
  const int *ke16, *kps, *ra16;
  const long *tS_off, *tA_off, *aS_off, *aSH_off;
  long tS_size, tA_size, aSP_size, aSH_size, aAP_size, aAH_size;
  const __nv_bfloat16 *tS_P, *tS_H, *tA_P, *tA_H;
  __nv_bfloat16 *aS_P, *aS_H, *aA_P, *aA_H;
  float *dsyn;   // [member][jh][m][16]: U, V, zeta, Phi at the southern then the northern latitude (complex)
  float2 *fold;  // [m][slot][parity][member][jh]: folded analysis inputs
  int *err;
  int lin_exact;        // see SplitPlan::lin_exact
  const float *lin32;   // [3][ntri]: the spectral Coriolis coefficients
};

namespace {

__host__ __device__ inline int pad16(int x) { return (x + 15) & ~15; }
__host__ __device__ inline int pad8(int x) { return (x + 7) & ~7; }
__host__ __device__ inline int pad64(int x) { return (x + 63) & ~63; }
// canonical chunked core-matrix order of an R-row operand: K chunks of BK columns (64, or the analysis's
// latitude chunk width when the grid has fewer latitude pairs), each [8-row group][8-column group][8 x 8]
__host__ __device__ inline long tile_off(int r, int k, int R, int BK = 64) {
  return static_cast<long>(k / BK) * R * BK + ((r >> 3) * (BK >> 3) + ((k % BK) >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

// round-to-nearest-even float -> bf16 on the host
inline uint16_t host_bf16(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return static_cast<uint16_t>(u >> 16);
}
inline double host_bf16_value(uint16_t b) {
  uint32_t u = static_cast<uint32_t>(b) << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
// hi, mid, lo BF16 pieces of a double: each piece rounds what the previous ones left
inline void split3(double x, uint16_t *out, long stride) {
  double r = x;
  for (int p = 0; p < 3; p++) {
    uint16_t b = host_bf16(static_cast<float>(r));
    out[p * stride] = b;
    r -= host_bf16_value(b);
  }
}
// FP32 value -> BF16 pieces (the FP32 value carries every bit the products keep)
__device__ __forceinline__ void fsplit(float x, __nv_bfloat16 *out, long stride, int pieces) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  out[0] = h;
  if (pieces > 1) {
    const float r = x - __bfloat162float(h);
    const __nv_bfloat16 l = __float2bfloat16_rn(r);
    out[stride] = l;
    if (pieces > 2) out[2 * stride] = __float2bfloat16_rn(r - __bfloat162float(l));
  }
}

// ------------------------------------------------------------------------------------------- tcgen05 helpers
// (tc_common.cuh: bounded mbarrier waits, bulk copies, chunk-layout descriptors, TMEM loads)
using tc::bulk_g2s;
using tc::chunk_desc;
using tc::gtimer;
using tc::idesc_m128;
using tc::su32;
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase) { return tc::wait(bar, phase); }
__device__ __forceinline__ void mbar_expect(uint32_t bar, uint32_t bytes) { tc::expect_tx(bar, bytes); }
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v) { tc::ld8(taddr, v); }
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) { tc::ld32(taddr, v); }

// One CTA's two GEMMs (H then P). Operand g = 0 (H) / 1 (P): nchunk[g] K chunks of bk columns. A is either streamed
// with B (a[g] != nullptr: chunk c of aR[g] rows at a[g] + c * aR[g] * bk, pieces a_ps[g] apart) or resident in
// shared memory (a_res[g]: chunk c, piece p at a_res[g] + (p * nchunk[g] + c) * aR[g] * bk * 2 bytes). B chunk c of
// bR rows at b[g] + c * b_cs. Accumulators at TMEM columns acc[g][seg], the second segment starting at K =
// kseg[g]. Only the first aR[g] accumulator rows are meaningful: an M = 128 MMA also reads whatever lies in the
// 16 KB after an A base, and the rows it makes from that are never read. Returns false when a bounded wait ran
// out (the error code is already recorded).
struct TwoGemm {
  const __nv_bfloat16 *a[2], *b[2];
  long a_ps[2], b_ps[2];
  long b_cs;  // elements between consecutive K chunks of B (bR * bk unless B is a row slice of a wider table)
  uint32_t a_res[2];
  int aR[2], aRmax, bR, nchunk[2], kseg[2];
  int bk = SPLIT_BK;  // K columns per chunk (16, 32 or 64)
  uint32_t acc[2][2];
};

// it0: iterations this CTA's pipeline already ran (a second call continues the barriers' phases); done_phase:
// the phase of `done` this call completes
__device__ bool run_two_gemm(const TwoGemm &G, int pieces, int terms, int ns, uint8_t *pipe, uint64_t *full, uint64_t *empty, uint64_t *done,
                             int *err, int it0 = 0, uint32_t done_phase = 0) {
  const int tid = threadIdx.x;
  const bool astream = G.a[0] != nullptr;
  const int bk = G.bk;
  const uint32_t sbo = static_cast<uint32_t>(bk) * 16u;  // bytes between 8-row groups of a chunk
  const int a_bytes = astream ? G.aRmax * bk * 2 : 0;
  const int b_bytes = G.bR * bk * 2;
  const int stage_bytes = pieces * (a_bytes + b_bytes);
  const int total = G.nchunk[0] + G.nchunk[1];
  __shared__ int s_fail, s_issued, s_consumed;
  if (tid == 0) {
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
  }
  __syncthreads();
  if (tid == 0) {
    // producer: bulk copies of each (operand, chunk)
    for (int it = 0; it < total; it++) {
      const int git = it0 + it;
      const int st = git % ns, g = it < G.nchunk[0] ? 0 : 1, c = g == 0 ? it : it - G.nchunk[0];
      if (git >= ns && !mbar_wait_bounded(su32(&empty[st]), ((git / ns) - 1) & 1)) {
        s_fail = 1;
        atomicExch(err, 2);
        break;
      }
      const uint32_t abytes = astream ? static_cast<uint32_t>(G.aR[g] * bk * 2) : 0u, bbytes = static_cast<uint32_t>(G.bR * bk * 2);
      mbar_expect(su32(&full[st]), static_cast<uint32_t>(pieces) * (abytes + bbytes));
      uint8_t *base = pipe + st * stage_bytes;
      for (int p = 0; p < pieces; p++) {
        if (astream)
          bulk_g2s(su32(base + p * a_bytes), G.a[g] + p * G.a_ps[g] + static_cast<long>(c) * G.aR[g] * bk, abytes, su32(&full[st]));
        bulk_g2s(su32(base + pieces * a_bytes + p * b_bytes), G.b[g] + p * G.b_ps[g] + static_cast<long>(c) * G.b_cs, bbytes,
                 su32(&full[st]));
      }
      s_issued = it + 1;
    }
  } else if (tid == 32) {
    // MMA issuer
    const uint32_t idesc = idesc_m128(G.bR);
    const int tp[6][2] = {{2, 0}, {1, 1}, {0, 2}, {1, 0}, {0, 1}, {0, 0}};
    const int t0 = terms == 6 ? 0 : (terms == 3 ? 3 : 5);
    bool started[2][2] = {{false, false}, {false, false}};
    bool ok = true;
    for (int it = 0; it < total && ok; it++) {
      const int git = it0 + it;
      const int st = git % ns, g = it < G.nchunk[0] ? 0 : 1, c = g == 0 ? it : it - G.nchunk[0];
      if (!mbar_wait_bounded(su32(&full[st]), (git / ns) & 1)) {
        s_fail = 1;
        atomicExch(err, 3);
        ok = false;
        break;
      }
      s_consumed = it + 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint8_t *base = pipe + st * stage_bytes;
      for (int kk = 0; kk < bk; kk += 16) {
        const int kg = c * bk + kk;
        const int seg = kg >= G.kseg[g] ? 1 : 0;
        for (int t = t0; t < 6; t++) {
          const int pa = tp[t][0], pb = tp[t][1];
          const uint32_t abase = astream ? su32(base + pa * a_bytes)
                                         : G.a_res[g] + static_cast<uint32_t>((pa * G.nchunk[g] + c) * G.aR[g] * bk * 2);
          const uint64_t ad = chunk_desc(abase + (kk / 8) * 128, sbo);
          const uint64_t bd = chunk_desc(su32(base + pieces * a_bytes + pb * b_bytes + (kk / 8) * 128), sbo);
          const uint32_t accum = started[g][seg] ? 1u : 0u;
          asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                           G.acc[g][seg]),
                       "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
                       : "memory");
          started[g][seg] = true;
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(&empty[st])) : "memory");
    }
    // completes `done` once every MMA this thread issued has finished (also after a failed wait, so that the
    // CTA can drain its own work before it frees tensor memory)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(done)) : "memory");
  }
  __syncthreads();
  if (tid == 0) {
    if (s_fail == 0) {
      if (!mbar_wait_bounded(su32(done), done_phase)) {
        s_fail = 1;
        atomicExch(err, 4);
      }
    } else {
      // a wait ran out: before the CTA returns (and frees its tensor memory and shared memory), wait a bounded
      // time for its own MMAs and for the bulk copies it issued that no MMA consumed
      tc::wait_for(su32(done), done_phase, 200000000ull);
      for (int it = s_consumed; it < s_issued; it++) {
        const int git = it0 + it;
        tc::wait_for(su32(&full[git % ns]), (git / ns) & 1, 200000000ull);
      }
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return s_fail == 0;
}

// tensor memory and barriers shared by the two GEMM kernels
__device__ __forceinline__ void split_setup(uint32_t *tslot, uint32_t ncols, uint64_t *full, uint64_t *empty, uint64_t *done, int ns) {
  const int tid = threadIdx.x;
  if ((tid >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < ns; s++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&full[s])), "r"(1) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(&empty[s])), "r"(1) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(done)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void split_teardown(uint32_t tmem, uint32_t ncols) {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

// ------------------------------------------------------------------------------------------- synthesis
// grid: (ntiles, latitude slices, M). D columns: H E/O at [0, nh16), [nh16, 2 nh16); P E/O at [2 nh16, 3 nh16), [3 nh16, 4 nh16)
__global__ void __launch_bounds__(SPLIT_THREADS, 1) split_syn(SphDev d, SplitDev sd, int B, int ns) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full[SPLIT_MAX_STAGES], empty[SPLIT_MAX_STAGES], done;
  __shared__ uint32_t tslot;
  // blockIdx.y: latitude slice [jh0, jh0 + nh16) of the table's sd.nh16 rows (two slices at T341, where four
  // accumulators of all latitudes would exceed the 512 tensor-memory columns)
  // m is the slowest grid index: CTAs start in order of decreasing work (K shrinks with m), and the small
  // high-m CTAs fill the last wave
  const int m = blockIdx.z, tile = blockIdx.x;
  const int mt = min(sd.nbt, B - tile * sd.nbt);
  const int nh16 = sd.syn_nh, jh0 = blockIdx.y * nh16;
  uint32_t ncols = 32;
  while (ncols < static_cast<uint32_t>(4 * nh16)) ncols <<= 1;
  split_setup(&tslot, ncols, full, empty, &done, ns);
  const uint32_t tmem = tslot;
  TwoGemm G;
  const long kp = sd.kps[m];
  const long aoffP = sd.aS_off[m] + static_cast<long>(tile) * sd.rSP * kp, aoffH = sd.aSH_off[m] + static_cast<long>(tile) * sd.rSH * kp;
  G.a[0] = sd.aS_H + aoffH;
  G.a[1] = sd.aS_P + aoffP;
  G.a_ps[0] = sd.aSH_size;
  G.a_ps[1] = sd.aSP_size;
  G.a_res[0] = G.a_res[1] = 0;
  // rows jh0.. of every chunk (8-row groups are 8 x bks elements)
  G.b[0] = sd.tS_H + sd.tS_off[m] + static_cast<long>(jh0) * sd.bks;
  G.b[1] = sd.tS_P + sd.tS_off[m] + static_cast<long>(jh0) * sd.bks;
  G.b_ps[0] = G.b_ps[1] = sd.tS_size;
  G.b_cs = static_cast<long>(sd.nh16) * sd.bks;
  G.bk = sd.bks;
  G.aR[0] = sd.rSH;
  G.aR[1] = sd.rSP;
  G.aRmax = sd.rSP;
  G.bR = nh16;
  G.nchunk[0] = G.nchunk[1] = static_cast<int>(kp / sd.bks);
  G.kseg[0] = G.kseg[1] = sd.ke16[m];
  G.acc[0][0] = tmem;
  G.acc[0][1] = tmem + nh16;
  G.acc[1][0] = tmem + 2 * nh16;
  G.acc[1][1] = tmem + 3 * nh16;
  const bool ok = run_two_gemm(G, sd.pieces, sd.terms, ns, smem, full, empty, &done, sd.err);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, row = warp * 32 + lane;
  // accumulator columns in blocks of 32 (TMEM -> shared memory by the warps that own live rows, then coalesced
  // stores by every thread): block cb covers jh in [32 cb, 32 cb + 32) of the four accumulators H E, H O, P E, P O
  float *tile_s = reinterpret_cast<float *>(smem);  // [4][8 mt][33]
  const int rows = 8 * mt;
  for (int cb = 0; ok && cb < nh16; cb += 32) {
    const int wcols = min(32, nh16 - cb);
    __syncthreads();
    if (warp * 32 < rows) {
      const uint32_t lanebase = tmem + (static_cast<uint32_t>(warp * 32) << 16);
      for (int a4 = 0; a4 < 4; a4++) {
        float v[32];
        if (wcols == 32) tmem_ld32(lanebase + a4 * nh16 + cb, v);
        else {
          tmem_ld8(lanebase + a4 * nh16 + cb, v);
          tmem_ld8(lanebase + a4 * nh16 + cb + 8, v + 8);
        }
        if (row < rows) {
#pragma unroll
          for (int i = 0; i < 32; i++)
            if (i < wcols) tile_s[(a4 * rows + row) * 33 + i] = v[i];
        }
      }
    }
    __syncthreads();
    // Fourier coefficients of both mirror latitudes: P sums south E + O, north E - O; H sums (opposite parity)
    // south E + O, north O - E; U = (i m chi P - psi H) / a, V = (i m psi P + chi H) / a (cpp/sphere.cpp:200-201)
    const float mm = static_cast<float>(m), ia = d.inv_a_f;
    for (int e = threadIdx.x; e < mt * 32; e += blockDim.x) {
      const int i = e & 31, ml = e >> 5, jh = jh0 + cb + i;
      if (i >= wcols || jh >= d.nh) continue;
      const float *PE = tile_s + (2 * rows + ml * 8) * 33 + i, *PO = tile_s + (3 * rows + ml * 8) * 33 + i;
      const float *HE = tile_s + (0 * rows + ml * 4) * 33 + i, *HO = tile_s + (1 * rows + ml * 4) * 33 + i;
      float4 *dst = reinterpret_cast<float4 *>(sd.dsyn + ((static_cast<long>(tile * sd.nbt + ml) * d.nh + jh) * d.M + m) * SPLIT_NQ);
#pragma unroll
      for (int side = 0; side < 2; side++) {
        float pv[8], hv[4];
#pragma unroll
        for (int q = 0; q < 8; q++) pv[q] = side == 0 ? PE[q * 33] + PO[q * 33] : PE[q * 33] - PO[q * 33];
#pragma unroll
        for (int q = 0; q < 4; q++) hv[q] = side == 0 ? HE[q * 33] + HO[q * 33] : HO[q * 33] - HE[q * 33];
        const float2 U = cscale(csub(imul(make_float2(pv[2], pv[3]), mm), make_float2(hv[0], hv[1])), ia);
        const float2 V = cscale(cadd(imul(make_float2(pv[0], pv[1]), mm), make_float2(hv[2], hv[3])), ia);
        dst[2 * side] = make_float4(U.x, U.y, V.x, V.y);
        dst[2 * side + 1] = make_float4(pv[4], pv[5], pv[6], pv[7]);
      }
    }
  }
  split_teardown(tmem, ncols);
}

// The k-th work item of a persistent CTA. Work items are numbered in order of decreasing size (m, the wavenumber,
// is the slowest index: K and the coefficient count shrink as m grows) and dealt to the CTAs in snake order
// (pass 0 to CTAs 0..G-1, pass 1 to G-1..0, ...), so every CTA gets an even share of the work (dealing m-fastest
// items in one direction left the busiest CTA with half again the mean). Returns a value >= nitems past the CTA's
// last item.
__device__ __forceinline__ int snake_item(int k) {
  const int g = static_cast<int>(gridDim.x), c = static_cast<int>(blockIdx.x);
  return k * g + ((k & 1) ? g - 1 - c : c);
}

// ------------------------------------------------------------------------------------------- synthesis, warp-specialised
// The same work as split_syn, by persistent CTAs whose warps take roles (as split_ana_ws): thread 0 streams the H
// and P operand and table chunks of the CTA's items (m, member tile, latitude slice; dealt by snake_item) through
// a ring of ns fixed-size stages; thread 32 issues the MMAs of item i into tensor-memory buffer i % 2 (four
// accumulators H E/O, P E/O of nh columns each) and commits it to accf[i % 2]; warps 2..9 copy a finished buffer
// to shared memory, release it (acce) and write the item's Fourier records while the next item loads and
// multiplies. Same products in the same order as split_syn, same epilogue arithmetic: the same bits. Every wait is
// bounded; after a failure each role stops and the CTA drains its own copies and MMAs before it frees its memory.
constexpr int SPLIT_SYN_WS_THREADS = 320;
template <int CTAS>
__global__ void __launch_bounds__(SPLIT_SYN_WS_THREADS, CTAS) split_syn_ws(SphDev d, SplitDev sd, int B, int ns, int buf_cols, int slot_bytes) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full[SPLIT_MAX_STAGES], empty[SPLIT_MAX_STAGES], accf[2], acce[2], done;
  __shared__ uint32_t tslot;
  __shared__ int s_fail, s_issued, s_consumed, s_epi_ok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nh = sd.syn_nh, nsl = sd.nh16 / nh;  // latitudes per slice, slices
  const int nitems = d.M * sd.ntiles * nsl;
  const int bk = sd.bks;
  const uint32_t ncols = 2u * static_cast<uint32_t>(buf_cols);
  uint8_t *pipe = smem;
  const int ldp = nh + 1;
  // staging of a finished buffer: H E, H O (rSH rows each), P E, P O (rSP rows each), row stride nh + 1
  float *stg = reinterpret_cast<float *>(smem + static_cast<size_t>(ns) * slot_bytes);
  const int a_bytes = sd.rSP * bk * 2;  // A piece region of a stage (the H operand's rows fit in it)
  const int b_bytes = nh * bk * 2;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tslot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int st = 0; st < ns; st++) {
      tc::bar_init(su32(&full[st]), 1);
      tc::bar_init(su32(&empty[st]), 1);
    }
    for (int b2 = 0; b2 < 2; b2++) {
      tc::bar_init(su32(&accf[b2]), 1);
      tc::bar_init(su32(&acce[b2]), 1);
    }
    tc::bar_init(su32(&done), 1);
    tc::bar_init_fence();
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;
  auto item_of = [&](int item, int &m, int &tile, int &jh0) {
    const int per_m = sd.ntiles * nsl;
    m = item / per_m;
    const int rest = item - m * per_m;
    tile = rest % sd.ntiles;
    jh0 = (rest / sd.ntiles) * nh;
  };
  if (tid == 0) {
    // producer
    int git = 0;
    bool ok = true;
    for (int k = 0, item = snake_item(0); item < nitems && ok; item = snake_item(++k)) {
      int m, tile, jh0;
      item_of(item, m, tile, jh0);
      const long kp = sd.kps[m];
      const int nchunk = static_cast<int>(kp / bk);
      for (int g = 0; g < 2 && ok; g++) {
        const int aR = g == 0 ? sd.rSH : sd.rSP;
        const uint32_t abytes = static_cast<uint32_t>(aR * bk * 2);
        const __nv_bfloat16 *A = g == 0 ? sd.aS_H + sd.aSH_off[m] + static_cast<long>(tile) * sd.rSH * kp
                                        : sd.aS_P + sd.aS_off[m] + static_cast<long>(tile) * sd.rSP * kp;
        const long aps = g == 0 ? sd.aSH_size : sd.aSP_size;
        const __nv_bfloat16 *Bt = (g == 0 ? sd.tS_H : sd.tS_P) + sd.tS_off[m] + static_cast<long>(jh0) * bk;
        const long b_cs = static_cast<long>(sd.nh16) * bk;
        for (int c = 0; c < nchunk; c++, git++) {
          const int st = git % ns;
          if (git >= ns && !mbar_wait_bounded(su32(&empty[st]), ((git / ns) - 1) & 1)) {
            s_fail = 1;
            atomicExch(sd.err, 2);
            ok = false;
            break;
          }
          mbar_expect(su32(&full[st]), static_cast<uint32_t>(sd.pieces) * (abytes + static_cast<uint32_t>(b_bytes)));
          uint8_t *base = pipe + static_cast<size_t>(st) * slot_bytes;
          for (int p = 0; p < sd.pieces; p++) {
            bulk_g2s(su32(base + p * a_bytes), A + p * aps + static_cast<long>(c) * aR * bk, abytes, su32(&full[st]));
            bulk_g2s(su32(base + sd.pieces * a_bytes + p * b_bytes), Bt + p * sd.tS_size + static_cast<long>(c) * b_cs,
                     static_cast<uint32_t>(b_bytes), su32(&full[st]));
          }
          s_issued = git + 1;
        }
      }
    }
  } else if (tid == 32) {
    // MMA issuer: per operand g, K columns below ke16[m] (even n) into the E accumulator, the rest into O
    const int tp[6][2] = {{2, 0}, {1, 1}, {0, 2}, {1, 0}, {0, 1}, {0, 0}};
    const int t0 = sd.terms == 6 ? 0 : (sd.terms == 3 ? 3 : 5);
    const uint32_t sbo = static_cast<uint32_t>(bk) * 16u;
    const uint32_t idesc = idesc_m128(nh);
    int git = 0, it = 0;
    bool ok = true;
    for (int k = 0, item = snake_item(0); item < nitems && ok; item = snake_item(++k)) {
      int m, tile, jh0;
      item_of(item, m, tile, jh0);
      const int nchunk = static_cast<int>(sd.kps[m] / bk), kseg = sd.ke16[m];
      const int bb = it & 1;
      if (it >= 2 && !mbar_wait_bounded(su32(&acce[bb]), ((it >> 1) - 1) & 1)) {
        s_fail = 1;
        atomicExch(sd.err, 5);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int g = 0; g < 2 && ok; g++) {
        bool started[2] = {false, false};
        for (int c = 0; c < nchunk; c++, git++) {
          const int st = git % ns;
          if (!mbar_wait_bounded(su32(&full[st]), (git / ns) & 1)) {
            s_fail = 1;
            atomicExch(sd.err, 3);
            ok = false;
            break;
          }
          s_consumed = git + 1;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          uint8_t *base = pipe + static_cast<size_t>(st) * slot_bytes;
          for (int kk = 0; kk < bk; kk += 16) {
            const int seg = c * bk + kk >= kseg ? 1 : 0;
            const uint32_t accc = tmem + static_cast<uint32_t>(bb * buf_cols + (2 * g + seg) * nh);
            for (int tt = t0; tt < 6; tt++) {
              const int pa = tp[tt][0], pb = tp[tt][1];
              const uint64_t ad = chunk_desc(su32(base + pa * a_bytes + (kk / 8) * 128), sbo);
              const uint64_t bd = chunk_desc(su32(base + sd.pieces * a_bytes + pb * b_bytes + (kk / 8) * 128), sbo);
              const uint32_t accum = started[seg] ? 1u : 0u;
              asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(accc),
                           "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
                           : "memory");
              started[seg] = true;
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(&empty[st])) : "memory");
        }
      }
      if (!ok) break;
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(&accf[bb])) : "memory");
      it++;
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(&done)) : "memory");
  } else if (warp >= 2) {
    // epilogue warps
    const int et = tid - 64;
    int it = 0;
    const float ia = d.inv_a_f;
    for (int k = 0, item = snake_item(0); item < nitems; item = snake_item(++k)) {
      int m, tile, jh0;
      item_of(item, m, tile, jh0);
      const int bb = it & 1;
      if (et == 0) s_epi_ok = mbar_wait_bounded(su32(&accf[bb]), (it >> 1) & 1) ? 1 : 0;
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (!s_epi_ok) {
        if (et == 0) {
          s_fail = 1;
          atomicExch(sd.err, 6);
        }
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int mt = min(sd.nbt, B - tile * sd.nbt);
      // accumulators -> staging: warp w reads lanes 32 (w % 4) .. + 31; warps 2..5 the even 32-column blocks of
      // the four accumulators, warps 6..9 the odd ones. H accumulators hold rSH meaningful rows, P rSP
      const int quarter = warp & 3, row = quarter * 32 + lane;
      const uint32_t lanebase = tmem + static_cast<uint32_t>(bb * buf_cols) + (static_cast<uint32_t>(quarter * 32) << 16);
      const int nblk = (nh + 31) / 32;
      for (int a4 = 0; a4 < 4; a4++) {
        const int rows_a = a4 < 2 ? sd.rSH : sd.rSP;
        if (quarter * 32 >= rows_a) continue;
        float *dst = stg + static_cast<size_t>(a4 < 2 ? a4 * sd.rSH : 2 * sd.rSH + (a4 - 2) * sd.rSP) * ldp;
        for (int cbk = (warp < 6 ? 0 : 1); cbk < nblk; cbk += 2) {
          const int c0 = cbk * 32;
          float v[32];
          if (c0 + 32 <= nh) {
            tmem_ld32(lanebase + a4 * nh + c0, v);
          } else {
            tmem_ld8(lanebase + a4 * nh + c0, v);
            tmem_ld8(lanebase + a4 * nh + c0 + 8, v + 8);
          }
          if (row < rows_a) {
            const int w = min(32, nh - c0);
#pragma unroll
            for (int i = 0; i < 32; i++)
              if (i < w) dst[row * ldp + c0 + i] = v[i];
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (et == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&acce[bb])) : "memory");
      // Fourier coefficients of both mirror latitudes (as split_syn): P sums south E + O, north E - O; H sums
      // south E + O, north O - E; U = (i m chi P - psi H) / a, V = (i m psi P + chi H) / a (cpp/sphere.cpp:200-201)
      const float mm = static_cast<float>(m);
      const float *HE0 = stg, *HO0 = stg + static_cast<size_t>(sd.rSH) * ldp, *PE0 = stg + static_cast<size_t>(2 * sd.rSH) * ldp,
                  *PO0 = stg + static_cast<size_t>(2 * sd.rSH + sd.rSP) * ldp;
      for (int e = et; e < mt * nh; e += SPLIT_WS_EPI) {
        const int ml = e / nh, i = e - ml * nh, jh = jh0 + i;
        if (jh >= d.nh) continue;
        const float *PE = PE0 + (ml * 8) * ldp + i, *PO = PO0 + (ml * 8) * ldp + i;
        const float *HE = HE0 + (ml * 4) * ldp + i, *HO = HO0 + (ml * 4) * ldp + i;
        float4 *dst = reinterpret_cast<float4 *>(sd.dsyn + ((static_cast<long>(tile * sd.nbt + ml) * d.nh + jh) * d.M + m) * SPLIT_NQ);
#pragma unroll
        for (int side = 0; side < 2; side++) {
          float pv[8], hv[4];
#pragma unroll
          for (int q = 0; q < 8; q++) pv[q] = side == 0 ? PE[q * ldp] + PO[q * ldp] : PE[q * ldp] - PO[q * ldp];
#pragma unroll
          for (int q = 0; q < 4; q++) hv[q] = side == 0 ? HE[q * ldp] + HO[q * ldp] : HO[q * ldp] - HE[q * ldp];
          const float2 U = cscale(csub(imul(make_float2(pv[2], pv[3]), mm), make_float2(hv[0], hv[1])), ia);
          const float2 V = cscale(cadd(imul(make_float2(pv[0], pv[1]), mm), make_float2(hv[2], hv[3])), ia);
          dst[2 * side] = make_float4(U.x, U.y, V.x, V.y);
          dst[2 * side + 1] = make_float4(pv[4], pv[5], pv[6], pv[7]);
        }
      }
      // the staging is free for the next item
      asm volatile("bar.sync 1, 256;" ::: "memory");
      it++;
    }
  }
  __syncthreads();
  if (tid == 0) {
    if (!s_fail) {
      if (!mbar_wait_bounded(su32(&done), 0)) atomicExch(sd.err, 4);
    } else {
      tc::wait_for(su32(&done), 0, 200000000ull);
      for (int g2 = s_consumed; g2 < s_issued; g2++) tc::wait_for(su32(&full[g2 % ns]), (g2 / ns) & 1, 200000000ull);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

// ------------------------------------------------------------------------------------------- grid (FP32)
// grid: (nh / jb, B). Fourier records of jb latitude pairs -> FFTs and products -> folded values. DIRECT: written
// as the analysis operands (BF16 pieces in the chunk layout, jb consecutive latitudes per store), which the
// analysis streams with bulk copies; otherwise written m-major as FP32 fold[m][slot][parity][member][jh] (jb
// latitudes per store), which the analysis gathers (cheaper for a few members, where jb is small)
// FMAX: the largest FFT stage group the instantiation takes (4: sixteen elements per thread, two CTAs per SM)
// LOGN: log2 of the transform length when it is fixed at compile time (the FFT groups then address shared memory
// with immediates), 0 for any length. Register budget: three CTAs per SM (77 registers) for the three-stage groups
// and for the four-stage groups of transforms up to 256 points, where the rows of a CTA's latitude pairs leave room
// for a third CTA or the fixed addressing frees the registers; two for the any-length and longer forms
template <bool DIRECT, int FMAX, int LOGN>
__global__ void __launch_bounds__(GRID_THREADS, FMAX < 4 || (LOGN > 0 && LOGN <= 8) ? 3 : 2) split_grid(SphDev d, SphTab<float> t, SplitDev sd, const double *__restrict__ fgrid,
                                                           const double *__restrict__ hsgrid) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float2 *sm = reinterpret_cast<float2 *>(smraw);  // rows f * jb + p: U, V, zeta, Phi and the fifth product of pair p
  const int JB = sd.jb;
  const int b = blockIdx.y, jh0 = blockIdx.x * JB;
  const int tile = b / sd.nbt, ml = b - tile * sd.nbt;
  constexpr int PSG = FMAX >= 4 ? 4 : 3;  // row padding: one element per 16 for sixteen-element FFT groups, else per 8
  const int logn = LOGN ? LOGN : d.logn;
  const int n = 1 << logn, M = d.M, rl = fft_row<PSG>(n);  // padded rows: element i at fft_at<PSG>(i)
  // the untilted Coriolis parameter 2 Omega mu of the CTA's latitudes (south, north), rounded to FP32 once
  __shared__ float cor[2 * SPLIT_JB_MAX];
  if (threadIdx.x < 2 * JB) {
    const int pr = threadIdx.x >> 1, js = jh0 + pr, j = (threadIdx.x & 1) ? d.nlat - 1 - js : js;
    cor[threadIdx.x] = static_cast<float>(d.om2[b] * d.mu[j]);
  }
  for (int e = threadIdx.x; e < 4 * JB * rl; e += blockDim.x) sm[e] = make_float2(0, 0);
  __syncthreads();
  for (int e = threadIdx.x; e < JB * M; e += blockDim.x) {
    const int pr = e / M, m = e - pr * M;
    const float4 *rec = reinterpret_cast<const float4 *>(sd.dsyn + ((static_cast<long>(b) * d.nh + jh0 + pr) * M + m) * SPLIT_NQ);
    const float4 s0 = rec[0], s1 = rec[1], n0 = rec[2], n1 = rec[3];
    const float2 A[4] = {make_float2(s0.x, s0.y), make_float2(s0.z, s0.w), make_float2(s1.x, s1.y), make_float2(s1.z, s1.w)};
    const float2 C[4] = {make_float2(n0.x, n0.y), make_float2(n0.z, n0.w), make_float2(n1.x, n1.y), make_float2(n1.z, n1.w)};
#pragma unroll
    for (int f = 0; f < 4; f++) {
      const float2 a = A[f], c = C[f];
      float2 *row = sm + static_cast<size_t>(f * JB + pr) * rl;
      if (m == 0) row[0] = make_float2(a.x, c.x);
      else {
        row[fft_at<PSG>(bitrev(m, logn))] = make_float2(a.x - c.y, a.y + c.x);
        row[fft_at<PSG>(bitrev(n - m, logn))] = make_float2(a.x + c.y, c.x - a.y);
      }
    }
  }
  __syncthreads();
  if constexpr (LOGN > 0) fft_inverse_dit_c<float2, PSG, FMAX, LOGN>(sm, 4 * JB, t.tw, sd.fgrp);
  else fft_inverse_dit<float2, PSG, FMAX>(sm, 4 * JB, n, logn, t.tw, sd.fgrp);
  const float g = static_cast<float>(d.g);
  for (int e = threadIdx.x; e < JB * n; e += blockDim.x) {
    const int pr = e >> logn, k = e & (n - 1);
    const int js = jh0 + pr, jn = d.nlat - 1 - js;
    const float r2om = t.r2om[js];
    const double *fr_s = fgrid + (static_cast<size_t>(b) * d.nlat + js) * n, *fr_n = fgrid + (static_cast<size_t>(b) * d.nlat + jn) * n;
    const double *hr_s = hsgrid + (static_cast<size_t>(b) * d.nlat + js) * n, *hr_n = hsgrid + (static_cast<size_t>(b) * d.nlat + jn) * n;
    const int gf = d.gflag[b];
    float2 *rU = sm + static_cast<size_t>(0 * JB + pr) * rl, *rV = sm + static_cast<size_t>(1 * JB + pr) * rl;
    float2 *rZ = sm + static_cast<size_t>(2 * JB + pr) * rl, *rP = sm + static_cast<size_t>(3 * JB + pr) * rl;
    float2 *rE = sm + static_cast<size_t>(4 * JB + pr) * rl;
    const int kp = fft_at<PSG>(k);
    const float2 U = rU[kp], V = rV[kp], Z = rZ[kp], P = rP[kp];
    float2 A, Bv, UP, VP, PE;
    // the FP64 Coriolis and orography rows (tilted or mountain members only) are rounded to FP32 on the integer
    // pipe: the same values as the hardware conversion, without the narrow FP64 pipe
    // linear-exact form: the untilted Coriolis parameter and Phi leave eta and Phi + E (their terms are added in
    // spectral space by the analysis), and P is Phi' (the synthesis left out Phi_00)
    const bool lx = sd.lin_exact != 0;
    {
      const float eta = Z.x + ((gf & 1) ? d2f_int(fr_s[k]) : (lx ? 0.0f : cor[2 * pr]));
      const float hs = (gf & 2) ? d2f_int(hr_s[k]) : 0.0f;
      A.x = U.x * eta; Bv.x = V.x * eta; UP.x = U.x * P.x; VP.x = V.x * P.x;
      PE.x = (lx ? 0.0f : P.x) + g * hs + (U.x * U.x + V.x * V.x) * r2om;
    }
    {
      const float eta = Z.y + ((gf & 1) ? d2f_int(fr_n[k]) : (lx ? 0.0f : cor[2 * pr + 1]));
      const float hs = (gf & 2) ? d2f_int(hr_n[k]) : 0.0f;
      A.y = U.y * eta; Bv.y = V.y * eta; UP.y = U.y * P.y; VP.y = V.y * P.y;
      PE.y = (lx ? 0.0f : P.y) + g * hs + (U.y * U.y + V.y * V.y) * r2om;
    }
    rU[kp] = A; rV[kp] = Bv; rZ[kp] = UP; rP[kp] = VP; rE[kp] = PE;
  }
  __syncthreads();
  if constexpr (LOGN > 0) fft_forward_dif_c<float2, PSG, FMAX, LOGN>(sm, 5 * JB, t.tw, sd.fgrp);
  else fft_forward_dif<float2, PSG, FMAX>(sm, 5 * JB, n, logn, t.tw, sd.fgrp);
  const float inv = 1.0f / n, hinv = 0.5f * inv;
  // one work item per (m, slot r): the folded values of this CTA's latitude pairs at both parities. Direct
  // operands: the five slots of one m are consecutive threads, so a warp's stores of one row pair land in the
  // same few core matrices; FP32 fold: consecutive m
  for (int e = threadIdx.x; e < M * 5; e += blockDim.x) {
    const int m = DIRECT ? e / 5 : e % M, r = DIRECT ? e - 5 * (e / 5) : e / M;
    {
      float2 f0[SPLIT_JB_MAX], f1[SPLIT_JB_MAX];
#pragma unroll
      for (int pr = 0; pr < SPLIT_JB_MAX; pr++) {
        if (pr >= JB) break;
        const int js = jh0 + pr;
        const float2 *row = sm + static_cast<size_t>(r * JB + pr) * rl;
        const float2 Ym = row[fft_at<PSG>(bitrev(m, logn))], Yc = conjd(row[fft_at<PSG>(bitrev((n - m) & (n - 1), logn))]);
        float2 Xs = cscale(cadd(Ym, Yc), hinv);
        const float2 tt = csub(Ym, Yc);
        float2 Xn = make_float2(hinv * tt.y, -hinv * tt.x);
        const float wt = r < 4 ? t.wd[js] : t.w[js];
        Xs = cscale(Xs, wt);
        Xn = cscale(Xn, wt);
        f0[pr] = cadd(Xs, Xn);
        f1[pr] = csub(Xs, Xn);
      }
      if constexpr (!DIRECT) {
#pragma unroll
        for (int par = 0; par < 2; par++) {
          const float2 *fv = par ? f1 : f0;
          float2 *o = sd.fold + ((static_cast<long>(m) * 10 + r * 2 + par) * gridDim.y + b) * d.nh + jh0;
          if (JB >= 2) {
#pragma unroll
            for (int pr = 0; pr < SPLIT_JB_MAX; pr += 2) {
              if (pr >= JB) break;
              reinterpret_cast<float4 *>(o)[pr / 2] = make_float4(fv[pr].x, fv[pr].y, fv[pr + 1].x, fv[pr + 1].y);
            }
          } else {
            o[0] = fv[0];
          }
        }
      } else {
      // the folded values go straight into the analysis operands (BF16 pieces, chunk layout): slot r at parity p
      // is a P row of (m, s = p) for r = 0, 1, 2, 4 and an H row of (m, s = 1 - p) for r = 0, 1, 3
#pragma unroll
      for (int par = 0; par < 2; par++) {
        const float2 *fv = par ? f1 : f0;
#pragma unroll
        for (int isH = 0; isH < 2; isH++) {
          if (isH ? (r == 2 || r == 4) : (r == 3)) continue;
          const int s_op = isH ? 1 - par : par;
          const int R = isH ? sd.rAH : sd.rAP;
          const int q = isH ? (r == 3 ? 2 : r) : (r == 4 ? 3 : r);
          const int row0 = isH ? ml * 6 + 2 * q : ml * 8 + 2 * q;
          __nv_bfloat16 *opnd = (isH ? sd.aA_H : sd.aA_P) + ((static_cast<long>(m) * 2 + s_op) * sd.ntiles + tile) * R * sd.nha;
          const long pstride = isH ? sd.aAH_size : sd.aAP_size;
#pragma unroll
          for (int ri = 0; ri < 2; ri++) {
            __nv_bfloat16 pc[3][SPLIT_JB_MAX];
#pragma unroll
            for (int pr = 0; pr < SPLIT_JB_MAX; pr++) {
              const float x = pr < JB ? (ri ? fv[pr].y : fv[pr].x) : 0.0f;
              const __nv_bfloat16 h = __float2bfloat16_rn(x);
              const float r1 = x - __bfloat162float(h);
              const __nv_bfloat16 l = __float2bfloat16_rn(r1);
              pc[0][pr] = h;
              pc[1][pr] = l;
              pc[2][pr] = __float2bfloat16_rn(r1 - __bfloat162float(l));
            }
            __nv_bfloat16 *dst = opnd + tile_off(row0 + ri, jh0, R, sd.bka);
#pragma unroll
            for (int pi = 0; pi < 3; pi++) {
              if (pi >= sd.pieces) break;
              __nv_bfloat16 *dp = dst + pi * pstride;
              if (JB == 8) {
                uint4 w;
                __nv_bfloat16 *wp = reinterpret_cast<__nv_bfloat16 *>(&w);
#pragma unroll
                for (int j = 0; j < 8; j++) wp[j] = pc[pi][j];
                *reinterpret_cast<uint4 *>(dp) = w;
              } else if (JB == 4) {
                uint2 w;
                __nv_bfloat16 *wp = reinterpret_cast<__nv_bfloat16 *>(&w);
                wp[0] = pc[pi][0];
                wp[1] = pc[pi][1];
                wp[2] = pc[pi][2];
                wp[3] = pc[pi][3];
                *reinterpret_cast<uint2 *>(dp) = w;
              } else if (JB == 2) {
                __nv_bfloat162 w;
                w.x = pc[pi][0];
                w.y = pc[pi][1];
                *reinterpret_cast<__nv_bfloat162 *>(dp) = w;
              } else {
                dp[0] = pc[pi][0];
              }
            }
          }
        }
      }
      }
    }
  }
}

// the grid kernel instantiation for a plan: operand form, FFT group bound and transform length (lengths 2^6 to
// 2^10, T21 to T341, compiled for their length; others take the any-length form)
using SplitGridFn = void (*)(SphDev, SphTab<float>, SplitDev, const double *, const double *);
template <bool DIRECT, int FMAX> inline SplitGridFn split_grid_for(int logn) {
  switch (logn) {
    case 6: return split_grid<DIRECT, FMAX, 6>;
    case 7: return split_grid<DIRECT, FMAX, 7>;
    case 8: return split_grid<DIRECT, FMAX, 8>;
    case 9: return split_grid<DIRECT, FMAX, 9>;
    case 10: return split_grid<DIRECT, FMAX, 10>;
    default: return split_grid<DIRECT, FMAX, 0>;
  }
}
inline SplitGridFn split_grid_kernel(int direct, int fmax, int logn) {
  if (fmax >= 4) return direct ? split_grid_for<true, 4>(logn) : split_grid_for<false, 4>(logn);
  return direct ? split_grid_for<true, 3>(logn) : split_grid_for<false, 3>(logn);
}

// ------------------------------------------------------------------------------------------- synthesis operands
// The next synthesis operands for coefficient (member b, m, n) from its value rounded to FP32: psi, chi, zeta, Phi
// (P rows) and psi, chi (H rows) at column k(n) of wavenumber m; kf = -a^2 / (n (n + 1)) in FP32.
__device__ __forceinline__ void pack_syn_coef(const SphDev &d, const SplitDev &sd, float kf, int b, int m, int n, float2 z, float2 dl, float2 f) {
  const int tile = b / sd.nbt, ml = b - tile * sd.nbt;
  const int ke16 = sd.ke16[m];
  const int k = ((n - m) & 1) ? ke16 + ((n - m - 1) >> 1) : ((n - m) >> 1);
  const long kp = sd.kps[m];
  const long baseP = sd.aS_off[m] + static_cast<long>(tile) * sd.rSP * kp;
  const long baseH = sd.aSH_off[m] + static_cast<long>(tile) * sd.rSH * kp;
  // the linear-exact form synthesises Phi' = Phi - Phi_00 P_00: the mean enters the tendencies separately
  const bool mean = sd.lin_exact && n == 0;
  const float v[8] = {z.x * kf, z.y * kf, dl.x * kf, dl.y * kf, z.x, z.y, mean ? 0.0f : f.x, mean ? 0.0f : f.y};
#pragma unroll
  for (int q = 0; q < 8; q++) fsplit(v[q], sd.aS_P + baseP + tile_off(ml * 8 + q, k, sd.rSP, sd.bks), sd.aSP_size, sd.pieces);
#pragma unroll
  for (int q = 0; q < 4; q++) fsplit(v[q], sd.aS_H + baseH + tile_off(ml * 4 + q, k, sd.rSH, sd.bks), sd.aSH_size, sd.pieces);
}

__device__ __forceinline__ float2 d2f2(double2 v) { return make_float2(d2f_int(v.x), d2f_int(v.y)); }

// The split path's private FP32 buffers (the state's copy, the RK4 accumulator, the stage inputs) order each m's
// coefficients by parity: n - m even first (index (n - m) / 2), then odd ((N - m) / 2 + 1 + (n - m - 1) / 2), so an
// analysis work item of one parity reads and writes them with unit stride. The FP64 state keeps the triangle order.
__device__ __forceinline__ int par_index(const SphDev &d, int m, int n) {
  const int k = n - m;
  return d.tri[m] + ((k & 1) ? (d.N - m) / 2 + 1 + (k >> 1) : (k >> 1));
}

// After the state was set from outside the stepping: its FP32 copy xf (stages 0-2 read it) and the synthesis
// operands. grid: (ceil(ntri/128), B)
__global__ void split_pack_state(SphDev d, SplitDev sd, const float *__restrict__ kfac32, const double2 *__restrict__ x, float2 *__restrict__ xf) {
  const int b = blockIdx.y, q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.ntri) return;
  const size_t i = static_cast<size_t>(b) * 3 * d.ntri + q;
  const float2 z = d2f2(x[i]), dl = d2f2(x[i + d.ntri]), f = d2f2(x[i + 2 * d.ntri]);
  const int n = d.trin[q], m = d.trim[q];
  const size_t ip = static_cast<size_t>(b) * 3 * d.ntri + par_index(d, m, n);
  xf[ip] = z;
  xf[ip + d.ntri] = dl;
  xf[ip + 2 * d.ntri] = f;
  pack_syn_coef(d, sd, kfac32[n], b, m, n, z, dl, f);
}

// ------------------------------------------------------------------------------------------- analysis + RK4
// The analysis epilogue of one coefficient (member b = tile member ml, wavenumber m, parity s, index r: n = m + s + 2r)
// from the accumulators staged in shared memory (dsm, row stride ldp): the tendencies (cpp/sphere.cpp:380-389) with
// the linear terms of the linear-exact form, the RK4 stage update, the next stage input and the next synthesis
// operands. Shared by both analysis kernels, so both give the same bits.
// Precision: the state x0 is FP64 and only the last stage touches it (x0 + c (k1 + 2 k2 + 2 k3 + k4), del^4
// filter, in FP64); xf holds it rounded to FP32. The tendencies are FP32 (their nonlinear part carries the BF16
// pieces' 2^-16 rounding), so the accumulator k1 + 2 k2 + 2 k3 (acc) and the stage inputs xf + c k of stages 0-2,
// which the next stage only reads in FP32, are formed in FP32.
__device__ __forceinline__ void ana_coef(const SphDev &d, const SplitDev &sd, const SphTab<float> &t, const StageArgs &sa,
                                         double2 *__restrict__ x0, float2 *__restrict__ xf, const float2 *__restrict__ xin,
                                         float2 *__restrict__ xout, float2 *__restrict__ acc, const float *dsm, int ldp, int m, int tile, int ml,
                                         int s, int r, int cb1, int ra0, int ra1) {
  const int b = tile * sd.nbt + ml, n = m + s + 2 * r;
  const int cbs = s ? cb1 : 0, ras = s ? ra1 : ra0;
  const float *H = dsm + (ml * 6) * ldp + cbs + r, *P = dsm + (ml * 8) * ldp + cbs + ras + r;
  const float2 aH = make_float2(H[0 * ldp], H[1 * ldp]), bH = make_float2(H[2 * ldp], H[3 * ldp]), vH = make_float2(H[4 * ldp], H[5 * ldp]);
  const float2 aP = make_float2(P[0 * ldp], P[1 * ldp]), bP = make_float2(P[2 * ldp], P[3 * ldp]);
  const float2 uP = make_float2(P[4 * ldp], P[5 * ldp]), eP = make_float2(P[6 * ldp], P[7 * ldp]);
  const float mm = static_cast<float>(m);
  // cpp/sphere.cpp:380-389
  float2 kz = csub(bH, imul(aP, mm));
  float2 kd = cadd(cadd(imul(bP, mm), aH), cscale(eP, t.lapl[n]));
  float2 kf = csub(vH, imul(uP, mm));
  const int q = d.tri[m] + n - m;
  // the FP64 state in triangle order (q); the FP32 buffers in parity order: this coefficient at qp, its
  // neighbours n + 1 and n - 1 (the other parity) at qu and ql
  const int ne = (d.N - m) / 2 + 1;  // coefficients of even n - m
  const int qp = d.tri[m] + (s ? ne + r : r), qu = d.tri[m] + (s ? r + 1 : ne + r), ql = d.tri[m] + (s ? r : ne + r - 1);
  const size_t mb = static_cast<size_t>(b) * 3 * d.ntri, base = mb + q, basep = mb + qp;
  // the stage input in FP32: the state's copy at stage 0, else the previous stage's output (a separate buffer:
  // neighbouring n belong to other CTAs)
  const float2 *yin = sa.stage == 0 ? xf : xin;
  if (sd.lin_exact && q != 0) {
    // the terms linear in the stage input y, in FP32 like the rest of the tendencies but outside the BF16 products:
    // n(n+1)/a^2 Phi_n in d delta; -Phi_mean delta_n in d Phi (D(U, V) = delta exactly for n <= T); for an untilted
    // axis the Coriolis terms -D(f U, f V) and D(f V, -f U) with f = 2 Omega mu, which couple n - 1, n, n + 1 of
    // the same m
    auto yat = [&](int field, int qq) -> float2 { return yin[mb + static_cast<size_t>(field) * d.ntri + qq]; };
    const float2 yz = yat(0, qp), yd = yat(1, qp), yf = yat(2, qp);
    const float phibar = xf[mb + 2 * d.ntri].x * t.Ps[0];
    const float lp = t.lapl[n];
    kd.x += lp * yf.x;
    kd.y += lp * yf.y;
    kf.x -= phibar * yd.x;
    kf.y -= phibar * yd.y;
    if (!(d.gflag[b] & 1)) {
      const float om = static_cast<float>(d.om2[b]);
      const float cA = sd.lin32[q], cB = sd.lin32[d.ntri + q], cC = sd.lin32[2 * d.ntri + q];
      const float2 zu = n < d.N ? yat(0, qu) : make_float2(0, 0), du = n < d.N ? yat(1, qu) : make_float2(0, 0);
      const float2 zl = n > m ? yat(0, ql) : make_float2(0, 0), dd = n > m ? yat(1, ql) : make_float2(0, 0);
      // -D(fU, fV)_n = -2 Omega (cA delta_{n+1} + cB delta_{n-1} - i cC zeta_n)
      kz.x -= om * (cA * du.x + cB * dd.x + cC * yz.y);
      kz.y -= om * (cA * du.y + cB * dd.y - cC * yz.x);
      // D(fV, -fU)_n = 2 Omega (cA zeta_{n+1} + cB zeta_{n-1} + i cC delta_n)
      kd.x += om * (cA * zu.x + cB * zl.x - cC * yd.y);
      kd.y += om * (cA * zu.y + cB * zl.y + cC * yd.x);
    }
  }
  if (q == 0) kz = kd = kf = make_float2(0, 0);
  const float2 k[3] = {kz, kd, kf};
  float2 nv[3];
  if (sa.stage < 3) {
    // every load of the three fields is issued before any store (the buffers never alias)
    float2 yv[3], av[3];
#pragma unroll
    for (int f = 0; f < 3; f++) {
      yv[f] = xf[basep + static_cast<size_t>(f) * d.ntri];
      av[f] = sa.stage > 0 ? acc[basep + static_cast<size_t>(f) * d.ntri] : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int f = 0; f < 3; f++) {
      const size_t i = basep + static_cast<size_t>(f) * d.ntri;
      acc[i] = sa.stage == 0 ? k[f] : make_float2(fmaf(2.0f, k[f].x, av[f].x), fmaf(2.0f, k[f].y, av[f].y));
      nv[f] = make_float2(fmaf(sa.c32, k[f].x, yv[f].x), fmaf(sa.c32, k[f].y, yv[f].y));
      // the next stage input is kept when the linear-exact form reads it (the split synthesis reads the packed
      // operands written below)
      if (xout != nullptr) xout[i] = nv[f];
    }
  } else {
    double2 xv[3];
    float2 av[3];
#pragma unroll
    for (int f = 0; f < 3; f++) {
      xv[f] = x0[base + static_cast<size_t>(f) * d.ntri];
      av[f] = acc[basep + static_cast<size_t>(f) * d.ntri];
    }
#pragma unroll
    for (int f = 0; f < 3; f++) {
      const double2 sum = make_double2(f2d_int(av[f].x + k[f].x), f2d_int(av[f].y + k[f].y));
      const double2 val = make_double2(fma(sa.c, sum.x, xv[f].x), fma(sa.c, sum.y, xv[f].y));
      const double fac = sa.filt[(f == 2 ? 1 : 0) * d.M + n];
      const double2 x1 = q == 0 ? val : cscale(val, fac);
      x0[base + static_cast<size_t>(f) * d.ntri] = x1;
      nv[f] = d2f2(x1);
      xf[basep + static_cast<size_t>(f) * d.ntri] = nv[f];
    }
  }
  pack_syn_coef(d, sd, t.kfac[n], b, m, n, nv[0], nv[1], nv[2]);
}


// BOTH = false: grid (M, 2, ntiles), one parity s = blockIdx.y per CTA. BOTH = true: grid (M, 1, ntiles), both
// parities in one CTA one after the other (the GEMM pipeline's barriers continue their phases), so the epilogue
// walks every n of m in order and the FP64 state is read and written with unit stride. Accumulator columns of
// parity s: H at [cb_s, cb_s + ra_s), P at [cb_s + ra_s, cb_s + 2 ra_s), cb_0 = 0, cb_1 = 2 ra_0 (BOTH).
// MINB: CTAs per SM the register budget allows (2: up to 128 registers a thread; 3: up to 80, for plans whose
// shared memory admits three CTAs per SM)
template <bool BOTH, bool DIRECT, int MINB>
__global__ void __launch_bounds__(SPLIT_ANA_THREADS, MINB) split_ana(SphDev d, SplitDev sd, SphTab<float> t, StageArgs sa, int B, int ns,
                                                             double2 *__restrict__ x0, float2 *__restrict__ xf, const float2 *__restrict__ xin,
                                                             float2 *__restrict__ xout, float2 *__restrict__ acc) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full[SPLIT_MAX_STAGES], empty[SPLIT_MAX_STAGES], done;
  __shared__ uint32_t tslot;
  // work items (m, parity or both, member tile); a CTA takes items blockIdx.x, blockIdx.x + gridDim.x, ... with one
  // TMEM allocation and one set of barriers whose phases continue from item to item. With one CTA per item, m is
  // the slowest index (CTAs start in order of decreasing work: fewer coefficients as m grows, so the small items
  // fill the last wave); with fewer CTAs, m is the fastest (each CTA gets a mix of m)
  const int per_m = (BOTH ? 1 : 2) * sd.ntiles;
  const int nitems = d.M * per_m;
  const bool m_slowest = static_cast<int>(gridDim.x) >= nitems;
  uint32_t ncols = 32;
  while (ncols < static_cast<uint32_t>(BOTH ? sd.ana_cols_both : sd.ana_cols_one)) ncols <<= 1;
  // DIRECT: A operands streamed with the tables; otherwise gathered from the FP32 fold into resident shared memory
  // (H rows then P rows, every chunk and piece, in the chunk layout) ahead of the pipeline buffers
  const int nchunk = sd.nha / sd.bka;
  const int aH_bytes = DIRECT ? 0 : sd.pieces * nchunk * sd.rAH * sd.bka * 2, aP_bytes = DIRECT ? 0 : sd.pieces * nchunk * sd.rAP * sd.bka * 2;
  uint8_t *aH = smem, *aP = smem + aH_bytes, *pipe = smem + aH_bytes + aP_bytes;
  bool ok = true, setup_done = false;
  int pipe_it = 0, calls = 0;
  for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
  const int m = m_slowest ? item / per_m : item % d.M, rest = m_slowest ? item % per_m : item / d.M;
  const int s_first = BOTH ? 0 : rest % 2, s_last = BOTH ? 1 : s_first;
  const int tile = BOTH ? rest : rest / 2;
  const int mt = min(sd.nbt, B - tile * sd.nbt);
  const int R0 = (d.N - m) / 2 + 1, R1 = (d.N - m + 1) / 2;  // coefficients of each parity
  if ((s_first ? R1 : R0) == 0) continue;
  const int ra0 = sd.ra16[2 * m], ra1 = sd.ra16[2 * m + 1];
  const int cb1 = BOTH ? 2 * ra0 : 0;                               // cb_0 = 0
  const int ld = BOTH ? 2 * (ra0 + ra1) : 2 * (s_first ? ra1 : ra0);  // accumulator columns (and dsm row length)
  // the previous item's epilogue has finished reading shared memory and tensor memory
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  for (int s = s_first; s <= s_last && ok; s++) {
  if ((s ? R1 : R0) == 0) break;
  if (!DIRECT) {
    // gather the folded grid values of this (m, s) into the resident A operands: P quantities a, b, u, e at
    // parity s and H quantities a, b, v at parity 1 - s. One work item = (member, quantity, 8 latitudes): eight
    // consecutive float2 loads, then one 16-byte store per (real/imaginary row, piece) into the chunk layout.
    const int ph = 1 - s;
    const long pstrideP = static_cast<long>(nchunk) * sd.rAP * sd.bka, pstrideH = static_cast<long>(nchunk) * sd.rAH * sd.bka;
    const long sstride = static_cast<long>(B) * d.nh;  // between slots/parities of fold[m][slot][parity][member][jh]
    const float2 *gm = sd.fold + static_cast<long>(m) * 10 * sstride + static_cast<long>(tile * sd.nbt) * d.nh;
    const int nkb = sd.nha >> 3;
    // consecutive threads take different operand rows of the same 8-latitude block: their 16-byte stores land in
    // different rows of the core matrices (different banks)
    for (int e = threadIdx.x; e < mt * 7 * nkb; e += blockDim.x) {
      const int kb = e / (mt * 7), rest = e - kb * (mt * 7), qi = rest % 7, ml = rest / 7;
      // qi 0..3: P slots 0, 1, 2, 4 at parity s; 4..6: H slots 0, 1, 3 at parity 1 - s
      const int slot = qi < 3 ? qi : (qi == 3 ? 4 : (qi == 6 ? 3 : qi - 4));
      const int par = qi < 4 ? s : ph;
      const int j0 = kb * 8;
      float2 v[8];
      const float2 *g = gm + static_cast<long>(slot * 2 + par) * sstride + static_cast<long>(ml) * d.nh + j0;
#pragma unroll
      for (int j = 0; j < 8; j++) v[j] = j0 + j < d.nh ? g[j] : make_float2(0.0f, 0.0f);
      const bool isP = qi < 4;
      const int R = isP ? sd.rAP : sd.rAH;
      const int row = isP ? ml * 8 + 2 * qi : ml * 6 + 2 * (qi - 4);
      __nv_bfloat16 *base = reinterpret_cast<__nv_bfloat16 *>(isP ? aP : aH);
      const long pstride = isP ? pstrideP : pstrideH;
#pragma unroll
      for (int ri = 0; ri < 2; ri++) {
        uint4 k0, k1, k2;
        __nv_bfloat16 *b0 = reinterpret_cast<__nv_bfloat16 *>(&k0), *b1 = reinterpret_cast<__nv_bfloat16 *>(&k1),
                      *b2 = reinterpret_cast<__nv_bfloat16 *>(&k2);
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const float x = ri == 0 ? v[j].x : v[j].y;
          const __nv_bfloat16 h = __float2bfloat16_rn(x);
          const float r1 = x - __bfloat162float(h);
          const __nv_bfloat16 l = __float2bfloat16_rn(r1);
          b0[j] = h;
          b1[j] = l;
          b2[j] = __float2bfloat16_rn(r1 - __bfloat162float(l));
        }
        __nv_bfloat16 *dst = base + tile_off(row + ri, j0, R, sd.bka);
        *reinterpret_cast<uint4 *>(dst) = k0;
        if (sd.pieces > 1) *reinterpret_cast<uint4 *>(dst + pstride) = k1;
        if (sd.pieces > 2) *reinterpret_cast<uint4 *>(dst + 2 * pstride) = k2;
      }
    }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (!setup_done) {
    split_setup(&tslot, ncols, full, empty, &done, ns);
    setup_done = true;
  } else {
    __syncthreads();
  }
  const uint32_t tmem = tslot;
  const int ra16 = s ? ra1 : ra0;
  TwoGemm G;
  if (DIRECT) {
    G.a[0] = sd.aA_H + ((static_cast<long>(m) * 2 + s) * sd.ntiles + tile) * sd.rAH * sd.nha;
    G.a[1] = sd.aA_P + ((static_cast<long>(m) * 2 + s) * sd.ntiles + tile) * sd.rAP * sd.nha;
    G.a_ps[0] = sd.aAH_size;
    G.a_ps[1] = sd.aAP_size;
    G.a_res[0] = G.a_res[1] = 0;
  } else {
    G.a[0] = G.a[1] = nullptr;
    G.a_ps[0] = G.a_ps[1] = 0;
    G.a_res[0] = su32(aH);
    G.a_res[1] = su32(aP);
  }
  G.b[0] = sd.tA_H + sd.tA_off[2 * m + s];
  G.b[1] = sd.tA_P + sd.tA_off[2 * m + s];
  G.b_ps[0] = G.b_ps[1] = sd.tA_size;
  G.aR[0] = sd.rAH;
  G.aR[1] = sd.rAP;
  G.aRmax = sd.rAP;
  G.bR = ra16;
  G.b_cs = static_cast<long>(ra16) * sd.bka;
  G.bk = sd.bka;
  G.nchunk[0] = G.nchunk[1] = nchunk;
  G.kseg[0] = G.kseg[1] = 1 << 30;
  G.acc[0][0] = G.acc[0][1] = tmem + (s ? cb1 : 0);
  G.acc[1][0] = G.acc[1][1] = tmem + (s ? cb1 : 0) + ra16;
  ok = run_two_gemm(G, sd.pieces, sd.terms, ns, pipe, full, empty, &done, sd.err, pipe_it, static_cast<uint32_t>(calls & 1));
  pipe_it += 2 * nchunk;
  calls++;
  }
  const uint32_t tmem = tslot;
  // accumulators -> shared memory [row][ld + 1] (the operand and pipeline buffers are free now); the odd row
  // stride puts the rows that one warp writes at once on different banks
  const int ldp = ld + 1;
  float *dsm = reinterpret_cast<float *>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, row = warp * 32 + lane;
  if (ok && warp * 32 < 8 * mt) {
    const uint32_t lanebase = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    int c = 0;
    for (; c + 32 <= ld; c += 32) {
      float v[32];
      tmem_ld32(lanebase + c, v);
      if (row < 8 * mt) {
#pragma unroll
        for (int i = 0; i < 32; i++) dsm[row * ldp + c + i] = v[i];
      }
    }
    for (; c < ld; c += 8) {
      float v[8];
      tmem_ld8(lanebase + c, v);
      if (row < 8 * mt) {
#pragma unroll
        for (int i = 0; i < 8; i++) dsm[row * ldp + c + i] = v[i];
      }
    }
  }
  __syncthreads();
  if (ok) {
    const int cnt = BOTH ? d.N - m + 1 : (s_first ? R1 : R0);
    for (int e = threadIdx.x; e < mt * cnt; e += blockDim.x) {
      const int ml = e / cnt, j = e - ml * cnt;
      const int s = BOTH ? (j & 1) : s_first, r = BOTH ? (j >> 1) : j;
      ana_coef(d, sd, t, sa, x0, xf, xin, xout, acc, dsm, ldp, m, tile, ml, s, r, cb1, ra0, ra1);
    }
  }
  }
  if (setup_done) split_teardown(tslot, ncols);
}

// ------------------------------------------------------------------------------------------- analysis, warp-specialised
// The same work as split_ana (direct operands), by persistent CTAs whose warps take roles, so that one item's
// epilogue runs while the next item's operands load and multiply: thread 0 streams the H and P chunks of the CTA's
// items (m, parity or both, member tile) through a ring of ns fixed-size stages; thread 32 issues the MMAs of item i
// into tensor-memory accumulator buffer i % 2 and commits it to accf[i % 2]; warps 2..9 (256 threads) wait for it,
// copy it to shared memory, release the buffer (acce[i % 2]) and run the epilogue (ana_coef, the same arithmetic as
// split_ana). Items are dealt by snake_item. Every wait is bounded; after a failure each role stops,
// the CTA drains its own copies and MMAs and frees its tensor memory.
template <bool BOTH, int CTAS>
__global__ void __launch_bounds__(SPLIT_WS_THREADS, CTAS) split_ana_ws(SphDev d, SplitDev sd, SphTab<float> t, StageArgs sa, int B, int ns,
                                                                       int buf_cols, int slot_bytes, double2 *__restrict__ x0, float2 *__restrict__ xf,
                                                                       const float2 *__restrict__ xin, float2 *__restrict__ xout,
                                                                       float2 *__restrict__ acc) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full[SPLIT_MAX_STAGES], empty[SPLIT_MAX_STAGES], accf[2], acce[2], done;
  __shared__ uint32_t tslot;
  __shared__ int s_fail, s_issued, s_consumed, s_epi_ok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int per_m = (BOTH ? 1 : 2) * sd.ntiles;
  const int nitems = d.M * per_m;
  const int nchunk = sd.nha / sd.bka;
  const int bk = sd.bka;
  const uint32_t ncols = 2u * static_cast<uint32_t>(buf_cols);
  uint8_t *pipe = smem;
  float *dsm = reinterpret_cast<float *>(smem + static_cast<size_t>(ns) * slot_bytes);
  const int a_bytes = sd.rAP * bk * 2;  // A piece region of a stage (the H operand's 6 rows per member fit in it)
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tslot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int st = 0; st < ns; st++) {
      tc::bar_init(su32(&full[st]), 1);
      tc::bar_init(su32(&empty[st]), 1);
    }
    for (int b2 = 0; b2 < 2; b2++) {
      tc::bar_init(su32(&accf[b2]), 1);
      tc::bar_init(su32(&acce[b2]), 1);
    }
    tc::bar_init(su32(&done), 1);
    tc::bar_init_fence();
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;
  // the item sequence every role walks (snake_item): (m, parity or both, tile), m the slowest index
  auto item_of = [&](int item, int &m, int &s_first, int &s_last, int &tile, int &R0, int &R1) {
    m = item / per_m;
    const int rest = item - m * per_m;
    s_first = BOTH ? 0 : rest % 2;
    tile = BOTH ? rest : rest / 2;
    R0 = (d.N - m) / 2 + 1;
    R1 = (d.N - m + 1) / 2;
    s_last = BOTH ? (R1 > 0 ? 1 : 0) : s_first;
  };
  if (tid == 0) {
    // producer
    int git = 0;
    bool ok = true;
    for (int k = 0, item = snake_item(0); item < nitems && ok; item = snake_item(++k)) {
      int m, s_first, s_last, tile, R0, R1;
      item_of(item, m, s_first, s_last, tile, R0, R1);
      if ((s_first ? R1 : R0) == 0) continue;
      for (int s = s_first; s <= s_last && ok; s++) {
        const int ra = sd.ra16[2 * m + s];
        const uint32_t bbytes = static_cast<uint32_t>(ra * bk * 2);
        for (int g = 0; g < 2 && ok; g++) {
          const int aR = g == 0 ? sd.rAH : sd.rAP;
          const uint32_t abytes = static_cast<uint32_t>(aR * bk * 2);
          const __nv_bfloat16 *A = (g == 0 ? sd.aA_H : sd.aA_P) + ((static_cast<long>(m) * 2 + s) * sd.ntiles + tile) * aR * sd.nha;
          const long aps = g == 0 ? sd.aAH_size : sd.aAP_size;
          const __nv_bfloat16 *Bt = (g == 0 ? sd.tA_H : sd.tA_P) + sd.tA_off[2 * m + s];
          for (int c = 0; c < nchunk; c++, git++) {
            const int st = git % ns;
            if (git >= ns && !mbar_wait_bounded(su32(&empty[st]), ((git / ns) - 1) & 1)) {
              s_fail = 1;
              atomicExch(sd.err, 2);
              ok = false;
              break;
            }
            mbar_expect(su32(&full[st]), static_cast<uint32_t>(sd.pieces) * (abytes + bbytes));
            uint8_t *base = pipe + static_cast<size_t>(st) * slot_bytes;
            for (int p = 0; p < sd.pieces; p++) {
              bulk_g2s(su32(base + p * a_bytes), A + p * aps + static_cast<long>(c) * aR * bk, abytes, su32(&full[st]));
              bulk_g2s(su32(base + sd.pieces * a_bytes + p * static_cast<int>(bbytes)), Bt + p * sd.tA_size + static_cast<long>(c) * ra * bk, bbytes,
                       su32(&full[st]));
            }
            s_issued = git + 1;
          }
        }
      }
    }
  } else if (tid == 32) {
    // MMA issuer
    const int tp[6][2] = {{2, 0}, {1, 1}, {0, 2}, {1, 0}, {0, 1}, {0, 0}};
    const int t0 = sd.terms == 6 ? 0 : (sd.terms == 3 ? 3 : 5);
    const uint32_t sbo = static_cast<uint32_t>(bk) * 16u;
    int git = 0, it = 0;
    bool ok = true;
    for (int k = 0, item = snake_item(0); item < nitems && ok; item = snake_item(++k)) {
      int m, s_first, s_last, tile, R0, R1;
      item_of(item, m, s_first, s_last, tile, R0, R1);
      if ((s_first ? R1 : R0) == 0) continue;
      const int bb = it & 1;
      // the epilogue has copied out what this buffer held two items ago
      if (it >= 2 && !mbar_wait_bounded(su32(&acce[bb]), ((it >> 1) - 1) & 1)) {
        s_fail = 1;
        atomicExch(sd.err, 5);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int ra0 = sd.ra16[2 * m];
      const int cb1 = BOTH ? 2 * ra0 : 0;
      for (int s = s_first; s <= s_last && ok; s++) {
        const int ra = sd.ra16[2 * m + s];
        const uint32_t idesc = idesc_m128(ra);
        const int bbytes = ra * bk * 2;
        for (int g = 0; g < 2 && ok; g++) {
          const uint32_t accc = tmem + static_cast<uint32_t>(bb * buf_cols + (s ? cb1 : 0) + (g ? ra : 0));
          for (int c = 0; c < nchunk; c++, git++) {
            const int st = git % ns;
            if (!mbar_wait_bounded(su32(&full[st]), (git / ns) & 1)) {
              s_fail = 1;
              atomicExch(sd.err, 3);
              ok = false;
              break;
            }
            s_consumed = git + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            uint8_t *base = pipe + static_cast<size_t>(st) * slot_bytes;
            for (int kk = 0; kk < bk; kk += 16) {
              for (int tt = t0; tt < 6; tt++) {
                const int pa = tp[tt][0], pb = tp[tt][1];
                const uint64_t ad = chunk_desc(su32(base + pa * a_bytes + (kk / 8) * 128), sbo);
                const uint64_t bd = chunk_desc(su32(base + sd.pieces * a_bytes + pb * bbytes + (kk / 8) * 128), sbo);
                const uint32_t accum = (c > 0 || kk > 0 || tt > t0) ? 1u : 0u;
                asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(accc),
                             "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
                             : "memory");
              }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(&empty[st])) : "memory");
          }
        }
      }
      if (!ok) break;
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(&accf[bb])) : "memory");
      it++;
    }
    // completes `done` when every MMA issued has finished (the drain after a failure waits on it)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(&done)) : "memory");
  } else if (warp >= 2) {
    // epilogue warps
    const int et = tid - 64;
    int it = 0;
    for (int k = 0, item = snake_item(0); item < nitems; item = snake_item(++k)) {
      int m, s_first, s_last, tile, R0, R1;
      item_of(item, m, s_first, s_last, tile, R0, R1);
      if ((s_first ? R1 : R0) == 0) continue;
      const int bb = it & 1;
      if (et == 0) s_epi_ok = mbar_wait_bounded(su32(&accf[bb]), (it >> 1) & 1) ? 1 : 0;
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (!s_epi_ok) {
        if (et == 0) {
          s_fail = 1;
          atomicExch(sd.err, 6);
        }
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int mt = min(sd.nbt, B - tile * sd.nbt);
      const int ra0 = sd.ra16[2 * m], ra1 = sd.ra16[2 * m + 1];
      const int cb1 = BOTH ? 2 * ra0 : 0;
      const int ld = BOTH ? 2 * (ra0 + (s_last ? ra1 : 0)) : 2 * (s_first ? ra1 : ra0);
      const int ldp = ld + 1;
      // accumulators -> shared memory: warp w reads tensor-memory lanes 32 (w % 4) .. + 31; warps 2..5 take the even
      // 32-column blocks, warps 6..9 the odd ones
      const int quarter = warp & 3, row = quarter * 32 + lane;
      const uint32_t lanebase = tmem + static_cast<uint32_t>(bb * buf_cols) + (static_cast<uint32_t>(quarter * 32) << 16);
      if (quarter * 32 < 8 * mt) {
        for (int c = (warp < 6 ? 0 : 32); c < ld; c += 64) {
          float v[32];
          tmem_ld32(lanebase + c, v);
          if (row < 8 * mt) {
#pragma unroll
            for (int i = 0; i < 32; i++) dsm[row * ldp + c + i] = v[i];
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (et == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&acce[bb])) : "memory");
      const int cnt = BOTH ? d.N - m + 1 : (s_first ? R1 : R0);
      for (int e = et; e < mt * cnt; e += SPLIT_WS_EPI) {
        const int ml = e / cnt, j = e - ml * cnt;
        const int s = BOTH ? (j & 1) : s_first, r = BOTH ? (j >> 1) : j;
        ana_coef(d, sd, t, sa, x0, xf, xin, xout, acc, dsm, ldp, m, tile, ml, s, r, cb1, ra0, ra1);
      }
      // the shared accumulator copy is free for the next item
      asm volatile("bar.sync 1, 256;" ::: "memory");
      it++;
    }
  }
  __syncthreads();
  if (tid == 0) {
    // every MMA issued has finished (and its arrivals landed) before the CTA releases its memory; after a failure the
    // waits are short and also cover the copies no MMA consumed
    if (!s_fail) {
      if (!mbar_wait_bounded(su32(&done), 0)) atomicExch(sd.err, 4);
    } else {
      tc::wait_for(su32(&done), 0, 200000000ull);
      for (int g2 = s_consumed; g2 < s_issued; g2++) tc::wait_for(su32(&full[g2 % ns]), (g2 / ns) & 1, 200000000ull);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

}  // namespace

// Pack the tables, size the operand buffers (once per engine).
inline void build_split_plan(SplitPlan &sp, const HostTables &h, int B, int terms) {
  const int N = h.N, M = h.M, nh = h.nh;
  // the synthesis keeps four accumulators of its latitudes in the 512 tensor-memory columns: slices of at most 128
  if (pad16(nh) > 256) throw InvalidArgument("split precision supports truncations up to 341");
  sp.terms = terms;
  sp.pieces = terms == 6 ? 3 : 2;
  sp.nbt = std::min(B, SPLIT_NBT);
  sp.ntiles = (B + sp.nbt - 1) / sp.nbt;
  sp.nh16 = pad16(nh);
  sp.nh64 = pad64(nh);
  sp.bka = nh >= 32 ? 32 : pad16(nh);
  sp.bks = N <= 85 ? 32 : 64;
  sp.nha = (nh + sp.bka - 1) / sp.bka * sp.bka;
  sp.syn_split = 4 * sp.nh16 > 512 ? 2 : 1;
  sp.syn_nh = sp.nh16 / sp.syn_split;
  sp.rSP = 8 * sp.nbt;
  sp.rSH = pad8(4 * sp.nbt);
  sp.rAP = 8 * sp.nbt;
  sp.rAH = pad8(6 * sp.nbt);
  sp.ke16.assign(M, 0);
  sp.kps.assign(M, 0);
  sp.ra16.assign(2 * M, 0);
  sp.tS_off.assign(M, 0);
  sp.tA_off.assign(2 * M, 0);
  sp.aS_off.assign(M, 0);
  sp.aSH_off.assign(M, 0);
  long ts = 0, ta = 0, as = 0, ash = 0;
  int ra_max = 16;
  for (int m = 0; m <= N; m++) {
    const int ke = (N - m) / 2 + 1, ko = (N - m + 1) / 2;
    sp.ke16[m] = pad16(ke);
    sp.kps[m] = (sp.ke16[m] + ko + sp.bks - 1) / sp.bks * sp.bks;
    sp.tS_off[m] = ts;
    ts += static_cast<long>(sp.nh16) * sp.kps[m];
    sp.aS_off[m] = as;
    as += static_cast<long>(sp.ntiles) * sp.rSP * sp.kps[m];
    sp.aSH_off[m] = ash;
    ash += static_cast<long>(sp.ntiles) * sp.rSH * sp.kps[m];
    for (int s = 0; s < 2; s++) {
      const int R = s == 0 ? ke : ko;
      sp.ra16[2 * m + s] = std::max(16, pad16(R));
      sp.tA_off[2 * m + s] = ta;
      ta += static_cast<long>(sp.ra16[2 * m + s]) * sp.nha;
      ra_max = std::max(ra_max, sp.ra16[2 * m + s]);
    }
  }
  sp.ra_max = ra_max;
  sp.tS_size = ts;
  sp.tA_size = ta;
  sp.aSP_size = as;
  sp.aSH_size = ash;
  sp.aAP_size = static_cast<long>(M) * 2 * sp.ntiles * sp.rAP * sp.nha;
  sp.aAH_size = static_cast<long>(M) * 2 * sp.ntiles * sp.rAH * sp.nha;
  // tables in the chunked core-matrix order, three pieces each
  std::vector<uint16_t> tSP(3 * ts, 0), tSH(3 * ts, 0), tAP(3 * ta, 0), tAH(3 * ta, 0);
  for (int m = 0; m <= N; m++) {
    const int ke16 = sp.ke16[m], kpm = sp.kps[m];
    for (int k = 0; k < kpm; k++) {
      const int n = k < ke16 ? m + 2 * k : m + 1 + 2 * (k - ke16);
      if (n > N || (k < ke16 && ((n - m) & 1))) continue;
      const size_t q = static_cast<size_t>(h.tri[m] + n - m);
      for (int jh = 0; jh < nh; jh++) {
        const long o = sp.tS_off[m] + tile_off(jh, k, sp.nh16, sp.bks);
        split3(h.P[q * nh + jh], &tSP[o], ts);
        split3(h.H[q * nh + jh], &tSH[o], ts);
      }
    }
    for (int s = 0; s < 2; s++) {
      const int R = s == 0 ? (N - m) / 2 + 1 : (N - m + 1) / 2;
      for (int r = 0; r < R; r++) {
        const int n = m + s + 2 * r;
        const size_t q = static_cast<size_t>(h.tri[m] + n - m);
        for (int jh = 0; jh < nh; jh++) {
          const long o = sp.tA_off[2 * m + s] + tile_off(r, jh, sp.ra16[2 * m + s], sp.bka);
          split3(h.P[q * nh + jh], &tAP[o], ta);
          split3(h.H[q * nh + jh], &tAH[o], ta);
        }
      }
    }
  }
  auto up = [](DevBuf<__nv_bfloat16> &dst, const std::vector<uint16_t> &src) {
    dst.alloc(src.size());
    LMW_CUDA(cudaMemcpy(dst.p, src.data(), src.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
  };
  up(sp.tS_P, tSP);
  up(sp.tS_H, tSH);
  up(sp.tA_P, tAP);
  up(sp.tA_H, tAH);
  // per-stage operands: padding rows and columns are never written and stay zero
  sp.aS_P.alloc(3 * sp.aSP_size);
  sp.aS_H.alloc(3 * sp.aSH_size);
  sp.aA_P.alloc(3 * sp.aAP_size);
  sp.aA_H.alloc(3 * sp.aAH_size);
  for (auto *b : {&sp.aS_P, &sp.aS_H, &sp.aA_P, &sp.aA_H}) LMW_CUDA(cudaMemset(b->p, 0, b->bytes()));
  sp.dsyn.alloc(static_cast<size_t>(B) * nh * M * SPLIT_NQ);
  LMW_CUDA(cudaMemset(sp.dsyn.p, 0, sp.dsyn.bytes()));
  sp.err.alloc(1);
  LMW_CUDA(cudaMemset(sp.err.p, 0, sizeof(int)));
  auto upi = [](DevBuf<int> &dst, const std::vector<int> &src) {
    dst.alloc(src.size());
    LMW_CUDA(cudaMemcpy(dst.p, src.data(), src.size() * sizeof(int), cudaMemcpyHostToDevice));
  };
  auto upl = [](DevBuf<long> &dst, const std::vector<long> &src) {
    dst.alloc(src.size());
    LMW_CUDA(cudaMemcpy(dst.p, src.data(), src.size() * sizeof(long), cudaMemcpyHostToDevice));
  };
  upi(sp.ke16_d, sp.ke16);
  upi(sp.kps_d, sp.kps);
  upi(sp.ra16_d, sp.ra16);
  upl(sp.tS_off_d, sp.tS_off);
  upl(sp.tA_off_d, sp.tA_off);
  upl(sp.aS_off_d, sp.aS_off);
  upl(sp.aSH_off_d, sp.aSH_off);
  const int pieces = sp.pieces;
  const size_t budget = 220 * 1024;
  const size_t syn_stage = static_cast<size_t>(pieces) * (sp.rSP + sp.syn_nh) * sp.bks * 2;
  // the pipeline never needs more stages than a CTA has chunks (two GEMMs of kps / bks chunks); two CTAs per SM
  // when two stages fit in half of the shared memory
  int max_chunks = 0;
  for (int m = 0; m <= N; m++) max_chunks = std::max(max_chunks, 2 * static_cast<int>(sp.kps[m] / sp.bks));
  const size_t half_budget = SPLIT_HALF_SM;
  if (2 * syn_stage + SPLIT_MARGIN <= half_budget) sp.ns_syn = static_cast<int>(std::min<size_t>(std::min(SPLIT_MAX_STAGES, max_chunks), (half_budget - SPLIT_MARGIN) / syn_stage));
  else sp.ns_syn = static_cast<int>(std::min<size_t>(std::min(SPLIT_MAX_STAGES, max_chunks), (budget - SPLIT_MARGIN) / syn_stage));
  sp.ns_syn = std::max(sp.ns_syn, 2);
  if (sp.ns_syn * syn_stage + SPLIT_MARGIN > budget) throw InvalidArgument("split precision: the synthesis pipeline does not fit in shared memory");
  sp.smem_syn = std::max(sp.ns_syn * syn_stage + SPLIT_MARGIN, static_cast<size_t>(4 * 8 * sp.nbt * 33 * sizeof(float)));
  // latitude pairs per grid CTA: four when that still gives two CTAs per SM
  sp.jb = 1;
  for (int jb = SPLIT_JB_MAX; jb > 1; jb /= 2)
    if (nh % jb == 0 && static_cast<long>(nh / jb) * B >= 2 * 152) {
      sp.jb = jb;
      break;
    }
  // the analysis either gathers its A operands into resident shared memory (variant 0) or streams them with
  // its tables (variant 1, the default for batches)
  const size_t nchunk = sp.nha / sp.bka;
  sp.ana_res_bytes_v[0] = static_cast<size_t>(pieces) * nchunk * (sp.rAH + sp.rAP) * sp.bka * 2;
  sp.ana_stage_bytes_v[0] = static_cast<size_t>(pieces) * ra_max * sp.bka * 2;
  sp.ana_res_bytes_v[1] = 0;
  sp.ana_stage_bytes_v[1] = static_cast<size_t>(pieces) * (sp.rAP + ra_max) * sp.bka * 2;
  sp.direct = sp.nbt >= 8 ? 1 : 0;
  const size_t ana_res = sp.ana_res_bytes_v[sp.direct], ana_stage = sp.ana_stage_bytes_v[sp.direct];
  // two analysis CTAs per SM when a 3-stage pipeline fits in half of the shared memory
  const size_t half = SPLIT_HALF_SM;
  if (ana_res + 3 * ana_stage + SPLIT_MARGIN <= half && static_cast<size_t>(sp.rAP) * (2 * ra_max + 1) * sizeof(float) <= half)
    sp.ns_ana = 3;
  else
    sp.ns_ana = static_cast<int>(std::min<size_t>(SPLIT_MAX_STAGES, (budget - SPLIT_MARGIN - ana_res) / ana_stage));
  if (sp.ns_ana < 2) throw InvalidArgument("split precision: the analysis pipeline does not fit in shared memory");
  sp.smem_ana = std::max(ana_res + sp.ns_ana * ana_stage + SPLIT_MARGIN, static_cast<size_t>(sp.rAP) * (2 * ra_max + 1) * sizeof(float));
  sp.syn_stage_bytes = syn_stage;
  sp.syn_min_bytes = static_cast<size_t>(4 * 8 * sp.nbt * 33 * sizeof(float));
  sp.ana_min_bytes = static_cast<size_t>(sp.rAP) * (2 * ra_max + 1) * sizeof(float);
  for (int m = 0; m <= N; m++) sp.ra_pair = std::max(sp.ra_pair, sp.ra16[2 * m] + sp.ra16[2 * m + 1]);
  sp.ana_both_min_bytes = static_cast<size_t>(sp.rAP) * (2 * sp.ra_pair + 1) * sizeof(float);
  sp.budget_bytes = budget;
  // coefficients of the spectral Coriolis terms (eps of cpp/sphere.cpp:11): for q = (m, n), eps_{n+1} n/(n+1)
  // (n < T), eps_n (n+1)/n (n > m) and m/(n(n+1)) (n >= 1)
  std::vector<double> lin(3 * static_cast<size_t>(h.ntri), 0.0);
  auto eps = [](int n, int m) { return std::sqrt(static_cast<double>(n * n - m * m) / static_cast<double>(4 * n * n - 1)); };
  for (int m = 0; m <= N; m++)
    for (int n = std::max(m, 1); n <= N; n++) {
      const size_t q = static_cast<size_t>(h.tri[m] + n - m);
      lin[q] = n < N ? eps(n + 1, m) * n / (n + 1.0) : 0.0;
      lin[h.ntri + q] = n > m ? eps(n, m) * (n + 1.0) / n : 0.0;
      lin[2 * h.ntri + q] = static_cast<double>(m) / (static_cast<double>(n) * (n + 1));
    }
  std::vector<float> lin32(lin.begin(), lin.end());
  sp.lin32.alloc(lin32.size());
  LMW_CUDA(cudaMemcpy(sp.lin32.p, lin32.data(), lin32.size() * sizeof(float), cudaMemcpyHostToDevice));
}

// bytes past the end of a warp-specialised kernel's layout (ns stage slots of `slot` bytes, then `tail` bytes of
// staging) that an M = 128 MMA reads: it reads 128 rows (16 row groups of bk x 16 bytes) from the A base of the last
// piece of the last slot, whatever the operand's row count
inline size_t ws_margin(int ns, size_t slot, size_t last_piece_offset, int bk, size_t tail) {
  const size_t end = static_cast<size_t>(ns - 1) * slot + last_piece_offset + static_cast<size_t>(128) * bk * 2;
  const size_t have = static_cast<size_t>(ns) * slot + tail;
  return end > have ? ((end - have + 15) & ~static_cast<size_t>(15)) : 0;
}

// shared-memory layout of the warp-specialised analysis for one parity (both = 0) or both per item and ns stages:
// stage slots of a fixed size, then the accumulator copy, then what an M = 128 MMA may read past the end (ws_margin).
// Returns false when the form does not fit (tensor memory: two accumulator buffers per CTA, `ctas` CTAs per SM).
inline bool ws_layout(const SplitPlan &sp, int both, int ns, int ctas, size_t *smem, int *buf_cols, int *slot) {
  const int ldmax = both ? 2 * sp.ra_pair : 2 * sp.ra_max;
  int bc = 32;
  while (bc < ldmax) bc <<= 1;
  const size_t sl = static_cast<size_t>(sp.pieces) * (sp.rAP + sp.ra_max) * sp.bka * 2;
  const size_t dsm = (static_cast<size_t>(sp.rAP) * (ldmax + 1) * sizeof(float) + 15) & ~static_cast<size_t>(15);
  const size_t total = ns * sl + dsm + ws_margin(ns, sl, static_cast<size_t>(sp.pieces - 1) * sp.rAP * sp.bka * 2, sp.bka, dsm);
  *smem = total;
  *buf_cols = bc;
  *slot = static_cast<int>(sl);
  if (2 * bc * ctas > 512) return false;
  if (total > sp.budget_bytes) return false;
  if (ctas == 2 && 2 * (total + 1024 + 2048) > 233472) return false;
  return ctas == 1 || ctas == 2;
}

// shared-memory layout of the warp-specialised synthesis with `sl` latitude slices and ns stages: stage slots,
// then the staging of one accumulator buffer (H E/O with rSH rows, P E/O with rSP rows, stride nh + 1), then what an
// M = 128 MMA may read past the end (ws_margin). Returns false when it does not fit (tensor memory: two buffers of
// four nh-column accumulators per CTA, `ctas` CTAs per SM).
inline bool syn_ws_layout(const SplitPlan &sp, int sl, int ns, int ctas, size_t *smem, int *buf_cols, int *slot) {
  if (sl < 1 || sp.nh16 % sl != 0) return false;
  const int nh = sp.nh16 / sl;
  if (nh < 16 || nh % 16 != 0 || nh > 256) return false;
  int bc = 32;
  while (bc < 4 * nh) bc <<= 1;
  const size_t st = static_cast<size_t>(sp.pieces) * (sp.rSP + nh) * sp.bks * 2;
  const size_t stg = (static_cast<size_t>(2 * sp.rSH + 2 * sp.rSP) * (nh + 1) * sizeof(float) + 15) & ~static_cast<size_t>(15);
  const size_t total = ns * st + stg + ws_margin(ns, st, static_cast<size_t>(sp.pieces - 1) * sp.rSP * sp.bks * 2, sp.bks, stg);
  *smem = total;
  *buf_cols = bc;
  *slot = static_cast<int>(st);
  if (2 * bc * ctas > 512) return false;
  if (total > sp.budget_bytes) return false;
  if (ctas == 2 && 2 * (total + 1024 + 2048) > 233472) return false;
  return ctas == 1 || ctas == 2;
}

inline SplitDev split_dev(const SplitPlan &sp) {
  SplitDev s;
  s.pieces = sp.pieces;
  s.terms = sp.terms;
  s.nbt = sp.nbt;
  s.ntiles = sp.ntiles;
  s.nh16 = sp.nh16;
  s.nh64 = sp.nh64;
  s.bka = sp.bka;
  s.bks = sp.bks;
  s.nha = sp.nha;
  s.rAP = sp.rAP;
  s.rAH = sp.rAH;
  s.rSP = sp.rSP;
  s.rSH = sp.rSH;
  s.jb = sp.jb;
  s.syn_nh = sp.syn_nh;
  s.fgrp = sp.fgrp;
  s.ana_cols_one = 2 * sp.ra_max;
  s.ana_cols_both = 2 * sp.ra_pair;
  s.ke16 = sp.ke16_d.p;
  s.kps = sp.kps_d.p;
  s.ra16 = sp.ra16_d.p;
  s.tS_off = sp.tS_off_d.p;
  s.tA_off = sp.tA_off_d.p;
  s.aS_off = sp.aS_off_d.p;
  s.aSH_off = sp.aSH_off_d.p;
  s.tS_size = sp.tS_size;
  s.tA_size = sp.tA_size;
  s.aSP_size = sp.aSP_size;
  s.aSH_size = sp.aSH_size;
  s.aAP_size = sp.aAP_size;
  s.aAH_size = sp.aAH_size;
  s.tS_P = sp.tS_P.p;
  s.tS_H = sp.tS_H.p;
  s.tA_P = sp.tA_P.p;
  s.tA_H = sp.tA_H.p;
  s.aS_P = sp.aS_P.p;
  s.aS_H = sp.aS_H.p;
  s.aA_P = sp.aA_P.p;
  s.aA_H = sp.aA_H.p;
  s.dsyn = sp.dsyn.p;
  s.fold = nullptr;
  s.err = sp.err.p;
  s.lin_exact = sp.lin_exact;
  s.lin32 = sp.lin32.p;
  return s;
}

}  // namespace lmw
