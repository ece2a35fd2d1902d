// Batched split-BF16 GEMM on tcgen05 (sm_103a): operands staged in shared memory in the canonical K-major
// core-matrix layout (8 rows x 16 bytes per core matrix), accumulators in tensor memory, one elected thread
// issuing tcgen05.mma, completion tracked by an mbarrier through tcgen05.commit, and the epilogue reading the
// accumulators back with tcgen05.ld. Every wait on the tensor cores is bounded in time: when it runs out the CTA
// records an error code, waits (bounded) once more for its own MMAs, releases its tensor memory and returns.
#include <algorithm>
#include <cstdint>

#include "tc_common.cuh"
#include "tc_gemm.h"

namespace lmw {
namespace {

constexpr int BK = 64;             // K elements per shared-memory stage
constexpr int GEMM_THREADS = 128;  // 4 warps: the 128 accumulator rows (TMEM lanes) of an M = 128 MMA
constexpr int A_TILE = 128 * BK * 2;
constexpr int B_TILE_MAX = 256 * BK * 2;
// three A pieces, three B pieces, plus slack so that no descriptor can address past the allocation
constexpr int SMEM_BYTES = 3 * A_TILE + 3 * B_TILE_MAX + 16384;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return tc::su32(p); }

// shared-memory matrix descriptor: start address, leading (K-direction) and stride (8-row group) byte offsets,
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  return d;
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(M >> 4) << 24);
}

__global__ void __launch_bounds__(GEMM_THREADS, 1)
    tc_gemm_kernel(const GemmProblem *__restrict__ probs, int terms, int *err, int variant) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int status;
  const GemmProblem P = probs[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n = P.n;
  const int pieces = terms == 6 ? 3 : (terms == 3 ? 2 : 1);
  uint32_t ncols = 32;
  while (ncols < static_cast<uint32_t>(P.nseg * n)) ncols <<= 1;
  uint8_t *sA = smem, *sB = smem + 3 * A_TILE;
  const int b_tile = n * BK * 2;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    status = 0;
  }
  // rows of A past arows stay zero for the whole K loop
  for (int e = tid; e < 3 * A_TILE / 16; e += GEMM_THREADS) reinterpret_cast<uint4 *>(sA)[e] = make_uint4(0, 0, 0, 0);
  const int arows = P.arows;
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = idesc_bf16(128, n);
  // K-direction stride between core matrices and stride between 8-row groups, per operand
  const uint32_t a_kstride = 16 * 128, a_mstride = 128;
  const uint32_t b_kstride = static_cast<uint32_t>(n / 8) * 128, b_mstride = 128;
  const uint32_t a_lbo = variant ? a_mstride : a_kstride, a_sbo = variant ? a_kstride : a_mstride;
  const uint32_t b_lbo = variant ? b_mstride : b_kstride, b_sbo = variant ? b_kstride : b_mstride;
  // (A piece, B piece) per term, smallest products first
  const int tp[6][2] = {{2, 0}, {1, 1}, {0, 2}, {1, 0}, {0, 1}, {0, 0}};
  const int t0 = terms == 6 ? 0 : (terms == 3 ? 3 : 5);
  bool started[3] = {false, false, false};
  uint32_t phase = 0;
  const int ktot = P.kseg[P.nseg];
  for (int k0 = 0; k0 < ktot; k0 += BK) {
    const int kc = min(BK, ktot - k0);
    const int kq_n = kc / 8;  // 16-byte chunks per row in this stage
    for (int pc = 0; pc < pieces; pc++) {
      const __nv_bfloat16 *srcA = P.a + pc * P.a_ps, *srcB = P.b + pc * P.b_ps;
      uint8_t *dA = sA + pc * A_TILE, *dB = sB + pc * b_tile;
      for (int e = tid; e < arows * kq_n; e += GEMM_THREADS) {
        const int row = e / kq_n, kq = e - row * kq_n;
        const uint4 v = *reinterpret_cast<const uint4 *>(srcA + static_cast<size_t>(row) * P.lda + k0 + kq * 8);
        *reinterpret_cast<uint4 *>(dA + (kq * 16 + (row >> 3)) * 128 + (row & 7) * 16) = v;
      }
      for (int e = tid; e < n * kq_n; e += GEMM_THREADS) {
        const int row = e / kq_n, kq = e - row * kq_n;
        const uint4 v = *reinterpret_cast<const uint4 *>(srcB + static_cast<size_t>(row) * P.ldb + k0 + kq * 8);
        *reinterpret_cast<uint4 *>(dB + (kq * (n / 8) + (row >> 3)) * 128 + (row & 7) * 16) = v;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int kk = 0; kk < kc; kk += 16) {
        const int kg = k0 + kk;
        int s = 0;
        while (s + 1 < P.nseg && kg >= P.kseg[s + 1]) s++;
        const uint32_t dcol = tmem + static_cast<uint32_t>(s * n);
        for (int t = t0; t < 6; t++) {
          const uint64_t ad = sdesc(smem_u32(sA + tp[t][0] * A_TILE + (kk / 8) * a_kstride), a_lbo, a_sbo);
          const uint64_t bd = sdesc(smem_u32(sB + tp[t][1] * b_tile + (kk / 8) * b_kstride), b_lbo, b_sbo);
          const uint32_t accum = started[s] ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dcol),
              "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
              : "memory");
          started[s] = true;
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&bar)) : "memory");
      if (!tc::wait(smem_u32(&bar), phase)) {
        status = 1;
        atomicExch(err, 1);
        tc::wait(smem_u32(&bar), phase);  // give the MMAs in flight one more bounded chance
      }
    }
    phase ^= 1;
    __syncthreads();
    if (status) break;
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!status && warp * 32 < arows) {
    // epilogue: warp w owns accumulator rows 32w .. 32w+31 (TMEM lanes), 8 columns per load
    const int row = warp * 32 + lane;
    const int total = P.nseg * n;
    for (int c = 0; c < total; c += 8) {
      uint32_t r[8];
      const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c);
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                   : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                   : "r"(taddr)
                   : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const int s = c / n;
      const bool live = P.kseg[s + 1] > P.kseg[s];
      if (row < arows) {
        float *dst = P.d + static_cast<size_t>(row) * P.ldd + c;
#pragma unroll
        for (int i = 0; i < 8; i++) dst[i] = live ? __uint_as_float(r[i]) : 0.0f;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

__global__ void split_bf16_kernel(const float *__restrict__ in, __nv_bfloat16 *__restrict__ out, long n, long lo, int pieces) {
  for (long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; i < n; i += static_cast<long>(gridDim.x) * blockDim.x) {
    const float x = in[i];
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const float r = x - __bfloat162float(h);
    const __nv_bfloat16 l = __float2bfloat16_rn(r);
    out[i] = h;
    if (pieces > 1) out[i + lo] = l;
    if (pieces > 2) out[i + 2 * lo] = __float2bfloat16_rn(r - __bfloat162float(l));
  }
}

}  // namespace

void tc_gemm_launch(const GemmProblem *probs_dev, int nprob, int terms, int *err, cudaStream_t stream, int layout_variant) {
  static bool attr = false;
  if (!attr) {
    LMW_CUDA(cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    attr = true;
  }
  if (nprob <= 0) return;
  tc_gemm_kernel<<<nprob, GEMM_THREADS, SMEM_BYTES, stream>>>(probs_dev, terms, err, layout_variant);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
}

void split_bf16_launch(const float *in, __nv_bfloat16 *out, long n, long lo, int pieces, cudaStream_t stream) {
  if (n <= 0) return;
  int blocks = static_cast<int>(std::min<long>((n + 255) / 256, 4096));
  split_bf16_kernel<<<blocks, 256, 0, stream>>>(in, out, n, lo, pieces);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
}

// Self-test of the GEMM on one problem from host arrays: D (128 x N) = A (128 x K) * B (N x K)^T, FP32 in and
// out, the split and the MMAs on the device. Returns 0, or the kernel's error code.
int tc_gemm_selftest(const float *A, const float *B, float *D, int N, int K, int terms, int variant) {
  if (N % 16 || N < 16 || N > 256 || K % 16 || K <= 0) throw InvalidArgument("self-test needs 16 <= N <= 256 and K, N multiples of 16");
  if (terms != 1 && terms != 3 && terms != 6) throw InvalidArgument("terms must be 1, 3 or 6");
  // the alternative stride convention keeps every descriptor inside the shared-memory allocation only for N <= 64
  if (variant != 0 && N > 64) throw InvalidArgument("layout 1 is limited to N <= 64");
  const int pieces = terms == 6 ? 3 : (terms == 3 ? 2 : 1);
  const long na = 128L * K, nb = static_cast<long>(N) * K;
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  __nv_bfloat16 *sA = nullptr, *sB = nullptr;
  GemmProblem *dp = nullptr;
  int *derr = nullptr;
  cudaStream_t st = nullptr;
  auto cleanup = [&] {
    cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(sA); cudaFree(sB); cudaFree(dp); cudaFree(derr);
    if (st) cudaStreamDestroy(st);
  };
  try {
    LMW_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    LMW_CUDA(cudaMalloc(&dA, na * sizeof(float)));
    LMW_CUDA(cudaMalloc(&dB, nb * sizeof(float)));
    LMW_CUDA(cudaMalloc(&dD, 128L * N * sizeof(float)));
    LMW_CUDA(cudaMalloc(&sA, 3 * na * sizeof(__nv_bfloat16)));
    LMW_CUDA(cudaMalloc(&sB, 3 * nb * sizeof(__nv_bfloat16)));
    LMW_CUDA(cudaMalloc(&dp, sizeof(GemmProblem)));
    LMW_CUDA(cudaMalloc(&derr, sizeof(int)));
    alloc_counter().fetch_add(7, std::memory_order_relaxed);
    LMW_CUDA(cudaMemset(derr, 0, sizeof(int)));
    LMW_CUDA(cudaMemcpy(dA, A, na * sizeof(float), cudaMemcpyHostToDevice));
    LMW_CUDA(cudaMemcpy(dB, B, nb * sizeof(float), cudaMemcpyHostToDevice));
    split_bf16_launch(dA, sA, na, na, pieces, st);
    split_bf16_launch(dB, sB, nb, nb, pieces, st);
    GemmProblem p;
    p.a = sA;
    p.b = sB;
    p.d = dD;
    p.a_ps = na;
    p.b_ps = nb;
    p.lda = K;
    p.ldb = K;
    p.ldd = N;
    p.arows = 128;
    p.n = N;
    p.nseg = 1;
    p.kseg[0] = 0;
    p.kseg[1] = K;
    p.kseg[2] = p.kseg[3] = K;
    LMW_CUDA(cudaMemcpy(dp, &p, sizeof p, cudaMemcpyHostToDevice));
    tc_gemm_launch(dp, 1, terms, derr, st, variant);
    LMW_CUDA(cudaStreamSynchronize(st));
    int herr = 0;
    LMW_CUDA(cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost));
    LMW_CUDA(cudaMemcpy(D, dD, 128L * N * sizeof(float), cudaMemcpyDeviceToHost));
    cleanup();
    return herr;
  } catch (...) {
    cleanup();
    throw;
  }
}

}  // namespace lmw
