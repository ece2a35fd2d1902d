// FP64 FMA throughput probe: every SM runs independent dependent-chain DFMA streams long enough to hide
// latency; the result is the denominator of the FP64 paths' roofline.
#include "lmw_internal.h"

namespace lmw {
namespace {
constexpr int PEAK_THREADS = 256, CHAINS = 8, ITERS = 4096;

__global__ void __launch_bounds__(PEAK_THREADS) fp64_fma_probe(double *out, double a, double b) {
  double x[CHAINS];
  for (int c = 0; c < CHAINS; c++) x[c] = threadIdx.x * 1e-9 + c;
  for (int i = 0; i < ITERS; i++)
#pragma unroll
    for (int c = 0; c < CHAINS; c++) x[c] = fma(x[c], a, b);
  double s = 0;
  for (int c = 0; c < CHAINS; c++) s += x[c];
  if (s == 1.2345) out[0] = s;  // keeps the chains live; never true for these inputs
}
}  // namespace

double measure_fp64_peak() {
  int dev = 0, sms = 0;
  LMW_CUDA(cudaGetDevice(&dev));
  LMW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double *out = nullptr;
  LMW_CUDA(cudaMalloc(&out, sizeof(double)));
  cudaEvent_t e0, e1;
  LMW_CUDA(cudaEventCreate(&e0));
  LMW_CUDA(cudaEventCreate(&e1));
  const int blocks = sms * 8;
  fp64_fma_probe<<<blocks, PEAK_THREADS>>>(out, 0.999999, 1e-7);
  LMW_CUDA(cudaEventRecord(e0));
  const int reps = 5;
  for (int r = 0; r < reps; r++) fp64_fma_probe<<<blocks, PEAK_THREADS>>>(out, 0.999999, 1e-7);
  LMW_CUDA(cudaEventRecord(e1));
  LMW_LAUNCH_CHECK();
  LMW_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  LMW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  g_launches += reps + 1;
  const double flops = 2.0 * CHAINS * ITERS * static_cast<double>(PEAK_THREADS) * blocks * reps;
  return flops / (ms * 1e-3) / 1e12;
}
}  // namespace lmw
