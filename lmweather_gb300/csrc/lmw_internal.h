// Internal declarations shared by the engine's translation units (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <utility>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

namespace lmw {

// The reference's two exception kinds (std::invalid_argument / std::runtime_error) plus device failures.
struct InvalidArgument : std::invalid_argument {
  using std::invalid_argument::invalid_argument;
};
struct RuntimeError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct DeviceError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

void cuda_check(cudaError_t e, const char *what, const char *file, int line);
#define LMW_CUDA(call) ::lmw::cuda_check((call), #call, __FILE__, __LINE__)
#define LMW_LAUNCH_CHECK() ::lmw::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)

// std::to_string(double) formatting ("%f"), which the reference uses in its run() messages
std::string fmt_f(double x);
// the text writers' number format ("%.10g") and file write, with the reference's error text
// ("<who>: cannot write <path>", a runtime_error) (cpp/main.cpp:84-92)
std::string fmt_g(double x);
void write_text(const std::string &path, const std::string &text, const char *who);
// runs fn with the C ABI's exception-to-status mapping and per-thread message (for entry points defined outside
// capi.cu)
int run_guarded(const std::function<void()> &fn);

// Counts this library's device and pinned-host allocations (cudaMalloc, cudaMallocHost), process-wide; a
// caller can check that an entry point which promises not to allocate leaves it unchanged.
inline std::atomic<uint64_t> &alloc_counter() {
  static std::atomic<uint64_t> n{0};
  return n;
}

// Device buffer owned by an engine object.
template <class T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count == 0) return;
    LMW_CUDA(cudaMalloc(reinterpret_cast<void **>(&p), count * sizeof(T)));
    alloc_counter().fetch_add(1, std::memory_order_relaxed);
    n = count;
  }
  void zero(cudaStream_t s) {
    if (p) LMW_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
  void swap(DevBuf &o) {
    std::swap(p, o.p);
    std::swap(n, o.n);
  }
};

// Pinned host staging buffer.
template <class T> struct HostBuf {
  T *p = nullptr;
  size_t n = 0;
  HostBuf() = default;
  HostBuf(const HostBuf &) = delete;
  HostBuf &operator=(const HostBuf &) = delete;
  ~HostBuf() {
    if (p) cudaFreeHost(p);
  }
  void alloc(size_t count) {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    if (count == 0) return;
    LMW_CUDA(cudaMallocHost(reinterpret_cast<void **>(&p), count * sizeof(T)));
    alloc_counter().fetch_add(1, std::memory_order_relaxed);
    n = count;
  }
};

// Counts this library's kernel launches (for the benchmark's launch accounting).
extern thread_local uint64_t g_launches;

int conversion_selftest_run(const uint32_t *f, int nf, const uint64_t *x, int nx, int *mismatches);
int wait_selftest_run(int timeout_us, int *completed, int *ran_out);
void division_selftest_run(const uint64_t *x, int nx, const double *y, int ny, long long *counts);

// Device-wide reduction results of one guard/diagnostic pass.
struct Reduce {
  double sum[8];
  double max[4];
};

}  // namespace lmw
