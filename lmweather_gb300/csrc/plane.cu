// Beta-plane C-grid shallow water on the GPU (FP64), the lmweather Plane model (cpp/plane.cpp).
//
// One fused kernel per RK4 stage: a CTA loads a (TY+2) x (TX+2) tile of h, u, v (periodic in x, rows
// clamped at the walls) into shared memory, forms the Bernoulli function B and the absolute vorticity eta
// for the tile plus its one-cell halo, evaluates du, dv, dh, and applies the RK4 stage update in the same
// pass (stage input, accumulator and, at the last stage, the state). Every arithmetic expression follows
// the reference's order of evaluation and this file is compiled with --fmad=false, so that the result is
// bitwise identical to cpp/plane.cpp:59-158 built without FMA contraction.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "fixed_div.cuh"

namespace lmw {
namespace {

constexpr int TX = 32, TY = 8;

struct PlaneDev {
  int nx, ny, lin;
  double dxx, dyy, dxx2, dyy2, g, depth, f0, beta, visc, drag, ly, hly;  // hly = 0.5 ly (exact)
  double zh[4], zl[4];  // two-term reciprocals of dxx, dyy, dxx2, dyy2 (in that order), for div_fixed
  int fastdiv;                      // every divisor and its reciprocal are normal numbers
};

// the stencil's divisions by the grid spacings: div_fixed when the host found the spacings normal, else IEEE
__device__ __forceinline__ double div_by(const PlaneDev &p, double x, double y, int k) {
  int fast;
  return p.fastdiv ? div_fixed(x, y, p.zh[k], p.zl[k], fast) : x / y;
}

__device__ __forceinline__ int wrapx(int i, int nx) { return ((i % nx) + nx) % nx; }

// stage 0..3 with coefficients c = 0.5 dt, 0.5 dt, dt, dt/6 (cpp/plane.cpp:143-158)
__global__ void __launch_bounds__(TX *TY) plane_stage(PlaneDev p, int stage, double c, const double *__restrict__ hi,
                                                      const double *__restrict__ ui, const double *__restrict__ vi,
                                                      double *h0, double *u0, double *v0, double *ah, double *au, double *av,
                                                      double *ho, double *uo, double *vo) {
  __shared__ double sh[TY + 2][TX + 2], su[TY + 2][TX + 2], sv[TY + 2][TX + 2];
  __shared__ double sB[TY + 1][TX + 1], sE[TY + 1][TX + 1];
  const int nx = p.nx, ny = p.ny;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int tid = threadIdx.y * TX + threadIdx.x;
  // tile load: local (ly, lx) <-> global (j0 - 1 + ly, i0 - 1 + lx), periodic in x
  for (int e = tid; e < (TY + 2) * (TX + 2); e += TX * TY) {
    int ly = e / (TX + 2), lx = e % (TX + 2);
    int jg = j0 - 1 + ly, ig = wrapx(i0 - 1 + lx, nx);
    double hv = 0, uv = 0, vv = 0;
    if (jg >= 0 && jg < ny) {
      size_t o = static_cast<size_t>(jg) * nx + ig;
      hv = hi[o];
      uv = ui[o];
    }
    if (jg >= 0 && jg <= ny) vv = vi[static_cast<size_t>(jg) * nx + ig];
    sh[ly][lx] = hv;
    su[ly][lx] = uv;
    sv[ly][lx] = vv;
  }
  __syncthreads();
  // Bernoulli B at cells (j0-1+ly, i0-1+lx) and absolute vorticity at corners (j0+ly, i0+lx), cpp/plane.cpp:70-92
  for (int e = tid; e < (TY + 1) * (TX + 1); e += TX * TY) {
    int ly = e / (TX + 1), lx = e % (TX + 1);
    int jb = j0 - 1 + ly;
    double b = 0;
    if (jb >= 0 && jb < ny) {
      double k = 0;
      if (!p.lin) {
        double ua = su[ly][lx], ub = su[ly][lx + 1], va = sv[ly][lx], vb = sv[ly + 1][lx];
        k = 0.5 * (0.5 * (ua * ua + ub * ub) + 0.5 * (va * va + vb * vb));
      }
      b = p.g * sh[ly][lx] + k;
    }
    sB[ly][lx] = b;
    int je = j0 + ly;
    double eta = 0;
    if (je <= ny) {
      double f = p.f0 + p.beta * (je * p.dyy - p.hly);
      double zeta = 0;
      if (!p.lin) {
        double dvdx = div_by(p, sv[ly + 1][lx + 1] - sv[ly + 1][lx], p.dxx, 0);
        double uj = je < ny ? su[ly + 1][lx + 1] : su[ly][lx + 1];
        double ujm = je > 0 ? su[ly][lx + 1] : su[ly + 1][lx + 1];
        zeta = dvdx - div_by(p, uj - ujm, p.dyy, 1);
      }
      eta = f + zeta;
    }
    sE[ly][lx] = eta;
  }
  __syncthreads();
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = i0 + tx, j = j0 + ty;
  if (i >= nx || j >= ny) return;
  const double U = su[ty + 1][tx + 1], V = sv[ty + 1][tx + 1], Hc = sh[ty + 1][tx + 1];
  // du at the u point (i, j): cpp/plane.cpp:94-105
  double du;
  {
    double q = 0.5 * (sE[ty][tx] + sE[ty + 1][tx]);
    double vbar = 0.25 * (sv[ty + 1][tx] + sv[ty + 1][tx + 1] + sv[ty + 2][tx] + sv[ty + 2][tx + 1]);
    double r = q * vbar - div_by(p, sB[ty + 1][tx + 1] - sB[ty + 1][tx], p.dxx, 0) - p.drag * U;
    if (p.visc != 0) {
      double uy1 = j + 1 < ny ? su[ty + 2][tx + 1] : U, uy0 = j > 0 ? su[ty][tx + 1] : U;
      r += p.visc * (div_by(p, su[ty + 1][tx + 2] - 2 * U + su[ty + 1][tx], p.dxx2, 2) + div_by(p, uy1 - 2 * U + uy0, p.dyy2, 3));
    }
    du = r;
  }
  // dv at the v point (i, j), interior rows only: cpp/plane.cpp:106-117
  double dv = 0;
  if (j >= 1) {
    double q = 0.5 * (sE[ty][tx] + sE[ty][tx + 1]);
    double ubar = 0.25 * (su[ty][tx + 1] + su[ty][tx + 2] + su[ty + 1][tx + 1] + su[ty + 1][tx + 2]);
    double r = -q * ubar - div_by(p, sB[ty + 1][tx + 1] - sB[ty][tx + 1], p.dyy, 1) - p.drag * V;
    if (p.visc != 0) {
      double vy1 = j + 1 < ny ? sv[ty + 2][tx + 1] : 0.0, vy0 = j - 1 > 0 ? sv[ty][tx + 1] : 0.0;
      r += p.visc * (div_by(p, sv[ty + 1][tx + 2] - 2 * V + sv[ty + 1][tx], p.dxx2, 2) + div_by(p, vy1 - 2 * V + vy0, p.dyy2, 3));
    }
    dv = r;
  }
  // dh: continuity in flux form, cpp/plane.cpp:119-128
  double dh;
  {
    double hw = p.lin ? p.depth : 0.5 * (sh[ty + 1][tx] + Hc);
    double fe = (p.lin ? p.depth : 0.5 * (Hc + sh[ty + 1][tx + 2])) * su[ty + 1][tx + 2];
    double fw = hw * U;
    double fn = 0, fs = 0;
    if (j + 1 < ny) fn = (p.lin ? p.depth : 0.5 * (Hc + sh[ty + 2][tx + 1])) * sv[ty + 2][tx + 1];
    if (j > 0) fs = (p.lin ? p.depth : 0.5 * (sh[ty][tx + 1] + Hc)) * V;
    dh = -(div_by(p, fe - fw, p.dxx, 0) + div_by(p, fn - fs, p.dyy, 1));
  }
  const size_t o = static_cast<size_t>(j) * nx + i;
  // RK4 bookkeeping: cpp/plane.cpp:146-156 (acc = k1 + 2 k2 + 2 k3, state += dt/6 (acc + k4))
  auto upd = [&](double k, double *x0, double *acc, double *out, size_t idx) {
    if (stage == 0) {
      out[idx] = x0[idx] + c * k;
      acc[idx] = k;
    } else if (stage < 3) {
      out[idx] = x0[idx] + c * k;
      acc[idx] = acc[idx] + 2 * k;
    } else {
      x0[idx] = x0[idx] + c * (acc[idx] + k);
    }
  };
  upd(dh, h0, ah, ho, o);
  upd(du, u0, au, uo, o);
  upd(dv, v0, av, vo, o);  // rows 0 (wall) .. ny-1; dv = 0 on the wall
  if (j == ny - 1) upd(0.0, v0, av, vo, o + nx);  // the northern wall row ny
}

// ---------------------------------------------------------------- reductions (guards and diagnostics)
// per block: sum h, sum u, sum v, energy sum, pv^2 sum; max speed, max h
constexpr int RED_THREADS = 256;
constexpr int RED_SUMS = 5, RED_MAXS = 2;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

__global__ void __launch_bounds__(RED_THREADS) plane_reduce(PlaneDev p, const double *__restrict__ h, const double *__restrict__ u,
                                                            const double *__restrict__ v, double *part) {
  const int nx = p.nx, ny = p.ny;
  const size_t ncell = static_cast<size_t>(nx) * ny, nv = static_cast<size_t>(nx) * (ny + 1);
  double s[RED_SUMS] = {0, 0, 0, 0, 0}, mx[RED_MAXS] = {0, -INFINITY};
  for (size_t e = blockIdx.x * (size_t)RED_THREADS + threadIdx.x; e < nv; e += (size_t)gridDim.x * RED_THREADS) {
    s[2] += v[e];
    if (e >= ncell) continue;
    int j = static_cast<int>(e / nx), i = static_cast<int>(e % nx);
    double hh = h[e];
    s[0] += hh;
    s[1] += u[e];
    double uc = 0.5 * (u[e] + u[static_cast<size_t>(j) * nx + (i + 1) % nx]);
    double vc = 0.5 * (v[e] + v[e + nx]);
    s[3] += 0.5 * hh * (uc * uc + vc * vc) + 0.5 * p.g * hh * hh;
    mx[0] = fmax(mx[0], hypot(uc, vc));
    mx[1] = fmax(mx[1], hh);
    if (j >= 1) {  // PV anomaly at interior corners, cpp/plane.cpp:228-243
      int im = (i + nx - 1) % nx;
      double hav = 0.25 * (h[static_cast<size_t>(j - 1) * nx + im] + h[static_cast<size_t>(j - 1) * nx + i] +
                           h[static_cast<size_t>(j) * nx + im] + hh);
      double dvdx = (v[e] - v[static_cast<size_t>(j) * nx + im]) / p.dxx;
      double z = dvdx - (u[e] - u[e - nx]) / p.dyy;
      double q = z - p.f0 * (hav - p.depth) / p.depth;
      s[4] += q * q;
    }
  }
  __shared__ double red[RED_THREADS / 32][RED_SUMS + RED_MAXS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < RED_SUMS; k++) s[k] = warp_sum(s[k]);
  for (int k = 0; k < RED_MAXS; k++) mx[k] = warp_max(mx[k]);
  if (lane == 0) {
    for (int k = 0; k < RED_SUMS; k++) red[wid][k] = s[k];
    for (int k = 0; k < RED_MAXS; k++) red[wid][RED_SUMS + k] = mx[k];
  }
  __syncthreads();
  if (threadIdx.x < RED_SUMS + RED_MAXS) {
    int k = threadIdx.x;
    double a = red[0][k];
    for (int w = 1; w < RED_THREADS / 32; w++) a = k < RED_SUMS ? a + red[w][k] : fmax(a, red[w][k]);
    part[static_cast<size_t>(blockIdx.x) * (RED_SUMS + RED_MAXS) + k] = a;
  }
}

__global__ void plane_reduce_final(const double *part, int nblk, Reduce *out) {
  int k = threadIdx.x;
  if (k >= RED_SUMS + RED_MAXS) return;
  double a = part[k];
  for (int b = 1; b < nblk; b++) {
    double x = part[static_cast<size_t>(b) * (RED_SUMS + RED_MAXS) + k];
    a = k < RED_SUMS ? a + x : fmax(a, x);
  }
  if (k < RED_SUMS) out->sum[k] = a;
  else out->max[k - RED_SUMS] = a;
}

// ---------------------------------------------------------------- point and harmonic diagnostics
// One thread: kind 0..2 -> bilinear value of h, u or v at (x, y) (cpp/plane.cpp:245-264: each field on its own
// points, periodic in x, rows clamped); kind 3 -> relative vorticity at corner (ci, cj) (cpp/plane.cpp:220-226).
// Compiled without FMA contraction, so the value is the reference's bit for bit.
__global__ void plane_point(PlaneDev p, const double *__restrict__ h, const double *__restrict__ u, const double *__restrict__ v, int kind,
                            double x, double y, int ci, int cj, double *out) {
  const int nx = p.nx, ny = p.ny;
  if (kind == 3) {
    const int im = (ci + nx - 1) % nx;
    const double dvdx = (v[static_cast<size_t>(cj) * nx + ci % nx] - v[static_cast<size_t>(cj) * nx + im]) / p.dxx;
    const double uj = cj < ny ? u[static_cast<size_t>(cj) * nx + ci % nx] : u[static_cast<size_t>(ny - 1) * nx + ci % nx];
    const double ujm = cj > 0 ? u[static_cast<size_t>(cj - 1) * nx + ci % nx] : u[ci % nx];
    out[0] = dvdx - (uj - ujm) / p.dyy;
    return;
  }
  const double xs = kind == 1 ? 0.0 : 0.5, ys = kind == 2 ? 0.0 : 0.5;
  const double fx = x / p.dxx - xs, fy = y / p.dyy - ys;
  const int rows = kind == 2 ? ny + 1 : ny;
  const double fl = floor(fx);
  const int i0 = static_cast<int>(fl), j0 = static_cast<int>(floor(fy));
  const double ax = fx - fl, ay = fy - floor(fy);
  const double *f = kind == 0 ? h : kind == 1 ? u : v;
  auto get = [&](int i, int j) {
    i = wrapx(i, nx);
    j = max(0, min(rows - 1, j));
    return f[static_cast<size_t>(j) * nx + i];
  };
  out[0] = (1 - ax) * ((1 - ay) * get(i0, j0) + ay * get(i0, j0 + 1)) + ax * ((1 - ay) * get(i0 + 1, j0) + ay * get(i0 + 1, j0 + 1));
}

constexpr int HARM_THREADS = 256;
constexpr double kPiPlane = 3.14159265358979323846;

// one CTA per row: c_m = (1/nx) sum_i f_i exp(-2 pi i m (i + shift) / nx) of rows j0.. of f (cpp/plane.cpp:266-270);
// out[r] = (re, im)
__global__ void __launch_bounds__(HARM_THREADS) plane_row_harmonics(const double *__restrict__ f, int nx, int j0, int m, double shift,
                                                                    double2 *out) {
  __shared__ double red[2][HARM_THREADS / 32];
  const double *row = f + static_cast<size_t>(j0 + blockIdx.x) * nx;
  double cr = 0, ci = 0;
  for (int i = threadIdx.x; i < nx; i += HARM_THREADS) {
    const double th = -2 * kPiPlane * m * (i + shift) / nx;
    double sn, cs;
    sincos(th, &sn, &cs);
    cr += row[i] * cs;
    ci += row[i] * sn;
  }
  cr = warp_sum(cr);
  ci = warp_sum(ci);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][wid] = cr;
    red[1][wid] = ci;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int w = 0; w < HARM_THREADS / 32; w++) {
      a += red[0][w];
      b += red[1][w];
    }
    out[blockIdx.x] = make_double2(a / static_cast<double>(nx), b / static_cast<double>(nx));
  }
}

// sum over rows of |c_m|^2 divided by ny (cpp/plane.cpp:291-299), one thread in row order
__global__ void plane_harmonic_energy_sum(const double2 *__restrict__ c, int rows, int ny, double *out) {
  double s = 0;
  for (int r = 0; r < rows; r++) s += c[r].x * c[r].x + c[r].y * c[r].y;
  out[0] = s / ny;
}

PlaneDev make_dev(const PlaneConfig &c) {
  PlaneDev d;
  d.nx = c.nx;
  d.ny = c.ny;
  d.lin = c.linear ? 1 : 0;
  d.dxx = c.lx / c.nx;
  d.dyy = c.ly / c.ny;
  d.dxx2 = d.dxx * d.dxx;
  d.dyy2 = d.dyy * d.dyy;
  d.g = c.gravity;
  d.depth = c.depth;
  d.f0 = c.f0;
  d.beta = c.beta;
  d.visc = c.viscosity;
  d.drag = c.drag;
  d.ly = c.ly;
  d.hly = 0.5 * c.ly;
  const double dv[4] = {d.dxx, d.dyy, d.dxx2, d.dyy2};
  d.fastdiv = 1;
  for (int k = 0; k < 4; k++)
    if (!fixed_div_reciprocal(dv[k], d.zh[k], d.zl[k])) d.fastdiv = 0;
  return d;
}

// splitmix64 and the Irwin-Hall normal of cpp/plane.cpp:12-17,37-41 (host, for the seeded initialisers)
uint64_t splitmix(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
double irwin_hall(uint64_t &st) {
  double s = 0;
  for (int i = 0; i < 12; i++) s += static_cast<double>(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
  return s - 6.0;
}

// Scratch of lmw_plane_step_noalloc: the two RK4 stage inputs and the accumulator (three fields each), in
// device memory reserved when the library is loaded, so that the entry point never allocates. Each field slot
// holds kNoAllocFieldCap doubles: up to kNoAllocMaxCells cells for h and u, plus one row (nx <= 4000) for v.
constexpr size_t kNoAllocMaxCells = 262144;
constexpr size_t kNoAllocFieldCap = kNoAllocMaxCells + 4096;
static __device__ __align__(256) double g_noalloc_scratch[9 * kNoAllocFieldCap];

// div_fixed against the IEEE division on every pair (x[i], y[k]): counts[0] = results that differ in any bit,
// counts[1] = pairs the fast path answered (the rest took the IEEE division)
__global__ void division_selftest(const unsigned long long *__restrict__ xb, int nx, const double *__restrict__ y,
                                  const double *__restrict__ zh, const double *__restrict__ zl, int ny,
                                  unsigned long long *counts) {
  const long long total = static_cast<long long>(nx) * ny;
  unsigned long long bad = 0, fastn = 0;
  for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double x = __longlong_as_double(static_cast<long long>(xb[e % nx]));
    const int k = static_cast<int>(e / nx);
    int fast = 0;
    const double a = div_fixed(x, y[k], zh[k], zl[k], fast);
    const double b = x / y[k];
    bad += __double_as_longlong(a) != __double_as_longlong(b) ? 1 : 0;
    fastn += fast;
  }
  if (bad) atomicAdd(&counts[0], bad);
  if (fastn) atomicAdd(&counts[1], fastn);
}

}  // namespace

void division_selftest_run(const uint64_t *x, int nx, const double *y, int ny, long long *counts) {
  if (nx < 0 || ny < 0 || nx > (1 << 26) || ny > 4096) throw InvalidArgument("counts out of range");
  std::vector<double> zh(std::max(ny, 1)), zl(std::max(ny, 1));
  for (int k = 0; k < ny; k++)
    if (!fixed_div_reciprocal(y[k], zh[k], zl[k]))
      throw InvalidArgument("divisor " + std::to_string(k) + " or its reciprocal is not a normal number");
  DevBuf<unsigned long long> xd, cd;
  DevBuf<double> yd, hd, ld;
  xd.alloc(std::max(nx, 1));
  yd.alloc(std::max(ny, 1));
  hd.alloc(std::max(ny, 1));
  ld.alloc(std::max(ny, 1));
  cd.alloc(2);
  if (nx) LMW_CUDA(cudaMemcpy(xd.p, x, nx * sizeof(unsigned long long), cudaMemcpyHostToDevice));
  if (ny) {
    LMW_CUDA(cudaMemcpy(yd.p, y, ny * sizeof(double), cudaMemcpyHostToDevice));
    LMW_CUDA(cudaMemcpy(hd.p, zh.data(), ny * sizeof(double), cudaMemcpyHostToDevice));
    LMW_CUDA(cudaMemcpy(ld.p, zl.data(), ny * sizeof(double), cudaMemcpyHostToDevice));
  }
  LMW_CUDA(cudaMemset(cd.p, 0, 2 * sizeof(unsigned long long)));
  if (nx > 0 && ny > 0) {
    division_selftest<<<1024, 256>>>(xd.p, nx, yd.p, hd.p, ld.p, ny, cd.p);
    LMW_LAUNCH_CHECK();
    g_launches += 1;
  }
  unsigned long long c[2];
  LMW_CUDA(cudaMemcpy(c, cd.p, sizeof(c), cudaMemcpyDeviceToHost));
  for (int k = 0; k < 2; k++) counts[k] = static_cast<long long>(c[k]);
}

// Device address of g_noalloc_scratch in the calling thread's current CUDA context. In host code the symbol's
// name is only a host-side stand-in, never a device address. A module's globals live in one context: after
// cudaDeviceReset, or in a second context made on the same device with the driver API, the array is loaded
// again at another address. So the address is cached per context (keyed by the driver's unique context id,
// which is never reused within a process) and looked up, with that context current, on the first call made
// in it.
using CtxGetCurrentFn = int (*)(void **);
using CtxGetIdFn = int (*)(void *, unsigned long long *);
static unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  if (!get_current || !get_id) throw DeviceError("lmw_plane_step_noalloc: the driver offers no context id (cuCtxGetId)");
  void *ctx = nullptr;
  if (get_current(&ctx) != 0) throw DeviceError("lmw_plane_step_noalloc: cuCtxGetCurrent failed");
  if (ctx == nullptr) {
    // no context bound to this thread yet: a runtime call on the module binds the device's primary context
    void *p = nullptr;
    LMW_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    if (get_current(&ctx) != 0 || ctx == nullptr) throw DeviceError("lmw_plane_step_noalloc: no current CUDA context");
  }
  unsigned long long id = 0;
  if (get_id(ctx, &id) != 0) throw DeviceError("lmw_plane_step_noalloc: cuCtxGetId failed");
  return id;
}

static double *noalloc_scratch() {
  static std::mutex mu;
  static std::vector<std::pair<unsigned long long, double *>> cache;  // (context id, array address)
  const unsigned long long id = current_context_id();
  std::lock_guard<std::mutex> lock(mu);
  for (const auto &e : cache)
    if (e.first == id) return e.second;
  void *p = nullptr;
  LMW_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  cache.emplace_back(id, static_cast<double *>(p));
  return static_cast<double *>(p);
}

void plane_step_noalloc(const PlaneConfig &c, double *h, double *u, double *v, double dt, int steps, cudaStream_t stream) {
  if (c.nx < 4 || c.ny < 4 || c.nx > 4000 || c.ny > 4000 || static_cast<int64_t>(c.nx) * c.ny > 8000000)
    throw InvalidArgument("grid must be at least 4 x 4 and at most 8 million cells");
  if (!(c.lx > 0 && c.ly > 0)) throw InvalidArgument("domain sizes must be positive");
  const size_t cells = static_cast<size_t>(c.nx) * c.ny;
  if (cells > kNoAllocMaxCells)
    throw InvalidArgument("lmw_plane_step_noalloc: the grid has " + std::to_string(cells) + " cells; this entry point's fixed scratch holds at most " +
                          std::to_string(kNoAllocMaxCells) + " cells (use lmw_plane_create for larger grids)");
  if (!h || !u || !v) throw InvalidArgument("lmw_plane_step_noalloc: field pointer is null");
  if (steps < 0) throw InvalidArgument("lmw_plane_step_noalloc: steps must not be negative");
  if (!std::isfinite(dt)) throw InvalidArgument("lmw_plane_step_noalloc: dt must be finite");
  double *sc = noalloc_scratch();
  // rows 0 and ny of v are the walls; the model keeps them at zero (lmw_plane_set_v does the same), and a
  // nonzero value there would never be cleared (dv = 0 on the walls) and would enter the fluxes and vorticity
  LMW_CUDA(cudaMemsetAsync(v, 0, static_cast<size_t>(c.nx) * sizeof(double), stream));
  LMW_CUDA(cudaMemsetAsync(v + static_cast<size_t>(c.ny) * c.nx, 0, static_cast<size_t>(c.nx) * sizeof(double), stream));
  double *ha = sc, *ua = sc + kNoAllocFieldCap, *va = sc + 2 * kNoAllocFieldCap;
  double *hb = sc + 3 * kNoAllocFieldCap, *ub = sc + 4 * kNoAllocFieldCap, *vb = sc + 5 * kNoAllocFieldCap;
  double *ah = sc + 6 * kNoAllocFieldCap, *au = sc + 7 * kNoAllocFieldCap, *av = sc + 8 * kNoAllocFieldCap;
  // every stage-0 launch writes all of a and the accumulator before any later stage reads them: nothing in the
  // scratch has to start at zero
  PlaneDev d = make_dev(c);
  dim3 grid((c.nx + TX - 1) / TX, (c.ny + TY - 1) / TY), block(TX, TY);
  const double half = 0.5 * dt, c6 = dt / 6;
  for (int s = 0; s < steps; s++) {
    plane_stage<<<grid, block, 0, stream>>>(d, 0, half, h, u, v, h, u, v, ah, au, av, ha, ua, va);
    plane_stage<<<grid, block, 0, stream>>>(d, 1, half, ha, ua, va, h, u, v, ah, au, av, hb, ub, vb);
    plane_stage<<<grid, block, 0, stream>>>(d, 2, dt, hb, ub, vb, h, u, v, ah, au, av, ha, ua, va);
    plane_stage<<<grid, block, 0, stream>>>(d, 3, c6, ha, ua, va, h, u, v, ah, au, av, nullptr, nullptr, nullptr);
    LMW_LAUNCH_CHECK();
    g_launches += 4;
  }
}

PlaneEngine::PlaneEngine(const PlaneConfig &c) : p(c) {
  // cpp/plane.cpp:20-25
  if (c.nx < 4 || c.ny < 4 || c.nx > 4000 || c.ny > 4000 || static_cast<int64_t>(c.nx) * c.ny > 8000000)
    throw InvalidArgument("grid must be at least 4 x 4 and at most 8 million cells");
  if (!(c.lx > 0 && c.ly > 0)) throw InvalidArgument("domain sizes must be positive");
  LMW_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  for (DevBuf<double> *b : {&h0, &u0, &ha, &ua, &hb, &ub, &ah, &au}) b->alloc(ncell());
  for (DevBuf<double> *b : {&v0, &va, &vb, &av}) b->alloc(nvpt());
  nblk_red = 2 * 152;
  part.alloc(static_cast<size_t>(nblk_red) * (RED_SUMS + RED_MAXS));
  dred.alloc(1);
  hred.alloc(1);
  stage.alloc(nvpt());
  diag.alloc(2 + 4 * static_cast<size_t>(c.ny));  // one scalar, then a complex per row of u and v
  reset();
}

PlaneEngine::~PlaneEngine() {
  if (graph) cudaGraphExecDestroy(graph);
  if (stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
}

void PlaneEngine::upload(double *dst, const double *src, size_t n) {
  for (size_t off = 0; off < n; off += stage.n) {
    size_t c = std::min(stage.n, n - off);
    LMW_CUDA(cudaStreamSynchronize(stream));
    std::memcpy(stage.p, src + off, c * sizeof(double));
    LMW_CUDA(cudaMemcpyAsync(dst + off, stage.p, c * sizeof(double), cudaMemcpyHostToDevice, stream));
  }
  LMW_CUDA(cudaStreamSynchronize(stream));
}

// cpp/plane.cpp:27-32
void PlaneEngine::reset() {
  std::vector<double> hh(ncell(), p.depth);
  upload(h0.p, hh.data(), ncell());
  u0.zero(stream);
  v0.zero(stream);
  LMW_CUDA(cudaStreamSynchronize(stream));
  t = 0;
}

// cpp/plane.cpp:312-318
void PlaneEngine::set_h(const double *g, size_t n) {
  if (n != ncell()) throw InvalidArgument("grid size mismatch");
  upload(h0.p, g, n);
}
void PlaneEngine::set_u(const double *g, size_t n) {
  if (n != ncell()) throw InvalidArgument("grid size mismatch");
  upload(u0.p, g, n);
}
void PlaneEngine::set_v(const double *g, size_t n) {
  if (n != nvpt()) throw InvalidArgument("grid size mismatch");
  std::vector<double> vv(g, g + n);
  for (int i = 0; i < p.nx; i++) {
    vv[i] = 0;
    vv[static_cast<size_t>(p.ny) * p.nx + i] = 0;
  }
  upload(v0.p, vv.data(), n);
}

void PlaneEngine::get(double *h, double *u, double *v) {
  LMW_CUDA(cudaStreamSynchronize(stream));
  if (h) LMW_CUDA(cudaMemcpy(h, h0.p, ncell() * sizeof(double), cudaMemcpyDeviceToHost));
  if (u) LMW_CUDA(cudaMemcpy(u, u0.p, ncell() * sizeof(double), cudaMemcpyDeviceToHost));
  if (v) LMW_CUDA(cudaMemcpy(v, v0.p, nvpt() * sizeof(double), cudaMemcpyDeviceToHost));
}

// cpp/plane.cpp:34-57: seeded smooth noise. An initialiser, run once on the host in the reference's
// operation order (bitwise identical), then added to the device height.
void PlaneEngine::perturb(double amplitude, uint64_t seed) {
  const int nx = p.nx, ny = p.ny;
  const size_t N = ncell();
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 777;
  std::vector<double> n(N), tt(N), h(N);
  for (auto &x : n) x = irwin_hall(st);
  for (int pass = 0; pass < 3; pass++) {
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++)
        tt[static_cast<size_t>(j) * nx + i] = 0.25 * n[static_cast<size_t>(j) * nx + (i + nx - 1) % nx] + 0.5 * n[static_cast<size_t>(j) * nx + i] +
                                              0.25 * n[static_cast<size_t>(j) * nx + (i + 1) % nx];
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        int jm = std::max(j - 1, 0), jp = std::min(j + 1, ny - 1);
        n[static_cast<size_t>(j) * nx + i] = 0.25 * tt[static_cast<size_t>(jm) * nx + i] + 0.5 * tt[static_cast<size_t>(j) * nx + i] +
                                             0.25 * tt[static_cast<size_t>(jp) * nx + i];
      }
  }
  double mean = 0, ms = 0;
  for (double x : n) mean += x;
  mean /= n.size();
  for (double &x : n) {
    x -= mean;
    ms += x * x;
  }
  double rms = std::sqrt(ms / n.size());
  double scale = rms > 0 ? amplitude / rms : 0;
  get(h.data(), nullptr, nullptr);
  for (size_t i = 0; i < N; i++) h[i] += n[i] * scale;
  upload(h0.p, h.data(), N);
}

// Zonal jet in geostrophic balance plus white height noise (this project's benchmark initialiser; the same
// definition as the oracle's or_plane_jet_grids).
void PlaneEngine::jet(double u0v, double width, double noise_rms, uint64_t seed) {
  const int nx = p.nx, ny = p.ny;
  const double dyy = dy();
  auto cor = [&](double y) { return p.f0 + p.beta * (y - 0.5 * p.ly); };
  std::vector<double> prof(ny), hy(ny);
  for (int j = 0; j < ny; j++) {
    double y = (j + 0.5) * dyy;
    double c = std::cosh((y - 0.5 * p.ly) / width);
    prof[j] = u0v / (c * c);
  }
  hy[0] = 0;
  for (int j = 1; j < ny; j++) {
    double fa = cor((j - 0.5) * dyy) * prof[j - 1], fb = cor((j + 0.5) * dyy) * prof[j];
    hy[j] = hy[j - 1] - dyy / p.gravity * 0.5 * (fa + fb);
  }
  double mean = 0;
  for (int j = 0; j < ny; j++) mean += hy[j];
  mean /= ny;
  const size_t N = ncell();
  std::vector<double> noise(N), h(N), u(N);
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 777;
  for (auto &x : noise) x = irwin_hall(st);
  double nm = 0, ms = 0;
  for (double x : noise) nm += x;
  nm /= N;
  for (double &x : noise) {
    x -= nm;
    ms += x * x;
  }
  double rms = std::sqrt(ms / N);
  double sc = rms > 0 ? noise_rms / rms : 0;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      size_t k = static_cast<size_t>(j) * nx + i;
      h[k] = p.depth + (hy[j] - mean) + noise[k] * sc;
      u[k] = prof[j];
    }
  upload(h0.p, h.data(), N);
  upload(u0.p, u.data(), N);
  v0.zero(stream);
  LMW_CUDA(cudaStreamSynchronize(stream));
  t = 0;
}

void PlaneEngine::enqueue_step(double dt) {
  PlaneDev d = make_dev(p);
  dim3 grid((p.nx + TX - 1) / TX, (p.ny + TY - 1) / TY), block(TX, TY);
  const double half = 0.5 * dt, c6 = dt / 6;
  // stage inputs: x0 -> a -> b -> a
  plane_stage<<<grid, block, 0, stream>>>(d, 0, half, h0.p, u0.p, v0.p, h0.p, u0.p, v0.p, ah.p, au.p, av.p, ha.p, ua.p, va.p);
  plane_stage<<<grid, block, 0, stream>>>(d, 1, half, ha.p, ua.p, va.p, h0.p, u0.p, v0.p, ah.p, au.p, av.p, hb.p, ub.p, vb.p);
  plane_stage<<<grid, block, 0, stream>>>(d, 2, dt, hb.p, ub.p, vb.p, h0.p, u0.p, v0.p, ah.p, au.p, av.p, ha.p, ua.p, va.p);
  plane_stage<<<grid, block, 0, stream>>>(d, 3, c6, ha.p, ua.p, va.p, h0.p, u0.p, v0.p, ah.p, au.p, av.p, nullptr, nullptr, nullptr);
  LMW_LAUNCH_CHECK();
  g_launches += 4;
}

// a chunk of RK4 steps as one CUDA graph (captured once per step size and chunk length)
void PlaneEngine::launch_chunk(double dt, int steps) {
  if (steps <= 0) return;
  if (!graph || graph_dt != dt || graph_steps != steps) {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    cudaGraph_t g;
    uint64_t before = g_launches;
    LMW_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < steps; s++) enqueue_step(dt);
    LMW_CUDA(cudaStreamEndCapture(stream, &g));
    g_launches = before;
    LMW_CUDA(cudaGraphInstantiate(&graph, g, 0));
    cudaGraphDestroy(g);
    graph_dt = dt;
    graph_steps = steps;
  }
  LMW_CUDA(cudaGraphLaunch(graph, stream));
  g_launches += 4ull * steps;
}

double PlaneEngine::kernel_time(double dt, int reps) {
  PlaneDev d = make_dev(p);
  dim3 grid((p.nx + TX - 1) / TX, (p.ny + TY - 1) / TY), block(TX, TY);
  cudaEvent_t e0, e1;
  LMW_CUDA(cudaEventCreate(&e0));
  LMW_CUDA(cudaEventCreate(&e1));
  // stage 1 reads the base state and stage input a, writes stage input b and the accumulator: x0 is untouched
  plane_stage<<<grid, block, 0, stream>>>(d, 1, 0.5 * dt, ha.p, ua.p, va.p, h0.p, u0.p, v0.p, ah.p, au.p, av.p, hb.p, ub.p, vb.p);
  LMW_CUDA(cudaEventRecord(e0, stream));
  for (int r = 0; r < reps; r++)
    plane_stage<<<grid, block, 0, stream>>>(d, 1, 0.5 * dt, ha.p, ua.p, va.p, h0.p, u0.p, v0.p, ah.p, au.p, av.p, hb.p, ub.p, vb.p);
  LMW_CUDA(cudaEventRecord(e1, stream));
  LMW_LAUNCH_CHECK();
  LMW_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  LMW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g_launches += reps + 1;
  return ms / reps;
}

void PlaneEngine::step(double dt) {
  enqueue_step(dt);
  t += dt;
  LMW_CUDA(cudaStreamSynchronize(stream));
}

void PlaneEngine::reduce(Reduce &r) {
  PlaneDev d = make_dev(p);
  plane_reduce<<<nblk_red, RED_THREADS, 0, stream>>>(d, h0.p, u0.p, v0.p, part.p);
  plane_reduce_final<<<1, 32, 0, stream>>>(part.p, nblk_red, dred.p);
  LMW_LAUNCH_CHECK();
  g_launches += 2;
  LMW_CUDA(cudaMemcpyAsync(hred.p, dred.p, sizeof(Reduce), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  r = *hred.p;
}

// cpp/plane.cpp:131-141
double PlaneEngine::stable_dt(double safety) {
  double hmax = p.linear ? p.depth : 0, umax = 0;
  if (!p.linear) {
    Reduce r;
    reduce(r);
    umax = r.max[0];
    hmax = std::max(hmax, r.max[1]);
  }
  if (!(hmax > 0)) throw RuntimeError("the depth must be positive to step the model");
  double c = std::sqrt(p.gravity * hmax) + umax;
  double inv = c * std::sqrt(1.0 / (dx() * dx()) + 1.0 / (dy() * dy()));
  double visc = p.viscosity * (4.0 / (dx() * dx()) + 4.0 / (dy() * dy()));
  return safety * 2.0 / (inv + visc + std::fabs(p.f0) + std::fabs(p.beta) * p.ly);
}

// cpp/plane.cpp:160-189
void PlaneEngine::run(double seconds, double dt) {
  if (!(seconds >= 0)) throw InvalidArgument("run: seconds must not be negative");
  if (seconds == 0) return;
  if (!(dt > 0)) dt = stable_dt(0.5);
  const double limit = stable_dt(std::sqrt(0.5));
  if (!(dt <= limit))
    throw InvalidArgument("run: dt = " + fmt_f(dt) + " s exceeds the RK4 stability limit of about " + fmt_f(limit) +
                          " s for the present state: use a smaller dt");
  int64_t n = static_cast<int64_t>(std::ceil(seconds / dt - 1e-9));
  if (n < 1) n = 1;
  if (n > 200000000) throw InvalidArgument("run: too many steps; use a larger dt");
  double hstep = seconds / static_cast<double>(n);
  int64_t i = 0;
  while (i < n) {
    // steps up to and including the next guard point ((i & 63) == 63 or the last step)
    int64_t next = std::min<int64_t>(n - 1, i | 63);
    int chunk = static_cast<int>(next - i + 1);
    if (chunk == 64) launch_chunk(hstep, 64);
    else for (int s = 0; s < chunk; s++) enqueue_step(hstep);
    for (int s = 0; s < chunk; s++) t += hstep;
    i = next + 1;
    Reduce r;
    reduce(r);
    double s = r.sum[0] + r.sum[1] + r.sum[2];
    if (!std::isfinite(s)) throw RuntimeError("the integration blew up (not finite): use a smaller dt");
    const double now = stable_dt(std::sqrt(0.5));
    if (!(hstep <= now))
      throw RuntimeError("run: dt = " + fmt_f(hstep) + " s exceeds the RK4 stability limit of about " + fmt_f(now) + " s reached at t = " +
                         fmt_f(t) + " s (the flow accelerated): use a smaller dt");
  }
}

// the small diagnostics read back a few doubles through the pinned staging buffer
double PlaneEngine::read_scalars(int n, double *out) {
  LMW_LAUNCH_CHECK();
  LMW_CUDA(cudaMemcpyAsync(stage.p, diag.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  for (int k = 0; k < n; k++) out[k] = stage.p[k];
  return out[0];
}

// cpp/plane.cpp:245-264 (h_at, u_at, v_at); any finite point is read in bounds (periodic x, clamped rows)
double PlaneEngine::probe(int kind, double x, double y) {
  if (kind < 0 || kind > 2) throw InvalidArgument("field must be 0 (h), 1 (u) or 2 (v)");
  if (!std::isfinite(x) || !std::isfinite(y)) throw InvalidArgument("point outside the domain");
  plane_point<<<1, 1, 0, stream>>>(make_dev(p), h0.p, u0.p, v0.p, kind, x, y, 0, 0, diag.p);
  g_launches += 1;
  double r;
  return read_scalars(1, &r);
}

// cpp/plane.cpp:220-226; corners i in 0..nx, j in 0..ny
double PlaneEngine::zeta_at_corner(int i, int j) {
  if (i < 0 || i > p.nx || j < 0 || j > p.ny) throw InvalidArgument("corner outside the grid");
  plane_point<<<1, 1, 0, stream>>>(make_dev(p), h0.p, u0.p, v0.p, 3, 0.0, 0.0, i, j, diag.p);
  g_launches += 1;
  double r;
  return read_scalars(1, &r);
}

void PlaneEngine::row_harmonic(int kind, int m, int j, double shift, double *re, double *im) {
  const double *f = kind == 0 ? h0.p : kind == 1 ? u0.p : v0.p;
  plane_row_harmonics<<<1, HARM_THREADS, 0, stream>>>(f, p.nx, j, m, shift, reinterpret_cast<double2 *>(diag.p));
  g_launches += 1;
  double c[2];
  read_scalars(2, c);
  *re = c[0];
  *im = c[1];
}

// crest x of f ~ cos(2 pi m x / lx + ph), in [0, lx/m) (cpp/plane.cpp:284-289)
static double crest_x(const PlaneConfig &p, int m, double re, double im) {
  const double ph = std::atan2(im, re);
  double x = -ph / (2 * kPiPlane * m) * p.lx;
  const double per = p.lx / m;
  x = std::fmod(x, per);
  return x < 0 ? x + per : x;
}

// cpp/plane.cpp:271-277
double PlaneEngine::zonal_amplitude(int m, int j) {
  if (m < 1 || m >= p.nx / 2 || j < 0 || j >= p.ny) throw InvalidArgument("zonal harmonic or row out of range");
  double re, im;
  row_harmonic(0, m, j, 0.5, &re, &im);
  return 2 * std::hypot(re, im);
}

// cpp/plane.cpp:278-290
double PlaneEngine::zonal_crest(int m, int j) {
  if (m < 1 || m >= p.nx / 2 || j < 0 || j >= p.ny) throw InvalidArgument("zonal harmonic or row out of range");
  double re, im;
  row_harmonic(0, m, j, 0.5, &re, &im);
  return crest_x(p, m, re, im);
}

// cpp/plane.cpp:300-310 (v rows 1..ny-1)
double PlaneEngine::v_zonal_crest(int m, int j) {
  if (m < 1 || m >= p.nx / 2 || j < 1 || j >= p.ny) throw InvalidArgument("zonal harmonic or v row out of range");
  double re, im;
  row_harmonic(2, m, j, 0.5, &re, &im);
  return crest_x(p, m, re, im);
}

// cpp/plane.cpp:291-299: every u row and the interior v rows, one CTA per row, summed on the device
double PlaneEngine::harmonic_energy(int m) {
  if (m < 1 || m >= p.nx / 2) throw InvalidArgument("zonal harmonic out of range");
  double2 *c = reinterpret_cast<double2 *>(diag.p) + 1;
  plane_row_harmonics<<<p.ny, HARM_THREADS, 0, stream>>>(u0.p, p.nx, 0, m, 0.0, c);
  plane_row_harmonics<<<p.ny - 1, HARM_THREADS, 0, stream>>>(v0.p, p.nx, 1, m, 0.5, c + p.ny);
  plane_harmonic_energy_sum<<<1, 1, 0, stream>>>(c, 2 * p.ny - 1, p.ny, diag.p);
  g_launches += 3;
  double r;
  return read_scalars(1, &r);
}

// ------------------------------------------------------------------------------------------------ text writers
// cpp/main.cpp:464-478: per cell x y h uc vc zeta (zeta the mean of the four corner vorticities), a blank line after
// each row; the fields come back once and the host forms the cell values in the reference's order
void PlaneEngine::save_csv(const std::string &path) {
  const int nx = p.nx, ny = p.ny;
  std::vector<double> h(ncell()), u(ncell()), v(nvpt());
  get(h.data(), u.data(), v.data());
  const double dxx = dx(), dyy = dy();
  auto zc = [&](int i, int j) {  // cpp/plane.cpp:220-226
    const int im = (i + nx - 1) % nx;
    const double dvdx = (v[static_cast<size_t>(j) * nx + i % nx] - v[static_cast<size_t>(j) * nx + im]) / dxx;
    const double uj = j < ny ? u[static_cast<size_t>(j) * nx + i % nx] : u[static_cast<size_t>(ny - 1) * nx + i % nx];
    const double ujm = j > 0 ? u[static_cast<size_t>(j - 1) * nx + i % nx] : u[i % nx];
    return dvdx - (uj - ujm) / dyy;
  };
  std::string t;
  t.reserve(ncell() * 80);
  for (int j = 0; j < ny; j++) {
    for (int i = 0; i < nx; i++) {
      const size_t e = static_cast<size_t>(j) * nx + i;
      const double uc = 0.5 * (u[e] + u[static_cast<size_t>(j) * nx + (i + 1) % nx]), vc = 0.5 * (v[e] + v[e + nx]);
      const double z = 0.25 * (zc(i, j) + zc(i + 1, j) + zc(i, j + 1) + zc(i + 1, j + 1));
      t += fmt_g((i + 0.5) * dxx) + " " + fmt_g((j + 0.5) * dyy) + " " + fmt_g(h[e]) + " " + fmt_g(uc) + " " + fmt_g(vc) + " " + fmt_g(z) + "\n";
    }
    t += "\n";
  }
  write_text(path, t, "Plane.save_csv");
}

// cpp/main.cpp:480-487: x and h along row j
void PlaneEngine::save_row(int j, const std::string &path) {
  if (j < 0 || j >= p.ny) throw InvalidArgument("Plane.save_row: row outside the grid");
  std::vector<double> h(ncell());
  get(h.data(), nullptr, nullptr);
  std::string t;
  for (int i = 0; i < p.nx; i++) t += fmt_g((i + 0.5) * dx()) + " " + fmt_g(h[static_cast<size_t>(j) * p.nx + i]) + "\n";
  write_text(path, t, "Plane.save_row");
}

// cpp/main.cpp:488-494: y and h along column i
void PlaneEngine::save_column(int i, const std::string &path) {
  if (i < 0 || i >= p.nx) throw InvalidArgument("Plane.save_column: column outside the grid");
  std::vector<double> h(ncell());
  get(h.data(), nullptr, nullptr);
  std::string t;
  for (int j = 0; j < p.ny; j++) t += fmt_g((j + 0.5) * dy()) + " " + fmt_g(h[static_cast<size_t>(j) * p.nx + i]) + "\n";
  write_text(path, t, "Plane.save_column");
}

// cpp/plane.cpp:191-243: mean_depth, energy, max_speed, pv_anomaly_rms
void PlaneEngine::diagnostics(double *out) {
  Reduce r;
  reduce(r);
  const double N = static_cast<double>(ncell());
  out[0] = r.sum[0] / N;
  out[1] = r.sum[3] / N;
  out[2] = r.max[0];
  out[3] = std::sqrt(r.sum[4] / static_cast<double>(static_cast<size_t>(p.nx) * (p.ny - 1)));
}

}  // namespace lmw
