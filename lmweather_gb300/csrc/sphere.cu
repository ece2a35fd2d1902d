// Spectral-transform shallow water on the sphere (the lmweather Sphere model, cpp/sphere.cpp), FP64 path.
//
// Per RK4 stage three kernels run on the engine stream:
//   sph_synth     per zonal wavenumber m (paired with T-m for load balance) and southern latitude jh: the
//                 six Legendre synthesis sums (psi P, chi P, psi H, chi H, zeta P, Phi P) split by the parity of
//                 n-m, which gives both mirror latitudes at once (hemispheric fold); writes the Fourier
//                 coefficients of U, V, zeta, Phi for both latitudes.
//   sph_grid      per latitude pair: the two latitudes ride in the real and imaginary parts of one complex
//                 FFT; inverse FFTs of U, V, zeta, Phi, the nonlinear products of cpp/sphere.cpp:348-359 in
//                 place, forward FFTs of the five products, then the quadrature weights and the fold
//                 (sum/difference of the mirror latitudes). The grid never leaves shared memory.
//   sph_analysis  per spectral coefficient (m, n): the seven folded Legendre analysis sums, the tendencies
//                 of cpp/sphere.cpp:372-389 and the RK4 stage update (cpp/sphere.cpp:416-434) with the del^4
//                 filter fused into the last stage.
// Layouts: state x[member][field][tri] complex128, tri(m, n) = packed triangle offset; Fourier
// coefficients four[member][lat][field][m]; folded analysis inputs fold[member][jh][slot][parity][m].
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>

#include "engine.h"
#include "fixed_div.cuh"
#include "sphere_common.cuh"
#include "sphere_tables.h"

namespace lmw {

struct SphereTables {
  HostTables host;
  DevBuf<double> Ps, Hs, Pa, Ha;  // coefficient-major [tri][jh] (synthesis) and latitude-major [jh][tri] (analysis)
  DevBuf<double> mu, w, wd, cosl, r2om, kfac, lapl;
  DevBuf<double2> tw;
  // FP32 copies for the reduced-precision stage kernels
  DevBuf<float> Ps32, Hs32, Pa32, Ha32, w32, wd32, r2om32, kfac32, lapl32;
  DevBuf<float2> tw32;  // exp(-2 pi i k / nlon), k < nlon/2
  DevBuf<int> trim, trin, tri;
};

namespace {

// ------------------------------------------------------------------------------------------------ synthesis
// Block: one wavenumber m and LATS southern latitudes (thread % LATS = latitude); the SYN_THREADS / LATS thread
// groups sum the terms n = m + c, m + c + NCH, ... (one parity of n - m per group), so the n-sum runs in NCH pieces
// at once; the pieces meet in shared memory. Reading the coefficient-major table is coalesced across latitudes.
// LATS = 32 (8 pieces) in general; LATS = 8 (32 pieces, four times the blocks) for grids of at most 32 latitude
// pairs (T <= 42), whose launches would otherwise occupy a fraction of the SMs. The choice depends on the grid
// only, so every member of a truncation is summed in the same order whatever the batch.
constexpr int SYN_THREADS = 256, SYN_Q = 12;
constexpr int SYN_CHUNKS = 8;  // n-sum pieces of the 32-latitude blocks (the tracer's synthesis uses this form)
__host__ __device__ constexpr int syn_lats(int nh) { return nh <= 32 ? 8 : 32; }

// x: [B][3][ntri] (zeta, delta, phi); four: [B][nlat][4][M] (U, V, zeta, Phi)
template <class R, int LATS>
__global__ void __launch_bounds__(SYN_THREADS) sph_synth(SphDev d, SphTab<R> t, const double2 *__restrict__ x,
                                                         typename V2<R>::type *__restrict__ four) {
  using C2 = typename V2<R>::type;
  constexpr int NCH = SYN_THREADS / LATS;
  __shared__ R part[NCH][SYN_Q][LATS + 1];
  const int b = blockIdx.z, m = blockIdx.y;
  const int lane = threadIdx.x % LATS, c = threadIdx.x / LATS;
  const int jh = blockIdx.x * LATS + lane;
  const bool live = jh < d.nh;
  const double2 *xz = x + static_cast<size_t>(b) * 3 * d.ntri, *xd = xz + d.ntri, *xf = xd + d.ntri;
  C2 sp = mk2(R(0), R(0)), sc = sp, hp = sp, hc = sp, zs = sp, fs = sp;
  const int base = d.tri[m];
  if (live) {
#pragma unroll 2
    for (int n = m + c; n <= d.N; n += NCH) {
      const int q = base + n - m;
      const R P = t.Ps[static_cast<size_t>(q) * d.nh + jh], H = t.Hs[static_cast<size_t>(q) * d.nh + jh];
      const double2 zd = xz[q], dd = xd[q], fd = xf[q];
      // FP32: the state is rounded on the integer pipe (the hardware conversion's values)
      const C2 z = mk2(to_arith<R>(zd.x), to_arith<R>(zd.y)), dl = mk2(to_arith<R>(dd.x), to_arith<R>(dd.y)),
               f = mk2(to_arith<R>(fd.x), to_arith<R>(fd.y));
      const R k = t.kfac[n];  // psi = -a^2/(n(n+1)) zeta, cpp/sphere.cpp:185-190
      const C2 psi = cscale(z, k), chi = cscale(dl, k);
      sp = cfma(sp, psi, P);
      sc = cfma(sc, chi, P);
      hp = cfma(hp, psi, H);
      hc = cfma(hc, chi, H);
      zs = cfma(zs, z, P);
      fs = cfma(fs, f, P);
    }
  }
  const R v[SYN_Q] = {sp.x, sp.y, sc.x, sc.y, hp.x, hp.y, hc.x, hc.y, zs.x, zs.y, fs.x, fs.y};
#pragma unroll
  for (int i = 0; i < SYN_Q; i++) part[c][i][lane] = v[i];
  __syncthreads();
  // even (n - m) pieces are those of even c, odd pieces those of odd c, each summed in the order of c
  R e[SYN_Q], o[SYN_Q];
  if constexpr (NCH <= 8) {
    if (threadIdx.x >= 2 * LATS || !live) return;
#pragma unroll
    for (int i = 0; i < SYN_Q; i++) {
      R se = 0, so = 0;
#pragma unroll
      for (int k = 0; k < NCH; k += 2) {
        se += part[k][i][lane];
        so += part[k + 1][i][lane];
      }
      e[i] = se;
      o[i] = so;
    }
  } else {
    // many pieces: every thread sums one (parity, value, latitude) first
    __shared__ R red[2][SYN_Q][LATS];
    for (int w = threadIdx.x; w < 2 * SYN_Q * LATS; w += SYN_THREADS) {
      const int par = w / (SYN_Q * LATS), i = (w / LATS) % SYN_Q, l = w % LATS;
      R acc = 0;
      for (int k = par; k < NCH; k += 2) acc += part[k][i][l];
      red[par][i][l] = acc;
    }
    __syncthreads();
    if (threadIdx.x >= 2 * LATS || !live) return;
#pragma unroll
    for (int i = 0; i < SYN_Q; i++) {
      e[i] = red[0][i][lane];
      o[i] = red[1][i][lane];
    }
  }
  const int side = threadIdx.x / LATS;  // 0: southern latitude (table latitude), 1: its northern mirror
  // southern latitude: even + odd; northern mirror: P sums even - odd, H sums odd - even
  R r[SYN_Q];
#pragma unroll
  for (int i = 0; i < SYN_Q; i++) {
    const bool hsum = i >= 4 && i < 8;
    r[i] = side == 0 ? e[i] + o[i] : (hsum ? o[i] - e[i] : e[i] - o[i]);
  }
  const R mm = static_cast<R>(m), ia = static_cast<R>(d.inv_a_f);
  const C2 SP = mk2(r[0], r[1]), SC = mk2(r[2], r[3]), HP = mk2(r[4], r[5]), HC = mk2(r[6], r[7]);
  // cpp/sphere.cpp:200-201: fu = (i m sc - hp)/a, fv = (i m sp + hc)/a
  C2 fu = csub(imul(SC, mm), HP), fv = cadd(imul(SP, mm), HC);
  if (sizeof(R) == 8) {
    if (d.div_a) {  // the same quotients as the IEEE division, in three FP64 operations each
      int fast;
      fu = mk2(R(div_fixed(fu.x, d.a, d.inv_a, d.inv_a_l, fast)), R(div_fixed(fu.y, d.a, d.inv_a, d.inv_a_l, fast)));
      fv = mk2(R(div_fixed(fv.x, d.a, d.inv_a, d.inv_a_l, fast)), R(div_fixed(fv.y, d.a, d.inv_a, d.inv_a_l, fast)));
    } else {
      fu = mk2(R(fu.x / d.a), R(fu.y / d.a));
      fv = mk2(R(fv.x / d.a), R(fv.y / d.a));
    }
  } else {
    fu = cscale(fu, ia);
    fv = cscale(fv, ia);
  }
  const int j = side == 0 ? jh : d.nlat - 1 - jh;
  C2 *out = four + (static_cast<size_t>(b) * d.nlat + j) * 4 * d.M;
  out[0 * d.M + m] = fu;
  out[1 * d.M + m] = fv;
  out[2 * d.M + m] = mk2(r[8], r[9]);
  out[3 * d.M + m] = mk2(r[10], r[11]);
}

// ------------------------------------------------------------------------------------------------ FFTs
// Radix-2 complex FFTs over `rows` rows of length n in shared memory, all threads of the block cooperating.
// Inverse: decimation in time from bit-reversed input to natural output. Forward: decimation in frequency
// from natural input to bit-reversed output. Twiddles exp(-2 pi i k / n) from the table (conjugated for the
// inverse), computed on the host in FP64.
// Radix-2 FFT stages fused in groups of up to three: a thread loads the 2^F elements that F consecutive stages
// combine (indices i0 + j 2^st), applies the F stages' butterflies in registers and stores them back, so each
// group costs one pass through shared memory and one barrier instead of F. The butterflies, their order and
// the twiddle factors are those of the plain radix-2 transform, so the results are bit for bit the same.
// Rows may be padded (PAD = p > 0): element i of a row sits at i + i / 2^p and rows are n + n / 2^p long, which spreads
// the strided accesses of the first stage groups over the shared-memory banks (p = 3 for groups of up to eight
// elements, p = 4 for the sixteen-element groups).
template <int PAD> __device__ __forceinline__ int fft_at(int i) { return PAD ? i + (i >> PAD) : i; }
template <int PAD> __host__ __device__ __forceinline__ int fft_row(int n) { return PAD ? n + (n >> PAD) : n; }

// FP32 twiddle tables hold tw[k + n/4] = -i tw[k] exactly (built that way), so FP32 groups derive the upper half
// of each stage's twiddles from the lower half; FP64 tables are the reference's cos/sin values and are all loaded.
template <class C2> constexpr bool TW_SYM = sizeof(C2) == 8;
// twiddle products of the butterflies. FP32: explicit single-rounding operations, so a twiddle derived by the
// rotation and the same twiddle loaded from the table multiply identically whatever the compiler would contract
// (every stage grouping gives the same bits); FP64: the plain product.
__device__ __forceinline__ float2 cmul_tw(float2 w, float2 x) {
  return make_float2(__fmaf_rn(w.x, x.x, -__fmul_rn(w.y, x.y)), __fmaf_rn(w.x, x.y, __fmul_rn(w.y, x.x)));
}
__device__ __forceinline__ double2 cmul_tw(double2 w, double2 x) { return cmul(w, x); }

template <class C2, int F, int PAD>
__device__ __forceinline__ void dit_group(C2 *s, int rows, int n, int logn, int st, const C2 *__restrict__ tw) {
  constexpr int E = 1 << F;
  const int halfn = n >> 1, lo = (1 << st) - 1;
  for (int e = threadIdx.x; e < (rows << (logn - F)); e += blockDim.x) {
    const int r = e >> (logn - F), q = e & ((1 << (logn - F)) - 1);
    const int i0 = ((q >> st) << (st + F)) + (q & lo);
    C2 *row = s + static_cast<size_t>(r) * fft_row<PAD>(n);
    C2 x[E];
#pragma unroll
    for (int j = 0; j < E; j++) x[j] = row[fft_at<PAD>(i0 + (j << st))];
#pragma unroll
    for (int f = 0; f < F; f++) {
      const int h = 1 << f, stride = halfn >> (st + f);
      // the stage's h twiddles; FP32: the upper half is the lower half times +i (the table is built with that
      // symmetry, so the value is the table's), which saves half the twiddle loads
      C2 wv[E / 2];
#pragma unroll
      for (int jj = 0; jj < h; jj++) {
        if (TW_SYM<C2> && jj >= (h >> 1) && h >= 2) wv[jj] = mk2(-wv[jj - (h >> 1)].y, wv[jj - (h >> 1)].x);
        else wv[jj] = conjd(tw[((q & lo) + (jj << st)) * stride]);
      }
#pragma unroll
      for (int j = 0; j < E; j++) {
        if (j & h) continue;
        const C2 w = wv[j & (h - 1)];
        const C2 t = cmul_tw(w, x[j + h]), u = x[j];
        x[j] = cadd(u, t);
        x[j + h] = csub(u, t);
      }
    }
#pragma unroll
    for (int j = 0; j < E; j++) row[fft_at<PAD>(i0 + (j << st))] = x[j];
  }
}
template <class C2, int F, int PAD>
__device__ __forceinline__ void dif_group(C2 *s, int rows, int n, int logn, int st, const C2 *__restrict__ tw) {
  constexpr int E = 1 << F;
  const int halfn = n >> 1, lo = (1 << st) - 1;
  for (int e = threadIdx.x; e < (rows << (logn - F)); e += blockDim.x) {
    const int r = e >> (logn - F), q = e & ((1 << (logn - F)) - 1);
    const int i0 = ((q >> st) << (st + F)) + (q & lo);
    C2 *row = s + static_cast<size_t>(r) * fft_row<PAD>(n);
    C2 x[E];
#pragma unroll
    for (int j = 0; j < E; j++) x[j] = row[fft_at<PAD>(i0 + (j << st))];
#pragma unroll
    for (int f = F - 1; f >= 0; f--) {
      const int h = 1 << f, stride = halfn >> (st + f);
      // FP32: the upper half of the stage's twiddles is the lower half times -i (see dit_group)
      C2 wv[E / 2];
#pragma unroll
      for (int jj = 0; jj < h; jj++) {
        if (TW_SYM<C2> && jj >= (h >> 1) && h >= 2) wv[jj] = mk2(wv[jj - (h >> 1)].y, -wv[jj - (h >> 1)].x);
        else wv[jj] = tw[((q & lo) + (jj << st)) * stride];
      }
#pragma unroll
      for (int j = 0; j < E; j++) {
        if (j & h) continue;
        const C2 u = x[j], v = x[j + h];
        x[j] = cadd(u, v);
        x[j + h] = cmul_tw(wv[j & (h - 1)], csub(u, v));
      }
    }
#pragma unroll
    for (int j = 0; j < E; j++) row[fft_at<PAD>(i0 + (j << st))] = x[j];
  }
}
// inverse transform (decimation in time) of `rows` rows in bit-reversed order, in place
// fmax: stages per group (1..FMAX); FMAX = 4 (16 elements per thread) raises the register count, so only kernels
// instantiated for it (with their own occupancy) take four-stage groups
template <class C2, int PAD = 0, int FMAX = 3>
__device__ void fft_inverse_dit(C2 *s, int rows, int n, int logn, const C2 *__restrict__ tw, int fmax = 3) {
  if (fmax > FMAX) fmax = FMAX;
  for (int st = 0; st < logn;) {
    const int F = logn - st >= fmax ? fmax : logn - st;
    if (FMAX >= 4 && F == 4) dit_group<C2, 4, PAD>(s, rows, n, logn, st, tw);
    else if (F == 3) dit_group<C2, 3, PAD>(s, rows, n, logn, st, tw);
    else if (F == 2) dit_group<C2, 2, PAD>(s, rows, n, logn, st, tw);
    else dit_group<C2, 1, PAD>(s, rows, n, logn, st, tw);
    __syncthreads();
    st += F;
  }
}
// forward transform (decimation in frequency) of `rows` rows in natural order, output bit-reversed, in place
template <class C2, int PAD = 0, int FMAX = 3>
__device__ void fft_forward_dif(C2 *s, int rows, int n, int logn, const C2 *__restrict__ tw, int fmax = 3) {
  if (fmax > FMAX) fmax = FMAX;
  for (int hi = logn; hi > 0;) {
    const int F = hi >= fmax ? fmax : hi;
    const int st = hi - F;
    if (FMAX >= 4 && F == 4) dif_group<C2, 4, PAD>(s, rows, n, logn, st, tw);
    else if (F == 3) dif_group<C2, 3, PAD>(s, rows, n, logn, st, tw);
    else if (F == 2) dif_group<C2, 2, PAD>(s, rows, n, logn, st, tw);
    else dif_group<C2, 1, PAD>(s, rows, n, logn, st, tw);
    __syncthreads();
    hi = st;
  }
}
// Compile-time forms of the same groups: the transform length 2^LOGN, the group's first stage ST and its size F
// are template constants, so every element and twiddle address of a thread is its base plus an immediate (no
// per-element index arithmetic). Where the padding lets a group's elements sit at a fixed step from their first
// one (rows unpadded, ST >= PAD, or a first group no wider than the padding period) the step is a constant;
// otherwise the element offsets are computed as in dit_group. Same butterflies, twiddles and order as
// dit_group / dif_group, so the same bits.
template <int PAD, int ST, int F> __host__ __device__ constexpr bool fft_fixed_step() { return PAD == 0 || ST >= PAD || (ST == 0 && F <= PAD); }
template <int PAD, int ST> __host__ __device__ constexpr int fft_step() { return PAD == 0 ? (1 << ST) : (ST >= PAD ? (1 << ST) + (1 << (ST - PAD)) : 1); }

template <class C2, int F, int PAD, int LOGN, int ST>
__device__ __forceinline__ void dit_group_c(C2 *s, int rows, const C2 *__restrict__ tw) {
  constexpr int E = 1 << F, N = 1 << LOGN, HALFN = N >> 1, LO = (1 << ST) - 1, QB = LOGN - F, RL = PAD ? N + (N >> PAD) : N;
  constexpr bool FIXED = fft_fixed_step<PAD, ST, F>();
  constexpr int STEP = fft_step<PAD, ST>();
  for (int e = threadIdx.x; e < (rows << QB); e += blockDim.x) {
    const int r = e >> QB, q = e & ((1 << QB) - 1);
    const int i0 = ((q >> ST) << (ST + F)) + (q & LO);
    C2 *row = s + r * RL, *p0 = row + fft_at<PAD>(i0);
    C2 x[E];
#pragma unroll
    for (int j = 0; j < E; j++) x[j] = FIXED ? p0[j * STEP] : row[fft_at<PAD>(i0 + (j << ST))];
#pragma unroll
    for (int f = 0; f < F; f++) {
      const int h = 1 << f, stride = HALFN >> (ST + f);
      const C2 *twb = tw + (q & LO) * stride;
      C2 wv[E / 2];
#pragma unroll
      for (int jj = 0; jj < h; jj++) {
        if (TW_SYM<C2> && jj >= (h >> 1) && h >= 2) wv[jj] = mk2(-wv[jj - (h >> 1)].y, wv[jj - (h >> 1)].x);
        else wv[jj] = conjd(twb[(jj << ST) * stride]);
      }
#pragma unroll
      for (int j = 0; j < E; j++) {
        if (j & h) continue;
        const C2 w = wv[j & (h - 1)];
        const C2 t = cmul_tw(w, x[j + h]), u = x[j];
        x[j] = cadd(u, t);
        x[j + h] = csub(u, t);
      }
    }
#pragma unroll
    for (int j = 0; j < E; j++) {
      if (FIXED) p0[j * STEP] = x[j];
      else row[fft_at<PAD>(i0 + (j << ST))] = x[j];
    }
  }
}
template <class C2, int F, int PAD, int LOGN, int ST>
__device__ __forceinline__ void dif_group_c(C2 *s, int rows, const C2 *__restrict__ tw) {
  constexpr int E = 1 << F, N = 1 << LOGN, HALFN = N >> 1, LO = (1 << ST) - 1, QB = LOGN - F, RL = PAD ? N + (N >> PAD) : N;
  constexpr bool FIXED = fft_fixed_step<PAD, ST, F>();
  constexpr int STEP = fft_step<PAD, ST>();
  for (int e = threadIdx.x; e < (rows << QB); e += blockDim.x) {
    const int r = e >> QB, q = e & ((1 << QB) - 1);
    const int i0 = ((q >> ST) << (ST + F)) + (q & LO);
    C2 *row = s + r * RL, *p0 = row + fft_at<PAD>(i0);
    C2 x[E];
#pragma unroll
    for (int j = 0; j < E; j++) x[j] = FIXED ? p0[j * STEP] : row[fft_at<PAD>(i0 + (j << ST))];
#pragma unroll
    for (int f = F - 1; f >= 0; f--) {
      const int h = 1 << f, stride = HALFN >> (ST + f);
      const C2 *twb = tw + (q & LO) * stride;
      C2 wv[E / 2];
#pragma unroll
      for (int jj = 0; jj < h; jj++) {
        if (TW_SYM<C2> && jj >= (h >> 1) && h >= 2) wv[jj] = mk2(wv[jj - (h >> 1)].y, -wv[jj - (h >> 1)].x);
        else wv[jj] = twb[(jj << ST) * stride];
      }
#pragma unroll
      for (int j = 0; j < E; j++) {
        if (j & h) continue;
        const C2 u = x[j], v = x[j + h];
        x[j] = cadd(u, v);
        x[j + h] = cmul_tw(wv[j & (h - 1)], csub(u, v));
      }
    }
#pragma unroll
    for (int j = 0; j < E; j++) {
      if (FIXED) p0[j * STEP] = x[j];
      else row[fft_at<PAD>(i0 + (j << ST))] = x[j];
    }
  }
}
// the group schedules of fft_inverse_dit / fft_forward_dif for a stage-group size FG, unrolled at compile time
template <class C2, int PAD, int LOGN, int FG, int ST = 0>
__device__ __forceinline__ void dit_sched(C2 *s, int rows, const C2 *__restrict__ tw) {
  if constexpr (ST < LOGN) {
    constexpr int F = LOGN - ST >= FG ? FG : LOGN - ST;
    dit_group_c<C2, F, PAD, LOGN, ST>(s, rows, tw);
    __syncthreads();
    dit_sched<C2, PAD, LOGN, FG, ST + F>(s, rows, tw);
  }
}
template <class C2, int PAD, int LOGN, int FG, int HI = LOGN>
__device__ __forceinline__ void dif_sched(C2 *s, int rows, const C2 *__restrict__ tw) {
  if constexpr (HI > 0) {
    constexpr int F = HI >= FG ? FG : HI;
    dif_group_c<C2, F, PAD, LOGN, HI - F>(s, rows, tw);
    __syncthreads();
    dif_sched<C2, PAD, LOGN, FG, HI - F>(s, rows, tw);
  }
}
// fft_inverse_dit / fft_forward_dif for a length 2^LOGN fixed at compile time (fmax: stages per group, 2..FMAX)
template <class C2, int PAD, int FMAX, int LOGN>
__device__ void fft_inverse_dit_c(C2 *s, int rows, const C2 *__restrict__ tw, int fmax) {
  if constexpr (FMAX >= 4) {
    if (fmax >= 4) {
      dit_sched<C2, PAD, LOGN, 4>(s, rows, tw);
      return;
    }
  }
  if constexpr (FMAX >= 3) {
    if (fmax >= 3) {
      dit_sched<C2, PAD, LOGN, 3>(s, rows, tw);
      return;
    }
  }
  dit_sched<C2, PAD, LOGN, 2>(s, rows, tw);
}
template <class C2, int PAD, int FMAX, int LOGN>
__device__ void fft_forward_dif_c(C2 *s, int rows, const C2 *__restrict__ tw, int fmax) {
  if constexpr (FMAX >= 4) {
    if (fmax >= 4) {
      dif_sched<C2, PAD, LOGN, 4>(s, rows, tw);
      return;
    }
  }
  if constexpr (FMAX >= 3) {
    if (fmax >= 3) {
      dif_sched<C2, PAD, LOGN, 3>(s, rows, tw);
      return;
    }
  }
  dif_sched<C2, PAD, LOGN, 2>(s, rows, tw);
}
__device__ __forceinline__ int bitrev(int k, int logn) { return static_cast<int>(__brev(static_cast<unsigned>(k)) >> (32 - logn)); }

// Load the Fourier coefficients of `rows` fields at latitudes js (real part) and jn (imaginary part) into
// bit-reversed rows: Y[m] = X_s[m] + i X_n[m], Y[n-m] = conj(X_s[m]) + i conj(X_n[m]); Im X[0] is dropped
// as in cpp/sphere.cpp:132.
template <class C2, int PAD = 0>
__device__ void load_pair_spectra(C2 *s, int rows, const SphDev &d, const C2 *__restrict__ fs, const C2 *__restrict__ fn, int fstride) {
  const int n = d.nlon, rl = fft_row<PAD>(n);
  for (int e = threadIdx.x; e < rows * rl; e += blockDim.x) s[e] = mk2(decltype(C2::x)(0), decltype(C2::x)(0));
  __syncthreads();
  for (int e = threadIdx.x; e < rows * d.M; e += blockDim.x) {
    const int r = e / d.M, m = e - r * d.M;
    C2 a = fs[r * fstride + m], c = fn[r * fstride + m];
    C2 *row = s + static_cast<size_t>(r) * rl;
    if (m == 0) {
      row[0] = mk2(a.x, c.x);
    } else {
      row[fft_at<PAD>(bitrev(m, d.logn))] = mk2(a.x - c.y, a.y + c.x);
      row[fft_at<PAD>(bitrev(n - m, d.logn))] = mk2(a.x + c.y, c.x - a.y);
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------------------------ grid stage
constexpr int GRID_THREADS = 256;

// four: [B][nlat][4][M]; fold: [B][nh][NSLOT][2][M]; fgrid/hsgrid: [B][nlat][nlon]
template <class R>
__global__ void __launch_bounds__(GRID_THREADS) sph_grid(SphDev d, SphTab<R> t, const typename V2<R>::type *__restrict__ four,
                                                         const double *__restrict__ fgrid, const double *__restrict__ hsgrid,
                                                         typename V2<R>::type *__restrict__ fold) {
  using C2 = typename V2<R>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2 *sm = reinterpret_cast<C2 *>(smraw);
  const int b = blockIdx.y, jh = blockIdx.x;
  const int js = jh, jn = d.nlat - 1 - jh, n = d.nlon, rl = fft_row<3>(n);  // padded rows
  const C2 *f_s = four + (static_cast<size_t>(b) * d.nlat + js) * 4 * d.M;
  const C2 *f_n = four + (static_cast<size_t>(b) * d.nlat + jn) * 4 * d.M;
  load_pair_spectra<C2, 3>(sm, 4, d, f_s, f_n, d.M);
  fft_inverse_dit<C2, 3>(sm, 4, n, d.logn, t.tw);
  // nonlinear products, cpp/sphere.cpp:348-359 (real part: southern latitude, imaginary part: northern)
  const R r2om = t.r2om[js], g = static_cast<R>(d.g);  // 1 / (2 (1 - mu^2)), the same at the mirror latitude
  const double *fr_s = fgrid + (static_cast<size_t>(b) * d.nlat + js) * n, *fr_n = fgrid + (static_cast<size_t>(b) * d.nlat + jn) * n;
  const double *hr_s = hsgrid + (static_cast<size_t>(b) * d.nlat + js) * n, *hr_n = hsgrid + (static_cast<size_t>(b) * d.nlat + jn) * n;
  const int gf = d.gflag[b];
  // the FP64 Coriolis and orography values in the arithmetic type; FP32 rounds them on the integer pipe (the
  // hardware conversion's values, without the narrow FP64 pipe)
  const R f0s = to_arith<R>(d.om2[b] * d.mu[js]), f0n = to_arith<R>(d.om2[b] * d.mu[jn]);
  C2 *rU = sm, *rV = sm + rl, *rZ = sm + 2 * rl, *rP = sm + 3 * rl, *rE = sm + 4 * rl;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int kp = fft_at<3>(k);
    const C2 U = rU[kp], V = rV[kp], Z = rZ[kp], P = rP[kp];
    C2 A, Bv, UP, VP, PE;
    {
      R eta = Z.x + ((gf & 1) ? to_arith<R>(fr_s[k]) : f0s);
      const R hs = (gf & 2) ? to_arith<R>(hr_s[k]) : R(0);
      A.x = U.x * eta; Bv.x = V.x * eta; UP.x = U.x * P.x; VP.x = V.x * P.x;
      PE.x = P.x + g * hs + (U.x * U.x + V.x * V.x) * r2om;
    }
    {
      R eta = Z.y + ((gf & 1) ? to_arith<R>(fr_n[k]) : f0n);
      const R hs = (gf & 2) ? to_arith<R>(hr_n[k]) : R(0);
      A.y = U.y * eta; Bv.y = V.y * eta; UP.y = U.y * P.y; VP.y = V.y * P.y;
      PE.y = P.y + g * hs + (U.y * U.y + V.y * V.y) * r2om;
    }
    rU[kp] = A; rV[kp] = Bv; rZ[kp] = UP; rP[kp] = VP; rE[kp] = PE;
  }
  __syncthreads();
  fft_forward_dif<C2, 3>(sm, NSLOT, n, d.logn, t.tw);
  // separate the two latitudes, normalise by nlon (cpp/sphere.cpp:128), weight and fold
  const R inv = R(1) / n, wd = t.wd[js], wj = t.w[js];
  C2 *o = fold + (static_cast<size_t>(b) * d.nh + jh) * NSLOT * 2 * d.M;
  for (int e = threadIdx.x; e < NSLOT * d.M; e += blockDim.x) {
    const int r = e / d.M, m = e - r * d.M;
    const C2 *row = sm + static_cast<size_t>(r) * rl;
    const C2 Ym = row[fft_at<3>(bitrev(m, d.logn))], Yc = conjd(row[fft_at<3>(bitrev((n - m) & (n - 1), d.logn))]);
    // X_s = (Ym + conj(Y_{n-m}))/2, X_n = -i (Ym - conj(Y_{n-m}))/2
    const R hinv = R(0.5) * inv;
    C2 Xs = cscale(cadd(Ym, Yc), hinv);
    C2 tt = csub(Ym, Yc);
    C2 Xn = mk2(hinv * tt.y, -hinv * tt.x);
    const R wt = r < 4 ? wd : wj;
    Xs = cscale(Xs, wt);
    Xn = cscale(Xn, wt);
    o[(r * 2 + 0) * d.M + m] = cadd(Xs, Xn);
    o[(r * 2 + 1) * d.M + m] = csub(Xs, Xn);
  }
}

// ------------------------------------------------------------------------------------------------ analysis + RK4
// Block: spectral coefficients (thread % COEF = coefficient, coalesced latitude-major tables) and latitude pieces
// (thread / COEF = c sums the latitude pairs jh = c, c + NCH, ...); the pieces meet in shared memory and the
// threads of piece 0 form the tendencies and apply the RK4 stage update. ANA_CHUNKS: the pieces of the 32-coefficient
// blocks (the tracer's analysis uses this form).
constexpr int ANA_CHUNKS = 8, ANA_THREADS = 32 * ANA_CHUNKS, ANA_Q = 14;



// x0: state, xs: stage input (written for stages 0-2), acc: RK4 accumulator. All [B][3][ntri].
// COEF coefficients per block (thread % COEF) and ANA_THREADS / COEF latitude pieces: 32 x 8 in general, 8 x 32 for
// grids of at most 32 latitude pairs (T <= 42), chosen by the grid only (ana_coef) like the synthesis's blocks.
__host__ __device__ constexpr int ana_coef(int nh) { return nh <= 32 ? 8 : 32; }
template <class R, int COEF>
__global__ void __launch_bounds__(ANA_THREADS) sph_analysis(SphDev d, SphTab<R> t, const typename V2<R>::type *__restrict__ fold,
                                                            StageArgs sa, double2 *__restrict__ x0, double2 *__restrict__ xs,
                                                            double2 *__restrict__ acc) {
  using C2 = typename V2<R>::type;
  constexpr int NCH = ANA_THREADS / COEF;
  __shared__ R part[NCH][ANA_Q][COEF + 1];
  const int b = blockIdx.y;
  const int lane = threadIdx.x % COEF, c = threadIdx.x / COEF;
  const int q = blockIdx.x * COEF + lane;
  const bool live = q < d.ntri;
  const int m = live ? d.trim[q] : 0, n = live ? d.trin[q] : 0, par = (n - m) & 1;
  const C2 *fb = fold + static_cast<size_t>(b) * d.nh * NSLOT * 2 * d.M;
  const int sP = par * d.M + m, sH = (1 - par) * d.M + m;  // parity slot for P and H terms
  C2 aP = mk2(R(0), R(0)), bH = aP, bP = aP, aH = aP, uP = aP, vH = aP, eP = aP;
  if (live) {
#pragma unroll 2
    for (int jh = c; jh < d.nh; jh += NCH) {
      const R P = t.Pa[static_cast<size_t>(jh) * d.ntri + q], H = t.Ha[static_cast<size_t>(jh) * d.ntri + q];
      const C2 *g = fb + static_cast<size_t>(jh) * NSLOT * 2 * d.M;
      aP = cfma(aP, g[0 * 2 * d.M + sP], P);
      aH = cfma(aH, g[0 * 2 * d.M + sH], H);
      bP = cfma(bP, g[1 * 2 * d.M + sP], P);
      bH = cfma(bH, g[1 * 2 * d.M + sH], H);
      uP = cfma(uP, g[2 * 2 * d.M + sP], P);
      vH = cfma(vH, g[3 * 2 * d.M + sH], H);
      eP = cfma(eP, g[4 * 2 * d.M + sP], P);
    }
  }
  const R v[ANA_Q] = {aP.x, aP.y, aH.x, aH.y, bP.x, bP.y, bH.x, bH.y, uP.x, uP.y, vH.x, vH.y, eP.x, eP.y};
#pragma unroll
  for (int i = 0; i < ANA_Q; i++) part[c][i][lane] = v[i];
  __syncthreads();
  R tsum[ANA_Q];
  if constexpr (NCH <= 8) {
    if (c != 0 || !live) return;
#pragma unroll
    for (int i = 0; i < ANA_Q; i++) {
      R acc_i = 0;
#pragma unroll
      for (int k = 0; k < NCH; k++) acc_i += part[k][i][lane];
      tsum[i] = acc_i;
    }
  } else {
    // many pieces: every thread sums one (value, coefficient) first, in the order of the pieces
    __shared__ R red[ANA_Q][COEF];
    for (int w = threadIdx.x; w < ANA_Q * COEF; w += ANA_THREADS) {
      const int i = w / COEF, l = w % COEF;
      R acc_i = 0;
      for (int k = 0; k < NCH; k++) acc_i += part[k][i][l];
      red[i][l] = acc_i;
    }
    __syncthreads();
    if (c != 0 || !live) return;
#pragma unroll
    for (int i = 0; i < ANA_Q; i++) tsum[i] = red[i][lane];
  }
  aP = mk2(tsum[0], tsum[1]); aH = mk2(tsum[2], tsum[3]); bP = mk2(tsum[4], tsum[5]); bH = mk2(tsum[6], tsum[7]);
  uP = mk2(tsum[8], tsum[9]); vH = mk2(tsum[10], tsum[11]); eP = mk2(tsum[12], tsum[13]);
  const R mm = static_cast<R>(m);
  // cpp/sphere.cpp:380-383: dz = -D(A,B), dd = D(B,-A) + n(n+1)/a^2 (Phi + E), df = -D(U Phi, V Phi)
  C2 kz = csub(bH, imul(aP, mm));
  C2 kd = cadd(cadd(imul(bP, mm), aH), cscale(eP, t.lapl[n]));
  C2 kf = csub(vH, imul(uP, mm));
  if (q == 0 || sa.zero) kz = kd = kf = mk2(R(0), R(0));  // cpp/sphere.cpp:387-389
  const size_t base = static_cast<size_t>(b) * 3 * d.ntri + q;
  // the RK4 state accumulates in FP64 whatever the precision of the tendencies (FP32 widened on the integer pipe)
  const double2 k[3] = {make_double2(from_arith(kz.x), from_arith(kz.y)), make_double2(from_arith(kd.x), from_arith(kd.y)),
                        make_double2(from_arith(kf.x), from_arith(kf.y))};
  // every load of the three fields is issued before any store (the buffers never alias)
  double2 xv[3], av[3];
#pragma unroll
  for (int f = 0; f < 3; f++) {
    xv[f] = x0[base + static_cast<size_t>(f) * d.ntri];
    av[f] = sa.stage > 0 ? acc[base + static_cast<size_t>(f) * d.ntri] : make_double2(0.0, 0.0);
  }
#pragma unroll
  for (int f = 0; f < 3; f++) {
    const size_t i = base + static_cast<size_t>(f) * d.ntri;
    if (sa.stage == 0) {
      acc[i] = k[f];
      xs[i] = cadd(xv[f], cscale(k[f], sa.c));
    } else if (sa.stage < 3) {
      acc[i] = cadd(av[f], cscale(k[f], 2.0));
      xs[i] = cadd(xv[f], cscale(k[f], sa.c));
    } else {
      // cpp/sphere.cpp:428-434: x += dt/6 (k1 + 2k2 + 2k3 + k4), then the del^4 filter
      double2 val = cadd(xv[f], cscale(cadd(av[f], k[f]), sa.c));
      const double fac = sa.filt[(f == 2 ? 1 : 0) * d.M + n];
      x0[i] = q == 0 ? val : cscale(val, fac);
    }
  }
}

// ------------------------------------------------------------------------------------------------ grid analysis
// set_state_grid on the device (cpp/sphere.cpp:208-234): U = u cos, V = v cos, Phi = g h, forward FFTs,
// weights and fold into slots (U wd, V wd, Phi w).
__global__ void __launch_bounds__(GRID_THREADS) sph_grid_in(SphDev d, const double *__restrict__ h, const double *__restrict__ u,
                                                            const double *__restrict__ v, double2 *__restrict__ fold) {
  extern __shared__ double2 sm[];
  const int jh = blockIdx.x, js = jh, jn = d.nlat - 1 - jh, n = d.nlon;
  const double c = d.cosl[js];
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    size_t os = static_cast<size_t>(js) * n + k, on = static_cast<size_t>(jn) * n + k;
    sm[k] = make_double2(u[os] * c, u[on] * c);
    sm[n + k] = make_double2(v[os] * c, v[on] * c);
    sm[2 * n + k] = make_double2(d.g * h[os], d.g * h[on]);
  }
  __syncthreads();
  fft_forward_dif(sm, 3, n, d.logn, d.tw);
  const double inv = 1.0 / n, wd = d.wd[js], wj = d.w[js];
  double2 *o = fold + static_cast<size_t>(jh) * 3 * 2 * d.M;
  for (int e = threadIdx.x; e < 3 * d.M; e += blockDim.x) {
    const int r = e / d.M, m = e - r * d.M;
    const double2 *row = sm + static_cast<size_t>(r) * n;
    const double2 Ym = row[bitrev(m, d.logn)], Yc = conjd(row[bitrev((n - m) & (n - 1), d.logn)]);
    double2 Xs = cscale(cadd(Ym, Yc), 0.5 * inv);
    double2 t = csub(Ym, Yc);
    double2 Xn = make_double2(0.5 * inv * t.y, -0.5 * inv * t.x);
    const double wt = r < 2 ? wd : wj;
    Xs = cscale(Xs, wt);
    Xn = cscale(Xn, wt);
    o[(r * 2 + 0) * d.M + m] = cadd(Xs, Xn);
    o[(r * 2 + 1) * d.M + m] = csub(Xs, Xn);
  }
}

// zeta = D(V, -U), delta = D(U, V) with (0,0) = 0, Phi = analysis(g h): written to the member's state
__global__ void __launch_bounds__(ANA_THREADS) sph_analysis_in(SphDev d, const double2 *__restrict__ fold, double2 *x) {
  const int q = blockIdx.x * ANA_THREADS + threadIdx.x;
  if (q >= d.ntri) return;
  const int m = d.trim[q], n = d.trin[q], par = (n - m) & 1;
  const int sP = par * d.M + m, sH = (1 - par) * d.M + m;
  double2 uP = make_double2(0, 0), uH = uP, vP = uP, vH = uP, pP = uP;
  for (int jh = 0; jh < d.nh; jh++) {
    const double P = d.Pa[static_cast<size_t>(jh) * d.ntri + q], H = d.Ha[static_cast<size_t>(jh) * d.ntri + q];
    const double2 *g = fold + static_cast<size_t>(jh) * 3 * 2 * d.M;
    uP = cfma(uP, g[0 * 2 * d.M + sP], P);
    uH = cfma(uH, g[0 * 2 * d.M + sH], H);
    vP = cfma(vP, g[1 * 2 * d.M + sP], P);
    vH = cfma(vH, g[1 * 2 * d.M + sH], H);
    pP = cfma(pP, g[2 * 2 * d.M + sP], P);
  }
  const double mm = static_cast<double>(m);
  double2 z = cadd(imul(vP, mm), uH);   // D(V, -U) = sum wd (i m V P + U H)
  double2 dl = csub(imul(uP, mm), vH);  // D(U, V) = sum wd (i m U P - V H)
  if (q == 0) z = dl = make_double2(0, 0);
  x[q] = z;
  x[d.ntri + q] = dl;
  x[2 * static_cast<size_t>(d.ntri) + q] = pP;
}

// ------------------------------------------------------------------------------------------------ diagnostics
// Per latitude pair: inverse FFTs of U, V, zeta, Phi; per-row sums of cpp/sphere.cpp:514-590 and maxima.
// rows: [B][nlat][DIAG_K]: KE row, PE row, enstrophy row, error num row, error den row, max wind, max h,
// max |h - ref|, max |ref|. Optional grids out: [4][nlat][nlon] (h, u, v, zeta) for member 0 of the call.
constexpr int DIAG_K = 9;

__device__ __forceinline__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
  return s;
}
__device__ __forceinline__ double block_max(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = -INFINITY;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s = fmax(s, red[i]);
  return s;
}

__global__ void __launch_bounds__(GRID_THREADS) sph_diag(SphDev d, const double2 *__restrict__ four, const double *__restrict__ fgrid,
                                                         const double *__restrict__ hsgrid, const double *__restrict__ refgrid,
                                                         double *__restrict__ rows, double *__restrict__ grids) {
  extern __shared__ double2 sm[];
  __shared__ double red[GRID_THREADS / 32];
  const int b = blockIdx.y, jh = blockIdx.x;
  const int js = jh, jn = d.nlat - 1 - jh, n = d.nlon;
  const double2 *f_s = four + (static_cast<size_t>(b) * d.nlat + js) * 4 * d.M;
  const double2 *f_n = four + (static_cast<size_t>(b) * d.nlat + jn) * 4 * d.M;
  load_pair_spectra(sm, 4, d, f_s, f_n, d.M);
  fft_inverse_dit(sm, 4, n, d.logn, d.tw);
  const double c = d.cosl[js];
  for (int side = 0; side < 2; side++) {
    const int j = side == 0 ? js : jn;
    const size_t go = (static_cast<size_t>(b) * d.nlat + j) * n;
    double acc[5] = {0, 0, 0, 0, 0}, mx[4] = {0, -INFINITY, 0, 0};
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      const double2 U = sm[k], V = sm[n + k], Z = sm[2 * n + k], P = sm[3 * n + k];
      const double Uv = side ? U.y : U.x, Vv = side ? V.y : V.x, Zv = side ? Z.y : Z.x, Pv = side ? P.y : P.x;
      const double h = Pv / d.g, u = Uv / c, v = Vv / c;
      const double f = fgrid[go + k], hs = hsgrid[go + k];
      acc[0] += 0.5 * h * (u * u + v * v);
      acc[1] += 0.5 * d.g * h * h + d.g * h * hs;
      acc[2] += 0.5 * (Zv + f) * (Zv + f) / h;
      const double r = refgrid[go + k] / d.g, dd = h - r;
      acc[3] += dd * dd;
      acc[4] += r * r;
      mx[0] = fmax(mx[0], hypot(u, v));
      mx[1] = fmax(mx[1], h);
      mx[2] = fmax(mx[2], fabs(dd));
      mx[3] = fmax(mx[3], fabs(r));
      if (grids) {
        const size_t gi = static_cast<size_t>(j) * n + k, ng = static_cast<size_t>(d.nlat) * n;
        grids[gi] = h;
        grids[ng + gi] = u;
        grids[2 * ng + gi] = v;
        grids[3 * ng + gi] = Zv;
      }
    }
    double out[DIAG_K];
    for (int i = 0; i < 5; i++) out[i] = block_sum(acc[i], red);
    for (int i = 0; i < 4; i++) out[5 + i] = block_max(mx[i], red);
    if (threadIdx.x == 0)
      for (int i = 0; i < DIAG_K; i++) rows[(static_cast<size_t>(b) * d.nlat + j) * DIAG_K + i] = out[i];
  }
}

// Per member: area means sum_j w_j row_j / nlon (cpp/sphere.cpp:520), error norms, and sum |coefficient|
// (cpp/sphere.cpp:449-455).
__global__ void __launch_bounds__(GRID_THREADS) sph_diag_final(SphDev d, const double *__restrict__ rows, const double2 *__restrict__ x,
                                                               int member0, Reduce *out) {
  __shared__ double red[GRID_THREADS / 32];
  __shared__ double part[9][GRID_THREADS / 32];
  const int b = member0 + blockIdx.x;
  const double2 *xb = x + static_cast<size_t>(b) * 3 * d.ntri;
  double s = 0;
  for (int i = threadIdx.x; i < 3 * d.ntri; i += blockDim.x) s += hypot(xb[i].x, xb[i].y);
  s = block_sum(s, red);
  // the latitude rows in parallel: sums 0-4 (weighted), maxima 5-8, each thread a strided subset of rows, then
  // the warps' and the block's partials
  double v[9] = {0, 0, 0, 0, 0, 0, -INFINITY, 0, 0};
  for (int j = threadIdx.x; j < d.nlat; j += blockDim.x) {
    const double *rw = rows + (static_cast<size_t>(b) * d.nlat + j) * DIAG_K;
    v[0] += d.w[j] * rw[0] / d.nlon;
    v[1] += d.w[j] * rw[1] / d.nlon;
    v[2] += d.w[j] * rw[2] / d.nlon;
    v[3] += d.w[j] * rw[3];
    v[4] += d.w[j] * rw[4];
    v[5] = fmax(v[5], rw[5]);
    v[6] = fmax(v[6], rw[6]);
    v[7] = fmax(v[7], rw[7]);
    v[8] = fmax(v[8], rw[8]);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      const double u = __shfl_down_sync(0xffffffffu, v[k], o);
      v[k] = k < 5 ? v[k] + u : fmax(v[k], u);
    }
    if (lane == 0) part[k][wid] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Reduce r;
    double ke = 0, pe = 0, en = 0, num = 0, den = 0, wmax = 0, hmax = -INFINITY, dmax = 0, rmax = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); w++) {
      ke += part[0][w];
      pe += part[1][w];
      en += part[2][w];
      num += part[3][w];
      den += part[4][w];
      wmax = fmax(wmax, part[5][w]);
      hmax = fmax(hmax, part[6][w]);
      dmax = fmax(dmax, part[7][w]);
      rmax = fmax(rmax, part[8][w]);
    }
    r.sum[0] = 0.5 * ke;
    r.sum[1] = 0.5 * pe;
    r.sum[2] = 0.5 * en;
    r.sum[3] = num;
    r.sum[4] = den;
    r.sum[5] = s;
    r.sum[6] = r.sum[7] = 0;
    r.max[0] = wmax;
    r.max[1] = hmax;
    r.max[2] = dmax;
    r.max[3] = rmax;
    out[blockIdx.x] = r;
  }
}

// The stability re-check of the reduced-precision engines (cpp/sphere.cpp:473-483 needs only the largest wind
// speed and height on the grid): FP32 inverse FFTs of U, V and Phi from the FP32 synthesis, per latitude row the
// maxima into rows[.][5] and rows[.][6] (the other entries zero), combined by sph_diag_final
__global__ void __launch_bounds__(GRID_THREADS) sph_guard32(SphDev d, SphTab<float> t, const float2 *__restrict__ four, double *__restrict__ rows) {
  extern __shared__ float2 smf[];
  __shared__ double red[GRID_THREADS / 32];
  const int b = blockIdx.y, jh = blockIdx.x;
  const int js = jh, jn = d.nlat - 1 - jh, n = d.nlon;
  const float2 *f_s = four + (static_cast<size_t>(b) * d.nlat + js) * 4 * d.M;
  const float2 *f_n = four + (static_cast<size_t>(b) * d.nlat + jn) * 4 * d.M;
  load_pair_spectra(smf, 4, d, f_s, f_n, d.M);
  fft_inverse_dit(smf, 4, n, d.logn, t.tw);
  const float ic = static_cast<float>(1.0 / d.cosl[js]), ig = static_cast<float>(1.0 / d.g);
  for (int side = 0; side < 2; side++) {
    const int j = side == 0 ? js : jn;
    float wmax = 0.0f, hmax = -INFINITY;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      const float2 U = smf[k], V = smf[n + k], P = smf[3 * n + k];
      const float u = (side ? U.y : U.x) * ic, v = (side ? V.y : V.x) * ic;
      wmax = fmaxf(wmax, sqrtf(u * u + v * v));
      hmax = fmaxf(hmax, (side ? P.y : P.x) * ig);
    }
    const double w = block_max(static_cast<double>(wmax), red), h = block_max(static_cast<double>(hmax), red);
    if (threadIdx.x == 0) {
      double *o = rows + (static_cast<size_t>(b) * d.nlat + j) * DIAG_K;
      for (int i = 0; i < DIAG_K; i++) o[i] = 0.0;
      o[5] = w;
      o[6] = h;
    }
  }
}

// synthesis of a single field's grid (reference grid for mark_reference): Phi rows of `four` -> grid
__global__ void __launch_bounds__(GRID_THREADS) sph_phi_grid(SphDev d, const double2 *__restrict__ four, double *__restrict__ out) {
  extern __shared__ double2 sm[];
  const int b = blockIdx.y, jh = blockIdx.x;
  const int js = jh, jn = d.nlat - 1 - jh, n = d.nlon;
  const double2 *f_s = four + (static_cast<size_t>(b) * d.nlat + js) * 4 * d.M + 3 * d.M;
  const double2 *f_n = four + (static_cast<size_t>(b) * d.nlat + jn) * 4 * d.M + 3 * d.M;
  load_pair_spectra(sm, 1, d, f_s, f_n, d.M);
  fft_inverse_dit(sm, 1, n, d.logn, d.tw);
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    out[(static_cast<size_t>(b) * d.nlat + js) * n + k] = sm[k].x;
    out[(static_cast<size_t>(b) * d.nlat + jn) * n + k] = sm[k].y;
  }
}

// ------------------------------------------------------------------------------------------------ transform hooks
// The reference's scalar transforms exposed for tests (cpp/sphere.cpp:138-177), in FP64 on the device.
// sph_hook_fold: per latitude pair, forward FFTs of A (and B when given), the weight (mode 0: w, the scalar
// analysis; mode 1: w / ((1 - mu^2) a), the divergence operator) and the hemispheric fold into
// fold[jh][row][parity][M] (parity 0: south + north, parity 1: south - north).
__global__ void __launch_bounds__(GRID_THREADS) sph_hook_fold(SphDev d, const double *__restrict__ A, const double *__restrict__ B, int mode,
                                                              double2 *__restrict__ fold) {
  extern __shared__ double2 sm[];
  const int jh = blockIdx.x, js = jh, jn = d.nlat - 1 - jh, n = d.nlon;
  const int rows = B ? 2 : 1;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const size_t os = static_cast<size_t>(js) * n + k, on = static_cast<size_t>(jn) * n + k;
    sm[k] = make_double2(A[os], A[on]);
    if (B) sm[n + k] = make_double2(B[os], B[on]);
  }
  __syncthreads();
  fft_forward_dif(sm, rows, n, d.logn, d.tw);
  const double inv = 1.0 / n, wt = mode ? d.wd[js] : d.w[js];
  double2 *o = fold + static_cast<size_t>(jh) * rows * 2 * d.M;
  for (int e = threadIdx.x; e < rows * d.M; e += blockDim.x) {
    const int r = e / d.M, m = e - r * d.M;
    const double2 *row = sm + static_cast<size_t>(r) * n;
    const double2 Ym = row[bitrev(m, d.logn)], Yc = conjd(row[bitrev((n - m) & (n - 1), d.logn)]);
    double2 Xs = cscale(cadd(Ym, Yc), 0.5 * inv);
    const double2 t = csub(Ym, Yc);
    double2 Xn = make_double2(0.5 * inv * t.y, -0.5 * inv * t.x);
    Xs = cscale(Xs, wt);
    Xn = cscale(Xn, wt);
    o[(r * 2 + 0) * d.M + m] = cadd(Xs, Xn);
    o[(r * 2 + 1) * d.M + m] = csub(Xs, Xn);
  }
}

// mode 0: spec = sum_j w F_m(A) P (analyze_scalar); mode 1: spec = sum_j wd (i m F_m(A) P - F_m(B) H)
// (analyze_divergence). Written into the reference layout spec[m (T+1) + n], or (packed != 0) into the engine's
// packed triangle spec[q].
__global__ void __launch_bounds__(ANA_THREADS) sph_hook_analysis(SphDev d, const double2 *__restrict__ fold, int mode, double2 *__restrict__ spec,
                                                                 int packed = 0) {
  const int q = blockIdx.x * ANA_THREADS + threadIdx.x;
  if (q >= d.ntri) return;
  const int m = d.trim[q], n = d.trin[q], par = (n - m) & 1;
  const int rows = mode ? 2 : 1;
  double2 a = make_double2(0, 0), b = a;
  for (int jh = 0; jh < d.nh; jh++) {
    const double2 *g = fold + static_cast<size_t>(jh) * rows * 2 * d.M;
    a = cfma(a, g[par * d.M + m], d.Pa[static_cast<size_t>(jh) * d.ntri + q]);
    if (mode) b = cfma(b, g[(2 + 1 - par) * d.M + m], d.Ha[static_cast<size_t>(jh) * d.ntri + q]);
  }
  spec[packed ? static_cast<size_t>(q) : static_cast<size_t>(m) * d.M + n] = mode ? csub(imul(a, static_cast<double>(m)), b) : a;
}

// F_m at both mirror latitudes of latitude pair jh from a spectrum in the reference layout (even n - m terms
// first, then the odd ones), into the Phi slot of four[lat][4][M] (the inverse FFTs follow in sph_phi_grid)
__global__ void sph_hook_synth(SphDev d, const double2 *__restrict__ spec, double2 *__restrict__ four) {
  const int jh = blockIdx.x * blockDim.x + threadIdx.x, m = blockIdx.y;
  if (jh >= d.nh) return;
  double2 se = make_double2(0, 0), so = se;
  for (int n = m; n <= d.N; n++) {
    const int q = d.tri[m] + n - m;
    const double P = d.Ps[static_cast<size_t>(q) * d.nh + jh];
    if ((n - m) & 1) so = cfma(so, spec[static_cast<size_t>(m) * d.M + n], P);
    else se = cfma(se, spec[static_cast<size_t>(m) * d.M + n], P);
  }
  const int js = jh, jn = d.nlat - 1 - jh;
  four[(static_cast<size_t>(js) * 4 + 3) * d.M + m] = cadd(se, so);
  four[(static_cast<size_t>(jn) * 4 + 3) * d.M + m] = csub(se, so);
}

const double kPi = 3.14159265358979323846;

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

}  // namespace
}  // namespace lmw

#include "sphere_split.cuh"
#include "sphere_tracer.cuh"

namespace lmw {

// ================================================================================================ engine

// The integer-pipe conversions against the hardware's, bit for bit: mismatches[0] counts float -> double,
// mismatches[1] double -> float differences (NaNs compare by NaN-ness).
__global__ void conversion_selftest(const unsigned *__restrict__ fb, int nf, const unsigned long long *__restrict__ db, int nd,
                                    int *__restrict__ mismatches) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nf) {
    const float f = __uint_as_float(fb[i]);
    const double a = f2d_int(f), b = static_cast<double>(f);
    const bool same = (a != a && b != b) || __double_as_longlong(a) == __double_as_longlong(b);
    if (!same) atomicAdd(&mismatches[0], 1);
  }
  if (i < nd) {
    const double x = __longlong_as_double(static_cast<long long>(db[i]));
    const float a = d2f_int(x), b = static_cast<float>(x);
    const bool same = (a != a && b != b) || __float_as_uint(a) == __float_as_uint(b);
    if (!same) atomicAdd(&mismatches[1], 1);
  }
}

// The bounded mbarrier wait of the tensor-core kernels, exercised on purpose: barrier 0 completes its phase (one
// arrival), barrier 1 never does (nothing arrives on it), so its wait must give up after timeout_ns and report it.
// out[0] = 1 when the completed phase was seen, out[1] = 1 when the other wait ran out.
__global__ void wait_selftest(unsigned long long timeout_ns, int *out) {
  __shared__ __align__(8) uint64_t bars[2];
  if (threadIdx.x == 0) {
    tc::bar_init(tc::su32(&bars[0]), 1);
    tc::bar_init(tc::su32(&bars[1]), 1);
    tc::bar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::su32(&bars[0])) : "memory");
    out[0] = tc::wait_for(tc::su32(&bars[0]), 0, timeout_ns) ? 1 : 0;
    out[1] = tc::wait_for(tc::su32(&bars[1]), 0, timeout_ns) ? 0 : 1;
  }
}

int wait_selftest_run(int timeout_us, int *completed, int *ran_out) {
  if (timeout_us < 1 || timeout_us > 1000000) throw InvalidArgument("timeout must be between 1 us and 1 s");
  DevBuf<int> o;
  o.alloc(2);
  LMW_CUDA(cudaMemset(o.p, 0, 2 * sizeof(int)));
  wait_selftest<<<1, 32>>>(static_cast<unsigned long long>(timeout_us) * 1000ull, o.p);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
  int h[2] = {0, 0};
  LMW_CUDA(cudaMemcpy(h, o.p, sizeof h, cudaMemcpyDeviceToHost));
  *completed = h[0];
  *ran_out = h[1];
  return 0;
}

void SphereEngine::inject_split_error(int code) {
  if (!split) throw InvalidArgument("the engine is not in split precision");
  LMW_CUDA(cudaStreamSynchronize(stream));
  LMW_CUDA(cudaMemcpy(split->err.p, &code, sizeof(int), cudaMemcpyHostToDevice));
}

int conversion_selftest_run(const uint32_t *f, int nf, const uint64_t *x, int nx, int *mismatches) {
  if (nf < 0 || nx < 0) throw InvalidArgument("counts must not be negative");
  DevBuf<unsigned> fd;
  DevBuf<unsigned long long> xd;
  DevBuf<int> md;
  fd.alloc(std::max(nf, 1));
  xd.alloc(std::max(nx, 1));
  md.alloc(2);
  if (nf) LMW_CUDA(cudaMemcpy(fd.p, f, nf * sizeof(unsigned), cudaMemcpyHostToDevice));
  if (nx) LMW_CUDA(cudaMemcpy(xd.p, x, nx * sizeof(unsigned long long), cudaMemcpyHostToDevice));
  LMW_CUDA(cudaMemset(md.p, 0, 2 * sizeof(int)));
  const int n = std::max(nf, nx);
  if (n > 0) conversion_selftest<<<(n + 255) / 256, 256>>>(fd.p, nf, xd.p, nx, md.p);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
  LMW_CUDA(cudaMemcpy(mismatches, md.p, 2 * sizeof(int), cudaMemcpyDeviceToHost));
  return 0;
}

static SphDev make_sph(const SphereEngine &e, const SphereTables &t) {
  SphDev d;
  d.N = e.N;
  d.M = e.M;
  d.nlat = e.nlat;
  d.nlon = e.nlon;
  d.nh = e.nh;
  d.ntri = e.ntri;
  d.logn = 0;
  while ((1 << d.logn) < e.nlon) d.logn++;
  d.a = e.p.radius;
  d.g = e.p.gravity;
  d.inv_a_f = static_cast<float>(1.0 / e.p.radius);
  d.div_a = fixed_div_reciprocal(e.p.radius, d.inv_a, d.inv_a_l) ? 1 : 0;
  d.Ps = t.Ps.p;
  d.Hs = t.Hs.p;
  d.Pa = t.Pa.p;
  d.Ha = t.Ha.p;
  d.mu = t.mu.p;
  d.w = t.w.p;
  d.wd = t.wd.p;
  d.cosl = t.cosl.p;
  d.r2om = t.r2om.p;
  d.kfac = t.kfac.p;
  d.lapl = t.lapl.p;
  d.tw = t.tw.p;
  d.trim = t.trim.p;
  d.trin = t.trin.p;
  d.gflag = e.gflag.p;
  d.om2 = e.om2.p;
  d.tri = t.tri.p;
  return d;
}

// The dynamic shared-memory limit is a property of each kernel function, shared by every engine of the
// process: raise it once to the device's opt-in maximum (engines of different truncations need different sizes).
static void allow_max_shared_memory() {
  static int done_for_device = -1;
  int dev = 0, optin = 0;
  LMW_CUDA(cudaGetDevice(&dev));
  if (done_for_device == dev) return;
  LMW_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const int dyn = optin - 2048;  // the kernels' static shared memory stays below 2 KB
  LMW_CUDA(cudaFuncSetAttribute(sph_grid<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  LMW_CUDA(cudaFuncSetAttribute(sph_grid<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  LMW_CUDA(cudaFuncSetAttribute(sph_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  LMW_CUDA(cudaFuncSetAttribute(sph_grid_in, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  LMW_CUDA(cudaFuncSetAttribute(split_syn, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  for (auto *k : {split_ana<false, false, 2>, split_ana<true, false, 2>, split_ana<false, true, 2>, split_ana<true, true, 2>,
                  split_ana<false, false, 3>, split_ana<true, false, 3>, split_ana<false, true, 3>, split_ana<true, true, 3>})
    LMW_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  for (auto *k : {split_ana_ws<false, 1>, split_ana_ws<true, 1>, split_ana_ws<false, 2>, split_ana_ws<true, 2>})
    LMW_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  LMW_CUDA(cudaFuncSetAttribute(split_syn_ws<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  LMW_CUDA(cudaFuncSetAttribute(split_syn_ws<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  for (int logn : {0, 6, 7, 8, 9, 10})
    for (int fmax : {3, 4})
      for (int direct : {0, 1}) LMW_CUDA(cudaFuncSetAttribute(split_grid_kernel(direct, fmax, logn), cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  done_for_device = dev;
}

static SphTab<double> tab64(const SphereTables &t) {
  return SphTab<double>{t.Ps.p, t.Hs.p, t.Pa.p, t.Ha.p, t.w.p, t.wd.p, t.r2om.p, t.kfac.p, t.lapl.p, t.tw.p};
}
static SphTab<float> tab32(const SphereTables &t) {
  return SphTab<float>{t.Ps32.p, t.Hs32.p, t.Pa32.p, t.Ha32.p, t.w32.p, t.wd32.p, t.r2om32.p, t.kfac32.p, t.lapl32.p, t.tw32.p};
}

SphereEngine::SphereEngine(const SphereConfig &c) : p(c) {
  // cpp/sphere.cpp:75-103
  if (c.truncation < 4 || c.truncation > c.max_truncation)
    throw InvalidArgument("truncation must be between 4 and " + std::to_string(c.max_truncation));
  if (c.members < 1) throw InvalidArgument("an ensemble needs at least one member");
  if (c.precision != kFP64 && c.precision != kFP32 && c.precision != kSplitBF16)
    throw InvalidArgument("precision must be 0 (FP64), 1 (FP32) or 2 (split BF16)");
  if (c.precision == kSplitBF16 && c.split_terms != 3 && c.split_terms != 6)
    throw InvalidArgument("split precision takes 3 or 6 BF16 products per term");
  B = c.members;
  tab = new SphereTables();
  HostTables &h = tab->host;
  h.build(c.truncation);
  N = h.N;
  M = h.M;
  nlat = h.nlat;
  nlon = h.nlon;
  nh = h.nh;
  ntri = h.ntri;
  t.assign(B, 0.0);
  omega_m.assign(B, c.omega);
  has_orog.assign(B, 0);
  LMW_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  // tables: coefficient-major for synthesis, latitude-major for analysis
  std::vector<double> Pa(static_cast<size_t>(nh) * ntri), Ha(Pa.size());
  for (int q = 0; q < ntri; q++)
    for (int jh = 0; jh < nh; jh++) {
      Pa[static_cast<size_t>(jh) * ntri + q] = h.P[static_cast<size_t>(q) * nh + jh];
      Ha[static_cast<size_t>(jh) * ntri + q] = h.H[static_cast<size_t>(q) * nh + jh];
    }
  auto up = [&](DevBuf<double> &dst, const std::vector<double> &src) {
    dst.alloc(src.size());
    LMW_CUDA(cudaMemcpy(dst.p, src.data(), src.size() * sizeof(double), cudaMemcpyHostToDevice));
  };
  up(tab->Ps, h.P);
  up(tab->Hs, h.H);
  up(tab->Pa, Pa);
  up(tab->Ha, Ha);
  up(tab->mu, h.mu);
  up(tab->w, h.w);
  std::vector<double> wd(nlat), cl(nlat);
  for (int j = 0; j < nlat; j++) {
    wd[j] = h.w[j] / (1 - h.mu[j] * h.mu[j]) / p.radius;  // cpp/sphere.cpp:371
    cl[j] = std::sqrt(1 - h.mu[j] * h.mu[j]);
  }
  up(tab->wd, wd);
  up(tab->cosl, cl);
  std::vector<double> r2(nlat), kf(M, 0.0), lp(M, 0.0);
  for (int j = 0; j < nlat; j++) r2[j] = 1.0 / (2 * (1 - h.mu[j] * h.mu[j]));
  for (int n = 1; n <= N; n++) {
    kf[n] = -p.radius * p.radius / (n * (n + 1.0));            // cpp/sphere.cpp:187
    lp[n] = n * (n + 1.0) / (p.radius * p.radius);             // cpp/sphere.cpp:382
  }
  up(tab->r2om, r2);
  up(tab->kfac, kf);
  up(tab->lapl, lp);
  std::vector<double2> tw(nlon / 2);
  for (int k = 0; k < nlon / 2; k++) {
    double ang = -2 * kPi * k / nlon;
    tw[k] = make_double2(std::cos(ang), std::sin(ang));
  }
  tab->tw.alloc(tw.size());
  LMW_CUDA(cudaMemcpy(tab->tw.p, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice));
  if (p.precision != kFP64) {
    auto up32 = [&](DevBuf<float> &dst, const std::vector<double> &src) {
      std::vector<float> f(src.begin(), src.end());
      dst.alloc(f.size());
      LMW_CUDA(cudaMemcpy(dst.p, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    };
    up32(tab->Ps32, h.P);
    up32(tab->Hs32, h.H);
    up32(tab->Pa32, Pa);
    up32(tab->Ha32, Ha);
    up32(tab->w32, h.w);
    up32(tab->wd32, wd);
    up32(tab->r2om32, r2);
    up32(tab->kfac32, kf);
    up32(tab->lapl32, lp);
    // FP32 twiddles: the first quarter rounded from FP64, the second quarter exactly -i times the first (the
    // FP32 FFT groups derive those from the first quarter)
    std::vector<float2> t32(tw.size());
    const size_t q4 = tw.size() / 2;
    for (size_t k = 0; k < tw.size(); k++)
      t32[k] = k < q4 || q4 == 0 ? make_float2(static_cast<float>(tw[k].x), static_cast<float>(tw[k].y)) : make_float2(t32[k - q4].y, -t32[k - q4].x);
    tab->tw32.alloc(t32.size());
    LMW_CUDA(cudaMemcpy(tab->tw32.p, t32.data(), t32.size() * sizeof(float2), cudaMemcpyHostToDevice));
  }
  std::vector<int> tm(ntri), tn(ntri);
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= N; n++) {
      tm[h.tri[m] + n - m] = m;
      tn[h.tri[m] + n - m] = n;
    }
  auto upi = [&](DevBuf<int> &dst, const std::vector<int> &src) {
    dst.alloc(src.size());
    LMW_CUDA(cudaMemcpy(dst.p, src.data(), src.size() * sizeof(int), cudaMemcpyHostToDevice));
  };
  upi(tab->trim, tm);
  upi(tab->trin, tn);
  upi(tab->tri, h.tri);
  const size_t nst = static_cast<size_t>(B) * 3 * ntri * 2;
  x0.alloc(nst);
  xs.alloc(nst);
  if (p.precision == kSplitBF16) xs2.alloc(nst);
  acc.alloc(nst);
  four.alloc(static_cast<size_t>(B) * nlat * 4 * M * 2);
  fold.alloc(static_cast<size_t>(B) * nh * NSLOT * 2 * M * 2);
  if (p.precision != kFP64) {
    four32.alloc(static_cast<size_t>(B) * nlat * 4 * M * 2);
    fold32.alloc(static_cast<size_t>(B) * nh * NSLOT * 2 * M * 2);
  }
  fgrid.alloc(static_cast<size_t>(B) * ngrid());
  hsgrid.alloc(static_cast<size_t>(B) * ngrid());
  refgrid.alloc(static_cast<size_t>(B) * ngrid());
  filt.alloc(2 * M);
  diagrows.alloc(static_cast<size_t>(B) * nlat * DIAG_K);
  gridin.alloc(4 * ngrid());
  dred.alloc(B);
  hred.alloc(B);
  gflag.alloc(B);
  om2.alloc(B);
  gflag.zero(stream);
  om2.zero(stream);
  gflag_h.assign(B, 0);
  hstage.alloc(std::max<size_t>(4 * ngrid(), static_cast<size_t>(3) * 2 * nspec_ref()));
  if (p.precision == kSplitBF16) {
    split = new SplitPlan();
    build_split_plan(*split, h, B, p.split_terms);
    {
      int dev = 0;
      LMW_CUDA(cudaGetDevice(&dev));
      LMW_CUDA(cudaDeviceGetAttribute(&split->nsm, cudaDevAttrMultiProcessorCount, dev));
    }

  }
  x0.zero(stream);
  xs.zero(stream);
  xs2.zero(stream);
  hsgrid.zero(stream);
  refgrid.zero(stream);
  allow_max_shared_memory();
  for (int b = 0; b < B; b++) set_axis_tilt(0, b);
  LMW_CUDA(cudaStreamSynchronize(stream));
  autotune_split();
}

SphereEngine::~SphereEngine() {
  for (const ChunkGraph &cg : graphs) cudaGraphExecDestroy(cg.exec);
  if (stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
  delete split;
  delete tab;
}

// the tensor-core kernels record a nonzero code when a bounded wait ran out
void SphereEngine::check_split_status() {
  if (!split) return;
  int e = 0;
  LMW_CUDA(cudaMemcpyAsync(&e, split->err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  if (e) throw DeviceError("a wait on the tensor cores timed out in the split-precision Legendre transforms");
}

static void check_member(const SphereEngine &e, int member) {
  if (member < 0 || member >= e.B) throw InvalidArgument("member index out of range");
}

// cpp/sphere.cpp:111-118 (with the member's own rotation rate)
void SphereEngine::upload_member_flags(int member) {
  const double o2 = 2 * omega_m[member];
  LMW_CUDA(cudaStreamSynchronize(stream));
  LMW_CUDA(cudaMemcpy(gflag.p + member, &gflag_h[member], sizeof(int), cudaMemcpyHostToDevice));
  LMW_CUDA(cudaMemcpy(om2.p + member, &o2, sizeof(double), cudaMemcpyHostToDevice));
}

void SphereEngine::set_axis_tilt(double alpha, int member) {
  check_member(*this, member);
  // an untilted grid is f = (2 Omega) mu exactly (the tilt terms are signed zeros): the grid kernels compute it
  gflag_h[member] = (gflag_h[member] & ~1) | (alpha != 0.0 ? 1 : 0);
  upload_member_flags(member);
  const HostTables &h = tab->host;
  std::vector<double> f(ngrid());
  for (int j = 0; j < nlat; j++)
    for (int k = 0; k < nlon; k++) {
      double lam = 2 * kPi * k / nlon, c = std::sqrt(1 - h.mu[j] * h.mu[j]);
      f[static_cast<size_t>(j) * nlon + k] = 2 * omega_m[member] * (-std::cos(lam) * c * std::sin(alpha) + h.mu[j] * std::cos(alpha));
    }
  LMW_CUDA(cudaStreamSynchronize(stream));
  LMW_CUDA(cudaMemcpy(fgrid.p + static_cast<size_t>(member) * ngrid(), f.data(), ngrid() * sizeof(double), cudaMemcpyHostToDevice));
}

void SphereEngine::set_omega(double omega, int member) {
  check_member(*this, member);
  omega_m[member] = omega;
  set_axis_tilt(0, member);
}

// cpp/sphere.cpp:105-109
void SphereEngine::set_orography(const double *hs, size_t n, int member) {
  check_member(*this, member);
  if (n != ngrid()) throw InvalidArgument("grid size mismatch");
  LMW_CUDA(cudaStreamSynchronize(stream));
  LMW_CUDA(cudaMemcpy(hsgrid.p + static_cast<size_t>(member) * ngrid(), hs, n * sizeof(double), cudaMemcpyHostToDevice));
  has_orog[member] = 1;
  gflag_h[member] |= 2;
  upload_member_flags(member);
}

void SphereEngine::synth_grids(int member_first, int count) {
  SphDev d = make_sph(*this, *tab);
  const size_t st = static_cast<size_t>(member_first) * 3 * ntri;
  const size_t fo = static_cast<size_t>(member_first) * nlat * 4 * M;
  const int L = syn_lats(nh);
  dim3 g((nh + L - 1) / L, M, count);
  auto *k = L == 8 ? sph_synth<double, 8> : sph_synth<double, 32>;
  k<<<g, SYN_THREADS, 0, stream>>>(d, tab64(*tab), reinterpret_cast<const double2 *>(x0.p) + st, reinterpret_cast<double2 *>(four.p) + fo);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
}

// cpp/sphere.cpp:236-239: remember the current height grid
void SphereEngine::mark_reference(int member) {
  check_member(*this, member);
  SphDev d = make_sph(*this, *tab);
  synth_grids(member, 1);
  const size_t smem = static_cast<size_t>(nlon) * sizeof(double2);
  sph_phi_grid<<<dim3(nh, 1), GRID_THREADS, smem, stream>>>(d, reinterpret_cast<const double2 *>(four.p) + static_cast<size_t>(member) * nlat * 4 * M,
                                                        refgrid.p + static_cast<size_t>(member) * ngrid());
  LMW_LAUNCH_CHECK();
  g_launches += 1;
  if (has_tracer) synth_tracer_grid(member, refq.p + static_cast<size_t>(member) * ngrid());
  LMW_CUDA(cudaStreamSynchronize(stream));
}

void SphereEngine::analyze_grids_to_state(int member) {
  split_packed = false;
  SphDev d = make_sph(*this, *tab);
  const size_t smem = 5 * static_cast<size_t>(nlon) * sizeof(double2);
  const size_t ng = ngrid();
  sph_grid_in<<<nh, GRID_THREADS, smem, stream>>>(d, gridin.p, gridin.p + ng, gridin.p + 2 * ng, reinterpret_cast<double2 *>(fold.p));
  sph_analysis_in<<<(ntri + ANA_THREADS - 1) / ANA_THREADS, ANA_THREADS, 0, stream>>>(
      d, reinterpret_cast<const double2 *>(fold.p), reinterpret_cast<double2 *>(x0.p) + static_cast<size_t>(member) * 3 * ntri);
  LMW_LAUNCH_CHECK();
  g_launches += 2;
}

// cpp/sphere.cpp:217-234
void SphereEngine::set_state_grid(const double *h, const double *u, const double *v, size_t n, int member) {
  check_member(*this, member);
  if (n != ngrid()) throw InvalidArgument("grid size mismatch");
  LMW_CUDA(cudaStreamSynchronize(stream));
  std::memcpy(hstage.p, h, n * sizeof(double));
  std::memcpy(hstage.p + n, u, n * sizeof(double));
  std::memcpy(hstage.p + 2 * n, v, n * sizeof(double));
  LMW_CUDA(cudaMemcpyAsync(gridin.p, hstage.p, 3 * n * sizeof(double), cudaMemcpyHostToDevice, stream));
  // grid_in expects (h, u, v) in this order
  analyze_grids_to_state(member);
  t[member] = 0;
  mark_reference(member);
}

// cpp/sphere.cpp:138-149, 150-162, 164-177: the transforms of one field, through device scratch (the member-0
// transform buffers, which every stage overwrites anyway)
void SphereEngine::hook_analysis(const double *A, const double *Bg, size_t n, double *spec) {
  if (n != ngrid()) throw InvalidArgument("grid size mismatch");
  LMW_CUDA(cudaStreamSynchronize(stream));
  if (hookspec.n < 2 * nspec_ref()) hookspec.alloc(2 * nspec_ref());
  SphDev d = make_sph(*this, *tab);
  std::memcpy(hstage.p, A, n * sizeof(double));
  if (Bg) std::memcpy(hstage.p + n, Bg, n * sizeof(double));
  LMW_CUDA(cudaMemcpyAsync(gridin.p, hstage.p, (Bg ? 2 : 1) * n * sizeof(double), cudaMemcpyHostToDevice, stream));
  LMW_CUDA(cudaMemsetAsync(hookspec.p, 0, hookspec.bytes(), stream));
  const size_t smem = 2 * static_cast<size_t>(nlon) * sizeof(double2);
  sph_hook_fold<<<nh, GRID_THREADS, smem, stream>>>(d, gridin.p, Bg ? gridin.p + n : nullptr, Bg ? 1 : 0, reinterpret_cast<double2 *>(fold.p));
  sph_hook_analysis<<<(ntri + ANA_THREADS - 1) / ANA_THREADS, ANA_THREADS, 0, stream>>>(d, reinterpret_cast<const double2 *>(fold.p), Bg ? 1 : 0,
                                                                                        reinterpret_cast<double2 *>(hookspec.p));
  LMW_LAUNCH_CHECK();
  g_launches += 2;
  LMW_CUDA(cudaMemcpyAsync(hstage.p, hookspec.p, 2 * nspec_ref() * sizeof(double), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  std::memcpy(spec, hstage.p, 2 * nspec_ref() * sizeof(double));
}

void SphereEngine::analyze_scalar(const double *grid, size_t n, double *spec) { hook_analysis(grid, nullptr, n, spec); }

void SphereEngine::analyze_divergence(const double *A, const double *Bg, size_t n, double *spec) {
  if (!A || !Bg) throw InvalidArgument("analyze_divergence: null grid");
  hook_analysis(A, Bg, n, spec);
}

void SphereEngine::synthesize_scalar(const double *spec, double *grid, size_t n) {
  if (n != ngrid()) throw InvalidArgument("grid size mismatch");
  LMW_CUDA(cudaStreamSynchronize(stream));
  if (hookspec.n < 2 * nspec_ref()) hookspec.alloc(2 * nspec_ref());
  SphDev d = make_sph(*this, *tab);
  std::memcpy(hstage.p, spec, 2 * nspec_ref() * sizeof(double));
  LMW_CUDA(cudaMemcpyAsync(hookspec.p, hstage.p, 2 * nspec_ref() * sizeof(double), cudaMemcpyHostToDevice, stream));
  sph_hook_synth<<<dim3((nh + 127) / 128, M), 128, 0, stream>>>(d, reinterpret_cast<const double2 *>(hookspec.p), reinterpret_cast<double2 *>(four.p));
  const size_t smem = static_cast<size_t>(nlon) * sizeof(double2);
  sph_phi_grid<<<dim3(nh, 1), GRID_THREADS, smem, stream>>>(d, reinterpret_cast<const double2 *>(four.p), gridin.p);
  LMW_LAUNCH_CHECK();
  g_launches += 2;
  LMW_CUDA(cudaMemcpyAsync(hstage.p, gridin.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  std::memcpy(grid, hstage.p, n * sizeof(double));
}

void SphereEngine::to_packed(const double *ref, double *packed) {
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= N; n++) {
      size_t q = static_cast<size_t>(tab->host.tri[m] + n - m), r = static_cast<size_t>(m) * M + n;
      packed[2 * q] = ref[2 * r];
      packed[2 * q + 1] = ref[2 * r + 1];
    }
}
void SphereEngine::from_packed(const double *packed, double *ref) {
  std::memset(ref, 0, nspec_ref() * 2 * sizeof(double));
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= N; n++) {
      size_t q = static_cast<size_t>(tab->host.tri[m] + n - m), r = static_cast<size_t>(m) * M + n;
      ref[2 * r] = packed[2 * q];
      ref[2 * r + 1] = packed[2 * q + 1];
    }
}

// packed triangles [B][3][ntri] <-> reference layout [3][B][M*M] (zeros where n < m). grid: (ceil(M*M/256), 3, B)
__global__ void state_to_ref(SphDev d, const double2 *__restrict__ x, double2 *__restrict__ ref, int B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, f = blockIdx.y, b = blockIdx.z;
  if (i >= d.M * d.M) return;
  const int m = i / d.M, n = i - m * d.M;
  ref[(static_cast<size_t>(f) * B + b) * d.M * d.M + i] =
      n >= m ? x[(static_cast<size_t>(b) * 3 + f) * d.ntri + d.tri[m] + n - m] : make_double2(0.0, 0.0);
}
__global__ void state_from_ref(SphDev d, const double2 *__restrict__ ref, double2 *__restrict__ x, int B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, f = blockIdx.y, b = blockIdx.z;
  if (i >= d.M * d.M) return;
  const int m = i / d.M, n = i - m * d.M;
  if (n >= m) x[(static_cast<size_t>(b) * 3 + f) * d.ntri + d.tri[m] + n - m] = ref[(static_cast<size_t>(f) * B + b) * d.M * d.M + i];
}

double *SphereEngine::device_refstates() {
  const size_t need = static_cast<size_t>(3) * B * M * M * 2;
  if (refstates.n < need) refstates.alloc(need);
  return refstates.p;
}
double *SphereEngine::states_to_ref() {
  double *r = device_refstates();
  SphDev d = make_sph(*this, *tab);
  state_to_ref<<<dim3((M * M + 255) / 256, 3, B), 256, 0, stream>>>(d, reinterpret_cast<const double2 *>(x0.p), reinterpret_cast<double2 *>(r), B);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
  return r;
}
void SphereEngine::states_from_ref() {
  SphDev d = make_sph(*this, *tab);
  state_from_ref<<<dim3((M * M + 255) / 256, 3, B), 256, 0, stream>>>(d, reinterpret_cast<const double2 *>(refstates.p), reinterpret_cast<double2 *>(x0.p), B);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
  split_packed = false;
}

void SphereEngine::set_state(const double *zeta, const double *delta, const double *phi, double time, int member) {
  check_member(*this, member);
  split_packed = false;
  LMW_CUDA(cudaStreamSynchronize(stream));
  const size_t pk = static_cast<size_t>(ntri) * 2;
  to_packed(zeta, hstage.p);
  to_packed(delta, hstage.p + pk);
  to_packed(phi, hstage.p + 2 * pk);
  LMW_CUDA(cudaMemcpyAsync(x0.p + static_cast<size_t>(member) * 3 * pk, hstage.p, 3 * pk * sizeof(double), cudaMemcpyHostToDevice, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  t[member] = time;
}

void SphereEngine::get_state(double *zeta, double *delta, double *phi, int member) {
  check_member(*this, member);
  const size_t pk = static_cast<size_t>(ntri) * 2;
  LMW_CUDA(cudaMemcpyAsync(hstage.p, x0.p + static_cast<size_t>(member) * 3 * pk, 3 * pk * sizeof(double), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  if (zeta) from_packed(hstage.p, zeta);
  if (delta) from_packed(hstage.p + pk, delta);
  if (phi) from_packed(hstage.p + 2 * pk, phi);
}

// cpp/sphere.cpp:301-311
void SphereEngine::add_mode(int n, int m, double amplitude, double mean_depth, int member) {
  check_member(*this, member);
  if (m < 0 || n < std::max(m, 1) || n > N) throw InvalidArgument("mode (n, m) needs 0 <= m <= n <= truncation and n >= 1");
  std::vector<double> z(2 * nspec_ref(), 0.0), ph(2 * nspec_ref(), 0.0);
  ph[0] = p.gravity * mean_depth * std::sqrt(2.0);
  ph[2 * (static_cast<size_t>(m) * M + n)] += p.gravity * amplitude * (m == 0 ? 1.0 : 0.5);
  set_state(z.data(), z.data(), ph.data(), 0.0, member);
  mark_reference(member);
}

// cpp/sphere.cpp:313-336. The seeded coefficients and their grid rms are formed on the host in the reference's
// order; the scaled increment is added to the device state.
void SphereEngine::perturb(double amplitude, uint64_t seed, int max_wave, int member) {
  check_member(*this, member);
  if (max_wave < 1 || max_wave > N) throw InvalidArgument("max_wave must be between 1 and the truncation");
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 12345;
  std::vector<cplx> add(nspec_ref(), 0);
  for (int m = 0; m <= max_wave; m++)
    for (int n = std::max(m, 1); n <= max_wave; n++) {
      double re = irwin_hall(st), im = m == 0 ? 0.0 : irwin_hall(st);
      add[static_cast<size_t>(m) * M + n] = cplx(re, im);
    }
  std::vector<double> g;
  tab->host.synthesize(add, g);
  const std::vector<double> &w = tab->host.w;
  double ms = 0, wsum = 0;
  for (int j = 0; j < nlat; j++)
    for (int k = 0; k < nlon; k++) {
      double x = g[static_cast<size_t>(j) * nlon + k];
      ms += w[j] * x * x;
      wsum += w[j];
    }
  double rms = std::sqrt(ms / wsum);
  double scale = rms > 0 ? amplitude / rms * p.gravity : 0;
  std::vector<double> z(2 * nspec_ref()), d(2 * nspec_ref()), ph(2 * nspec_ref());
  get_state(z.data(), d.data(), ph.data(), member);
  cplx *phc = reinterpret_cast<cplx *>(ph.data());
  for (size_t i = 0; i < nspec_ref(); i++) phc[i] += add[i] * scale;
  set_state(z.data(), d.data(), ph.data(), 0.0, member);
  mark_reference(member);
}

// Seeded balanced turbulence (this project's benchmark initialiser; the same definition as the oracle's
// or_sphere_turbulence_grids): complex-Gaussian vorticity for 1 <= n <= nforce with a kinetic-energy spectrum
// proportional to n^-3 and the largest grid wind equal to max_wind, zero divergence, h = mean + f psi / g less
// the area mean of f psi / g.
void SphereEngine::turbulence(uint64_t seed, double mean_height, double max_wind, int nforce, int member) {
  check_member(*this, member);
  const HostTables &h = tab->host;
  const double a = p.radius, a2 = a * a;
  std::vector<cplx> z(nspec_ref(), 0), zero(nspec_ref(), 0), psi(nspec_ref(), 0);
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 424242;
  nforce = std::min(nforce, N);
  for (int n = 1; n <= nforce; n++) {
    for (int m = 0; m <= n; m++) {
      double re = irwin_hall(st), im = m == 0 ? 0.0 : irwin_hall(st);
      z[static_cast<size_t>(m) * M + n] = cplx(re, im);
    }
    double e = 0;
    for (int m = 0; m <= n; m++) {
      cplx c = z[static_cast<size_t>(m) * M + n];
      e += 0.25 * (m == 0 ? 1.0 : 2.0) * a2 * (c.real() * c.real() + c.imag() * c.imag()) / (n * (n + 1.0));
    }
    double target = 1.0 / (static_cast<double>(n) * n * n);
    double sc = e > 0 ? std::sqrt(target / e) : 0.0;
    for (int m = 0; m <= n; m++) z[static_cast<size_t>(m) * M + n] *= sc;
  }
  std::vector<double> U, V;
  h.winds(z, zero, a, U, V);
  double wmax = 0;
  for (int j = 0; j < nlat; j++) {
    double c = std::sqrt(1 - h.mu[j] * h.mu[j]);
    for (int k = 0; k < nlon; k++) {
      size_t i = static_cast<size_t>(j) * nlon + k;
      double sp = std::sqrt(U[i] * U[i] + V[i] * V[i]) / c;
      wmax = wmax < sp ? sp : wmax;
    }
  }
  double gsc = wmax > 0 ? max_wind / wmax : 0.0;
  for (auto &c : z) c *= gsc;
  h.winds(z, zero, a, U, V);
  std::vector<double> hh, uu(ngrid()), vv(ngrid());
  for (int j = 0; j < nlat; j++) {
    double c = std::sqrt(1 - h.mu[j] * h.mu[j]);
    for (int k = 0; k < nlon; k++) {
      size_t i = static_cast<size_t>(j) * nlon + k;
      uu[i] = U[i] / c;
      vv[i] = V[i] / c;
    }
  }
  for (int m = 0; m <= N; m++)
    for (int n = std::max(m, 1); n <= N; n++) psi[static_cast<size_t>(m) * M + n] = z[static_cast<size_t>(m) * M + n] * (-a2 / (n * (n + 1.0)));
  h.synthesize(psi, hh);
  for (int j = 0; j < nlat; j++) {
    double f = 2 * omega_m[member] * h.mu[j];
    for (int k = 0; k < nlon; k++) {
      size_t i = static_cast<size_t>(j) * nlon + k;
      hh[i] = f * hh[i] / p.gravity;
    }
  }
  // remove the Gaussian-quadrature area mean of the balanced part: the mean height is mean_height
  double sum = 0;
  for (int j = 0; j < nlat; j++) {
    double row = 0;
    for (int k = 0; k < nlon; k++) row += hh[static_cast<size_t>(j) * nlon + k];
    sum += h.w[j] * row / nlon;
  }
  const double hmean = 0.5 * sum;
  for (auto &x : hh) x = mean_height + (x - hmean);
  set_state_grid(hh.data(), uu.data(), vv.data(), ngrid(), member);
}

// del^4 filter factors for this step size (cpp/sphere.cpp:392-405), by total wavenumber n
void SphereEngine::upload_filter(double dt) {
  if (filt_dt == dt) return;
  std::vector<double> f(2 * M, 1.0);
  if (p.diffusion > 0) {
    const double a2 = p.radius * p.radius;
    for (int n = 1; n <= N; n++) {
      double l = n * (n + 1.0);
      double kv = (l - 2) / a2, kp = l / a2;
      f[n] = std::exp(-p.diffusion * kv * kv * dt);
      f[M + n] = std::exp(-p.diffusion * kp * kp * dt);
    }
  }
  LMW_CUDA(cudaStreamSynchronize(stream));
  LMW_CUDA(cudaMemcpy(filt.p, f.data(), 2 * M * sizeof(double), cudaMemcpyHostToDevice));
  filt_dt = dt;
}

// One RK4 stage in the engine's precision: FP64 tables and buffers, or FP32 (tendencies in FP32, the state in FP64)
template <class R>
static void stage_kernels(const SphDev &d, const SphTab<R> &t, int B, int stage, double dt, const double *filt, const double2 *in,
                          typename V2<R>::type *four, typename V2<R>::type *fold, double2 *x0, double2 *xs, double2 *acc,
                          const double *fgrid, const double *hsgrid, cudaStream_t stream, int which = -1, int zero = 0) {
  const size_t smem = 5 * static_cast<size_t>(fft_row<3>(d.nlon)) * sizeof(typename V2<R>::type);  // padded FFT rows
  StageArgs sa;
  sa.stage = stage;
  sa.c = stage < 2 ? 0.5 * dt : (stage == 2 ? dt : dt / 6);
  sa.filt = filt;
  sa.zero = zero;
  if (which < 0 || which == 0) {
    if (syn_lats(d.nh) == 8)
      sph_synth<R, 8><<<dim3((d.nh + 7) / 8, d.M, B), SYN_THREADS, 0, stream>>>(d, t, in, four);
    else
      sph_synth<R, 32><<<dim3((d.nh + 31) / 32, d.M, B), SYN_THREADS, 0, stream>>>(d, t, in, four);
  }
  if (which < 0 || which == 1) sph_grid<R><<<dim3(d.nh, B), GRID_THREADS, smem, stream>>>(d, t, four, fgrid, hsgrid, fold);
  if (which < 0 || which == 2)
  {
    if (ana_coef(d.nh) == 8)
      sph_analysis<R, 8><<<dim3((d.ntri + 7) / 8, B), ANA_THREADS, 0, stream>>>(d, t, fold, sa, x0, xs, acc);
    else
      sph_analysis<R, 32><<<dim3((d.ntri + 31) / 32, B), ANA_THREADS, 0, stream>>>(d, t, fold, sa, x0, xs, acc);
  }
}

// One RK4 stage in split precision: tensor-core synthesis, FP32 grid stage, tensor-core analysis with the RK4
// update (which also packs the next stage's synthesis operands)
// xs, xs2: the stage inputs (rounded to FP32, in the first half of each FP64 buffer) that the linear-exact form keeps,
// in turn (stage 0 writes xs, 1 reads xs and writes xs2, 2 reads xs2 and writes xs, 3 reads xs): an analysis CTA
// reads neighbouring coefficients that other CTAs update. The second half of xs holds the state rounded to FP32
// (written by the last stage and by split_pack_state); acc is the FP32 RK4 accumulator (first half).
static void split_stage(const SphDev &d, const SphTab<float> &t, const SplitPlan &sp, int B, int stage, double dt,
                        const double *filt, float2 *fold, double2 *x0, double2 *xs, double2 *xs2, double2 *acc, const double *fgrid,
                        const double *hsgrid, cudaStream_t stream, int which = -1) {
  SplitDev sd = split_dev(sp);
  sd.fold = fold;
  StageArgs sa;
  sa.stage = stage;
  sa.c = stage < 2 ? 0.5 * dt : (stage == 2 ? dt : dt / 6);
  sa.c32 = static_cast<float>(sa.c);
  sa.filt = filt;
  if (which < 0 || which == 0) {
    if (sp.syn_ws > 0) {
      size_t smem = 0;
      int buf_cols = 0, slot = 0;
      if (!syn_ws_layout(sp, sp.syn_split, sp.ns_syn, sp.syn_ws, &smem, &buf_cols, &slot))
        throw InvalidArgument("split precision: the warp-specialised synthesis does not fit");
      const int items = d.M * sp.ntiles * sp.syn_split;
      auto *k = sp.syn_ws == 2 ? split_syn_ws<2> : split_syn_ws<1>;
      k<<<std::min(items, sp.nsm * sp.syn_ws), SPLIT_SYN_WS_THREADS, smem, stream>>>(d, sd, B, sp.ns_syn, buf_cols, slot);
    } else {
      split_syn<<<dim3(sp.ntiles, sp.syn_split, d.M), SPLIT_THREADS, sp.smem_syn, stream>>>(d, sd, B, sp.ns_syn);
    }
  }
  if (which < 0 || which == 1) {
    const dim3 grid(d.nh / sp.jb, B);
    const size_t bytes = 5 * static_cast<size_t>(sp.jb) * fft_row<3>(d.nlon) * sizeof(float2);
    // the FFT group bound sets the kernel's register budget: 4 (sixteen elements a thread) two CTAs per SM,
    // else three
    auto *k = split_grid_kernel(sp.direct, sp.fgrp >= 4 ? 4 : 3, sp.grid_fixed ? d.logn : 0);
    k<<<grid, GRID_THREADS, bytes, stream>>>(d, t, sd, fgrid, hsgrid);
  }
  if (which < 0 || which == 2) {
    if (sp.ana_both && 2 * sp.ra_pair > 512) throw InvalidArgument("split precision: both parities' accumulators exceed tensor memory");
    const int items = d.M * (sp.ana_both ? 1 : 2) * sp.ntiles;
    float2 *ys = reinterpret_cast<float2 *>(xs), *ys2 = reinterpret_cast<float2 *>(xs2);
    float2 *xf = ys + static_cast<size_t>(B) * 3 * d.ntri, *ac = reinterpret_cast<float2 *>(acc);
    const float2 *xin = stage == 1 || stage == 3 ? ys : (stage == 2 ? ys2 : nullptr);
    float2 *xout = !sp.lin_exact || stage == 3 ? nullptr : (stage == 1 ? ys2 : ys);
    if (sp.ana_ws > 0 && sp.direct) {
      size_t smem = 0;
      int buf_cols = 0, slot = 0;
      if (!ws_layout(sp, sp.ana_both, sp.ns_ana, sp.ana_ws, &smem, &buf_cols, &slot))
        throw InvalidArgument("split precision: the warp-specialised analysis does not fit");
      const int grid = std::min(items, sp.nsm * sp.ana_ws);
      auto *k = sp.ana_ws == 2 ? (sp.ana_both ? split_ana_ws<true, 2> : split_ana_ws<false, 2>)
                               : (sp.ana_both ? split_ana_ws<true, 1> : split_ana_ws<false, 1>);
      k<<<grid, SPLIT_WS_THREADS, smem, stream>>>(d, sd, t, sa, B, sp.ns_ana, buf_cols, slot, x0, xf, xin, xout, ac);
      return;
    }
    const int grid = sp.ana_grid > 0 ? std::min(items, sp.ana_grid) : items;
    auto *k = sp.ana_minb >= 3
                  ? (sp.ana_both ? (sp.direct ? split_ana<true, true, 3> : split_ana<true, false, 3>)
                                 : (sp.direct ? split_ana<false, true, 3> : split_ana<false, false, 3>))
                  : (sp.ana_both ? (sp.direct ? split_ana<true, true, 2> : split_ana<true, false, 2>)
                                 : (sp.direct ? split_ana<false, true, 2> : split_ana<false, false, 2>));
    k<<<grid, SPLIT_ANA_THREADS, sp.smem_ana, stream>>>(d, sd, t, sa, B, sp.ns_ana, x0, xf, xin, xout, ac);
  }
}

void SphereEngine::launch_stage(int stage, double dt) {
  SphDev d = make_sph(*this, *tab);
  const double2 *in = reinterpret_cast<const double2 *>(stage == 0 ? x0.p : xs.p);
  double2 *X0 = reinterpret_cast<double2 *>(x0.p), *XS = reinterpret_cast<double2 *>(xs.p), *AC = reinterpret_cast<double2 *>(acc.p);
  if (p.precision == kFP64 && has_tracer) {
    // the tracer's kernels read the flow's stage input and its synthesised winds before the flow's analysis
    // overwrites the stage input
    for (int k = 0; k < 3; k++) {
      stage_kernels<double>(d, tab64(*tab), B, stage, dt, filt.p, in, reinterpret_cast<double2 *>(four.p), reinterpret_cast<double2 *>(fold.p),
                            X0, XS, AC, fgrid.p, hsgrid.p, stream, k, advect_only ? 1 : 0);
      tracer_stage(stage, dt, k);
    }
    g_launches += 6;
  } else if (p.precision == kFP64) {
    stage_kernels<double>(d, tab64(*tab), B, stage, dt, filt.p, in, reinterpret_cast<double2 *>(four.p), reinterpret_cast<double2 *>(fold.p),
                          X0, XS, AC, fgrid.p, hsgrid.p, stream);
    g_launches += 3;
  } else if (p.precision == kFP32) {
    stage_kernels<float>(d, tab32(*tab), B, stage, dt, filt.p, in, reinterpret_cast<float2 *>(four32.p), reinterpret_cast<float2 *>(fold32.p),
                         X0, XS, AC, fgrid.p, hsgrid.p, stream);
    g_launches += 3;
  } else {
    split_stage(d, tab32(*tab), *split, B, stage, dt, filt.p, reinterpret_cast<float2 *>(fold32.p), X0, XS, XS2(), AC, fgrid.p,
                hsgrid.p, stream);
    g_launches += 3;
  }
  LMW_LAUNCH_CHECK();
}

// ------------------------------------------------------------------------------------------------ tracer
void SphereEngine::ensure_tracer() {
  if (p.precision != kFP64) throw InvalidArgument("the tracer is supported in FP64 precision only");
  if (tq0.p) return;
  const size_t nq = static_cast<size_t>(B) * ntri * 2;
  tq0.alloc(nq);
  tqs.alloc(nq);
  tqacc.alloc(nq);
  fourq.alloc(static_cast<size_t>(B) * nlat * 2 * M * 2);
  foldq.alloc(static_cast<size_t>(B) * nh * TRC_SLOT * 2 * M * 2);
  refq.alloc(static_cast<size_t>(B) * ngrid());
  tgrid.alloc(static_cast<size_t>(B) * ngrid());
  for (auto *b : {&tq0, &tqs, &tqacc, &fourq, &foldq, &refq, &tgrid}) b->zero(stream);
  LMW_CUDA(cudaStreamSynchronize(stream));
  graphs_clear();
}

// part 0: q and delta synthesis, 1: grid products, 2: analysis and RK4 update of q
void SphereEngine::tracer_stage(int stage, double dt, int part) {
  SphDev d = make_sph(*this, *tab);
  const double2 *in = reinterpret_cast<const double2 *>(stage == 0 ? x0.p : xs.p);
  const double2 *qin = reinterpret_cast<const double2 *>(stage == 0 ? tq0.p : tqs.p);
  if (part == 0) {
    trc_synth<<<dim3((nh + 31) / 32, M, B), SYN_THREADS, 0, stream>>>(d, tab64(*tab), in, qin, reinterpret_cast<double2 *>(fourq.p));
  } else if (part == 1) {
    const size_t smem = 4 * static_cast<size_t>(fft_row<3>(nlon)) * sizeof(double2);
    trc_grid<<<dim3(nh, B), GRID_THREADS, smem, stream>>>(d, tab64(*tab), reinterpret_cast<const double2 *>(four.p),
                                                          reinterpret_cast<const double2 *>(fourq.p), reinterpret_cast<double2 *>(foldq.p));
  } else {
    StageArgs sa;
    sa.stage = stage;
    sa.c = stage < 2 ? 0.5 * dt : (stage == 2 ? dt : dt / 6);
    sa.filt = filt.p;
    trc_analysis<<<dim3((ntri + 31) / 32, B), ANA_THREADS, 0, stream>>>(d, tab64(*tab), reinterpret_cast<const double2 *>(foldq.p), sa,
                                                                        reinterpret_cast<double2 *>(tq0.p), reinterpret_cast<double2 *>(tqs.p),
                                                                        reinterpret_cast<double2 *>(tqacc.p));
  }
  LMW_LAUNCH_CHECK();
}

// cpp/sphere.cpp:264-270: q from its grid (analysis), and the grid it was set from as the reference of the
// tracer errors (its synthesis)
void SphereEngine::set_tracer_grid(const double *qg, size_t n, int member) {
  check_member(*this, member);
  if (n != ngrid()) throw InvalidArgument("grid size mismatch");
  ensure_tracer();
  // analyze_scalar (cpp/sphere.cpp:138-149) on the device, straight into the member's packed tracer state
  LMW_CUDA(cudaStreamSynchronize(stream));
  std::memcpy(hstage.p, qg, n * sizeof(double));
  LMW_CUDA(cudaMemcpyAsync(gridin.p, hstage.p, n * sizeof(double), cudaMemcpyHostToDevice, stream));
  SphDev d = make_sph(*this, *tab);
  const size_t smem = 2 * static_cast<size_t>(nlon) * sizeof(double2);
  sph_hook_fold<<<nh, GRID_THREADS, smem, stream>>>(d, gridin.p, nullptr, 0, reinterpret_cast<double2 *>(fold.p));
  sph_hook_analysis<<<(ntri + ANA_THREADS - 1) / ANA_THREADS, ANA_THREADS, 0, stream>>>(
      d, reinterpret_cast<const double2 *>(fold.p), 0, reinterpret_cast<double2 *>(tq0.p) + static_cast<size_t>(member) * ntri, 1);
  LMW_LAUNCH_CHECK();
  g_launches += 2;
  if (!has_tracer) {
    has_tracer = true;
    graphs_clear();
  }
  synth_tracer_grid(member, refq.p + static_cast<size_t>(member) * ngrid());
  LMW_CUDA(cudaStreamSynchronize(stream));
}

void SphereEngine::set_tracer_state(const double *qr, int member) {
  check_member(*this, member);
  ensure_tracer();
  LMW_CUDA(cudaStreamSynchronize(stream));
  to_packed(qr, hstage.p);
  LMW_CUDA(cudaMemcpy(tq0.p + static_cast<size_t>(member) * ntri * 2, hstage.p, static_cast<size_t>(ntri) * 2 * sizeof(double),
                      cudaMemcpyHostToDevice));
  if (!has_tracer) {
    has_tracer = true;
    graphs_clear();
  }
}

void SphereEngine::set_advect_only(bool on) {
  if (advect_only != on) graphs_clear();
  advect_only = on;
}

void SphereEngine::tracer_state(double *qr, int member) {
  check_member(*this, member);
  if (!has_tracer) {
    std::memset(qr, 0, nspec_ref() * 2 * sizeof(double));
    return;
  }
  LMW_CUDA(cudaStreamSynchronize(stream));
  LMW_CUDA(cudaMemcpy(hstage.p, tq0.p + static_cast<size_t>(member) * ntri * 2, static_cast<size_t>(ntri) * 2 * sizeof(double),
                      cudaMemcpyDeviceToHost));
  from_packed(hstage.p, qr);
}

// the tracer's grid of one member into dst (device), by the same synthesis for the diagnostics and the reference
// grid, so that a tracer compared with the grid it was just set from has exactly zero error (cpp/sphere.cpp:236-246)
void SphereEngine::synth_tracer_grid(int member, double *dst) {
  SphDev d = make_sph(*this, *tab);
  const size_t fo = static_cast<size_t>(member) * nlat * 2 * M;
  trc_synth<<<dim3((nh + 31) / 32, M, 1), SYN_THREADS, 0, stream>>>(d, tab64(*tab), reinterpret_cast<const double2 *>(x0.p) + static_cast<size_t>(member) * 3 * ntri,
                                                                  reinterpret_cast<const double2 *>(tq0.p) + static_cast<size_t>(member) * ntri,
                                                                  reinterpret_cast<double2 *>(fourq.p) + fo);
  trc_to_grid<<<dim3(nh, 1), GRID_THREADS, static_cast<size_t>(nlon) * sizeof(double2), stream>>>(d, reinterpret_cast<const double2 *>(fourq.p) + fo, dst);
  LMW_LAUNCH_CHECK();
  g_launches += 2;
}

void SphereEngine::tracer_grid(double *out, int member) {
  check_member(*this, member);
  if (!has_tracer) {
    std::memset(out, 0, ngrid() * sizeof(double));
    return;
  }
  LMW_CUDA(cudaStreamSynchronize(stream));
  synth_tracer_grid(member, tgrid.p + static_cast<size_t>(member) * ngrid());
  LMW_CUDA(cudaMemcpyAsync(out, tgrid.p + static_cast<size_t>(member) * ngrid(), ngrid() * sizeof(double), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
}

// cpp/sphere.cpp:271-284 and 571-590: out[0] mean, out[1] mass = area mean of h q, out[2] l2, out[3] linf error
// against the grid the tracer was set from
void SphereEngine::tracer_diagnostics(double *out, int member) {
  check_member(*this, member);
  if (!has_tracer) throw RuntimeError("no tracer: set one with tracer() first");
  std::vector<double> q(ngrid()), hgt(ngrid()), ref(ngrid(), 0.0);
  tracer_grid(q.data(), member);
  grid(0, hgt.data(), member);
  if (has_tracer)
    LMW_CUDA(cudaMemcpy(ref.data(), refq.p + static_cast<size_t>(member) * ngrid(), ngrid() * sizeof(double), cudaMemcpyDeviceToHost));
  double q00[2] = {0, 0};
  if (has_tracer)
    LMW_CUDA(cudaMemcpy(q00, tq0.p + static_cast<size_t>(member) * ntri * 2, sizeof(q00), cudaMemcpyDeviceToHost));
  const HostTables &h = tab->host;
  double sum = 0, num = 0, den = 0, mn = 0, mr = 0, qmin = q[0], qmax = q[0];
  for (int j = 0; j < nlat; j++) {
    double rowsum = 0;
    for (int k = 0; k < nlon; k++) {
      const size_t i = static_cast<size_t>(j) * nlon + k;
      rowsum += hgt[i] * q[i];
      qmin = std::min(qmin, q[i]);
      qmax = std::max(qmax, q[i]);
      const double dd = q[i] - ref[i];
      num += h.w[j] * dd * dd;
      den += h.w[j] * ref[i] * ref[i];
      mn = std::max(mn, std::fabs(dd));
      mr = std::max(mr, std::fabs(ref[i]));
    }
    sum += h.w[j] * rowsum / nlon;
  }
  out[0] = q00[0] / std::sqrt(2.0);
  out[1] = 0.5 * sum;
  out[2] = den > 0 ? std::sqrt(num / den) : 0.0;
  out[3] = mr > 0 ? mn / mr : 0.0;
  out[4] = qmin;  // cpp/sphere.cpp:285-286
  out[5] = qmax;
}

void SphereEngine::kernel_times(double dt, int reps, double *out) {
  upload_filter(dt);
  ensure_packed();
  SphDev d = make_sph(*this, *tab);
  double2 *X0 = reinterpret_cast<double2 *>(x0.p), *XS = reinterpret_cast<double2 *>(xs.p), *AC = reinterpret_cast<double2 *>(acc.p);
  // stage 1 reads x0 and writes the stage input and the accumulator: x0 is unchanged
  auto one = [&](int which) {
    if (p.precision == kFP64)
      stage_kernels<double>(d, tab64(*tab), B, 1, dt, filt.p, X0, reinterpret_cast<double2 *>(four.p), reinterpret_cast<double2 *>(fold.p), X0,
                            XS, AC, fgrid.p, hsgrid.p, stream, which);
    else if (p.precision == kFP32)
      stage_kernels<float>(d, tab32(*tab), B, 1, dt, filt.p, X0, reinterpret_cast<float2 *>(four32.p), reinterpret_cast<float2 *>(fold32.p),
                           X0, XS, AC, fgrid.p, hsgrid.p, stream, which);
    else
      split_stage(d, tab32(*tab), *split, B, 1, dt, filt.p, reinterpret_cast<float2 *>(fold32.p), X0, XS, XS2(), AC, fgrid.p,
                  hsgrid.p, stream, which);
  };
  cudaEvent_t e0, e1;
  LMW_CUDA(cudaEventCreate(&e0));
  LMW_CUDA(cudaEventCreate(&e1));
  for (int k = 0; k < 3; k++) {
    one(k);  // warm
    LMW_CUDA(cudaEventRecord(e0, stream));
    for (int r = 0; r < reps; r++) one(k);
    LMW_CUDA(cudaEventRecord(e1, stream));
    LMW_LAUNCH_CHECK();
    LMW_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    LMW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    out[k] = ms / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g_launches += 3ull * (reps + 1);
  split_packed = false;
}

// Measured choice of the split path's launch plan (each candidate timed after its producer kernel): latitude pairs per grid CTA (8, 4, 2, 1), FFT stages fused per
// shared-memory pass (4, 3 or 2), and the pipeline depth of the synthesis and analysis kernels (1-4 stages where
// they fit) and the analysis variant (one parity or both per CTA). Each kernel is timed alone for every candidate (CUDA events on the engine stream, stage 1 on the
// present state, which leaves the state unchanged); the arithmetic does not depend on the choice.
void SphereEngine::autotune_split() {
  if (!split) return;
  SplitPlan &sp = *split;
  const double dt = 60.0;
  upload_filter(dt);
  SphDev d = make_sph(*this, *tab);
  double2 *X0 = reinterpret_cast<double2 *>(x0.p), *XS = reinterpret_cast<double2 *>(xs.p), *AC = reinterpret_cast<double2 *>(acc.p);
  cudaEvent_t e0, e1;
  LMW_CUDA(cudaEventCreate(&e0));
  LMW_CUDA(cudaEventCreate(&e1));
  auto launch = [&](int which) {
    split_stage(d, tab32(*tab), sp, B, 1, dt, filt.p, reinterpret_cast<float2 *>(fold32.p), X0, XS, XS2(), AC, fgrid.p, hsgrid.p, stream,
                which);
    g_launches += 1;
  };
  // a candidate is timed right after the kernel that produces its input (the analysis after the grid kernel, the
  // grid kernel after the synthesis, the synthesis after the analysis), so the caches hold what they hold in a run
  auto timed = [&](int which) {
    const int prev = (which + 2) % 3;
    launch(prev);
    launch(which);
    double total = 0;
    for (int r = 0; r < 5; r++) {
      launch(prev);
      LMW_CUDA(cudaEventRecord(e0, stream));
      launch(which);
      LMW_CUDA(cudaEventRecord(e1, stream));
      LMW_LAUNCH_CHECK();
      LMW_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      LMW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      total += ms;
    }
    return total;
  };
  ensure_packed();
  // warm the device (clocks) on the default plan before any measurement
  for (int r = 0; r < 10; r++)
    for (int k = 0; k < 3; k++) launch(k);
  struct Cand {
    int which, jb, fg, ns, dir;
    size_t bytes;
    double best;
    int mb = 2;  // analysis register budget (CTAs per SM)
    int ws = 0;  // the warp-specialised form (analysis or synthesis) with this many CTAs per SM
  };
  std::vector<Cand> cands;
  int dev = 0, optin = 0;
  LMW_CUDA(cudaGetDevice(&dev));
  LMW_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  // the grid and analysis candidates come in two variants of their interface (dir 1: the grid kernel writes the
  // analysis operands, which the analysis streams; dir 0: FP32 fold, gathered by the analysis)
  for (int dir = 1; dir >= 0; dir--)
    for (int jb = SPLIT_JB_MAX; jb >= 1; jb /= 2)
      if (nh % jb == 0 && 5 * static_cast<size_t>(jb) * fft_row<3>(nlon) * sizeof(float2) <= static_cast<size_t>(optin - 2048))
        for (int fg = 4; fg >= 2; fg--) cands.push_back({1, jb, fg, 0, dir, 0, 1e30});
  // one stage (no double buffering inside a CTA) leaves room for a third CTA per SM, whose copies overlap the others'
  for (int ns = 1; ns <= SPLIT_MAX_STAGES; ns++) {
    // synthesis: latitude slices per (m, tile) (each CTA keeps four accumulators of its slice in tensor memory,
    // so narrower slices let more CTAs share an SM) at this pipeline depth
    for (int sl = 1; sl <= 4; sl *= 2) {
      const int snh = sp.nh16 / sl;
      if (sp.nh16 % sl != 0 || snh < 16 || snh % 16 != 0 || 4 * snh > 512) continue;
      const size_t st = static_cast<size_t>(sp.pieces) * (sp.rSP + snh) * sp.bks * 2;
      const size_t bs = std::max(ns * st + SPLIT_MARGIN, sp.syn_min_bytes);
      if (bs <= sp.budget_bytes) cands.push_back({0, sl, 0, ns, 0, bs, 1e30});
      // the warp-specialised persistent form, one or two CTAs per SM
      if (ns >= 2)
        for (int ctas = 1; ctas <= 2; ctas++) {
          size_t wsm = 0;
          int bc = 0, slot = 0;
          if (syn_ws_layout(sp, sl, ns, ctas, &wsm, &bc, &slot)) cands.push_back({0, sl, 0, ns, 0, wsm, 1e30, 2, ctas});
        }
    }
    for (int dir = 1; dir >= 0; dir--)
      for (int both = 0; both <= 1; both++) {
        if (both && 2 * sp.ra_pair > 512) continue;  // both parities' accumulators must fit the 512 tensor-memory columns
        const size_t ba = std::max(sp.ana_res_bytes_v[dir] + ns * sp.ana_stage_bytes_v[dir] + SPLIT_MARGIN,
                                   both ? sp.ana_both_min_bytes : sp.ana_min_bytes);
        if (ba > sp.budget_bytes) continue;
        // one CTA per work item (persistent CTAs, ana_grid > 0, measured no faster on GB300 and are not tried)
        cands.push_back({2, both, 0, ns, dir, ba, 1e30, 2});
        // the 80-register form only pays where three CTAs fit in shared memory
        if (3 * (ba + 1024) <= 233472) cands.push_back({2, both, 0, ns, dir, ba, 1e30, 3});
        // the warp-specialised persistent form (direct operands), one or two CTAs per SM
        if (dir == 1 && ns >= 2)
          for (int ctas = 1; ctas <= 2; ctas++) {
            size_t wsm = 0;
            int bc = 0, sl = 0;
            if (ws_layout(sp, both, ns, ctas, &wsm, &bc, &sl)) cands.push_back({2, both, 0, ns, dir, wsm, 1e30, 2, ctas});
          }
      }
  }
  const int jb0 = sp.jb, fg0 = sp.fgrp, nss0 = sp.ns_syn, nsa0 = sp.ns_ana, ab0 = sp.ana_both, ag0 = sp.ana_grid, dir0 = sp.direct,
            mb0 = sp.ana_minb, sl0 = sp.syn_split, ws0 = sp.ana_ws, sws0 = sp.syn_ws;
  const size_t sms0 = sp.smem_syn, sma0 = sp.smem_ana;
  auto apply = [&](const Cand &c) {
    sp.jb = jb0;
    sp.fgrp = fg0;
    sp.ns_syn = nss0;
    sp.smem_syn = sms0;
    sp.ns_ana = nsa0;
    sp.smem_ana = sma0;
    sp.ana_both = ab0;
    sp.ana_grid = ag0;
    sp.direct = dir0;
    sp.ana_minb = mb0;
    sp.ana_ws = ws0;
    sp.syn_ws = sws0;
    sp.syn_split = sl0;
    sp.syn_nh = sp.nh16 / sl0;
    if (c.which == 1) {
      sp.jb = c.jb;
      sp.fgrp = c.fg;
      sp.direct = c.dir;
    } else if (c.which == 0) {
      sp.ns_syn = c.ns;
      sp.smem_syn = c.bytes;
      sp.syn_split = c.jb;  // the synthesis candidates carry their latitude slices in jb
      sp.syn_nh = sp.nh16 / c.jb;
      sp.syn_ws = c.ws;
    } else {
      sp.ns_ana = c.ns;
      sp.smem_ana = c.bytes;
      sp.ana_both = c.jb;  // the analysis candidates carry the variant in jb and the CTA count in fg
      sp.ana_grid = c.fg;
      sp.direct = c.dir;
      sp.ana_minb = c.mb;
      sp.ana_ws = c.ws;
    }
  };
  // two rounds in opposite orders; each candidate keeps its faster round
  for (int round = 0; round < 2; round++)
    for (size_t i = 0; i < cands.size(); i++) {
      Cand &c = cands[round == 0 ? i : cands.size() - 1 - i];
      apply(c);
      c.best = std::min(c.best, timed(c.which));
    }
  auto pick = [&](int which, int dir) -> const Cand * {
    const Cand *b = nullptr;
    for (const Cand &c : cands)
      if (c.which == which && (which == 0 || c.dir == dir) && (!b || c.best < b->best)) b = &c;
    return b;
  };
  // the interface variant with the lower grid + analysis time, then its best candidates
  int dir = dir0;
  double tbest = 1e30;
  for (int v = 0; v <= 1; v++) {
    const Cand *g = pick(1, v), *a = pick(2, v);
    if (g && a && g->best + a->best < tbest) {
      tbest = g->best + a->best;
      dir = v;
    }
  }
  const Cand *bg = pick(1, dir), *bs = pick(0, 0), *ba = pick(2, dir);
  sp.direct = dir;
  sp.jb = bg ? bg->jb : jb0;
  sp.fgrp = bg ? bg->fg : fg0;
  sp.ns_syn = bs ? bs->ns : nss0;
  sp.smem_syn = bs ? bs->bytes : sms0;
  sp.syn_split = bs ? bs->jb : sl0;
  sp.syn_nh = sp.nh16 / sp.syn_split;
  sp.syn_ws = bs ? bs->ws : sws0;
  sp.ns_ana = ba ? ba->ns : nsa0;
  sp.smem_ana = ba ? ba->bytes : sma0;
  sp.ana_both = ba ? ba->jb : ab0;
  sp.ana_grid = ba ? ba->fg : ag0;
  sp.ana_minb = ba ? ba->mb : mb0;
  sp.ana_ws = ba ? ba->ws : ws0;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  check_split_status();
  split_packed = false;
}

void SphereEngine::split_plan(int *out) const {
  out[0] = split ? split->jb : 0;
  out[1] = split ? split->fgrp : 0;
  out[2] = split ? split->ns_syn : 0;
  out[3] = split ? split->ns_ana : 0;
  out[4] = split ? split->ana_both : 0;
  out[5] = split ? split->ana_grid : 0;
  out[6] = split ? split->direct : 0;
  out[7] = split ? split->ana_minb : 0;
  out[8] = split ? split->syn_split : 0;
  out[9] = split ? split->ana_ws : 0;
  out[10] = split ? split->grid_fixed : 0;
  out[11] = split ? split->syn_ws : 0;
}

void SphereEngine::set_split_form(int linear_exact) {
  if (!split) throw InvalidArgument("the engine is not in split precision");
  if (linear_exact != 0 && linear_exact != 1) throw InvalidArgument("split form: linear_exact must be 0 or 1");
  LMW_CUDA(cudaStreamSynchronize(stream));
  split->lin_exact = linear_exact;
  split_packed = false;  // the synthesis operands of Phi_00 differ between the forms
  graphs_clear();
}

void SphereEngine::set_split_plan(const int *in) {
  if (!split) throw InvalidArgument("the engine is not in split precision");
  SplitPlan &sp = *split;
  const int jb = in[0], fg = in[1], nss = in[2], nsa = in[3], both = in[4], grid = in[5], dir = in[6], mb = in[7], sl = in[8], ws = in[9], gfix = in[10], sws = in[11];
  int dev = 0, optin = 0;
  LMW_CUDA(cudaGetDevice(&dev));
  LMW_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (!(jb == 1 || jb == 2 || jb == 4 || jb == 8) || jb > SPLIT_JB_MAX || nh % jb != 0 ||
      5 * static_cast<size_t>(jb) * fft_row<3>(nlon) * sizeof(float2) > static_cast<size_t>(optin - 2048))
    throw InvalidArgument("split plan: latitude pairs per grid CTA must be 1, 2, 4 or 8, divide the latitude pairs and fit in shared memory");
  if (fg < 2 || fg > 4) throw InvalidArgument("split plan: FFT stages per pass must be 2, 3 or 4");
  if (nss < 1 || nss > SPLIT_MAX_STAGES || nsa < 1 || nsa > SPLIT_MAX_STAGES)
    throw InvalidArgument("split plan: pipeline stages must be between 1 and " + std::to_string(SPLIT_MAX_STAGES));
  if ((both != 0 && both != 1) || (dir != 0 && dir != 1) || grid < 0) throw InvalidArgument("split plan: flags must be 0 or 1, the CTA count not negative");
  if (both && 2 * sp.ra_pair > 512) throw InvalidArgument("split plan: both parities' accumulators exceed tensor memory");
  if (!(sl == 1 || sl == 2 || sl == 4) || sp.nh16 % sl != 0 || (sp.nh16 / sl) % 16 != 0 || 4 * (sp.nh16 / sl) > 512)
    throw InvalidArgument("split plan: synthesis latitude slices must be 1, 2 or 4, leave slices of a multiple of 16 latitudes and fit tensor memory");
  const size_t bs = std::max(nss * static_cast<size_t>(sp.pieces) * (sp.rSP + sp.nh16 / sl) * sp.bks * 2 + SPLIT_MARGIN, sp.syn_min_bytes);
  const size_t ba = std::max(sp.ana_res_bytes_v[dir] + nsa * sp.ana_stage_bytes_v[dir] + SPLIT_MARGIN, both ? sp.ana_both_min_bytes : sp.ana_min_bytes);
  if (bs > sp.budget_bytes || ba > sp.budget_bytes) throw InvalidArgument("split plan: the pipelines do not fit in shared memory");
  if (mb != 2 && mb != 3) throw InvalidArgument("split plan: the analysis register budget must be 2 or 3 CTAs per SM");
  if (gfix != 0 && gfix != 1) throw InvalidArgument("split plan: the grid kernel's fixed-length flag must be 0 or 1");
  size_t swsm = 0;
  if (sws != 0) {
    int bc = 0, slot = 0;
    if (nss < 2 || !syn_ws_layout(sp, sl, nss, sws, &swsm, &bc, &slot))
      throw InvalidArgument("split plan: the warp-specialised synthesis takes 1 or 2 CTAs per SM, at least 2 stages, and must fit shared "
                            "and tensor memory");
  }
  size_t wsm = 0;
  if (ws != 0) {
    int bc = 0, slot = 0;
    if (!dir || nsa < 2 || !ws_layout(sp, both, nsa, ws, &wsm, &bc, &slot))
      throw InvalidArgument("split plan: the warp-specialised analysis takes 1 or 2 CTAs per SM, direct operands, at least 2 stages, and must fit "
                            "shared and tensor memory");
  }
  LMW_CUDA(cudaStreamSynchronize(stream));
  sp.jb = jb;
  sp.fgrp = fg;
  sp.ns_syn = nss;
  sp.smem_syn = bs;
  sp.ns_ana = nsa;
  sp.smem_ana = ba;
  sp.ana_both = both;
  sp.ana_grid = grid;
  sp.direct = dir;
  sp.ana_minb = mb;
  sp.ana_ws = ws;
  sp.grid_fixed = gfix;
  sp.syn_ws = sws;
  if (ws) sp.smem_ana = wsm;
  if (sws) sp.smem_syn = swsm;
  sp.syn_split = sl;
  sp.syn_nh = sp.nh16 / sl;
  graphs_clear();
}

// the split path keeps its synthesis operands packed from the state; pack them after a change from outside
void SphereEngine::ensure_packed() {
  if (!split || split_packed) return;
  SphDev d = make_sph(*this, *tab);
  split_pack_state<<<dim3((ntri + 127) / 128, B), 128, 0, stream>>>(d, split_dev(*split), tab->kfac32.p, reinterpret_cast<const double2 *>(x0.p),
                                                                     reinterpret_cast<float2 *>(xs.p) + static_cast<size_t>(B) * 3 * ntri);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
  split_packed = true;
}

void SphereEngine::enqueue_step(double dt) {
  upload_filter(dt);
  ensure_packed();
  for (int s = 0; s < 4; s++) launch_stage(s, dt);
  launches_step = 12;
}

void SphereEngine::graphs_clear() {
  for (const ChunkGraph &cg : graphs) cudaGraphExecDestroy(cg.exec);
  graphs.clear();
}

void SphereEngine::launch_chunk(double dt, int steps) {
  if (steps <= 0) return;
  upload_filter(dt);
  ensure_packed();
  cudaGraphExec_t exec = nullptr;
  for (const ChunkGraph &cg : graphs)
    if (cg.dt == dt && cg.steps == steps) exec = cg.exec;
  if (!exec) {
    if (graphs.size() >= 4) {
      cudaGraphExecDestroy(graphs.front().exec);
      graphs.erase(graphs.begin());
    }
    cudaGraph_t g;
    uint64_t before = g_launches;
    LMW_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < steps; s++)
      for (int k = 0; k < 4; k++) launch_stage(k, dt);
    LMW_CUDA(cudaStreamEndCapture(stream, &g));
    g_launches = before;
    LMW_CUDA(cudaGraphInstantiate(&exec, g, 0));
    cudaGraphDestroy(g);
    graphs.push_back({dt, steps, exec});
  }
  LMW_CUDA(cudaGraphLaunch(exec, stream));
  g_launches += 12ull * steps;
}

void SphereEngine::step(double dt) {
  enqueue_step(dt);
  for (int b = 0; b < B; b++) t[b] += dt;
  LMW_CUDA(cudaStreamSynchronize(stream));
  check_split_status();
}

void SphereEngine::reduce_guard(Reduce &r, int member) {
  SphDev d = make_sph(*this, *tab);
  synth_grids(member, 1);
  const size_t smem = 4 * static_cast<size_t>(nlon) * sizeof(double2);
  const size_t go = static_cast<size_t>(member) * ngrid();
  sph_diag<<<dim3(nh, 1), GRID_THREADS, smem, stream>>>(d, reinterpret_cast<const double2 *>(four.p) + static_cast<size_t>(member) * nlat * 4 * M,
                                                        fgrid.p + go, hsgrid.p + go, refgrid.p + go, diagrows.p, nullptr);
  sph_diag_final<<<1, GRID_THREADS, 0, stream>>>(d, diagrows.p, reinterpret_cast<const double2 *>(x0.p) + static_cast<size_t>(member) * 3 * ntri,
                                                0, dred.p);
  LMW_LAUNCH_CHECK();
  g_launches += 2;
  LMW_CUDA(cudaMemcpyAsync(hred.p, dred.p, sizeof(Reduce), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
  r = hred.p[0];
}

// guard reductions of every member in one pass, read back once: FP64 synthesis and grid reductions, or (exact =
// false, reduced-precision engines) the FP32 synthesis and the FP32 maxima of the stability re-check
void SphereEngine::reduce_guard_all(bool exact) {
  SphDev d = make_sph(*this, *tab);
  if (!exact && p.precision != kFP64 && !has_tracer) {
    const int L = syn_lats(nh);
    auto *k = L == 8 ? sph_synth<float, 8> : sph_synth<float, 32>;
    k<<<dim3((nh + L - 1) / L, M, B), SYN_THREADS, 0, stream>>>(d, tab32(*tab), reinterpret_cast<const double2 *>(x0.p),
                                                              reinterpret_cast<float2 *>(four32.p));
    sph_guard32<<<dim3(nh, B), GRID_THREADS, 4 * static_cast<size_t>(nlon) * sizeof(float2), stream>>>(
        d, tab32(*tab), reinterpret_cast<const float2 *>(four32.p), diagrows.p);
    g_launches += 2;
  } else {
    synth_grids(0, B);
    const size_t smem = 4 * static_cast<size_t>(nlon) * sizeof(double2);
    sph_diag<<<dim3(nh, B), GRID_THREADS, smem, stream>>>(d, reinterpret_cast<const double2 *>(four.p), fgrid.p, hsgrid.p, refgrid.p, diagrows.p,
                                                          nullptr);
  }
  sph_diag_final<<<B, GRID_THREADS, 0, stream>>>(d, diagrows.p, reinterpret_cast<const double2 *>(x0.p), 0, dred.p);
  if (has_tracer) trc_abs_sum<<<B, GRID_THREADS, 0, stream>>>(d, reinterpret_cast<const double2 *>(tq0.p), dred.p);
  LMW_LAUNCH_CHECK();
  g_launches += 2;
  LMW_CUDA(cudaMemcpyAsync(hred.p, dred.p, B * sizeof(Reduce), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
}

// RK4 limit of member b from its guard reduction (cpp/sphere.cpp:438-447)
double SphereEngine::limit_from(const Reduce &r, int b, double safety) const {
  double hmax = std::max(0.0, r.max[1]);
  if (!(hmax > 0)) throw RuntimeError("the height field must be positive to step the model");
  // cpp/sphere.cpp:438-447; advect-only: the frozen flow's advection alone
  double omega = advect_only ? (N / p.radius) * r.max[0] : (N / p.radius) * (std::sqrt(p.gravity * hmax) + r.max[0]) + 2 * omega_m[b];
  if (!(omega > 0)) return 1e9;
  return safety / omega;
}

// the smallest stable step over the members
double SphereEngine::stable_dt_all(double safety) {
  reduce_guard_all();
  double dt = 1e300;
  for (int b = 0; b < B; b++) dt = std::min(dt, limit_from(hred.p[b], b, safety));
  return dt;
}

// cpp/sphere.cpp:438-447
double SphereEngine::stable_dt(double safety, int member) {
  Reduce r;
  reduce_guard(r, member);
  double hmax = std::max(0.0, r.max[1]), wmax = r.max[0];
  if (!(hmax > 0)) throw RuntimeError("the height field must be positive to step the model");
  double omega = (N / p.radius) * (std::sqrt(p.gravity * hmax) + wmax) + 2 * omega_m[member];
  if (!(omega > 0)) return 1e9;
  return safety / omega;
}

// cpp/sphere.cpp:457-466: equal steps, the stability pre-check over every member
SphereEngine::RunPlan SphereEngine::plan_run(double seconds, double dt) {
  RunPlan rp;
  if (!(seconds >= 0)) throw InvalidArgument("run: seconds must not be negative");
  if (advect_only && !has_tracer) throw InvalidArgument("advect_only: set a tracer first (Sphere.tracer)");
  if (seconds == 0) return rp;
  // one guard reduction gives both the automatic step (stable_dt(1.5)) and the limit (cpp/sphere.cpp:461-466)
  reduce_guard_all();
  double auto_dt = 1e300, limit = 1e300;
  for (int b = 0; b < B; b++) {
    auto_dt = std::min(auto_dt, limit_from(hred.p[b], b, 1.5));
    limit = std::min(limit, limit_from(hred.p[b], b, 2.0 * std::sqrt(2.0)));
  }
  if (!(dt > 0)) dt = auto_dt;
  if (!(dt <= limit))
    throw InvalidArgument("run: dt = " + fmt_f(dt) + " s exceeds the RK4 stability limit of about " + fmt_f(limit) +
                          " s for the present state: use a smaller dt");
  int64_t n = static_cast<int64_t>(std::ceil(seconds / dt - 1e-9));
  if (n < 1) n = 1;
  if (n > 50000000) throw InvalidArgument("run: more than 5e7 steps; use a larger dt");
  rp.n = n;
  rp.h = seconds / static_cast<double>(n);
  upload_filter(rp.h);
  return rp;
}

// enqueue the steps up to the next guard point (no synchronisation); true when a guard check is due
bool SphereEngine::advance(RunPlan &rp) {
  if (rp.i >= rp.n) return false;
  int64_t next = std::min<int64_t>(rp.n - 1, rp.i | 63);
  int chunk = static_cast<int>(next - rp.i + 1);
  if (chunk >= 4) launch_chunk(rp.h, chunk);
  else for (int s = 0; s < chunk; s++) enqueue_step(rp.h);
  for (int s = 0; s < chunk; s++)
    for (int b = 0; b < B; b++) t[b] += rp.h;
  rp.i = next + 1;
  rp.guard_due = (next & 63) == 63;
  return true;
}

// cpp/sphere.cpp:473-483: every 64 steps the finiteness check and the stability re-check, and a final
// finiteness check, over every member
void SphereEngine::guard(RunPlan &rp) {
  const bool last = rp.i >= rp.n;
  if (!rp.guard_due && !last) return;
  check_split_status();
  // reduced-precision engines re-check with FP32 grids (a decision about the stability margin, not a result)
  reduce_guard_all(false);
  for (int b = 0; b < B; b++) {
    const Reduce &r = hred.p[b];
    if (!std::isfinite(r.sum[5])) throw RuntimeError("the integration blew up (not finite): use a smaller dt");
    if (rp.guard_due) {
      const double now = limit_from(r, b, 2.0 * std::sqrt(2.0));
      if (!(rp.h <= now))
        throw RuntimeError("run: dt = " + fmt_f(rp.h) + " s exceeds the RK4 stability limit of about " + fmt_f(now) + " s reached at t = " +
                           fmt_f(t[b]) + " s (the flow accelerated): use a smaller dt");
    }
  }
  rp.guard_due = false;
}

void SphereEngine::run(double seconds, double dt) {
  RunPlan rp = plan_run(seconds, dt);
  while (advance(rp)) guard(rp);
}

// cpp/sphere.cpp:510-590
void SphereEngine::diagnostics(double *out, int member) {
  check_member(*this, member);
  Reduce r;
  reduce_guard(r, member);
  const size_t pk = static_cast<size_t>(ntri) * 2;
  double phi00[2];
  LMW_CUDA(cudaMemcpy(phi00, x0.p + static_cast<size_t>(member) * 3 * pk + 2 * pk, sizeof(phi00), cudaMemcpyDeviceToHost));
  out[0] = phi00[0] / std::sqrt(2.0) / p.gravity;
  out[1] = r.sum[0];
  out[2] = r.sum[1];
  out[3] = r.sum[0] + r.sum[1];
  out[4] = r.sum[2];
  out[5] = r.max[0];
  out[6] = std::sqrt(r.sum[3] / r.sum[4]);
  out[7] = r.max[2] / r.max[3];
}

void SphereEngine::grid(int which, double *out, int member) {
  check_member(*this, member);
  if (which < 0 || which > 3) throw InvalidArgument("grid field must be 0 (height), 1 (u), 2 (v) or 3 (vorticity)");
  SphDev d = make_sph(*this, *tab);
  synth_grids(member, 1);
  const size_t smem = 4 * static_cast<size_t>(nlon) * sizeof(double2);
  const size_t go = static_cast<size_t>(member) * ngrid();
  sph_diag<<<dim3(nh, 1), GRID_THREADS, smem, stream>>>(d, reinterpret_cast<const double2 *>(four.p) + static_cast<size_t>(member) * nlat * 4 * M,
                                                        fgrid.p + go, hsgrid.p + go, refgrid.p + go, diagrows.p, gridin.p);
  LMW_LAUNCH_CHECK();
  g_launches += 1;
  LMW_CUDA(cudaMemcpyAsync(out, gridin.p + static_cast<size_t>(which) * ngrid(), ngrid() * sizeof(double), cudaMemcpyDeviceToHost, stream));
  LMW_CUDA(cudaStreamSynchronize(stream));
}

// cpp/sphere.cpp:536-551 (from the spectral state)
// ------------------------------------------------------------------------------------------------ point probes
double SphereEngine::probe(int which, double lat, double lon, int member) {
  check_member(*this, member);
  if (which < 0 || which > 4) throw InvalidArgument("probe: which must be 0 (height), 1 (u), 2 (v), 3 (vorticity) or 4 (tracer)");
  if (which == 4 && !has_tracer) throw RuntimeError("no tracer: set one with tracer() first");
  const size_t ns = nspec_ref() * 2;
  std::vector<double> z(ns), dl(ns), f(ns), q(ns);
  get_state(z.data(), dl.data(), f.data(), member);
  if (which == 4) tracer_state(q.data(), member);
  auto at = [&](const std::vector<double> &v, int m, int n) { return cplx(v[2 * (static_cast<size_t>(m) * M + n)], v[2 * (static_cast<size_t>(m) * M + n) + 1]); };
  const double mu = std::sin(lat), a = p.radius;
  std::vector<double> col;
  double sum = 0;
  for (int m = 0; m <= N; m++) {
    legendre_column(m, N, mu, col);
    cplx g(0, 0);
    if (which == 1 || which == 2) {
      cplx sp(0, 0), sc(0, 0), hp(0, 0), hc(0, 0);
      for (int n = std::max(m, 1); n <= N; n++) {
        const double k = -a * a / (n * (n + 1.0));
        const double P = col[n - m];
        const double H = -n * legendre_eps(n + 1, m) * col[n + 1 - m] + (n > m ? (n + 1) * legendre_eps(n, m) * col[n - 1 - m] : 0.0);
        const cplx ps = at(z, m, n) * k, ch = at(dl, m, n) * k;
        sp += ps * P;
        sc += ch * P;
        hp += ps * H;
        hc += ch * H;
      }
      const cplx im(0, static_cast<double>(m));
      g = which == 1 ? (im * sc - hp) / a : (im * sp + hc) / a;
    } else {
      const std::vector<double> &src = which == 0 ? f : (which == 3 ? z : q);
      for (int n = m; n <= N; n++) g += at(src, m, n) * col[n - m];
    }
    sum += (m == 0 ? 1.0 : 2.0) * (g * std::exp(cplx(0, m * lon))).real();
  }
  if (which == 0) return sum / p.gravity;
  if (which == 1 || which == 2) return sum / std::cos(lat);
  return sum;
}

double SphereEngine::mode_coefficient(int n, int m, bool imag, int member) {
  check_member(*this, member);
  if (m < 0 || n < m || n > N) throw InvalidArgument("mode (n, m) outside the truncation");
  const size_t ns = nspec_ref() * 2;
  std::vector<double> f(ns);
  get_state(nullptr, nullptr, f.data(), member);
  const size_t i = static_cast<size_t>(m) * M + n;
  const cplx c = cplx(f[2 * i], f[2 * i + 1]) / p.gravity;
  return imag ? c.imag() : c.real();
}

double SphereEngine::wave_crest(int m, double lat, int member) {
  check_member(*this, member);
  if (m < 1 || m > N) throw InvalidArgument("zonal wavenumber must be between 1 and the truncation");
  const size_t ns = nspec_ref() * 2;
  std::vector<double> f(ns), col;
  get_state(nullptr, nullptr, f.data(), member);
  legendre_column(m, N, std::sin(lat), col);
  cplx g(0, 0);
  for (int n = m; n <= N; n++) {
    const size_t i = static_cast<size_t>(m) * M + n;
    g += cplx(f[2 * i], f[2 * i + 1]) * col[n - m];
  }
  return -std::arg(g) / m;
}

// ------------------------------------------------------------------------------------------------ text writers
// The wx layer's files (cpp/main.cpp:328-335, 357-384), written from grids synthesised on the device.
static constexpr double kDegree = 3.14159265358979323846 / 180.0;

// one line per grid point: lon lat h u v vorticity tracer orography (degrees, m, m/s, 1/s), a blank line after
// each latitude row
void SphereEngine::save_csv(const std::string &path, int member) {
  check_member(*this, member);
  const size_t n = ngrid();
  std::vector<double> hh(n), uu(n), vv(n), zz(n), qq(n, 0.0), hs(n);
  grid(0, hh.data(), member);
  grid(1, uu.data(), member);
  grid(2, vv.data(), member);
  grid(3, zz.data(), member);
  if (has_tracer) tracer_grid(qq.data(), member);
  LMW_CUDA(cudaMemcpy(hs.data(), hsgrid.p + static_cast<size_t>(member) * n, n * sizeof(double), cudaMemcpyDeviceToHost));
  const HostTables &h = tab->host;
  std::string t;
  t.reserve(n * 96);
  for (int j = 0; j < nlat; j++) {
    const std::string lat = fmt_g(std::asin(h.mu[j]) / kDegree);
    for (int k = 0; k < nlon; k++) {
      const size_t i = static_cast<size_t>(j) * nlon + k;
      t += fmt_g(2 * 3.14159265358979323846 * k / nlon / kDegree) + " " + lat + " " + fmt_g(hh[i]) + " " + fmt_g(uu[i]) + " " + fmt_g(vv[i]) + " " +
           fmt_g(zz[i]) + " " + fmt_g(qq[i]) + " " + fmt_g(hs[i]) + "\n";
    }
    t += "\n";
  }
  write_text(path, t, "Sphere.save_csv");
}

// one line per latitude: lat, zonal means of h and u
void SphereEngine::save_zonal_mean(const std::string &path, int member) {
  check_member(*this, member);
  const size_t n = ngrid();
  std::vector<double> hh(n), uu(n);
  grid(0, hh.data(), member);
  grid(1, uu.data(), member);
  const HostTables &h = tab->host;
  std::string t;
  for (int j = 0; j < nlat; j++) {
    double sh = 0, su = 0;
    for (int k = 0; k < nlon; k++) {
      sh += hh[static_cast<size_t>(j) * nlon + k];
      su += uu[static_cast<size_t>(j) * nlon + k];
    }
    t += fmt_g(std::asin(h.mu[j]) / kDegree) + " " + fmt_g(sh / nlon) + " " + fmt_g(su / nlon) + "\n";
  }
  write_text(path, t, "Sphere.save_zonal_mean");
}

// one line per total wavenumber n >= 1: n, kinetic and potential energy in that degree
void SphereEngine::save_spectrum(const std::string &path, int member) {
  std::vector<double> ke(N + 1), pe(N + 1);
  spectrum(ke.data(), pe.data(), member);
  std::string t;
  for (int n = 1; n <= N; n++) t += std::to_string(n) + " " + fmt_g(ke[n]) + " " + fmt_g(pe[n]) + "\n";
  write_text(path, t, "Sphere.save_spectrum");
}

void SphereEngine::spectrum(double *ke, double *pe, int member) {
  std::vector<double> z(2 * nspec_ref()), dd(2 * nspec_ref()), ph(2 * nspec_ref());
  get_state(z.data(), dd.data(), ph.data(), member);
  for (int n = 0; n <= N; n++) ke[n] = pe[n] = 0;
  const double a2 = p.radius * p.radius, g2 = p.gravity * p.gravity;
  for (int m = 0; m <= N; m++) {
    double cm = m == 0 ? 1.0 : 2.0;
    for (int n = std::max(m, 1); n <= N; n++) {
      size_t q = 2 * (static_cast<size_t>(m) * M + n);
      double nz = z[q] * z[q] + z[q + 1] * z[q + 1], nd = dd[q] * dd[q] + dd[q + 1] * dd[q + 1], np = ph[q] * ph[q] + ph[q + 1] * ph[q + 1];
      ke[n] += 0.25 * cm * a2 * (nz + nd) / (n * (n + 1.0));
      pe[n] += 0.25 * cm * p.gravity * np / g2;
    }
  }
}

}  // namespace lmw
