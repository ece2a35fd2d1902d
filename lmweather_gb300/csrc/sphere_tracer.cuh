// Passive tracer q on the FP64 path (included by sphere.cu): the reference's tracer tendency
// dq = A(q delta) - D(U q, V q) (cpp/sphere.cpp:250-263), i.e. -v . grad q, advanced by the same RK4 stages as the
// flow and filtered with Phi's del^4 factor. Three kernels per stage beside the flow's three:
//   trc_synth     per (m, 32 latitudes): Fourier coefficients of q and delta at both mirror latitudes
//   trc_grid      per latitude pair: U, V (from the flow's synthesis), q, delta -> inverse FFTs -> U q, V q, q delta
//                 -> forward FFTs -> weighted, folded analysis inputs
//   trc_analysis  per 32 coefficients: the two analysis sums, the tendency and the RK4 update of q
#pragma once

namespace lmw {
namespace {

constexpr int TRC_Q = 4;     // per chunk: q P and delta P sums (complex)
constexpr int TRC_SLOT = 3;  // folded inputs: U q w_d, V q w_d, q delta w

// x: flow stage input [B][3][ntri]; q: tracer stage input [B][ntri]; fourq: [B][nlat][2][M] (q, delta)
__global__ void __launch_bounds__(SYN_THREADS) trc_synth(SphDev d, SphTab<double> t, const double2 *__restrict__ x,
                                                         const double2 *__restrict__ qin, double2 *__restrict__ fourq) {
  __shared__ double part[SYN_CHUNKS][TRC_Q][33];
  const int b = blockIdx.z, m = blockIdx.y;
  const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
  const int jh = blockIdx.x * 32 + lane;
  const bool live = jh < d.nh;
  const double2 *xd = x + static_cast<size_t>(b) * 3 * d.ntri + d.ntri, *xq = qin + static_cast<size_t>(b) * d.ntri;
  double2 qs = make_double2(0, 0), ds = qs;
  const int base = d.tri[m];
  if (live) {
#pragma unroll 2
    for (int n = m + c; n <= d.N; n += SYN_CHUNKS) {
      const int q = base + n - m;
      const double P = t.Ps[static_cast<size_t>(q) * d.nh + jh];
      qs = cfma(qs, xq[q], P);
      ds = cfma(ds, xd[q], P);
    }
  }
  part[c][0][lane] = qs.x;
  part[c][1][lane] = qs.y;
  part[c][2][lane] = ds.x;
  part[c][3][lane] = ds.y;
  __syncthreads();
  if (threadIdx.x >= 64 || !live) return;
  const int side = threadIdx.x >> 5;
  double r[TRC_Q];
#pragma unroll
  for (int i = 0; i < TRC_Q; i++) {
    double se = 0, so = 0;
#pragma unroll
    for (int k = 0; k < SYN_CHUNKS; k += 2) {
      se += part[k][i][lane];
      so += part[k + 1][i][lane];
    }
    r[i] = side == 0 ? se + so : se - so;  // P sums: southern even + odd, northern even - odd
  }
  const int j = side == 0 ? jh : d.nlat - 1 - jh;
  double2 *out = fourq + (static_cast<size_t>(b) * d.nlat + j) * 2 * d.M;
  out[m] = make_double2(r[0], r[1]);
  out[d.M + m] = make_double2(r[2], r[3]);
}

// four: the flow's [B][nlat][4][M] (U, V rows 0 and 1); fourq: [B][nlat][2][M]; foldq: [B][nh][TRC_SLOT][2][M]
__global__ void __launch_bounds__(GRID_THREADS) trc_grid(SphDev d, SphTab<double> t, const double2 *__restrict__ four,
                                                        const double2 *__restrict__ fourq, double2 *__restrict__ foldq) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double2 *sm = reinterpret_cast<double2 *>(smraw);
  const int b = blockIdx.y, jh = blockIdx.x;
  const int js = jh, jn = d.nlat - 1 - jh, n = d.nlon, rl = fft_row<3>(n);
  load_pair_spectra<double2, 3>(sm, 2, d, four + (static_cast<size_t>(b) * d.nlat + js) * 4 * d.M,
                                   four + (static_cast<size_t>(b) * d.nlat + jn) * 4 * d.M, d.M);
  load_pair_spectra<double2, 3>(sm + 2 * rl, 2, d, fourq + (static_cast<size_t>(b) * d.nlat + js) * 2 * d.M,
                                   fourq + (static_cast<size_t>(b) * d.nlat + jn) * 2 * d.M, d.M);
  fft_inverse_dit<double2, 3>(sm, 4, n, d.logn, t.tw);
  // cpp/sphere.cpp:255-258: A = U q, B = V q, C = q delta (real part: southern latitude, imaginary: northern)
  double2 *rU = sm, *rV = sm + rl, *rQ = sm + 2 * rl, *rD = sm + 3 * rl;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int kp = fft_at<3>(k);
    const double2 U = rU[kp], V = rV[kp], Q = rQ[kp], D = rD[kp];
    rU[kp] = make_double2(U.x * Q.x, U.y * Q.y);
    rV[kp] = make_double2(V.x * Q.x, V.y * Q.y);
    rQ[kp] = make_double2(Q.x * D.x, Q.y * D.y);
  }
  __syncthreads();
  fft_forward_dif<double2, 3>(sm, TRC_SLOT, n, d.logn, t.tw);
  const double inv = 1.0 / n, wd = t.wd[js], wj = t.w[js];
  double2 *o = foldq + (static_cast<size_t>(b) * d.nh + jh) * TRC_SLOT * 2 * d.M;
  for (int e = threadIdx.x; e < TRC_SLOT * d.M; e += blockDim.x) {
    const int r = e / d.M, m = e - r * d.M;
    const double2 *row = sm + static_cast<size_t>(r) * rl;
    const double2 Ym = row[fft_at<3>(bitrev(m, d.logn))], Yc = conjd(row[fft_at<3>(bitrev((n - m) & (n - 1), d.logn))]);
    const double hinv = 0.5 * inv;
    double2 Xs = cscale(cadd(Ym, Yc), hinv);
    const double2 tt = csub(Ym, Yc);
    double2 Xn = make_double2(hinv * tt.y, -hinv * tt.x);
    const double wt = r < 2 ? wd : wj;
    Xs = cscale(Xs, wt);
    Xn = cscale(Xn, wt);
    o[(r * 2 + 0) * d.M + m] = cadd(Xs, Xn);
    o[(r * 2 + 1) * d.M + m] = csub(Xs, Xn);
  }
}

// q0: tracer state, qs: stage input, qacc: RK4 accumulator, all [B][ntri]
__global__ void __launch_bounds__(ANA_THREADS) trc_analysis(SphDev d, SphTab<double> t, const double2 *__restrict__ foldq, StageArgs sa,
                                                           double2 *q0, double2 *qs, double2 *qacc) {
  __shared__ double part[ANA_CHUNKS][6][33];
  const int b = blockIdx.y;
  const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
  const int q = blockIdx.x * 32 + lane;
  const bool live = q < d.ntri;
  const int m = live ? d.trim[q] : 0, n = live ? d.trin[q] : 0, par = (n - m) & 1;
  const double2 *fb = foldq + static_cast<size_t>(b) * d.nh * TRC_SLOT * 2 * d.M;
  const int sP = par * d.M + m, sH = (1 - par) * d.M + m;
  double2 aP = make_double2(0, 0), bH = aP, cP = aP;
  if (live) {
#pragma unroll 2
    for (int jh = c; jh < d.nh; jh += ANA_CHUNKS) {
      const double P = t.Pa[static_cast<size_t>(jh) * d.ntri + q], H = t.Ha[static_cast<size_t>(jh) * d.ntri + q];
      const double2 *g = fb + static_cast<size_t>(jh) * TRC_SLOT * 2 * d.M;
      aP = cfma(aP, g[0 * 2 * d.M + sP], P);
      bH = cfma(bH, g[1 * 2 * d.M + sH], H);
      cP = cfma(cP, g[2 * 2 * d.M + sP], P);
    }
  }
  const double v[6] = {aP.x, aP.y, bH.x, bH.y, cP.x, cP.y};
#pragma unroll
  for (int i = 0; i < 6; i++) part[c][i][lane] = v[i];
  __syncthreads();
  if (c != 0 || !live) return;
  double s[6];
#pragma unroll
  for (int i = 0; i < 6; i++) {
    double a = 0;
#pragma unroll
    for (int k = 0; k < ANA_CHUNKS; k++) a += part[k][i][lane];
    s[i] = a;
  }
  aP = make_double2(s[0], s[1]);
  bH = make_double2(s[2], s[3]);
  cP = make_double2(s[4], s[5]);
  // dq = A(q delta) - D(U q, V q), D(A, B) = i m A_P - B_H (cpp/sphere.cpp:259-262)
  const double2 kq = csub(cP, csub(imul(aP, static_cast<double>(m)), bH));
  const size_t i = static_cast<size_t>(b) * d.ntri + q;
  if (sa.stage == 0) {
    qacc[i] = kq;
    qs[i] = cadd(q0[i], cscale(kq, sa.c));
  } else if (sa.stage < 3) {
    qacc[i] = cadd(qacc[i], cscale(kq, 2.0));
    qs[i] = cadd(q0[i], cscale(kq, sa.c));
  } else {
    const double2 val = cadd(q0[i], cscale(cadd(qacc[i], kq), sa.c));
    q0[i] = q == 0 ? val : cscale(val, sa.filt[d.M + n]);  // Phi's del^4 factor (cpp/sphere.cpp:400-404)
  }
}

// Fourier rows of q (row 0 of fourq) -> grid (the tracer grid of the diagnostics)
__global__ void __launch_bounds__(GRID_THREADS) trc_to_grid(SphDev d, const double2 *__restrict__ fourq, double *__restrict__ out) {
  extern __shared__ double2 smq[];
  const int b = blockIdx.y, jh = blockIdx.x;
  const int js = jh, jn = d.nlat - 1 - jh, n = d.nlon;
  load_pair_spectra(smq, 1, d, fourq + (static_cast<size_t>(b) * d.nlat + js) * 2 * d.M, fourq + (static_cast<size_t>(b) * d.nlat + jn) * 2 * d.M,
                    d.M);
  fft_inverse_dit(smq, 1, n, d.logn, d.tw);
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    out[(static_cast<size_t>(b) * d.nlat + js) * n + k] = smq[k].x;
    out[(static_cast<size_t>(b) * d.nlat + jn) * n + k] = smq[k].y;
  }
}

// sum of |q| per member (the tracer's share of the finiteness guard, cpp/sphere.cpp:449-455)
__global__ void __launch_bounds__(GRID_THREADS) trc_abs_sum(SphDev d, const double2 *__restrict__ q, Reduce *out) {
  __shared__ double red[GRID_THREADS / 32];
  const double2 *qb = q + static_cast<size_t>(blockIdx.x) * d.ntri;
  double s = 0;
  for (int i = threadIdx.x; i < d.ntri; i += blockDim.x) s += hypot(qb[i].x, qb[i].y);
  s = block_sum(s, red);
  if (threadIdx.x == 0) out[blockIdx.x].sum[5] += s;
}

}  // namespace
}  // namespace lmw
