// surface.cuh -- TFSF 1-D auxiliary grid, NF-FF running DFT, far-field
// integration, sparse lumped-element and probe kernels, step counter.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace xg {

// ------------------------------------------------------------------------
// TFSF3D::updateIncidentField (src/tfsf/tfsf_3d.cpp:153-183) for one step,
// in one block.  state = [e_inc (L) | h_inc (L-1) | a | b].  The projected
// arrays of this step go to buffer (t & 1) of `inc`.
struct AuxParams {
  int L;
  double *state;
  double *inc;
  float *incf;             // FP32 copy of inc (FP32 form), or null
  const double *source;    // e0 * w(t dt)
  double ceihi, chiei, c1, c2;
  double te[3], th[3];
  const long long *step;
  long long total;
  int *status;
};

// Body of the 1-D line update for one block (all of its threads).
__device__ __forceinline__ void tfsf_aux_block(const AuxParams &p) {
  const long long t = *p.step;
  if (t >= p.total) {
    if (threadIdx.x == 0) atomicExch(p.status, 6);
    return;
  }
  const int L = p.L;
  double *e = p.state;
  double *h = p.state + L;
  double *ab = p.state + 2 * L - 1;
  __shared__ double xy[2];
  if (threadIdx.x == 0) {
    e[0] = p.source[t];
    xy[0] = e[L - 2];
    xy[1] = e[L - 1];
  }
  __syncthreads();
  for (int i = 1 + threadIdx.x; i < L - 1; i += blockDim.x) e[i] = 1.0 * e[i] + p.ceihi * (h[i] - h[i - 1]);
  __syncthreads();
  if (threadIdx.x == 0) {
    const double x = xy[0], y = xy[1];
    e[L - 1] = -ab[0] + p.c1 * (e[L - 2] + ab[1]) + p.c2 * (x + y);
    ab[0] = x;
    ab[1] = y;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < L - 1; i += blockDim.x) h[i] = 1.0 * h[i] + p.chiei * (e[i + 1] - e[i]);
  __syncthreads();
  double *out = p.inc + (t & 1) * 6 * L;
  float *outf = p.incf ? p.incf + (t & 1) * 6 * L : nullptr;
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const double ev = e[i];
    double o[6] = {p.te[0] * ev, p.te[1] * ev, p.te[2] * ev, 0, 0, 0};
    if (i < L - 1) {
      const double hv = h[i];
      o[3] = p.th[0] * hv;
      o[4] = p.th[1] * hv;
      o[5] = p.th[2] * hv;
    }
    const int nc = i < L - 1 ? 6 : 3;
    for (int c = 0; c < nc; ++c) {
      out[c * L + i] = o[c];
      if (outf) outf[c * L + i] = static_cast<float>(o[c]);
    }
  }
}

__global__ void k_tfsf_aux(AuxParams p) { tfsf_aux_block(p); }

// ------------------------------------------------------------------------
// NffftFd::update (src/nffft/nffft_fd.cpp:108-203) with the face-centre
// interpolations of EMF (src/electromagnetic_field/linear_interpolation_emf.cpp:286-421).
// blockIdx.z selects the face pair (0: x, 1: y, 2: z).  Accumulators are
// complex FP64 in both precisions.  Device layout: X faces [n][j][k],
// Y faces [n][i][k] (k contiguous; the reference's order is [n][k][i]),
// Z faces [n][i][j].
template <typename T>
struct NfParams {
  Dims d;
  const T *E[3];
  const T *H[3];
  int lo[3], hi[3];
  int nf;
  double2 *acc[24];
  const double2 *pj, *pm;   // [nf][total]
  const float2 *pjf, *pmf;  // the same tables rounded to FP32 (FP32 form only)
  long long total;
  const long long *step;
  T *buf[3];                // per face pair: [batch][8][face cells] surface values
  int batch;
};

// Samples face pair `face` at face coordinates (u, v) (u the fastest axis)
// for step *step - lag.  part 0 takes all eight values of a face pair; part
// 1 the four from E (the M currents), part 2 the four from H (the J
// currents): E is final once the step's E update and corrections are done,
// H once its H update is, so each half can be taken while the other field
// is still being updated.
template <typename T>
__device__ __forceinline__ void nffft_sample(const NfParams<T> &p, int face, int u, int v, int part = 0,
                                             int lag = 0) {
  const long long t = *p.step - lag;
  if (t < 0 || t >= p.total) return;
  const int li = p.lo[0], lj = p.lo[1], lk = p.lo[2], ri = p.hi[0], rj = p.hi[1], rk = p.hi[2];
  const long long si = p.d.si, sj = p.d.sj;
  const T *ex = p.E[0], *ey = p.E[1], *ez = p.E[2], *hx = p.H[0], *hy = p.H[1], *hz = p.H[2];
  // the face-centre averages are taken in the field precision: FP64 as the
  // reference does; FP32 in the FP32 form, whose samples are stored as FP32
  auto at = [&](const T *f, int i, int j, int k) -> T {
    return f[static_cast<long long>(i) * si + static_cast<long long>(j) * sj + k];
  };
  const T half = T(0.5), quarter = T(0.25), neg = T(-1);
  const bool want_e = part != 2, want_h = part != 1;
  T val[8] = {};
  long long cell, plane;
  int base;
  if (face == 0) {  // X faces: j in [lj, rj), k in [lk, rk); jy, jz, my, mz
    const int k = lk + u, j = lj + v;
    if (k >= rk || j >= rj) return;
    // M = -/+ E face centres, J = +/- H face centres
    if (want_e) val[2] = neg * (half * (at(ez, li, j, k) + at(ez, li, j + 1, k)));            // my_xn
    if (want_e) val[3] = half * (at(ey, li, j, k) + at(ey, li, j, k + 1));                   // mz_xn
    if (want_h) val[0] = quarter * (at(hz, li, j, k) + at(hz, li, j, k + 1) + at(hz, li - 1, j, k) + at(hz, li - 1, j, k + 1));
    if (want_h) val[1] = neg * (quarter * (at(hy, li, j, k) + at(hy, li, j + 1, k) + at(hy, li - 1, j, k) + at(hy, li - 1, j + 1, k)));
    if (want_e) val[6] = half * (at(ez, ri, j, k) + at(ez, ri, j + 1, k));                   // my_xp
    if (want_e) val[7] = neg * (half * (at(ey, ri, j, k) + at(ey, ri, j, k + 1)));            // mz_xp
    if (want_h) val[4] = neg * (quarter * (at(hz, ri, j, k) + at(hz, ri, j, k + 1) + at(hz, ri - 1, j, k) + at(hz, ri - 1, j, k + 1)));
    if (want_h) val[5] = quarter * (at(hy, ri, j, k) + at(hy, ri, j + 1, k) + at(hy, ri - 1, j, k) + at(hy, ri - 1, j + 1, k));
    cell = static_cast<long long>(j - lj) * (rk - lk) + (k - lk);
    plane = static_cast<long long>(rj - lj) * (rk - lk);
    base = 0;
  } else if (face == 1) {  // Y faces: k in [lk, rk), i in [li, ri); jz, jx, mz, mx
    const int k = lk + u, i = li + v;
    if (k >= rk || i >= ri) return;
    if (want_e) val[2] = neg * (half * (at(ex, i, lj, k) + at(ex, i, lj + 1, k)));            // mz_yn
    if (want_e) val[3] = half * (at(ez, i, lj, k) + at(ez, i + 1, lj, k));                   // mx_yn
    if (want_h) val[0] = quarter * (at(hx, i + 1, lj, k) + at(hx, i, lj, k) + at(hx, i + 1, lj - 1, k) + at(hx, i, lj - 1, k));
    if (want_h) val[1] = neg * (quarter * (at(hz, i, lj, k) + at(hz, i, lj, k + 1) + at(hz, i, lj - 1, k) + at(hz, i, lj - 1, k + 1)));
    if (want_e) val[6] = half * (at(ex, i, rj, k) + at(ex, i, rj + 1, k));                   // mz_yp
    if (want_e) val[7] = neg * (half * (at(ez, i, rj, k) + at(ez, i + 1, rj, k)));            // mx_yp
    if (want_h) val[4] = neg * (quarter * (at(hx, i + 1, rj, k) + at(hx, i, rj, k) + at(hx, i + 1, rj - 1, k) + at(hx, i, rj - 1, k)));
    if (want_h) val[5] = quarter * (at(hz, i, rj, k) + at(hz, i, rj, k + 1) + at(hz, i, rj - 1, k) + at(hz, i, rj - 1, k + 1));
    cell = static_cast<long long>(i - li) * (rk - lk) + (k - lk);
    plane = static_cast<long long>(ri - li) * (rk - lk);
    base = 8;
  } else {  // Z faces: i in [li, ri), j in [lj, rj); jx, jy, mx, my
    const int j = lj + u, i = li + v;
    if (j >= rj || i >= ri) return;
    if (want_e) val[2] = neg * (half * (at(ey, i, j, lk) + at(ey, i + 1, j, lk)));            // mx_zn
    if (want_e) val[3] = half * (at(ex, i, j, lk) + at(ex, i, j, lk + 1));                   // my_zn
    if (want_h) val[0] = quarter * (at(hy, i, j, lk) + at(hy, i, j + 1, lk) + at(hy, i, j, lk - 1) + at(hy, i, j + 1, lk - 1));
    if (want_h) val[1] = neg * (quarter * (at(hx, i + 1, j, lk) + at(hx, i, j, lk) + at(hx, i + 1, j, lk - 1) + at(hx, i, j, lk - 1)));
    if (want_e) val[6] = half * (at(ey, i, j, rk) + at(ey, i + 1, j, rk));                   // mx_zp
    if (want_e) val[7] = neg * (half * (at(ex, i, j, rk) + at(ex, i, j, rk + 1)));            // my_zp
    if (want_h) val[4] = neg * (quarter * (at(hy, i, j, rk) + at(hy, i, j + 1, rk) + at(hy, i, j, rk - 1) + at(hy, i, j + 1, rk - 1)));
    if (want_h) val[5] = quarter * (at(hx, i + 1, j, rk) + at(hx, i, j, rk) + at(hx, i + 1, j, rk - 1) + at(hx, i, j, rk - 1));
    cell = static_cast<long long>(i - li) * (rj - lj) + (j - lj);
    plane = static_cast<long long>(ri - li) * (rj - lj);
    base = 16;
  }
  // store the step's surface values in slot t % batch; k_nffft_accumulate
  // folds a whole batch into the FP64 accumulators (values 0, 1, 4, 5 come
  // from H, 2, 3, 6, 7 from E)
  T *buf = p.buf[base / 8] + (static_cast<long long>(t % p.batch) * 8) * plane + cell;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const bool from_e = (q & 2) != 0;
    if (part == 0 || (part == 1) == from_e) buf[q * plane] = val[q];
  }
}

template <typename T>
__global__ void k_nffft(NfParams<T> p, int part, int lag) {
  nffft_sample(p, blockIdx.z, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y, part,
               lag);
}

// acc[n] += v[s] * phase[n][t0 + s] for the `count` (<= 8) buffered steps
// ending at step *step - lag.  FP64 form: added one step at a time in step
// order, the same additions in the same order as accumulating every step
// (nffft_fd.cpp:117-203).  FP32 form: the batch's products are summed in FP32
// (the samples are FP32 already) and the partial sum is added to the FP64
// running sum, which carries the thousands-of-steps accumulation.
constexpr int kMaxNfBatch = 8;

template <typename T>
__device__ __forceinline__ void nffft_fold(const NfParams<T> &p, int group, long long cell, int count, int lag) {
  const int lo_a = group == 0 ? p.lo[1] : p.lo[0], hi_a = group == 0 ? p.hi[1] : p.hi[0];
  const int lo_b = group == 2 ? p.lo[1] : p.lo[2], hi_b = group == 2 ? p.hi[1] : p.hi[2];
  const long long plane = static_cast<long long>(hi_a - lo_a) * (hi_b - lo_b);
  if (cell >= plane) return;
  const long long t_last = *p.step - lag;
  const long long t0 = t_last - count + 1;
  if (t0 < 0 || t_last >= p.total || count > kMaxNfBatch) return;
  const T *buf = p.buf[group] + cell;
  for (int q = 0; q < 8; ++q) {
    T v[kMaxNfBatch];
#pragma unroll
    for (int s = 0; s < kMaxNfBatch; ++s)
      v[s] = s < count ? buf[(static_cast<long long>((t0 + s) % p.batch) * 8 + q) * plane] : T(0);
    const bool j_term = (q % 4) < 2;   // J terms use the (t+1/2) phase, M terms t
    for (int n = 0; n < p.nf; ++n) {
      double2 *a = p.acc[group * 8 + q] + n * plane + cell;
      double2 r = *a;
      if constexpr (sizeof(T) == 8) {
        const double2 *ph = (j_term ? p.pj : p.pm) + n * p.total + t0;
#pragma unroll
        for (int s = 0; s < kMaxNfBatch; ++s)
          if (s < count) {
            const double2 f = ph[s];
            r.x = fma(static_cast<double>(v[s]), f.x, r.x);
            r.y = fma(static_cast<double>(v[s]), f.y, r.y);
          }
      } else {
        const float2 *ph = (j_term ? p.pjf : p.pmf) + n * p.total + t0;
        float2 part = make_float2(0.f, 0.f);
#pragma unroll
        for (int s = 0; s < kMaxNfBatch; ++s)
          if (s < count) {
            const float2 f = ph[s];
            part.x = fmaf(static_cast<float>(v[s]), f.x, part.x);
            part.y = fmaf(static_cast<float>(v[s]), f.y, part.y);
          }
        r.x += static_cast<double>(part.x);
        r.y += static_cast<double>(part.y);
      }
      *a = r;
    }
  }
}

template <typename T>
__global__ void k_nffft_accumulate(NfParams<T> p, int count, int lag) {
  nffft_fold(p, blockIdx.z, blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x, count, lag);
}

// ------------------------------------------------------------------------
// NffftFd::calculateFarfield{,X,Y,Z} (src/nffft/nffft_fd.cpp:379-556): one
// block per (frequency, theta, phi).  Each thread sums a strided share of
// the surface, the block reduces with warp shuffles, thread 0 projects and
// writes E/H theta/phi, N/L theta/phi and the power pattern.
struct FarParams {
  int lo[3], hi[3];
  int nf, nt, np;
  const double2 *acc[24];
  const double *theta, *phi, *k;
  double dl[3];
  double eta0, pi;
  double2 *out[8];
  double *power[2];
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

__global__ void __launch_bounds__(256) k_far_field(FarParams p) {
  const int q = blockIdx.x;
  const int n = q / (p.nt * p.np), t = (q / p.np) % p.nt, pp = q % p.np;
  const double cos_t = cos(p.theta[t]), sin_t = sin(p.theta[t]);
  const double cos_p = cos(p.phi[pp]), sin_p = sin(p.phi[pp]);
  const double stcp = sin_t * cos_p, stsp = sin_t * sin_p;
  const int li = p.lo[0], lj = p.lo[1], lk = p.lo[2], ri = p.hi[0], rj = p.hi[1], rk = p.hi[2];
  const int bx = ri - li, by = rj - lj, bz = rk - lk;
  // s[0..3]: X faces jy jz my mz; s[4..7]: Y faces jz jx mz mx; s[8..11]: Z faces jx jy mx my
  double2 s[12];
#pragma unroll
  for (int r = 0; r < 12; ++r) s[r] = make_double2(0.0, 0.0);
  {
    const double dk = p.dl[0] * p.k[n];
    const long long cnt = static_cast<long long>(by) * bz;
    for (long long c = threadIdx.x; c < cnt; c += blockDim.x) {
      const int a = static_cast<int>(c / bz), b = static_cast<int>(c % bz);
      const int j = lj + a, k = lk + b;
      double sn, cn, sp, cp;
      sincos(dk * (li * stcp + (j + 0.5) * stsp + (k + 0.5) * cos_t), &sn, &cn);
      sincos(dk * (ri * stcp + (j + 0.5) * stsp + (k + 0.5) * cos_t), &sp, &cp);
      const double2 pn = make_double2(cn, sn), pq = make_double2(cp, sp);
      const long long o = static_cast<long long>(n) * cnt + c;
#pragma unroll
      for (int r = 0; r < 4; ++r) s[r] = cadd(s[r], cadd(cmul(p.acc[r][o], pn), cmul(p.acc[4 + r][o], pq)));
    }
  }
  {
    const double dk = p.dl[1] * p.k[n];
    const long long cnt = static_cast<long long>(bz) * bx;
    for (long long c = threadIdx.x; c < cnt; c += blockDim.x) {
      const int a = static_cast<int>(c / bz), b = static_cast<int>(c % bz);   // device layout [i][k]
      const int i = li + a, k = lk + b;
      double sn, cn, sp, cp;
      sincos(dk * ((i + 0.5) * stcp + lj * stsp + (k + 0.5) * cos_t), &sn, &cn);
      sincos(dk * ((i + 0.5) * stcp + rj * stsp + (k + 0.5) * cos_t), &sp, &cp);
      const double2 pn = make_double2(cn, sn), pq = make_double2(cp, sp);
      const long long o = static_cast<long long>(n) * cnt + c;
#pragma unroll
      for (int r = 0; r < 4; ++r) s[4 + r] = cadd(s[4 + r], cadd(cmul(p.acc[8 + r][o], pn), cmul(p.acc[12 + r][o], pq)));
    }
  }
  {
    const double dk = p.dl[2] * p.k[n];
    const long long cnt = static_cast<long long>(bx) * by;
    for (long long c = threadIdx.x; c < cnt; c += blockDim.x) {
      const int a = static_cast<int>(c / by), b = static_cast<int>(c % by);
      const int i = li + a, j = lj + b;
      double sn, cn, sp, cp;
      sincos(dk * ((i + 0.5) * stcp + (j + 0.5) * stsp + lk * cos_t), &sn, &cn);
      sincos(dk * ((i + 0.5) * stcp + (j + 0.5) * stsp + rk * cos_t), &sp, &cp);
      const double2 pn = make_double2(cn, sn), pq = make_double2(cp, sp);
      const long long o = static_cast<long long>(n) * cnt + c;
#pragma unroll
      for (int r = 0; r < 4; ++r) s[8 + r] = cadd(s[8 + r], cadd(cmul(p.acc[16 + r][o], pn), cmul(p.acc[20 + r][o], pq)));
    }
  }
  // block reduction of the 24 doubles
  __shared__ double red[8][24];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < 12; ++r) {
    double x = s[r].x, y = s[r].y;
    for (int off = 16; off > 0; off >>= 1) {
      x += __shfl_down_sync(0xffffffffu, x, off);
      y += __shfl_down_sync(0xffffffffu, y, off);
    }
    if (lane == 0) { red[warp][2 * r] = x; red[warp][2 * r + 1] = y; }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int nw = blockDim.x / 32;
  double tot[24];
  for (int r = 0; r < 24; ++r) {
    double acc = 0;
    for (int w = 0; w < nw; ++w) acc += red[w][r];
    tot[r] = acc;
  }
  auto S = [&](int r) { return make_double2(tot[2 * r], tot[2 * r + 1]); };
  const double dy_dz = p.dl[1] * p.dl[2], dz_dx = p.dl[2] * p.dl[0], dx_dy = p.dl[0] * p.dl[1];
  double2 zero = make_double2(0.0, 0.0);
  // X adds a_y a_z f_y f_z; Y adds a_z a_x f_z f_x; Z adds a_x a_y f_x f_y (that order)
  double2 a_x = zero, a_y = zero, a_z = zero, f_x = zero, f_y = zero, f_z = zero;
  a_y = cadd(a_y, cscale(S(0), dy_dz)); a_z = cadd(a_z, cscale(S(1), dy_dz));
  f_y = cadd(f_y, cscale(S(2), dy_dz)); f_z = cadd(f_z, cscale(S(3), dy_dz));
  a_z = cadd(a_z, cscale(S(4), dz_dx)); a_x = cadd(a_x, cscale(S(5), dz_dx));
  f_z = cadd(f_z, cscale(S(6), dz_dx)); f_x = cadd(f_x, cscale(S(7), dz_dx));
  a_x = cadd(a_x, cscale(S(8), dx_dy)); a_y = cadd(a_y, cscale(S(9), dx_dy));
  f_x = cadd(f_x, cscale(S(10), dx_dy)); f_y = cadd(f_y, cscale(S(11), dx_dy));
  const double ctcp = cos_t * cos_p, ctsp = cos_t * sin_p;
  const double2 a_th = cadd(cadd(cscale(a_x, ctcp), cscale(a_y, ctsp)), cscale(a_z, -sin_t));
  const double2 a_ph = cadd(cscale(a_x, -sin_p), cscale(a_y, cos_p));
  const double2 f_th = cadd(cadd(cscale(f_x, ctcp), cscale(f_y, ctsp)), cscale(f_z, -sin_t));
  const double2 f_ph = cadd(cscale(f_x, -sin_p), cscale(f_y, cos_p));
  const double k = p.k[n], eta = p.eta0, fp = 4 * p.pi;
  const double coff = (k * k) / (32 * p.pi * p.pi * eta);
  // e_theta = (-i k)(eta a_th + f_ph)/(4 pi), e_phi = (i k)(-eta a_ph + f_th)/(4 pi),
  // h_theta = (i k)(a_ph - f_th/eta)/(4 pi), h_phi = (-i k)(a_th + f_ph/eta)/(4 pi)
  const double2 u1 = cadd(cscale(a_th, eta), f_ph);
  const double2 u2 = cadd(cscale(a_ph, -eta), f_th);
  const double2 u3 = make_double2(a_ph.x - f_th.x / eta, a_ph.y - f_th.y / eta);
  const double2 u4 = make_double2(a_th.x + f_ph.x / eta, a_th.y + f_ph.y / eta);
  const double2 mik = make_double2(-0.0, -k), pik = make_double2(0.0, k);
  auto div = [](double2 a, double s) { return make_double2(a.x / s, a.y / s); };
  p.out[0][q] = div(cmul(mik, u1), fp);
  p.out[1][q] = div(cmul(pik, u2), fp);
  p.out[2][q] = div(cmul(pik, u3), fp);
  p.out[3][q] = div(cmul(mik, u4), fp);
  p.out[4][q] = a_th;
  p.out[5][q] = a_ph;
  p.out[6][q] = f_th;
  p.out[7][q] = f_ph;
  const double m1 = hypot(u1.x, u1.y), m2 = hypot(u2.x, u2.y);
  p.power[0][q] = coff * (m1 * m1);
  p.power[1][q] = coff * (m2 * m2);
}

// ------------------------------------------------------------------------
// TFSF3D::updateE / updateH face corrections (src/tfsf/tfsf_3d.cpp:185-411).
// One thread per cell of the surface of the face box ([lo, hi] on every axis
// for E, [lo-1, hi] for H), split into six disjoint parts (the two x planes
// whole, the two y planes without their x edges, the two z planes without
// their x and y edges).  A thread applies every face correction its cell
// receives, per component, in the reference's face order (x, then y, then z).
template <typename T>
struct TfsfSurfParams {
  Dims d;
  T *F[6];
  TfsfDev tf;
  const long long *step;
};

__device__ __forceinline__ void add_corr(double &v, double corr) { v = v + corr; }
__device__ __forceinline__ void add_corr(float &v, float corr) { v = v + corr; }

// Maps a linear surface index to (i, j, k) on the surface of [a0,a1]x[b0,b1]x[c0,c1]
// (32-bit arithmetic: a surface holds far fewer than 2^31 cells).
__device__ __forceinline__ bool surface_cell(int q, int a0, int a1, int b0, int b1, int c0, int c1, int &i, int &j,
                                             int &k) {
  const int nb = b1 - b0 + 1, nc = c1 - c0 + 1, na_in = max(a1 - a0 - 1, 0), nb_in = max(b1 - b0 - 1, 0);
  const int px = nb * nc, py = na_in * nc, pz = na_in * nb_in;
  if (q < 2 * px) {
    i = q < px ? a0 : a1;
    const int r = q < px ? q : q - px;
    j = b0 + r / nc;
    k = c0 + r % nc;
    return true;
  }
  q -= 2 * px;
  if (q < 2 * py) {
    j = q < py ? b0 : b1;
    const int r = q < py ? q : q - py;
    i = a0 + 1 + r / nc;
    k = c0 + r % nc;
    return true;
  }
  q -= 2 * py;
  if (q < 2 * pz) {
    k = q < pz ? c0 : c1;
    const int r = q < pz ? q : q - pz;
    i = a0 + 1 + r / nb_in;
    j = b0 + 1 + r % nb_in;
    return true;
  }
  return false;
}

// Whether (i, j, k) lies on the surface of the TFSF E box [lo, hi] (the
// cells TFSF3D::updateE may correct) or of the H box [lo-1, hi].
__device__ __forceinline__ bool tfsf_on_e_surface(const TfsfDev &tf, int i, int j, int k) {
  return i >= tf.lo[0] && i <= tf.hi[0] && j >= tf.lo[1] && j <= tf.hi[1] && k >= tf.lo[2] && k <= tf.hi[2] &&
         (i == tf.lo[0] || i == tf.hi[0] || j == tf.lo[1] || j == tf.hi[1] || k == tf.lo[2] || k == tf.hi[2]);
}
__device__ __forceinline__ bool tfsf_h_terms(const TfsfDev &tf, int i, int j, int k) {
  if (tf.two_d)   // TFSF2D: the x and y faces of the one z cell
    return k >= tf.lo[2] && k < tf.hi[2] && i >= tf.lo[0] - 1 && i <= tf.hi[0] && j >= tf.lo[1] - 1 &&
           j <= tf.hi[1] && (i == tf.lo[0] - 1 || i == tf.hi[0] || j == tf.lo[1] - 1 || j == tf.hi[1]);
  return i >= tf.lo[0] - 1 && i <= tf.hi[0] && j >= tf.lo[1] - 1 && j <= tf.hi[1] && k >= tf.lo[2] - 1 &&
         k <= tf.hi[2] &&
         (i == tf.lo[0] - 1 || i == tf.hi[0] || j == tf.lo[1] - 1 || j == tf.hi[1] || k == tf.lo[2] - 1 ||
          k == tf.hi[2]);
}

// TFSF3D::updateE (src/tfsf/tfsf_3d.cpp:299-411) for one cell and one E
// component C: which of the component's two face corrections apply at
// (i, j, k) (bit 0: the first face pair, bit 1: the second) ...
template <int C>
__device__ __forceinline__ int tfsf_e_terms(const TfsfDev &tf, int i, int j, int k) {
  const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
  if (C == 0)   // Ex: y faces, z faces
    return (((j == lj || j == rj) && k >= lk && k <= rk && i >= li && i < ri) ? 1 : 0) |
           (((k == lk || k == rk) && i >= li && i < ri && j >= lj && j <= rj) ? 2 : 0);
  if (C == 1)   // Ey: x faces, z faces
    return (((i == li || i == ri) && j >= lj && j < rj && k >= lk && k <= rk) ? 1 : 0) |
           (((k == lk || k == rk) && i >= li && i <= ri && j >= lj && j < rj) ? 2 : 0);
  // Ez: x faces, y faces
  return (((i == li || i == ri) && j >= lj && j <= rj && k >= lk && k < rk) ? 1 : 0) |
         (((j == lj || j == rj) && k >= lk && k < rk && i >= li && i <= ri) ? 2 : 0);
}

// ... and adds them to e, first face pair first.  hinc: the incident H
// arrays of the previous step.
template <int C, typename T>
__device__ __forceinline__ void tfsf_e_add(const TfsfDev &tf, const decltype(tfsf_view<T>(tf).inc) hinc, int i, int j,
                                           int k, int terms, T &e) {
  const auto V = tfsf_view<T>(tf);
  using R = typename std::remove_const<typename std::remove_pointer<decltype(V.inc)>::type>::type;
  const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
  if (C == 0) {
    // Ex: y faces (j = lj: -= cay Hz_inc(i, lj-1, k); j = rj: += cay Hz_inc(i, rj, k)),
    //     z faces (k = lk: += caz Hy_inc(i, j, lk-1); k = rk: -= caz Hy_inc(i, j, rk))
    if (terms & 1) {
      const int jj = j == lj ? lj - 1 : rj;
      const R pr = V.ph[0][i - li + 1] + V.ph[1][jj - lj + 1] + V.pf[2][k - lk] - R(0.5);
      const R v = V.ca[1] * tfsf_interp(hinc + 5 * tf.L, pr);
      add_corr(e, j == lj ? -v : v);
    }
    if (terms & 2) {
      const int kk = k == lk ? lk - 1 : rk;
      const R pr = V.ph[0][i - li + 1] + V.pf[1][j - lj] + V.ph[2][kk - lk + 1] - R(0.5);
      const R v = V.ca[2] * tfsf_interp(hinc + 4 * tf.L, pr);
      add_corr(e, k == lk ? v : -v);
    }
  } else if (C == 1) {
    // Ey: x faces (i = li: += cax Hz_inc(li-1, j, k); i = ri: -= cax Hz_inc(ri, j, k)),
    //     z faces (k = lk: -= caz Hx_inc(i, j, lk-1); k = rk: += caz Hx_inc(i, j, rk))
    if (terms & 1) {
      const int ii = i == li ? li - 1 : ri;
      const R pr = V.ph[0][ii - li + 1] + V.ph[1][j - lj + 1] + V.pf[2][k - lk] - R(0.5);
      const R v = V.ca[0] * tfsf_interp(hinc + 5 * tf.L, pr);
      add_corr(e, i == li ? v : -v);
    }
    if (terms & 2) {
      const int kk = k == lk ? lk - 1 : rk;
      const R pr = V.pf[0][i - li] + V.ph[1][j - lj + 1] + V.ph[2][kk - lk + 1] - R(0.5);
      const R v = V.ca[2] * tfsf_interp(hinc + 3 * tf.L, pr);
      add_corr(e, k == lk ? -v : v);
    }
  } else {
    // Ez: x faces (i = li: -= cax Hy_inc(li-1, j, k); i = ri: += cax Hy_inc(ri, j, k)),
    //     y faces (j = lj: += cay Hx_inc(i, lj-1, k); j = rj: -= cay Hx_inc(i, rj, k))
    if (terms & 1) {
      const int ii = i == li ? li - 1 : ri;
      const R pr = V.ph[0][ii - li + 1] + V.pf[1][j - lj] + V.ph[2][k - lk + 1] - R(0.5);
      const R v = V.ca[0] * tfsf_interp(hinc + 4 * tf.L, pr);
      add_corr(e, i == li ? -v : v);
    }
    if (terms & 2) {
      const int jj = j == lj ? lj - 1 : rj;
      const R pr = V.pf[0][i - li] + V.ph[1][jj - lj + 1] + V.ph[2][k - lk + 1] - R(0.5);
      const R v = V.ca[1] * tfsf_interp(hinc + 3 * tf.L, pr);
      add_corr(e, j == lj ? v : -v);
    }
  }
}

// The E corrections of one cell, on its values in registers; w[c] tells
// which components have a term.
template <typename T>
__device__ __forceinline__ void tfsf_e_fused(const TfsfDev &tf, const decltype(tfsf_view<T>(tf).inc) hinc, int i,
                                             int j, int k, T &ex, T &ey, T &ez, bool w[3]) {
  const int t0 = tfsf_e_terms<0>(tf, i, j, k), t1 = tfsf_e_terms<1>(tf, i, j, k), t2 = tfsf_e_terms<2>(tf, i, j, k);
  if (t0) tfsf_e_add<0>(tf, hinc, i, j, k, t0, ex);
  if (t1) tfsf_e_add<1>(tf, hinc, i, j, k, t1, ey);
  if (t2) tfsf_e_add<2>(tf, hinc, i, j, k, t2, ez);
  w[0] = t0 != 0;
  w[1] = t1 != 0;
  w[2] = t2 != 0;
}

template <int C, typename T>
__device__ __forceinline__ void tfsf_e_component(const TfsfSurfParams<T> &p, const decltype(tfsf_view<T>(p.tf).inc) hinc,
                                                 int i, int j, int k, long long b) {
  const int terms = tfsf_e_terms<C>(p.tf, i, j, k);
  if (!terms) return;
  T e = p.F[C][b];
  tfsf_e_add<C>(p.tf, hinc, i, j, k, terms, e);
  p.F[C][b] = e;
}

// TFSF E corrections of surface cell q (surface_cell order).
template <typename T>
__device__ __forceinline__ void tfsf_e_surface(const TfsfSurfParams<T> &p, int q) {
  const TfsfDev &tf = p.tf;
  int i, j, k;
  if (!surface_cell(q, tf.lo[0], tf.hi[0], tf.lo[1], tf.hi[1], tf.lo[2], tf.hi[2], i, j, k)) return;
  const auto hinc = tfsf_view<T>(tf).inc + (((*p.step) + 1) & 1) * 6 * tf.L;   // incident H of the previous step
  const long long b = static_cast<long long>(i) * p.d.si + static_cast<long long>(j) * p.d.sj + k;
  if (!tf.two_d) {   // TFSF2D::updateE corrects Ez only (tfsf_2d.cpp:192-228)
    tfsf_e_component<0>(p, hinc, i, j, k, b);
    tfsf_e_component<1>(p, hinc, i, j, k, b);
  }
  tfsf_e_component<2>(p, hinc, i, j, k, b);
}

template <typename T>
__global__ void k_tfsf_e(TfsfSurfParams<T> p) {
  tfsf_e_surface(p, blockIdx.x * blockDim.x + threadIdx.x);
}

// TFSF3D::updateH (src/tfsf/tfsf_3d.cpp:185-297) at one cell (i, j, k) of
// the surface of the box one cell larger on the low sides: the corrections
// of its H components, added to hx, hy, hz (the values the cell holds after
// the H update); w[c] tells which components have a term.  einc: the
// incident E arrays of this step.
template <typename T>
__device__ __forceinline__ void tfsf_h_cell(const TfsfDev &tf, const decltype(tfsf_view<T>(tf).inc) einc, int i,
                                            int j, int k, T &hx, T &hy, T &hz, bool w[3]) {
  const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
  const auto V = tfsf_view<T>(tf);
  using R = typename std::remove_const<typename std::remove_pointer<decltype(V.inc)>::type>::type;
  w[0] = w[1] = w[2] = false;
  // Hx: y faces (j = lj-1: += cby Ez_inc(i, lj, k); j = rj: -= cby Ez_inc(i, rj, k)),
  //     z faces (k = lk-1: -= cbz Ey_inc(i, j, lk); k = rk: += cbz Ey_inc(i, j, rk))
  // TFSF2D::updateH (tfsf_2d.cpp:150-190) keeps the x- and y-face terms of
  // Hx and Hy: no z faces, no Hz
  const bool two_d = tf.two_d != 0;
  {
    const bool w1 = (j == lj - 1 || j == rj) && k >= lk && k < rk && i >= li && i <= ri;
    const bool w2 = !two_d && (k == lk - 1 || k == rk) && i >= li && i <= ri && j >= lj && j < rj;
    if (w1) {
      const int jj = j == rj ? rj : lj;
      const R pr = V.pf[0][i - li] + V.pf[1][jj - lj] + V.ph[2][k - lk + 1];
      const R v = V.cb[1] * tfsf_interp(einc + 2 * tf.L, pr);
      add_corr(hx, j == rj ? -v : v);
    }
    if (w2) {
      const int kk = k == rk ? rk : lk;
      const R pr = V.pf[0][i - li] + V.ph[1][j - lj + 1] + V.pf[2][kk - lk];
      const R v = V.cb[2] * tfsf_interp(einc + 1 * tf.L, pr);
      add_corr(hx, k == rk ? v : -v);
    }
    w[0] = w1 || w2;
  }
  // Hy: x faces (i = li-1: -= cbx Ez_inc(li, j, k); i = ri: += cbx Ez_inc(ri, j, k)),
  //     z faces (k = lk-1: += cbz Ex_inc(i, j, lk); k = rk: -= cbz Ex_inc(i, j, rk))
  {
    const bool w1 = (i == li - 1 || i == ri) && j >= lj && j <= rj && k >= lk && k < rk;
    const bool w2 = !two_d && (k == lk - 1 || k == rk) && i >= li && i < ri && j >= lj && j <= rj;
    if (w1) {
      const int ii = i == ri ? ri : li;
      const R pr = V.pf[0][ii - li] + V.pf[1][j - lj] + V.ph[2][k - lk + 1];
      const R v = V.cb[0] * tfsf_interp(einc + 2 * tf.L, pr);
      add_corr(hy, i == ri ? v : -v);
    }
    if (w2) {
      const int kk = k == rk ? rk : lk;
      const R pr = V.ph[0][i - li + 1] + V.pf[1][j - lj] + V.pf[2][kk - lk];
      const R v = V.cb[2] * tfsf_interp(einc + 0 * tf.L, pr);
      add_corr(hy, k == rk ? -v : v);
    }
    w[1] = w1 || w2;
  }
  // Hz: x faces (i = li-1: += cbx Ey_inc(li, j, k); i = ri: -= cbx Ey_inc(ri, j, k)),
  //     y faces (j = lj-1: -= cby Ex_inc(i, lj, k); j = rj: += cby Ex_inc(i, rj, k))
  if (!two_d) {
    const bool w1 = (i == li - 1 || i == ri) && j >= lj && j < rj && k >= lk && k <= rk;
    const bool w2 = (j == lj - 1 || j == rj) && k >= lk && k <= rk && i >= li && i < ri;
    if (w1) {
      const int ii = i == ri ? ri : li;
      const R pr = V.pf[0][ii - li] + V.ph[1][j - lj + 1] + V.pf[2][k - lk];
      const R v = V.cb[0] * tfsf_interp(einc + 1 * tf.L, pr);
      add_corr(hz, i == ri ? -v : v);
    }
    if (w2) {
      const int jj = j == rj ? rj : lj;
      const R pr = V.ph[0][i - li + 1] + V.pf[1][jj - lj] + V.pf[2][k - lk];
      const R v = V.cb[1] * tfsf_interp(einc + 0 * tf.L, pr);
      add_corr(hz, j == rj ? v : -v);
    }
    w[2] = w1 || w2;
  }
}

// The H corrections at surface cell q of the box one cell larger on the low
// sides, read from and written back to the fields.
template <typename T>
__device__ __forceinline__ void tfsf_h_surface(const TfsfSurfParams<T> &p, int q) {
  const TfsfDev &tf = p.tf;
  int i, j, k;
  if (!surface_cell(q, tf.lo[0] - 1, tf.hi[0], tf.lo[1] - 1, tf.hi[1], tf.lo[2] - 1, tf.hi[2], i, j, k)) return;
  const auto einc = tfsf_view<T>(tf).inc + ((*p.step) & 1) * 6 * tf.L;   // incident E of this step
  const long long b = static_cast<long long>(i) * p.d.si + static_cast<long long>(j) * p.d.sj + k;
  if (!tfsf_h_terms(tf, i, j, k)) return;
  // load only the components that get a term (tfsf_h_cell's conditions):
  // a face cell corrects one or two of its three
  const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
  const bool two_d = tf.two_d != 0;
  const bool ix = i >= li && i <= ri, iy = j >= lj && j <= rj;
  const bool hx_t = ((j == lj - 1 || j == rj) && k >= lk && k < rk && ix) ||
                    (!two_d && (k == lk - 1 || k == rk) && ix && j >= lj && j < rj);
  const bool hy_t = ((i == li - 1 || i == ri) && iy && k >= lk && k < rk) ||
                    (!two_d && (k == lk - 1 || k == rk) && i >= li && i < ri && iy);
  const bool hz_t = !two_d && (((i == li - 1 || i == ri) && j >= lj && j < rj && k >= lk && k <= rk) ||
                               ((j == lj - 1 || j == rj) && k >= lk && k <= rk && i >= li && i < ri));
  T hx = hx_t ? p.F[3][b] : T(0), hy = hy_t ? p.F[4][b] : T(0), hz = hz_t ? p.F[5][b] : T(0);
  bool w[3];
  tfsf_h_cell<T>(tf, einc, i, j, k, hx, hy, hz, w);
  if (w[0]) p.F[3][b] = hx;
  if (w[1]) p.F[4][b] = hy;
  if (w[2]) p.F[5][b] = hz;
}

template <typename T>
__global__ void k_tfsf_h(TfsfSurfParams<T> p) {
  tfsf_h_surface(p, blockIdx.x * blockDim.x + threadIdx.x);
}

// Number of cells on the surface of [a0,a1]x[b0,b1]x[c0,c1] (surface_cell's range).
inline long long surface_count(int a0, int a1, int b0, int b1, int c0, int c1) {
  const long long nb = b1 - b0 + 1, nc = c1 - c0 + 1, na_in = a1 - a0 - 1, nb_in = b1 - b0 - 1;
  return 2 * nb * nc + 2 * (na_in > 0 ? na_in : 0) * nc + 2 * (na_in > 0 ? na_in : 0) * (nb_in > 0 ? nb_in : 0);
}

// ------------------------------------------------------------------------
// Sparse per-step work.
template <typename T>
struct SparseParams {
  Dims d;
  T *F[6];
  const xfdtd_injection *inj;
  int n_inj;
  const double *waveforms;   // [n_waveforms][total]
  xfdtd_inductor_cell *ind;
  double *ind_j;
  int n_ind;
  const xfdtd_probe_term *terms;
  const int *probe_off;       // [n_probes + 1]
  int n_probes;
  double *probe_out;          // [n_probes][total]
  long long total;
  const long long *step;
};

template <typename T>
__device__ __forceinline__ long long sp_index(const Dims &d, long long i, long long j, long long k) {
  return i * d.si + j * d.sj + k;
}

// ------------------------------------------------------------------------
// Linear dispersive media: the E components of their cells, whose volume
// update left E as it was (identity table entry), get the medium's
// recursion -- LorentzMedium / DrudeMedium / DebyMedium::updateE{x,y,z},
// src/material/dispersive_material.cpp:38-113, 144-196, 212-275 -- in the
// field precision, with the terms in the reference's order.  State per
// listed component: J, and for Lorentz media the previous E and J.
template <typename T>
struct DispMedium {
  int kind;
  T ca, cb, cc, alpha, xi, gamma, k, beta;
};
struct DispCell {
  long long b;   // padded index of (i, j, k)
  int comp, medium;
};
template <typename T>
struct DispParams {
  Dims d;
  T *E[3];
  const T *H[3];
  const DispCell *cells;
  const DispMedium<T> *media;
  T *j, *jp, *ep;   // [n]
  int n;
  T dl, dt;
};

template <typename T>
__global__ void k_dispersive_e(DispParams<T> p) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n) return;
  const DispCell c = p.cells[q];
  const DispMedium<T> m = p.media[c.medium];
  const long long b = c.b, sj = p.d.sj, si = p.d.si;
  const T *hx = p.H[0], *hy = p.H[1], *hz = p.H[2];
  T curl;
  if (c.comp == 0) curl = -(hy[b] - hy[b - 1]) + (hz[b] - hz[b - sj]);
  else if (c.comp == 1) curl = -(hz[b] - hz[b - si]) + (hx[b] - hx[b - 1]);
  else curl = -(hx[b] - hx[b - sj]) + (hy[b] - hy[b - si]);
  T *E = p.E[c.comp] + b;
  const T e_old = *E;
  T J = p.j[q];
  const T half = T(0.5), one = T(1), two = T(2);
  if (m.kind == 1) {   // Lorentz
    const T Jp = p.jp[q], Ep = p.ep[q];
    T j_sum = T(0);
    j_sum += half * p.dl * ((one + m.alpha) * J + m.xi * Jp);
    const T e = m.ca * e_old + m.cb * Ep + m.cc * (curl - j_sum);
    *E = e;
    p.j[q] = m.alpha * J + m.xi * Jp + m.gamma * (e - Ep) / (two * p.dt);
    p.ep[q] = e_old;
    p.jp[q] = J;
  } else {   // Drude (2), Debye (3)
    T j_sum = T(0);
    j_sum += half * p.dl * ((one + m.k) * J);
    const T e = m.ca * e_old + m.cb * (curl - j_sum);
    *E = e;
    p.j[q] = m.kind == 2 ? m.k * J + m.beta * (e + e_old) : m.k * J + m.beta * (e - e_old) / p.dt;
  }
}

// CurrentSource / VoltageSource ::correctE and Inductor::correctE, in list order.
template <typename T>
__global__ void k_lumped_e(SparseParams<T> p) {
  const long long t = *p.step;
  if (t >= p.total) return;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < p.n_inj) {
    const xfdtd_injection &c = p.inj[q];
    T &e = p.F[c.comp][sp_index<T>(p.d, c.i, c.j, c.k)];
    e = static_cast<T>(static_cast<double>(e) + c.coff * p.waveforms[c.waveform * p.total + t]);
  }
  if (q < p.n_ind) {
    const xfdtd_inductor_cell &c = p.ind[q];
    T &e = p.F[c.comp][sp_index<T>(p.d, c.i, c.j, c.k)];
    double ev = static_cast<double>(e) + c.cecjc * p.ind_j[q];
    e = static_cast<T>(ev);
    p.ind_j[q] = c.cjcec * static_cast<double>(e) + p.ind_j[q];
  }
}

// Monitor::update as a linear functional per probe (one thread per probe).
template <typename T>
__global__ void k_probes(SparseParams<T> p) {
  const long long t = *p.step;
  if (t >= p.total) return;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n_probes) return;
  double acc = 0.0;
  for (int r = p.probe_off[q]; r < p.probe_off[q + 1]; ++r) {
    const xfdtd_probe_term &c = p.terms[r];
    acc += c.weight * static_cast<double>(p.F[c.comp][sp_index<T>(p.d, c.i, c.j, c.k)]);
  }
  p.probe_out[static_cast<long long>(q) * p.total + t] = acc;
}

// One snapshot series on the device: frames [n_frames][cells] of the
// field type, in step order.  The steps are the multiples of `every` and,
// when extra, the step `last` between two of them.
struct SnapDev {
  int comp;
  int extra;
  long long lo[3], n[3];
  long long every, last, n_regular, n_frames, cells;
  void *frames;
};

template <typename T>
struct SnapParams {
  Dims d;
  const T *F[6];
  const SnapDev *s;
  const long long *step;
};

// MovieMonitor::update over TimeDomainFieldMonitors: blockIdx.y is the
// series; blocks of a series that records nothing this step return.
template <typename T>
__global__ void k_snapshots(SnapParams<T> p) {
  const SnapDev &s = p.s[blockIdx.y];
  const long long t = *p.step;
  long long slot;
  if (t % s.every == 0) slot = t / s.every + ((s.extra && t > s.last) ? 1 : 0);
  else if (s.extra && t == s.last) slot = s.last / s.every + 1;
  else return;
  if (slot >= s.n_frames) return;
  T *out = static_cast<T *>(s.frames) + slot * s.cells;
  const T *f = p.F[s.comp];
  for (long long q = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; q < s.cells;
       q += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long k = q % s.n[2], r = q / s.n[2], j = r % s.n[1], i = r / s.n[1];
    out[q] = f[(s.lo[0] + i) * p.d.si + (s.lo[1] + j) * p.d.sj + s.lo[2] + k];
  }
}

__global__ void k_advance(long long *step) { *step += 1; }

// Non-finite scan: sets *flag when any value is NaN or Inf.
template <typename T>
__global__ void k_finite(const T *f, long long n, int *flag) {
  for (long long q = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; q < n;
       q += static_cast<long long>(gridDim.x) * blockDim.x) {
    if (!isfinite(static_cast<double>(f[q]))) {
      atomicExch(flag, 1);
      return;
    }
  }
}

}  // namespace xg
