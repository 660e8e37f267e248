// volume.cuh -- the fused Yee + CPML E and H kernels.
//
// One thread per cell (i, j, k) of the (nx+1)(ny+1)(nz+1) box, k on the
// fastest thread axis so that a warp reads 32 contiguous values.  The curl
// operands are read-only during the kernel (H in the E kernel, E in the H
// kernel) and go through the read-only data path; neighbours along k and j
// hit L1, neighbours along i (another block) hit L2.  Per cell the kernel
// applies, in the reference's order:
//
//   E:  updateE main update          src/simulation/simulation_update.cpp:170-196
//       PML::updateE psi recursions  src/boundary/perfect_match_layer.cpp:574-718
//   H:  updateH main update          src/simulation/simulation_update.cpp:84-100
//       PML::updateH psi recursions  src/boundary/perfect_match_layer.cpp:434-572
//
// (the TFSF face corrections, which the reference applies between the two,
// touch cells outside every CPML slab and run as surface kernels in
// surface.cuh).  The update coefficients come from the material table (18
// per entry, FDTDBasicCoff::initCoff, src/fdtd_basic_coff/fdtd_basic_coff.cpp:77-121),
// multiplied by 1/kappa inside CPML slabs (perfect_match_layer.cpp:190-206,
// 342-358).  The CPML's c_psi = coefficient * dl (same lines) is formed from
// the table entry as well.  Main updates skip the outer walls exactly where
// the reference's loops do; psi terms cover the full transverse extent of the
// component, walls included, as the reference's PML loops do.
//
// Cells whose three indices are all flagged "plain" (not an outer wall, not
// in a CPML slab) take a fast path with only the main update, written with
// the same expression as the general path so both give identical bits.  The
// split kernels run the plain box and the rest (the shell) as two launches;
// the batched kernels choose per warp: a warp with any non-plain cell runs
// the general path for all its cells.
#pragma once

#include "common.cuh"

namespace xg {

template <typename T, typename I, bool SMEM_TABLE>
__device__ __forceinline__ const T *load_table(const VolCore<T, I> &p, int half, int &ts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (!SMEM_TABLE) {
    ts = 18;
    return p.table + 9 * half;
  }
  T *st = reinterpret_cast<T *>(smem_raw);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  const int tid = (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x;
  for (int q = tid; q < p.n_mat * 9; q += nt) st[q] = p.table[(q / 9) * 18 + 9 * half + (q % 9)];
  __syncthreads();
  ts = 9;
  return st;
}

// The 9 coefficients of material m for one side (half 0: E, 1: H).  On a
// uniform grid the three components of a side share their coefficients
// (c0 = c3 = c6, c1 = c4 = c7, c2 = c5 = c8, bit for bit); the compact
// table holds c0, c1, c2 and a flag per material and side, one 16-byte load
// instead of nine gathered ones.  A material whose coefficients differ
// (flag != 0: a lumped element's override) takes them from the full table
// (tab: this side's half, stride ts).  CT = false reads every material
// from the full table: for few materials its nine loads hit L1 and need no
// second dependent load, and the autotuner keeps whichever form is faster.
template <typename T, typename I, bool CT>
__device__ __forceinline__ void coefs(const VolCore<T, I> &p, const T *tab, int ts, unsigned m, int half, T out[9]) {
  if constexpr (!CT) {
    const T *t = tab + m * static_cast<unsigned>(ts);
#pragma unroll
    for (int q = 0; q < 9; ++q) out[q] = t[q];
    return;
  }
  const T *cc = p.ctable + m * 8 + half * 4;
  T a, b, c, f;
  if constexpr (sizeof(T) == 4) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(cc));
    a = v.x, b = v.y, c = v.z, f = v.w;
  } else {
    const double2 v0 = __ldg(reinterpret_cast<const double2 *>(cc)), v1 = __ldg(reinterpret_cast<const double2 *>(cc) + 1);
    a = v0.x, b = v0.y, c = v1.x, f = v1.y;
  }
  if (f == T(0)) {
    out[0] = out[3] = out[6] = a;
    out[1] = out[4] = out[7] = b;
    out[2] = out[5] = out[8] = c;
  } else {
    const T *t = tab + m * static_cast<unsigned>(ts);
#pragma unroll
    for (int q = 0; q < 9; ++q) out[q] = t[q];
  }
}

// Rounded arithmetic with the contractions spelled out, so that every kernel
// that updates a cell (split E/H kernels, fused sweep) gives the same bits.
template <typename T>
__device__ __forceinline__ T fmad(T a, T b, T c) {
  if constexpr (sizeof(T) == 8) return __fma_rn(a, b, c);
  else return __fmaf_rn(a, b, c);
}
template <typename T>
__device__ __forceinline__ T mul(T a, T b) {
  if constexpr (sizeof(T) == 8) return __dmul_rn(a, b);
  else return __fmul_rn(a, b);
}
// c0 * f + ca * da + cb * db: the Yee main update of one component
template <typename T>
__device__ __forceinline__ T yee(T c0, T f, T ca, T da, T cb, T db) {
  return fmad(cb, db, fmad(ca, da, mul(c0, f)));
}

// The curl operands of one E cell: H at (i,j,k) and its k-1, j-1, i-1 neighbours.
template <typename T>
struct ECurl {
  T hx, hy, hz, hx_k, hy_k, hx_j, hz_j, hy_i, hz_i;
};
// The curl operands of one H cell: E at (i,j,k) and its k+1, j+1, i+1 neighbours.
template <typename T>
struct HCurl {
  T ex, ey, ez, ex_k, ey_k, ex_j, ez_j, ey_i, ez_i;
};

// Main E update of a plain cell (not on an outer wall, not in a CPML slab).
template <typename T>
__device__ __forceinline__ void e_plain(const T *c, const ECurl<T> &h, T &ex, T &ey, T &ez) {
  ex = yee(c[0], ex, c[1], h.hy - h.hy_k, c[2], h.hz - h.hz_j);
  ey = yee(c[3], ey, c[5], h.hx - h.hx_k, c[4], h.hz - h.hz_i);
  ez = yee(c[6], ez, c[7], h.hx - h.hx_j, c[8], h.hy - h.hy_i);
}

// Main H update of a plain cell.
template <typename T>
__device__ __forceinline__ void h_plain(const T *c, const HCurl<T> &e, T &hx, T &hy, T &hz) {
  hx = yee(c[0], hx, c[1], e.ey_k - e.ey, c[2], e.ez_j - e.ez);
  hy = yee(c[3], hy, c[4], e.ez_i - e.ez, c[5], e.ex_k - e.ex);
  hz = yee(c[6], hz, c[7], e.ex_j - e.ex, c[8], e.ey_i - e.ey);
}

// One CPML recursion: psi' = b psi + a d.  The field term is (c dl) psi'.
template <typename T>
__device__ __forceinline__ T psi_next(T b, T a, T d, T psi) {
  return fmad(a, d, mul(b, psi));
}

// The CPML profile values of one index on one axis (b, a, 1/kappa; 0, 0, 1
// outside the slabs).
template <typename T>
struct AxisCoef {
  T b, a, rk;
};
template <typename T>
__device__ __forceinline__ AxisCoef<T> axis_coef(int slot, const T *b, const T *a, const T *rk, int n) {
  AxisCoef<T> r{T(0), T(0), T(1)};
  if (slot >= 0) {
    r.b = __ldg(b + n);
    r.a = __ldg(a + n);
    r.rk = __ldg(rk + n);
  }
  return r;
}

// The CPML context of one cell: the slab slot on each axis (-1 outside the
// slabs, and on the axes a caller names plain) and the profile values at
// the cell's indices.
template <typename T>
struct SlabCtx {
  int xs, ys, zs;
  AxisCoef<T> X, Y, Z;
};

// One axis of it: the E (half 0) or H (half 1) slot and profiles of axis a
// at index n.
template <typename T, typename I>
__device__ __forceinline__ void slab_axis(const VolCore<T, I> &p, int a, int half, int n, int &slot, AxisCoef<T> &c) {
  const CpmlAxis<T> &cp = p.cp[a];
  slot = cp.n_layers ? __ldg((half ? cp.slot_h : cp.slot_e) + n) : -1;
  c = half ? axis_coef(slot, cp.b_m, cp.a_m, cp.rk_m, n) : axis_coef(slot, cp.b_e, cp.a_e, cp.rk_e, n);
}

template <typename T, typename I, int AXES>
__device__ __forceinline__ SlabCtx<T> slab_ctx(const VolCore<T, I> &p, int half, int i, int j, int k) {
  SlabCtx<T> x;
  x.xs = x.ys = x.zs = -1;
  x.X = x.Y = x.Z = AxisCoef<T>{T(0), T(0), T(1)};
  if (AXES & 1) slab_axis(p, 0, half, i, x.xs, x.X);
  if (AXES & 2) slab_axis(p, 1, half, j, x.ys, x.Y);
  if (AXES & 4) slab_axis(p, 2, half, k, x.zs, x.Z);
  return x;
}

// The six psi operands of one cell and side: E ex_y, ex_z, ey_x, ey_z,
// ez_x, ez_y (H likewise), 0 where the recursion does not run.
template <typename T>
struct PsiOps {
  T xy, xz, yx, yz, zx, zy;
};

// Psi offsets of one cell: X slabs (xs, j, k), Y slabs (i, ys, k), Z slabs
// (i, j, zs), each with k (or the slot) fastest.
template <typename T, typename I>
__device__ __forceinline__ void psi_offsets(const VolCore<T, I> &p, const SlabCtx<T> &x, int i, int j, int k,
                                            unsigned &ox, unsigned &oy, unsigned &oz) {
  const unsigned Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(p.d.ny + 1);
  ox = (static_cast<unsigned>(x.xs) * ny1 + j) * nzp + k;
  oy = (static_cast<unsigned>(i) * Ly + x.ys) * nzp + k;
  oz = (static_cast<unsigned>(i) * ny1 + j) * Lz + x.zs;
}

// The E psi operands of one cell (AXES as in e_general).
template <typename T, typename I, int AXES>
__device__ __forceinline__ PsiOps<T> e_psi_load(const VolCore<T, I> &p, const SlabCtx<T> &x, int i, int j, int k,
                                                const Psi<T> &pr) {
  constexpr bool SX = AXES & 1, SY = AXES & 2, SZ = AXES & 4;
  const bool ex_on = !SX || i < p.d.nx, ey_on = !SY || j < p.d.ny, ez_on = !SZ || k < p.d.nz;
  unsigned ox, oy, oz;
  psi_offsets(p, x, i, j, k, ox, oy, oz);
  PsiOps<T> s;
  s.xy = ex_on && x.ys >= 0 ? pr.ex_y[oy] : T(0);
  s.xz = ex_on && x.zs >= 0 ? pr.ex_z[oz] : T(0);
  s.yx = ey_on && x.xs >= 0 ? pr.ey_x[ox] : T(0);
  s.yz = ey_on && x.zs >= 0 ? pr.ey_z[oz] : T(0);
  s.zx = ez_on && x.xs >= 0 ? pr.ez_x[ox] : T(0);
  s.zy = ez_on && x.ys >= 0 ? pr.ez_y[oy] : T(0);
  return s;
}

// The H psi operands of one cell (AXES as in h_general).
template <typename T, typename I, int AXES>
__device__ __forceinline__ PsiOps<T> h_psi_load(const VolCore<T, I> &p, const SlabCtx<T> &x, int i, int j, int k) {
  constexpr bool SX = AXES & 1, SY = AXES & 2, SZ = AXES & 4;
  const bool i_lt = !SX || i < p.d.nx, j_lt = !SY || j < p.d.ny, k_lt = !SZ || k < p.d.nz;
  const bool hx_on = j_lt && k_lt, hy_on = i_lt && k_lt, hz_on = i_lt && j_lt;
  unsigned ox, oy, oz;
  psi_offsets(p, x, i, j, k, ox, oy, oz);
  const Psi<T> &ps = p.psi;
  PsiOps<T> s;
  s.xy = hx_on && x.ys >= 0 ? ps.hx_y[oy] : T(0);
  s.xz = hx_on && x.zs >= 0 ? ps.hx_z[oz] : T(0);
  s.yx = hy_on && x.xs >= 0 ? ps.hy_x[ox] : T(0);
  s.yz = hy_on && x.zs >= 0 ? ps.hy_z[oz] : T(0);
  s.zx = hz_on && x.xs >= 0 ? ps.hz_x[ox] : T(0);
  s.zy = hz_on && x.ys >= 0 ? ps.hz_y[oy] : T(0);
  return s;
}

// The arithmetic of the general E update of one cell, from its operands:
// curl operands h, coefficients c, CPML context x and psi operands ps
// (e_psi_load).  Psi is written to pw when store_psi.  w[c] reports whether
// component c was updated.  The arithmetic is that of the reference's
// loops, term by term.  AXES (bit 0 x, 1 y, 2 z) names the axes whose index
// may be special (wall or CPML slab); on the others the caller guarantees a
// plain index, and their tests and terms drop out at compile time (a CPML
// face cell has one special axis, an edge cell two).
template <typename T, typename I, int AXES>
__device__ __forceinline__ void e_general_ops(const VolCore<T, I> &p, const T *c, int i, int j, int k,
                                              const ECurl<T> &h, const SlabCtx<T> &x, const PsiOps<T> &ps,
                                              const Psi<T> &pw, bool store_psi, T &ex, T &ey, T &ez, bool w[3]) {
  constexpr bool SX = AXES & 1, SY = AXES & 2, SZ = AXES & 4;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const int xs = SX ? x.xs : -1, ys = SY ? x.ys : -1, zs = SZ ? x.zs : -1;
  const bool in_i = !SX || (i >= 1 && i < nx), in_j = !SY || (j >= 1 && j < ny), in_k = !SZ || (k >= 1 && k < nz);
  const bool ex_on = !SX || i < nx, ey_on = !SY || j < ny, ez_on = !SZ || k < nz;   // Ex, Ey, Ez exist here
  unsigned ox, oy, oz;
  psi_offsets(p, x, i, j, k, ox, oy, oz);
  const AxisCoef<T> &X = x.X, &Y = x.Y, &Z = x.Z;
  const T s_ex_y = ps.xy, s_ex_z = ps.xz, s_ey_x = ps.yx, s_ey_z = ps.yz, s_ez_x = ps.zx, s_ez_y = ps.zy;
  T cf[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) cf[q] = c[q];
  w[0] = w[1] = w[2] = false;

  // ---- Ex (nx, ny+1, nz+1) ----
  if (ex_on) {
    const T d_hz_y = h.hz - h.hz_j;   // Hz(j) - Hz(j-1)
    const T d_hy_z = h.hy - h.hy_k;   // Hy(k) - Hy(k-1)
    if (in_j && in_k) {
      T ca = cf[1], cb = cf[2];
      if (zs >= 0) ca = mul(ca, Z.rk);
      if (ys >= 0) cb = mul(cb, Y.rk);
      ex = yee(cf[0], ex, ca, d_hy_z, cb, d_hz_y);
      w[0] = true;
    }
    if (ys >= 0) {   // Y slabs: psi_eb of YN/YP, c_psi = cexhz * dy
      const T s = psi_next(Y.b, Y.a, d_hz_y, s_ex_y);
      if (store_psi) pw.ex_y[oy] = s;
      ex = fmad(mul(cf[2], p.dl[1]), s, ex);
      w[0] = true;
    }
    if (zs >= 0) {   // Z slabs: psi_ea of ZN/ZP, c_psi = cexhy * dz
      const T s = psi_next(Z.b, Z.a, d_hy_z, s_ex_z);
      if (store_psi) pw.ex_z[oz] = s;
      ex = fmad(mul(cf[1], p.dl[2]), s, ex);
      w[0] = true;
    }
  }

  // ---- Ey (nx+1, ny, nz+1) ----
  if (ey_on) {
    const T d_hz_x = h.hz - h.hz_i;  // Hz(i) - Hz(i-1)
    const T d_hx_z = h.hx - h.hx_k;  // Hx(k) - Hx(k-1)
    if (in_i && in_k) {
      T ca = cf[5], cb = cf[4];      // ceyhx, ceyhz
      if (zs >= 0) ca = mul(ca, Z.rk);
      if (xs >= 0) cb = mul(cb, X.rk);
      ey = yee(cf[3], ey, ca, d_hx_z, cb, d_hz_x);
      w[1] = true;
    }
    if (xs >= 0) {   // X slabs: psi_ea of XN/XP, c_psi = ceyhz * dx
      const T s = psi_next(X.b, X.a, d_hz_x, s_ey_x);
      if (store_psi) pw.ey_x[ox] = s;
      ey = fmad(mul(cf[4], p.dl[0]), s, ey);
      w[1] = true;
    }
    if (zs >= 0) {   // Z slabs: psi_eb of ZN/ZP, c_psi = ceyhx * dz
      const T s = psi_next(Z.b, Z.a, d_hx_z, s_ey_z);
      if (store_psi) pw.ey_z[oz] = s;
      ey = fmad(mul(cf[5], p.dl[2]), s, ey);
      w[1] = true;
    }
  }

  // ---- Ez (nx+1, ny+1, nz) ----
  if (ez_on) {
    const T d_hy_x = h.hy - h.hy_i;  // Hy(i) - Hy(i-1)
    const T d_hx_y = h.hx - h.hx_j;  // Hx(j) - Hx(j-1)
    if (in_i && in_j) {
      T ca = cf[7], cb = cf[8];      // cezhx, cezhy
      if (ys >= 0) ca = mul(ca, Y.rk);
      if (xs >= 0) cb = mul(cb, X.rk);
      ez = yee(cf[6], ez, ca, d_hx_y, cb, d_hy_x);
      w[2] = true;
    }
    if (xs >= 0) {   // X slabs: psi_eb of XN/XP, c_psi = cezhy * dx
      const T s = psi_next(X.b, X.a, d_hy_x, s_ez_x);
      if (store_psi) pw.ez_x[ox] = s;
      ez = fmad(mul(cf[8], p.dl[0]), s, ez);
      w[2] = true;
    }
    if (ys >= 0) {   // Y slabs: psi_ea of YN/YP, c_psi = cezhx * dy
      const T s = psi_next(Y.b, Y.a, d_hx_y, s_ez_y);
      if (store_psi) pw.ez_y[oy] = s;
      ez = fmad(mul(cf[7], p.dl[1]), s, ez);
      w[2] = true;
    }
  }
}

// General E update of one cell: outer walls and CPML slabs.  E psi is read
// from pr and, when store_psi, written to pw (SEPARATE_PSI) or back to pr
// (in place).  Every operand (coefficients, profiles, psi values) is loaded
// before the first store, so that the loads are in flight together.  AXES
// as in e_general_ops.
template <typename T, typename I, bool SEPARATE_PSI, int AXES = 7>
__device__ __forceinline__ void e_general(const VolCore<T, I> &p, const T *c, int i, int j, int k,
                                          const ECurl<T> &h, const Psi<T> &pr, const Psi<T> &pw_, bool store_psi,
                                          T &ex, T &ey, T &ez, bool w[3]) {
  const Psi<T> &pw = SEPARATE_PSI ? pw_ : pr;
  const SlabCtx<T> x = slab_ctx<T, I, AXES>(p, 0, i, j, k);
  const PsiOps<T> ps = e_psi_load<T, I, AXES>(p, x, i, j, k, pr);
  e_general_ops<T, I, AXES>(p, c, i, j, k, h, x, ps, pw, store_psi, ex, ey, ez, w);
}

// The arithmetic of the general H update of one cell (H psi in place), as
// e_general_ops.
template <typename T, typename I, int AXES>
__device__ __forceinline__ void h_general_ops(const VolCore<T, I> &p, const T *c, int i, int j, int k,
                                              const HCurl<T> &e, const SlabCtx<T> &x, const PsiOps<T> &pv,
                                              T &hx, T &hy, T &hz, bool w[3]) {
  constexpr bool SX = AXES & 1, SY = AXES & 2, SZ = AXES & 4;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const int xs = SX ? x.xs : -1, ys = SY ? x.ys : -1, zs = SZ ? x.zs : -1;
  const bool i_lt = !SX || i < nx, j_lt = !SY || j < ny, k_lt = !SZ || k < nz;
  const bool hx_on = j_lt && k_lt, hy_on = i_lt && k_lt, hz_on = i_lt && j_lt;   // Hx, Hy, Hz exist here
  unsigned ox, oy, oz;
  psi_offsets(p, x, i, j, k, ox, oy, oz);
  const Psi<T> &ps = p.psi;
  const AxisCoef<T> &X = x.X, &Y = x.Y, &Z = x.Z;
  const T s_hx_y = pv.xy, s_hx_z = pv.xz, s_hy_x = pv.yx, s_hy_z = pv.yz, s_hz_x = pv.zx, s_hz_y = pv.zy;
  T cf[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) cf[q] = c[q];
  w[0] = w[1] = w[2] = false;

  // ---- Hx (nx+1, ny, nz) ----
  if (hx_on) {
    const T d_ey_z = e.ey_k - e.ey;   // Ey(k+1) - Ey(k)
    const T d_ez_y = e.ez_j - e.ez;   // Ez(j+1) - Ez(j)
    if (i_lt) {
      T ca = cf[1], cb = cf[2];        // chxey, chxez
      if (zs >= 0) ca = mul(ca, Z.rk);
      if (ys >= 0) cb = mul(cb, Y.rk);
      hx = yee(cf[0], hx, ca, d_ey_z, cb, d_ez_y);
      w[0] = true;
    }
    if (ys >= 0) {   // Y slabs: psi_hb of YN/YP, c_psi = chxez * dy
      const T s = psi_next(Y.b, Y.a, d_ez_y, s_hx_y);
      ps.hx_y[oy] = s;
      hx = fmad(mul(cf[2], p.dl[1]), s, hx);
      w[0] = true;
    }
    if (zs >= 0) {   // Z slabs: psi_ha of ZN/ZP, c_psi = chxey * dz
      const T s = psi_next(Z.b, Z.a, d_ey_z, s_hx_z);
      ps.hx_z[oz] = s;
      hx = fmad(mul(cf[1], p.dl[2]), s, hx);
      w[0] = true;
    }
  }

  // ---- Hy (nx, ny+1, nz) ----
  if (hy_on) {
    const T d_ez_x = e.ez_i - e.ez;   // Ez(i+1) - Ez(i)
    const T d_ex_z = e.ex_k - e.ex;   // Ex(k+1) - Ex(k)
    if (j_lt) {
      T ca = cf[4], cb = cf[5];        // chyez, chyex
      if (xs >= 0) ca = mul(ca, X.rk);
      if (zs >= 0) cb = mul(cb, Z.rk);
      hy = yee(cf[3], hy, ca, d_ez_x, cb, d_ex_z);
      w[1] = true;
    }
    if (xs >= 0) {   // X slabs: psi_ha of XN/XP, c_psi = chyez * dx
      const T s = psi_next(X.b, X.a, d_ez_x, s_hy_x);
      ps.hy_x[ox] = s;
      hy = fmad(mul(cf[4], p.dl[0]), s, hy);
      w[1] = true;
    }
    if (zs >= 0) {   // Z slabs: psi_hb of ZN/ZP, c_psi = chyex * dz
      const T s = psi_next(Z.b, Z.a, d_ex_z, s_hy_z);
      ps.hy_z[oz] = s;
      hy = fmad(mul(cf[5], p.dl[2]), s, hy);
      w[1] = true;
    }
  }

  // ---- Hz (nx, ny, nz+1) ----
  if (hz_on) {
    const T d_ex_y = e.ex_j - e.ex;   // Ex(j+1) - Ex(j)
    const T d_ey_x = e.ey_i - e.ey;   // Ey(i+1) - Ey(i)
    if (k_lt) {
      T ca = cf[7], cb = cf[8];        // chzex, chzey
      if (ys >= 0) ca = mul(ca, Y.rk);
      if (xs >= 0) cb = mul(cb, X.rk);
      hz = yee(cf[6], hz, ca, d_ex_y, cb, d_ey_x);
      w[2] = true;
    }
    if (xs >= 0) {   // X slabs: psi_hb of XN/XP, c_psi = chzey * dx
      const T s = psi_next(X.b, X.a, d_ey_x, s_hz_x);
      ps.hz_x[ox] = s;
      hz = fmad(mul(cf[8], p.dl[0]), s, hz);
      w[2] = true;
    }
    if (ys >= 0) {   // Y slabs: psi_ha of YN/YP, c_psi = chzex * dy
      const T s = psi_next(Y.b, Y.a, d_ex_y, s_hz_y);
      ps.hz_y[oy] = s;
      hz = fmad(mul(cf[7], p.dl[1]), s, hz);
      w[2] = true;
    }
  }
}

// General H update of one cell: last planes and CPML slabs (H psi in place),
// operands first and AXES as in e_general_ops.
template <typename T, typename I, int AXES = 7>
__device__ __forceinline__ void h_general(const VolCore<T, I> &p, const T *c, int i, int j, int k,
                                          const HCurl<T> &e, T &hx, T &hy, T &hz, bool w[3]) {
  const SlabCtx<T> x = slab_ctx<T, I, AXES>(p, 1, i, j, k);
  const PsiOps<T> pv = h_psi_load<T, I, AXES>(p, x, i, j, k);
  h_general_ops<T, I, AXES>(p, c, i, j, k, e, x, pv, hx, hy, hz, w);
}

// E update of one cell by the general path.  It serves any cell: a plain
// cell gets the bits of the fast path (same expressions, no CPML terms).
// AXES as in e_general.
template <typename T, typename I, int AXES = 7, bool CT = false>
__device__ __forceinline__ void e_cell_general(const VolCore<T, I> &p, const T *tab, int ts, int i, int j, int k) {
  constexpr bool SX = AXES & 1, SY = AXES & 2, SZ = AXES & 4;
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const unsigned b = static_cast<unsigned>(i) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
  const T *__restrict__ Hx = p.H[0];
  const T *__restrict__ Hy = p.H[1];
  const T *__restrict__ Hz = p.H[2];
  T *__restrict__ Ex = p.E[0];
  T *__restrict__ Ey = p.E[1];
  T *__restrict__ Ez = p.E[2];
  ECurl<T> h;
  h.hx = __ldg(Hx + b);
  h.hy = __ldg(Hy + b);
  h.hz = __ldg(Hz + b);
  h.hx_k = !SZ || k > 0 ? __ldg(Hx + b - 1) : T(0);
  h.hy_k = !SZ || k > 0 ? __ldg(Hy + b - 1) : T(0);
  h.hx_j = !SY || j > 0 ? __ldg(Hx + b - usj) : T(0);
  h.hz_j = !SY || j > 0 ? __ldg(Hz + b - usj) : T(0);
  h.hy_i = !SX || i > 0 ? __ldg(Hy + b - usi) : T(0);
  h.hz_i = !SX || i > 0 ? __ldg(Hz + b - usi) : T(0);
  T c[9];
  coefs<T, I, CT>(p, tab, ts, static_cast<unsigned>(__ldg(p.idx + b)), 0, c);
  T ex = Ex[b], ey = Ey[b], ez = Ez[b];
  bool w[3];
  e_general<T, I, false, AXES>(p, c, i, j, k, h, p.psi, p.psi, true, ex, ey, ez, w);
  if (w[0]) Ex[b] = ex;
  if (w[1]) Ey[b] = ey;
  if (w[2]) Ez[b] = ez;
}

// NC plain cells (i0 .. i0+NC-1) of one (j, k) column: every load is issued
// before any store, and the H at i-1 of cell c+1 is cell c's own.
template <typename T, typename I, int NC, bool CT = false>
__device__ __forceinline__ void e_fast(const VolCore<T, I> &p, const T *tab, int ts, int i0, int j, int k) {
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const unsigned b0 = static_cast<unsigned>(i0) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
  const T *__restrict__ Hx = p.H[0];
  const T *__restrict__ Hy = p.H[1];
  const T *__restrict__ Hz = p.H[2];
  T *__restrict__ Ex = p.E[0];
  T *__restrict__ Ey = p.E[1];
  T *__restrict__ Ez = p.E[2];
  T hx[NC], hy[NC + 1], hz[NC + 1], hx_k[NC], hy_k[NC], hx_j[NC], hz_j[NC], ex[NC], ey[NC], ez[NC];
  unsigned m[NC];
  hy[0] = __ldg(Hy + b0 - usi);
  hz[0] = __ldg(Hz + b0 - usi);
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    const unsigned b = b0 + q * usi;
    hx[q] = __ldg(Hx + b);
    hy[q + 1] = __ldg(Hy + b);
    hz[q + 1] = __ldg(Hz + b);
    hx_k[q] = __ldg(Hx + b - 1);
    hy_k[q] = __ldg(Hy + b - 1);
    hx_j[q] = __ldg(Hx + b - usj);
    hz_j[q] = __ldg(Hz + b - usj);
    m[q] = __ldg(p.idx + b);
    ex[q] = Ex[b];
    ey[q] = Ey[b];
    ez[q] = Ez[b];
  }
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    const unsigned b = b0 + q * usi;
    const ECurl<T> h{hx[q], hy[q + 1], hz[q + 1], hx_k[q], hy_k[q], hx_j[q], hz_j[q], hy[q], hz[q]};
    T c[9];
    coefs<T, I, CT>(p, tab, ts, m[q], 0, c);
    e_plain(c, h, ex[q], ey[q], ez[q]);
    Ex[b] = ex[q];
    Ey[b] = ey[q];
    Ez[b] = ez[q];
  }
}

// The volume update runs as two kernels per side.  The interior kernel
// covers the box of cells that are plain on all three axes (no flag loads,
// no general path: its registers serve the fast path alone); the shell
// kernel covers every other cell, one thread per cell, by the general path.
// The two sets are disjoint and together cover the component box, so the
// pair does what one kernel over all cells with a per-cell choice would.
//
// Interior box [lo, hi] (inclusive, per axis).  k0: first k of the launch
// grid, lo[2] rounded down to the block's k extent, so that every row of
// threads starts on the row's alignment.
struct InteriorBox {
  int lo[3], hi[3];
  int k0;
  int px_lo, px_hi, py_lo, py_hi;   // plain runs on x and y and the interior's k range
  int pz_lo, pz_hi;                 //   (the wide and z-edge TMA launches of interior_tma.cuh)
};

// The shell: boxes of cells (origin, extent per axis), each covering whole
// 256-thread blocks from block0 on, cells numbered with k fastest.  Along k
// a box may skip a gap: its k offsets from ksplit on are shifted by kgap,
// so that the cells below and above the interior's k range of one row are
// numbered together (ext[2] counts both parts).  cls names the axes on
// which the box's indices may be special (AXES of e_general): 1, 2, 4 for
// the CPML faces, 5, 6, 7 for edges and corners.  Division by the extents
// uses multiply-shift constants (m, sh: q = n * m >> sh, exact for n <
// 2^31).
struct ShellBox {
  int lo[3];
  int ext[3];
  int ksplit, kgap;
  unsigned cells;
  int cls;
  unsigned long long m2, m1;   // divide by ext[2], by ext[1]
  int sh2, sh1;
  unsigned block0;
};
constexpr int kMaxShellBoxes = 18;
struct ShellBoxes {
  int n;
  unsigned blocks;   // total blocks
  ShellBox b[kMaxShellBoxes];
};

__device__ __forceinline__ unsigned div_magic(unsigned n, unsigned long long m, int sh) {
  return static_cast<unsigned>((static_cast<unsigned long long>(n) * m) >> sh);
}

// Box of shell block `blk` (binary search on block0) and this thread's cell
// in it; false past the box's last cell.
__device__ __forceinline__ bool shell_cell(const ShellBoxes &s, unsigned blk, int &cls, int &i, int &j, int &k) {
  int lo = 0, hi = s.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (blk >= s.b[mid].block0) lo = mid;
    else hi = mid - 1;
  }
  const ShellBox &bx = s.b[lo];
  const unsigned r = (blk - bx.block0) * 256u + threadIdx.x;
  if (r >= bx.cells) return false;
  const unsigned t = div_magic(r, bx.m2, bx.sh2);
  const unsigned u = div_magic(t, bx.m1, bx.sh1);
  const int kk = static_cast<int>(r - t * static_cast<unsigned>(bx.ext[2]));
  k = bx.lo[2] + kk + (kk >= bx.ksplit ? bx.kgap : 0);
  j = bx.lo[1] + static_cast<int>(t - u * static_cast<unsigned>(bx.ext[1]));
  i = bx.lo[0] + static_cast<int>(u);
  cls = bx.cls;
  return true;
}

// MINB: minimum resident blocks per SM requested from the register
// allocator (1 = no cap); NC: cells per thread along i.  The autotuner in
// engine.cu picks both (and the block shape) per plan.
template <typename T, typename I, bool SMEM_TABLE, int MINB, int NC, bool CT>
__global__ void __launch_bounds__(256, MINB) k_update_e(VolCore<T, I> p, InteriorBox in) {
  int ts;
  const T *tab = load_table<T, I, SMEM_TABLE>(p, 0, ts);
  const int k = in.k0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = in.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
  const int i0 = in.lo[0] + (blockIdx.z * blockDim.z + threadIdx.z) * NC;
  if (k < in.lo[2] || k > in.hi[2] || j > in.hi[1] || i0 > in.hi[0]) return;
  if (i0 + NC - 1 <= in.hi[0]) {
    e_fast<T, I, NC, CT>(p, tab, ts, i0, j, k);
    return;
  }
#pragma unroll
  for (int q = 0; q < NC; ++q)
    if (i0 + q <= in.hi[0]) e_fast<T, I, 1, CT>(p, tab, ts, i0 + q, j, k);
}

// E update of one shell cell of box class cls (coefficient table read
// through L1): the general path specialised per class.
template <typename T, typename I, bool CT = false>
__device__ __forceinline__ void e_shell_cell(const VolCore<T, I> &p, int cls, int i, int j, int k) {
  switch (cls) {
    case 1: e_cell_general<T, I, 1, CT>(p, p.table, 18, i, j, k); break;
    case 2: e_cell_general<T, I, 2, CT>(p, p.table, 18, i, j, k); break;
    case 4: e_cell_general<T, I, 4, CT>(p, p.table, 18, i, j, k); break;
    case 5: e_cell_general<T, I, 5, CT>(p, p.table, 18, i, j, k); break;
    case 6: e_cell_general<T, I, 6, CT>(p, p.table, 18, i, j, k); break;
    default: e_cell_general<T, I, 7, CT>(p, p.table, 18, i, j, k); break;
  }
}

// E update of the shell cells, the class uniform per block.
template <typename T, typename I, int MINB, bool CT>
__global__ void __launch_bounds__(256, MINB) k_update_e_shell(VolCore<T, I> p, const __grid_constant__ ShellBoxes s) {
  int cls, i, j, k;
  if (shell_cell(s, blockIdx.x, cls, i, j, k)) e_shell_cell<T, I, CT>(p, cls, i, j, k);
}

// H update of one cell by the general path (any cell, as e_cell_general).
template <typename T, typename I, int AXES = 7, bool CT = false>
__device__ __forceinline__ void h_cell_general(const VolCore<T, I> &p, const T *tab, int ts, int i, int j, int k) {
  constexpr bool SX = AXES & 1, SY = AXES & 2, SZ = AXES & 4;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const unsigned b = static_cast<unsigned>(i) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
  const T *__restrict__ Ex = p.E[0];
  const T *__restrict__ Ey = p.E[1];
  const T *__restrict__ Ez = p.E[2];
  T *__restrict__ Hx = p.H[0];
  T *__restrict__ Hy = p.H[1];
  T *__restrict__ Hz = p.H[2];
  HCurl<T> e;
  e.ex = __ldg(Ex + b);
  e.ey = __ldg(Ey + b);
  e.ez = __ldg(Ez + b);
  e.ey_i = !SX || i < nx ? __ldg(Ey + b + usi) : T(0);
  e.ez_i = !SX || i < nx ? __ldg(Ez + b + usi) : T(0);
  e.ex_k = !SZ || k < nz ? __ldg(Ex + b + 1) : T(0);
  e.ey_k = !SZ || k < nz ? __ldg(Ey + b + 1) : T(0);
  e.ex_j = !SY || j < ny ? __ldg(Ex + b + usj) : T(0);
  e.ez_j = !SY || j < ny ? __ldg(Ez + b + usj) : T(0);
  T c[9];
  coefs<T, I, CT>(p, tab, ts, static_cast<unsigned>(__ldg(p.idx + b)), 1, c);
  T hx = Hx[b], hy = Hy[b], hz = Hz[b];
  bool w[3];
  h_general<T, I, AXES>(p, c, i, j, k, e, hx, hy, hz, w);
  if (w[0]) Hx[b] = hx;
  if (w[1]) Hy[b] = hy;
  if (w[2]) Hz[b] = hz;
}

// NC plain cells of one column for H: the E at i+1 of cell c is cell c+1's own.
template <typename T, typename I, int NC, bool CT = false>
__device__ __forceinline__ void h_fast(const VolCore<T, I> &p, const T *tab, int ts, int i0, int j, int k) {
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const unsigned b0 = static_cast<unsigned>(i0) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
  const T *__restrict__ Ex = p.E[0];
  const T *__restrict__ Ey = p.E[1];
  const T *__restrict__ Ez = p.E[2];
  T *__restrict__ Hx = p.H[0];
  T *__restrict__ Hy = p.H[1];
  T *__restrict__ Hz = p.H[2];
  T ex[NC], ey[NC + 1], ez[NC + 1], ex_kp[NC], ey_kp[NC], ex_jp[NC], ez_jp[NC], hx[NC], hy[NC], hz[NC];
  unsigned m[NC];
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    const unsigned b = b0 + q * usi;
    ex[q] = __ldg(Ex + b);
    ey[q] = __ldg(Ey + b);
    ez[q] = __ldg(Ez + b);
    ex_kp[q] = __ldg(Ex + b + 1);
    ey_kp[q] = __ldg(Ey + b + 1);
    ex_jp[q] = __ldg(Ex + b + usj);
    ez_jp[q] = __ldg(Ez + b + usj);
    m[q] = __ldg(p.idx + b);
    hx[q] = Hx[b];
    hy[q] = Hy[b];
    hz[q] = Hz[b];
  }
  ey[NC] = __ldg(Ey + b0 + NC * usi);
  ez[NC] = __ldg(Ez + b0 + NC * usi);
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    const unsigned b = b0 + q * usi;
    const HCurl<T> e{ex[q], ey[q], ez[q], ex_kp[q], ey_kp[q], ex_jp[q], ez_jp[q], ey[q + 1], ez[q + 1]};
    T c[9];
    coefs<T, I, CT>(p, tab, ts, m[q], 1, c);
    h_plain(c, e, hx[q], hy[q], hz[q]);
    Hx[b] = hx[q];
    Hy[b] = hy[q];
    Hz[b] = hz[q];
  }
}

template <typename T, typename I, bool SMEM_TABLE, int MINB, int NC, bool CT>
__global__ void __launch_bounds__(256, MINB) k_update_h(VolCore<T, I> p, InteriorBox in) {
  int ts;
  const T *tab = load_table<T, I, SMEM_TABLE>(p, 1, ts);
  const int k = in.k0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = in.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
  const int i0 = in.lo[0] + (blockIdx.z * blockDim.z + threadIdx.z) * NC;
  if (k < in.lo[2] || k > in.hi[2] || j > in.hi[1] || i0 > in.hi[0]) return;
  if (i0 + NC - 1 <= in.hi[0]) {
    h_fast<T, I, NC, CT>(p, tab, ts, i0, j, k);
    return;
  }
#pragma unroll
  for (int q = 0; q < NC; ++q)
    if (i0 + q <= in.hi[0]) h_fast<T, I, 1, CT>(p, tab, ts, i0 + q, j, k);
}


template <typename T, typename I, bool CT = false>
__device__ __forceinline__ void h_shell_cell(const VolCore<T, I> &p, int cls, int i, int j, int k) {
  switch (cls) {
    case 1: h_cell_general<T, I, 1, CT>(p, p.table + 9, 18, i, j, k); break;
    case 2: h_cell_general<T, I, 2, CT>(p, p.table + 9, 18, i, j, k); break;
    case 4: h_cell_general<T, I, 4, CT>(p, p.table + 9, 18, i, j, k); break;
    case 5: h_cell_general<T, I, 5, CT>(p, p.table + 9, 18, i, j, k); break;
    case 6: h_cell_general<T, I, 6, CT>(p, p.table + 9, 18, i, j, k); break;
    default: h_cell_general<T, I, 7, CT>(p, p.table + 9, 18, i, j, k); break;
  }
}

template <typename T, typename I, int MINB, bool CT>
__global__ void __launch_bounds__(256, MINB) k_update_h_shell(VolCore<T, I> p, const __grid_constant__ ShellBoxes s) {
  int cls, i, j, k;
  if (shell_cell(s, blockIdx.x, cls, i, j, k)) h_shell_cell<T, I, CT>(p, cls, i, j, k);
}

}  // namespace xg
