// adjoint.cuh -- reverse-time (discrete adjoint) kernels of the split E/H
// update, for gradients of a field loss with respect to per-cell eps_r and
// sigma.
//
// One forward step t maps (E, H, psiE, psiH) to (E', H', psiE', psiH'):
//   E' = c0 E + ca dH_a + cb dH_b  (+ (c dl) psiE',  psiE' = b psiE + a dH)
//   H' = c0 H + ca dE'_a + cb dE'_b (+ (c dl) psiH', psiH' = b psiH + a dE')
// with the masks and CPML terms of e_general / h_general (volume.cuh).  Its
// transpose, applied to the adjoint state (lE, lH, mE, mH) of step t+1,
// gives that of step t.  Writing W for the adjoint weight an E cell puts on
// one of its H differences,
//   W = [main] ca L + [slab] a (mE + c dl L),      L = lE' of that cell,
// and U for the weight an H cell puts on one of its E differences (same
// form with lH', mH'), the transpose is
//   lE' += loss gradient + sum of the U of the H cells that read the cell
//   lH  =  [main] c0 lH' + sum of the W of the E cells that read the cell
//   mH  =  b (mH' + c dl lH')
//   lE  =  [main] c0 lE'                mE = b (mE' + c dl lE')
// and the parameter gradient gathers lE' dE'/dp with the forward state of
// step t.  The sources (lumped injections, TFSF corrections) are affine and
// drop out.  Two kernels per step, each a gather over neighbours with the
// forward's own index ranges:
//   k_adj_h(t):  lH(t) and mH(t) from lH', mH' and the W of lE'(t), mE'(t);
//   k_adj_e(t):  lE(t), mE(t), the gradient of step t, then (for the step
//                before) the loss gradient of step t-1 and the U of lH(t).
//
// Scaled adjoint fields.  The arrays hold, per cell and component, the
// adjoint value times that component's second curl coefficient (s: cexhz,
// ceyhx, cezhy for E; chxez, chyex, chzey for H; 1 where it is zero), so
// lE = stored / s.  On a uniform grid a material's two curl coefficients
// of a component are s and -s, bit for bit, so the weight a cell puts on
// each of its differences is + or - its stored value: a cell whose
// neighbours are plain (no CPML, no wall, such a material) gathers their
// stored values with no coefficient of theirs and scales the sum by its
// own s -- the forward update's shape, own coefficients only.  Planes that
// hold a material whose curl coefficients differ (lumped elements, thin
// wires, a non-uniform cell) carry kAdjGeneral and take the general path,
// which unscales each neighbour's value with its material's 1/s.
#pragma once

#include "common.cuh"
#include "volume.cuh"

namespace xg {

template <typename T, typename I>
struct AdjParams {
  VolParams<T, I> v;          // geometry, coefficient table, CPML profiles, flags
  T *lE[3], *lH[3];           // adjoint fields, padded layout
  Psi<T> m;                   // adjoint psi, layout of the forward psi
  // parameter gradient over the design box [lo, hi)
  int dlo[3], dhi[3];
  double *g_eps, *g_sig;      // [di][dj][dk]
  const double *dtab;         // per table entry: dc0/deps, dc0/dsig, dc/deps / c, dc/dsig / c
  const T *recE[3];           // E(t) over the design box
  const T *recH[3];           // H(t) over the design box grown by one cell on the low sides
  // loss: sum over a plane of F(comp)^2 after the steps of a window
  int loss_comp, plane_axis, plane_index;
  int plo[2], phi[2];         // ranges on the two other axes (in axis order)
  const T *plane_rec;         // the loss component over the plane after step t-1 (or null)
  int do_e_own;               // k_adj_e: the own-cell transpose and gradient of step t
  int do_gather;              // k_adj_e: the loss and U gather of step t-1
  const T *sc, *isc;          // per table entry: s and 1/s of Ex, Ey, Ez, Hx, Hy, Hz
  // k tiling of the launch (adj_k below): the k range whose cells can take
  // the plain path, [kp_lo, kp_hi], and the 32-wide tiles below it (kt_n0)
  // and over it (kt_n1); the rest cover the k above it
  int kp_lo, kp_hi, kt_n0, kt_n1;
};

// The k of this thread: blockIdx.x walks the 32-wide tiles below, over and
// above the plain k range, so that no warp mixes cells of the z slabs with
// plain cells (a warp is one row of 32 k).  Returns -1 past a range's end.
template <typename T, typename I>
__device__ __forceinline__ int adj_k(const AdjParams<T, I> &a, int nz) {
  const int t = static_cast<int>(blockIdx.x), l = static_cast<int>(threadIdx.x);
  int k, end;
  if (t < a.kt_n0) {
    k = t * 32 + l;
    end = a.kp_lo - 1;
  } else if (t < a.kt_n0 + a.kt_n1) {
    k = a.kp_lo + (t - a.kt_n0) * 32 + l;
    end = a.kp_hi;
  } else {
    k = a.kp_hi + 1 + (t - a.kt_n0 - a.kt_n1) * 32 + l;
    end = nz;
  }
  return k <= end ? k : -1;
}

// An x plane that holds a material whose two curl coefficients of some
// component are not s and -s: the adjoint kernels take the general path
// for the cells whose gathers reach it.
constexpr uint8_t kAdjGeneral = 8;

// ---- weights of one E cell on its H differences ------------------------
// which: 0 = Ex on dHy/dz, 1 = Ex on dHz/dy, 2 = Ey on dHx/dz, 3 = Ey on
// dHz/dx, 4 = Ez on dHx/dy, 5 = Ez on dHy/dx.  Zero outside the component.
template <typename T, typename I>
__device__ __forceinline__ T e_weight(const AdjParams<T, I> &a, int i, int j, int k, int which) {
  const VolParams<T, I> &p = a.v;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  if (i < 0 || j < 0 || k < 0 || i > nx || j > ny || k > nz) return T(0);
  const int comp = which >> 1;
  if ((comp == 0 && i >= nx) || (comp == 1 && j >= ny) || (comp == 2 && k >= nz)) return T(0);
  const unsigned b = static_cast<unsigned>(i) * static_cast<unsigned>(p.d.si) +
                     static_cast<unsigned>(j) * static_cast<unsigned>(p.d.sj) + static_cast<unsigned>(k);
  const unsigned id = static_cast<unsigned>(__ldg(p.idx + b));
  const T L = mul(a.lE[comp][b], a.isc[id * 6 + comp]);
  const T *c = p.table + id * 18;
  const int xs = p.cp[0].n_layers ? p.cp[0].slot_e[i] : -1;
  const int ys = p.cp[1].n_layers ? p.cp[1].slot_e[j] : -1;
  const int zs = p.cp[2].n_layers ? p.cp[2].slot_e[k] : -1;
  const bool in_i = i >= 1 && i < nx, in_j = j >= 1 && j < ny, in_k = k >= 1 && k < nz;
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);
  T w = T(0);
  switch (which) {
    case 0:   // Ex, (Hy(k) - Hy(k-1)): main ca = cexhy (x 1/kappa_z), psi_ex_z
      if (in_j && in_k) w = mul(zs >= 0 ? mul(c[1], p.cp[2].rk_e[k]) : c[1], L);
      if (zs >= 0) {
        const unsigned o = (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
        w = fmad(p.cp[2].a_e[k], fmad(mul(c[1], p.dl[2]), L, a.m.ex_z[o]), w);
      }
      break;
    case 1:   // Ex, (Hz(j) - Hz(j-1)): main cb = cexhz (x 1/kappa_y), psi_ex_y
      if (in_j && in_k) w = mul(ys >= 0 ? mul(c[2], p.cp[1].rk_e[j]) : c[2], L);
      if (ys >= 0) {
        const unsigned o = (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
        w = fmad(p.cp[1].a_e[j], fmad(mul(c[2], p.dl[1]), L, a.m.ex_y[o]), w);
      }
      break;
    case 2:   // Ey, (Hx(k) - Hx(k-1)): main ca = ceyhx (x 1/kappa_z), psi_ey_z
      if (in_i && in_k) w = mul(zs >= 0 ? mul(c[5], p.cp[2].rk_e[k]) : c[5], L);
      if (zs >= 0) {
        const unsigned o = (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
        w = fmad(p.cp[2].a_e[k], fmad(mul(c[5], p.dl[2]), L, a.m.ey_z[o]), w);
      }
      break;
    case 3:   // Ey, (Hz(i) - Hz(i-1)): main cb = ceyhz (x 1/kappa_x), psi_ey_x
      if (in_i && in_k) w = mul(xs >= 0 ? mul(c[4], p.cp[0].rk_e[i]) : c[4], L);
      if (xs >= 0) {
        const unsigned o = (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
        w = fmad(p.cp[0].a_e[i], fmad(mul(c[4], p.dl[0]), L, a.m.ey_x[o]), w);
      }
      break;
    case 4:   // Ez, (Hx(j) - Hx(j-1)): main ca = cezhx (x 1/kappa_y), psi_ez_y
      if (in_i && in_j) w = mul(ys >= 0 ? mul(c[7], p.cp[1].rk_e[j]) : c[7], L);
      if (ys >= 0) {
        const unsigned o = (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
        w = fmad(p.cp[1].a_e[j], fmad(mul(c[7], p.dl[1]), L, a.m.ez_y[o]), w);
      }
      break;
    default:   // Ez, (Hy(i) - Hy(i-1)): main cb = cezhy (x 1/kappa_x), psi_ez_x
      if (in_i && in_j) w = mul(xs >= 0 ? mul(c[8], p.cp[0].rk_e[i]) : c[8], L);
      if (xs >= 0) {
        const unsigned o = (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
        w = fmad(p.cp[0].a_e[i], fmad(mul(c[8], p.dl[0]), L, a.m.ez_x[o]), w);
      }
      break;
  }
  return w;
}

// ---- weights of one H cell on its E differences ------------------------
// which: 0 = Hx on dEy/dz, 1 = Hx on dEz/dy, 2 = Hy on dEz/dx, 3 = Hy on
// dEx/dz, 4 = Hz on dEx/dy, 5 = Hz on dEy/dx.  Zero outside the component.
template <typename T, typename I>
__device__ __forceinline__ T h_weight(const AdjParams<T, I> &a, int i, int j, int k, int which) {
  const VolParams<T, I> &p = a.v;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  if (i < 0 || j < 0 || k < 0 || i > nx || j > ny || k > nz) return T(0);
  const int comp = which >> 1;
  if ((comp == 0 && (j >= ny || k >= nz)) || (comp == 1 && (i >= nx || k >= nz)) || (comp == 2 && (i >= nx || j >= ny)))
    return T(0);
  const unsigned b = static_cast<unsigned>(i) * static_cast<unsigned>(p.d.si) +
                     static_cast<unsigned>(j) * static_cast<unsigned>(p.d.sj) + static_cast<unsigned>(k);
  const unsigned id = static_cast<unsigned>(__ldg(p.idx + b));
  const T L = mul(a.lH[comp][b], a.isc[id * 6 + 3 + comp]);
  const T *c = p.table + id * 18 + 9;
  const int xs = p.cp[0].n_layers ? p.cp[0].slot_h[i] : -1;
  const int ys = p.cp[1].n_layers ? p.cp[1].slot_h[j] : -1;
  const int zs = p.cp[2].n_layers ? p.cp[2].slot_h[k] : -1;
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);
  T w = T(0);
  switch (which) {
    case 0:   // Hx, (Ey(k+1) - Ey(k)): main ca = chxey (x 1/kappa_z), psi_hx_z
      if (i < nx) w = mul(zs >= 0 ? mul(c[1], p.cp[2].rk_m[k]) : c[1], L);
      if (zs >= 0) {
        const unsigned o = (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
        w = fmad(p.cp[2].a_m[k], fmad(mul(c[1], p.dl[2]), L, a.m.hx_z[o]), w);
      }
      break;
    case 1:   // Hx, (Ez(j+1) - Ez(j)): main cb = chxez (x 1/kappa_y), psi_hx_y
      if (i < nx) w = mul(ys >= 0 ? mul(c[2], p.cp[1].rk_m[j]) : c[2], L);
      if (ys >= 0) {
        const unsigned o = (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
        w = fmad(p.cp[1].a_m[j], fmad(mul(c[2], p.dl[1]), L, a.m.hx_y[o]), w);
      }
      break;
    case 2:   // Hy, (Ez(i+1) - Ez(i)): main ca = chyez (x 1/kappa_x), psi_hy_x
      if (j < ny) w = mul(xs >= 0 ? mul(c[4], p.cp[0].rk_m[i]) : c[4], L);
      if (xs >= 0) {
        const unsigned o = (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
        w = fmad(p.cp[0].a_m[i], fmad(mul(c[4], p.dl[0]), L, a.m.hy_x[o]), w);
      }
      break;
    case 3:   // Hy, (Ex(k+1) - Ex(k)): main cb = chyex (x 1/kappa_z), psi_hy_z
      if (j < ny) w = mul(zs >= 0 ? mul(c[5], p.cp[2].rk_m[k]) : c[5], L);
      if (zs >= 0) {
        const unsigned o = (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
        w = fmad(p.cp[2].a_m[k], fmad(mul(c[5], p.dl[2]), L, a.m.hy_z[o]), w);
      }
      break;
    case 4:   // Hz, (Ex(j+1) - Ex(j)): main ca = chzex (x 1/kappa_y), psi_hz_y
      if (k < nz) w = mul(ys >= 0 ? mul(c[7], p.cp[1].rk_m[j]) : c[7], L);
      if (ys >= 0) {
        const unsigned o = (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
        w = fmad(p.cp[1].a_m[j], fmad(mul(c[7], p.dl[1]), L, a.m.hz_y[o]), w);
      }
      break;
    default:   // Hz, (Ey(i+1) - Ey(i)): main cb = chzey (x 1/kappa_x), psi_hz_x
      if (k < nz) w = mul(xs >= 0 ? mul(c[8], p.cp[0].rk_m[i]) : c[8], L);
      if (xs >= 0) {
        const unsigned o = (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
        w = fmad(p.cp[0].a_m[i], fmad(mul(c[8], p.dl[0]), L, a.m.hz_x[o]), w);
      }
      break;
  }
  return w;
}

// ---- the same weights for cells of a material whose curl coefficients are
// -s and s (every cell outside the kAdjGeneral planes) --------------------
// With the stored value M = s L, the main term ca L is -M or M and the
// slab term a (m + c dl L) is a (m - dl M) or a (m + dl M): no coefficient
// of the neighbour is read, only its stored value, its psi adjoint and the
// 1-D CPML profile at its index.  Signs (which 0..5): E -, +, +, -, -, +;
// H -, +, -, +, -, +.
template <typename T, typename I>
__device__ __forceinline__ T e_weight_c(const AdjParams<T, I> &a, int i, int j, int k, int which) {
  const VolParams<T, I> &p = a.v;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  if (i < 0 || j < 0 || k < 0 || i > nx || j > ny || k > nz) return T(0);
  const int comp = which >> 1;
  if ((comp == 0 && i >= nx) || (comp == 1 && j >= ny) || (comp == 2 && k >= nz)) return T(0);
  const unsigned b = static_cast<unsigned>(i) * static_cast<unsigned>(p.d.si) +
                     static_cast<unsigned>(j) * static_cast<unsigned>(p.d.sj) + static_cast<unsigned>(k);
  const T M = a.lE[comp][b];
  const bool in_i = i >= 1 && i < nx, in_j = j >= 1 && j < ny, in_k = k >= 1 && k < nz;
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);
  T w = T(0);
  switch (which) {
    case 0: {   // Ex, (Hy(k) - Hy(k-1)): -s, psi_ex_z
      const int zs = Lz ? p.cp[2].slot_e[k] : -1;
      if (in_j && in_k) w = -(zs >= 0 ? mul(M, p.cp[2].rk_e[k]) : M);
      if (zs >= 0) w = fmad(p.cp[2].a_e[k], fmad(-p.dl[2], M, a.m.ex_z[(static_cast<unsigned>(i) * ny1 + j) * Lz + zs]), w);
      break;
    }
    case 1: {   // Ex, (Hz(j) - Hz(j-1)): +s, psi_ex_y
      const int ys = Ly ? p.cp[1].slot_e[j] : -1;
      if (in_j && in_k) w = ys >= 0 ? mul(M, p.cp[1].rk_e[j]) : M;
      if (ys >= 0) w = fmad(p.cp[1].a_e[j], fmad(p.dl[1], M, a.m.ex_y[(static_cast<unsigned>(i) * Ly + ys) * nzp + k]), w);
      break;
    }
    case 2: {   // Ey, (Hx(k) - Hx(k-1)): +s, psi_ey_z
      const int zs = Lz ? p.cp[2].slot_e[k] : -1;
      if (in_i && in_k) w = zs >= 0 ? mul(M, p.cp[2].rk_e[k]) : M;
      if (zs >= 0) w = fmad(p.cp[2].a_e[k], fmad(p.dl[2], M, a.m.ey_z[(static_cast<unsigned>(i) * ny1 + j) * Lz + zs]), w);
      break;
    }
    case 3: {   // Ey, (Hz(i) - Hz(i-1)): -s, psi_ey_x
      const int xs = p.cp[0].n_layers ? p.cp[0].slot_e[i] : -1;
      if (in_i && in_k) w = -(xs >= 0 ? mul(M, p.cp[0].rk_e[i]) : M);
      if (xs >= 0) w = fmad(p.cp[0].a_e[i], fmad(-p.dl[0], M, a.m.ey_x[(static_cast<unsigned>(xs) * ny1 + j) * nzp + k]), w);
      break;
    }
    case 4: {   // Ez, (Hx(j) - Hx(j-1)): -s, psi_ez_y
      const int ys = Ly ? p.cp[1].slot_e[j] : -1;
      if (in_i && in_j) w = -(ys >= 0 ? mul(M, p.cp[1].rk_e[j]) : M);
      if (ys >= 0) w = fmad(p.cp[1].a_e[j], fmad(-p.dl[1], M, a.m.ez_y[(static_cast<unsigned>(i) * Ly + ys) * nzp + k]), w);
      break;
    }
    default: {   // Ez, (Hy(i) - Hy(i-1)): +s, psi_ez_x
      const int xs = p.cp[0].n_layers ? p.cp[0].slot_e[i] : -1;
      if (in_i && in_j) w = xs >= 0 ? mul(M, p.cp[0].rk_e[i]) : M;
      if (xs >= 0) w = fmad(p.cp[0].a_e[i], fmad(p.dl[0], M, a.m.ez_x[(static_cast<unsigned>(xs) * ny1 + j) * nzp + k]), w);
      break;
    }
  }
  return w;
}

template <typename T, typename I>
__device__ __forceinline__ T h_weight_c(const AdjParams<T, I> &a, int i, int j, int k, int which) {
  const VolParams<T, I> &p = a.v;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  if (i < 0 || j < 0 || k < 0 || i > nx || j > ny || k > nz) return T(0);
  const int comp = which >> 1;
  if ((comp == 0 && (j >= ny || k >= nz)) || (comp == 1 && (i >= nx || k >= nz)) || (comp == 2 && (i >= nx || j >= ny)))
    return T(0);
  const unsigned b = static_cast<unsigned>(i) * static_cast<unsigned>(p.d.si) +
                     static_cast<unsigned>(j) * static_cast<unsigned>(p.d.sj) + static_cast<unsigned>(k);
  const T M = a.lH[comp][b];
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);
  T w = T(0);
  switch (which) {
    case 0: {   // Hx, (Ey(k+1) - Ey(k)): -s, psi_hx_z
      const int zs = Lz ? p.cp[2].slot_h[k] : -1;
      if (i < nx) w = -(zs >= 0 ? mul(M, p.cp[2].rk_m[k]) : M);
      if (zs >= 0) w = fmad(p.cp[2].a_m[k], fmad(-p.dl[2], M, a.m.hx_z[(static_cast<unsigned>(i) * ny1 + j) * Lz + zs]), w);
      break;
    }
    case 1: {   // Hx, (Ez(j+1) - Ez(j)): +s, psi_hx_y
      const int ys = Ly ? p.cp[1].slot_h[j] : -1;
      if (i < nx) w = ys >= 0 ? mul(M, p.cp[1].rk_m[j]) : M;
      if (ys >= 0) w = fmad(p.cp[1].a_m[j], fmad(p.dl[1], M, a.m.hx_y[(static_cast<unsigned>(i) * Ly + ys) * nzp + k]), w);
      break;
    }
    case 2: {   // Hy, (Ez(i+1) - Ez(i)): -s, psi_hy_x
      const int xs = p.cp[0].n_layers ? p.cp[0].slot_h[i] : -1;
      if (j < ny) w = -(xs >= 0 ? mul(M, p.cp[0].rk_m[i]) : M);
      if (xs >= 0) w = fmad(p.cp[0].a_m[i], fmad(-p.dl[0], M, a.m.hy_x[(static_cast<unsigned>(xs) * ny1 + j) * nzp + k]), w);
      break;
    }
    case 3: {   // Hy, (Ex(k+1) - Ex(k)): +s, psi_hy_z
      const int zs = Lz ? p.cp[2].slot_h[k] : -1;
      if (j < ny) w = zs >= 0 ? mul(M, p.cp[2].rk_m[k]) : M;
      if (zs >= 0) w = fmad(p.cp[2].a_m[k], fmad(p.dl[2], M, a.m.hy_z[(static_cast<unsigned>(i) * ny1 + j) * Lz + zs]), w);
      break;
    }
    case 4: {   // Hz, (Ex(j+1) - Ex(j)): -s, psi_hz_y
      const int ys = Ly ? p.cp[1].slot_h[j] : -1;
      if (k < nz) w = -(ys >= 0 ? mul(M, p.cp[1].rk_m[j]) : M);
      if (ys >= 0) w = fmad(p.cp[1].a_m[j], fmad(-p.dl[1], M, a.m.hz_y[(static_cast<unsigned>(i) * Ly + ys) * nzp + k]), w);
      break;
    }
    default: {   // Hz, (Ey(i+1) - Ey(i)): +s, psi_hz_x
      const int xs = p.cp[0].n_layers ? p.cp[0].slot_h[i] : -1;
      if (k < nz) w = xs >= 0 ? mul(M, p.cp[0].rk_m[i]) : M;
      if (xs >= 0) w = fmad(p.cp[0].a_m[i], fmad(p.dl[0], M, a.m.hz_x[(static_cast<unsigned>(xs) * ny1 + j) * nzp + k]), w);
      break;
    }
  }
  return w;
}

// lH(t) = [main] c0 lH' + W gather;  mH(t) = b (mH' + c dl lH').
// Three paths, by the cells the gather reaches: plain (no CPML, no wall:
// the stored values with no profile), compact (CPML or walls, materials
// with curl coefficients -s and s: e_weight_c), and the planes that carry
// kAdjGeneral (any material: e_weight, with each neighbour's coefficients).
template <typename T, typename I>
__global__ void __launch_bounds__(256) k_adj_h(AdjParams<T, I> a) {
  const VolParams<T, I> &p = a.v;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const int k = adj_k(a, nz);
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z;
  if (k < 0 || j > ny || i > nx) return;
  const unsigned b = static_cast<unsigned>(i) * static_cast<unsigned>(p.d.si) +
                     static_cast<unsigned>(j) * static_cast<unsigned>(p.d.sj) + static_cast<unsigned>(k);
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const unsigned id = static_cast<unsigned>(__ldg(p.idx + b));
  // The E cells reading H at this cell are those at this index and one
  // above on each axis.
  const uint8_t fx = __ldg(p.flags[0] + i) | (i < nx ? __ldg(p.flags[0] + i + 1) : uint8_t(0));
  const bool plain = i < nx && j < ny && k < nz &&
                     !((fx | __ldg(p.flags[1] + j) | __ldg(p.flags[1] + j + 1) | __ldg(p.flags[2] + k) |
                        __ldg(p.flags[2] + k + 1)) &
                       (kSpecialE | kSpecialH | kAdjGeneral));
  if (plain) {
    const T *lx = a.lE[0], *ly = a.lE[1], *lz = a.lE[2];
    const T gx = (ly[b] - ly[b + 1]) - (lz[b] - lz[b + usj]);
    const T gy = (lz[b] - lz[b + usi]) - (lx[b] - lx[b + 1]);
    const T gz = (lx[b] - lx[b + usj]) - (ly[b] - ly[b + usi]);
    const T c0 = p.table[id * 18 + 9], s = p.table[id * 18 + 11];
    a.lH[0][b] = fmad(c0, a.lH[0][b], mul(s, gx));
    a.lH[1][b] = fmad(c0, a.lH[1][b], mul(s, gy));
    a.lH[2][b] = fmad(c0, a.lH[2][b], mul(s, gz));
    return;
  }
  const int xs = p.cp[0].n_layers ? p.cp[0].slot_h[i] : -1;
  const int ys = p.cp[1].n_layers ? p.cp[1].slot_h[j] : -1;
  const int zs = p.cp[2].n_layers ? p.cp[2].slot_h[k] : -1;
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);
  if (!(fx & kAdjGeneral)) {
    const T gx = e_weight_c(a, i, j, k, 2) - e_weight_c(a, i, j, k + 1, 2) + e_weight_c(a, i, j, k, 4) -
                 e_weight_c(a, i, j + 1, k, 4);
    const T gy = e_weight_c(a, i, j, k, 0) - e_weight_c(a, i, j, k + 1, 0) + e_weight_c(a, i, j, k, 5) -
                 e_weight_c(a, i + 1, j, k, 5);
    const T gz = e_weight_c(a, i, j, k, 1) - e_weight_c(a, i, j + 1, k, 1) + e_weight_c(a, i, j, k, 3) -
                 e_weight_c(a, i + 1, j, k, 3);
    const T c0 = p.table[id * 18 + 9], s = p.table[id * 18 + 11];
    // own transpose on the stored value M = s lH': mH = b (mH' + c dl lH')
    // with c dl lH' = -dl M or dl M, and s lH = [main] c0 M + s g
    if (j < ny && k < nz) {   // Hx: psi_hx_y (+), psi_hx_z (-)
      const T M = a.lH[0][b];
      if (ys >= 0) {
        T *q = a.m.hx_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
        *q = mul(p.cp[1].b_m[j], fmad(p.dl[1], M, *q));
      }
      if (zs >= 0) {
        T *q = a.m.hx_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
        *q = mul(p.cp[2].b_m[k], fmad(-p.dl[2], M, *q));
      }
      a.lH[0][b] = fmad(s, gx, i < nx ? mul(c0, M) : M);
    }
    if (i < nx && k < nz) {   // Hy: psi_hy_x (-), psi_hy_z (+)
      const T M = a.lH[1][b];
      if (xs >= 0) {
        T *q = a.m.hy_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
        *q = mul(p.cp[0].b_m[i], fmad(-p.dl[0], M, *q));
      }
      if (zs >= 0) {
        T *q = a.m.hy_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
        *q = mul(p.cp[2].b_m[k], fmad(p.dl[2], M, *q));
      }
      a.lH[1][b] = fmad(s, gy, j < ny ? mul(c0, M) : M);
    }
    if (i < nx && j < ny) {   // Hz: psi_hz_x (+), psi_hz_y (-)
      const T M = a.lH[2][b];
      if (xs >= 0) {
        T *q = a.m.hz_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
        *q = mul(p.cp[0].b_m[i], fmad(p.dl[0], M, *q));
      }
      if (ys >= 0) {
        T *q = a.m.hz_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
        *q = mul(p.cp[1].b_m[j], fmad(-p.dl[1], M, *q));
      }
      a.lH[2][b] = fmad(s, gz, k < nz ? mul(c0, M) : M);
    }
    return;
  }
  const T gx = e_weight(a, i, j, k, 2) - e_weight(a, i, j, k + 1, 2) + e_weight(a, i, j, k, 4) - e_weight(a, i, j + 1, k, 4);
  const T gy = e_weight(a, i, j, k, 0) - e_weight(a, i, j, k + 1, 0) + e_weight(a, i, j, k, 5) - e_weight(a, i + 1, j, k, 5);
  const T gz = e_weight(a, i, j, k, 1) - e_weight(a, i, j + 1, k, 1) + e_weight(a, i, j, k, 3) - e_weight(a, i + 1, j, k, 3);
  const T *c = p.table + id * 18 + 9;
  const T *sc = a.sc + id * 6 + 3, *isc = a.isc + id * 6 + 3;
  // own transpose: mH = b (mH' + c dl lH'), lH = [main] c0 lH' (+ gather)
  if (j < ny && k < nz) {   // Hx
    const T L = mul(a.lH[0][b], isc[0]);
    if (ys >= 0) {
      T *q = a.m.hx_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      *q = mul(p.cp[1].b_m[j], fmad(mul(c[2], p.dl[1]), L, *q));
    }
    if (zs >= 0) {
      T *q = a.m.hx_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      *q = mul(p.cp[2].b_m[k], fmad(mul(c[1], p.dl[2]), L, *q));
    }
    a.lH[0][b] = mul(sc[0], (i < nx ? mul(c[0], L) : L) + gx);
  }
  if (i < nx && k < nz) {   // Hy
    const T L = mul(a.lH[1][b], isc[1]);
    if (xs >= 0) {
      T *q = a.m.hy_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      *q = mul(p.cp[0].b_m[i], fmad(mul(c[4], p.dl[0]), L, *q));
    }
    if (zs >= 0) {
      T *q = a.m.hy_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      *q = mul(p.cp[2].b_m[k], fmad(mul(c[5], p.dl[2]), L, *q));
    }
    a.lH[1][b] = mul(sc[1], (j < ny ? mul(c[3], L) : L) + gy);
  }
  if (i < nx && j < ny) {   // Hz
    const T L = mul(a.lH[2][b], isc[2]);
    if (xs >= 0) {
      T *q = a.m.hz_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      *q = mul(p.cp[0].b_m[i], fmad(mul(c[8], p.dl[0]), L, *q));
    }
    if (ys >= 0) {
      T *q = a.m.hz_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      *q = mul(p.cp[1].b_m[j], fmad(mul(c[7], p.dl[1]), L, *q));
    }
    a.lH[2][b] = mul(sc[2], (k < nz ? mul(c[6], L) : L) + gz);
  }
}

// Own E transpose and gradient of step t (do_e_own), then the loss and U
// gather of step t-1 (do_gather); the three paths of k_adj_h.
template <typename T, typename I>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 8 : 6) k_adj_e(AdjParams<T, I> a) {
  const VolParams<T, I> &p = a.v;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const int k = adj_k(a, nz);
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z;
  if (k < 0 || j > ny || i > nx) return;
  const unsigned b = static_cast<unsigned>(i) * static_cast<unsigned>(p.d.si) +
                     static_cast<unsigned>(j) * static_cast<unsigned>(p.d.sj) + static_cast<unsigned>(k);
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const bool ex = i < nx, ey = j < ny, ez = k < nz;   // components present at this index
  const unsigned id = static_cast<unsigned>(__ldg(p.idx + b));
  const T *c = p.table + id * 18;
  T M[3] = {ex ? a.lE[0][b] : T(0), ey ? a.lE[1][b] : T(0), ez ? a.lE[2][b] : T(0)};
  // gradient of step t over the design box (interior cells: main updates, no CPML)
  if (a.do_e_own && i >= a.dlo[0] && i < a.dhi[0] && j >= a.dlo[1] && j < a.dhi[1] && k >= a.dlo[2] &&
      k < a.dhi[2]) {
    const int di = i - a.dlo[0], dj = j - a.dlo[1], dk = k - a.dlo[2];
    const int ej = a.dhi[1] - a.dlo[1], ek = a.dhi[2] - a.dlo[2];
    const int hj = ej + 1, hk = ek + 1;
    auto E = [&](int comp) { return static_cast<double>(a.recE[comp][(di * ej + dj) * ek + dk]); };
    auto H = [&](int comp, int oi, int oj, int ok) {   // H(t) at (i+oi, j+oj, k+ok), o* in {-1, 0}
      return static_cast<double>(a.recH[comp][((di + 1 + oi) * hj + (dj + 1 + oj)) * hk + (dk + 1 + ok)]);
    };
    const double curl[3] = {
        static_cast<double>(c[1]) * (H(1, 0, 0, 0) - H(1, 0, 0, -1)) + static_cast<double>(c[2]) * (H(2, 0, 0, 0) - H(2, 0, -1, 0)),
        static_cast<double>(c[5]) * (H(0, 0, 0, 0) - H(0, 0, 0, -1)) + static_cast<double>(c[4]) * (H(2, 0, 0, 0) - H(2, -1, 0, 0)),
        static_cast<double>(c[7]) * (H(0, 0, 0, 0) - H(0, 0, -1, 0)) + static_cast<double>(c[8]) * (H(1, 0, 0, 0) - H(1, -1, 0, 0))};
    const double *dt = a.dtab + 4 * id;
    double ge = 0, gs = 0;
    for (int comp = 0; comp < 3; ++comp) {
      const double l = static_cast<double>(mul(M[comp], a.isc[id * 6 + comp]));
      ge += l * (dt[0] * E(comp) + dt[2] * curl[comp]);
      gs += l * (dt[1] * E(comp) + dt[3] * curl[comp]);
    }
    const int g = (di * ej + dj) * ek + dk;
    a.g_eps[g] += ge;
    a.g_sig[g] += gs;
  }
  // loss gradient of step t-1 at this cell: d/dF sum F^2 = 2 F over the plane
  T lossg = T(0);
  if (a.do_gather && a.plane_rec) {
    const int ax = a.plane_axis;
    const int idx3[3] = {i, j, k};
    const int u = idx3[ax == 0 ? 1 : 0], v = idx3[ax == 2 ? 1 : 2];
    if (idx3[ax] == a.plane_index && u >= a.plo[0] && u < a.phi[0] && v >= a.plo[1] && v < a.phi[1]) {
      const int nv = a.phi[1] - a.plo[1];
      lossg = T(2) * a.plane_rec[(u - a.plo[0]) * nv + (v - a.plo[1])];
    }
  }
  // The H cells of step t-1 reading E at this cell are those at this index
  // and one below on each axis.
  const uint8_t fx = __ldg(p.flags[0] + i) | (i >= 1 ? __ldg(p.flags[0] + i - 1) : uint8_t(0));
  const bool plain = i >= 1 && j >= 1 && k >= 1 && i < nx && j < ny && k < nz &&
                     !((fx | __ldg(p.flags[1] + j) | __ldg(p.flags[1] + j - 1) | __ldg(p.flags[2] + k) |
                        __ldg(p.flags[2] + k - 1)) &
                       (kSpecialE | kSpecialH | kAdjGeneral));
  if (plain) {
    if (a.do_e_own) {
      const T c0 = c[0];
      M[0] = mul(c0, M[0]);
      M[1] = mul(c0, M[1]);
      M[2] = mul(c0, M[2]);
    }
    if (a.do_gather) {
      const T *hx = a.lH[0], *hy = a.lH[1], *hz = a.lH[2];
      T u0 = (hy[b - 1] - hy[b]) - (hz[b - usj] - hz[b]);
      T u1 = (hz[b - usi] - hz[b]) - (hx[b - 1] - hx[b]);
      T u2 = (hx[b - usj] - hx[b]) - (hy[b - usi] - hy[b]);
      if (a.loss_comp == 0) u0 += lossg;
      else if (a.loss_comp == 1) u1 += lossg;
      else u2 += lossg;
      const T s = c[2];
      M[0] = fmad(s, u0, M[0]);
      M[1] = fmad(s, u1, M[1]);
      M[2] = fmad(s, u2, M[2]);
    }
  } else {
    const int xs = p.cp[0].n_layers ? p.cp[0].slot_e[i] : -1;
    const int ys = p.cp[1].n_layers ? p.cp[1].slot_e[j] : -1;
    const int zs = p.cp[2].n_layers ? p.cp[2].slot_e[k] : -1;
    const bool in_i = i >= 1 && i < nx, in_j = j >= 1 && j < ny, in_k = k >= 1 && k < nz;
    const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
    const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);
    if (!(fx & kAdjGeneral)) {
      // own transpose on the stored value M = s lE': mE = b (mE' + c dl lE')
      // with c dl lE' = -dl M or dl M; s lE = [main] c0 M, then + s U
      const T c0 = c[0], s = c[2];
      if (a.do_e_own) {
        if (ex) {   // psi_ex_y (+), psi_ex_z (-)
          if (ys >= 0) {
            T *q = a.m.ex_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
            *q = mul(p.cp[1].b_e[j], fmad(p.dl[1], M[0], *q));
          }
          if (zs >= 0) {
            T *q = a.m.ex_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
            *q = mul(p.cp[2].b_e[k], fmad(-p.dl[2], M[0], *q));
          }
          if (in_j && in_k) M[0] = mul(c0, M[0]);
        }
        if (ey) {   // psi_ey_x (-), psi_ey_z (+)
          if (xs >= 0) {
            T *q = a.m.ey_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
            *q = mul(p.cp[0].b_e[i], fmad(-p.dl[0], M[1], *q));
          }
          if (zs >= 0) {
            T *q = a.m.ey_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
            *q = mul(p.cp[2].b_e[k], fmad(p.dl[2], M[1], *q));
          }
          if (in_i && in_k) M[1] = mul(c0, M[1]);
        }
        if (ez) {   // psi_ez_x (+), psi_ez_y (-)
          if (xs >= 0) {
            T *q = a.m.ez_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
            *q = mul(p.cp[0].b_e[i], fmad(p.dl[0], M[2], *q));
          }
          if (ys >= 0) {
            T *q = a.m.ez_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
            *q = mul(p.cp[1].b_e[j], fmad(-p.dl[1], M[2], *q));
          }
          if (in_i && in_j) M[2] = mul(c0, M[2]);
        }
      }
      if (a.do_gather) {
        T u[3] = {T(0), T(0), T(0)};
        u[a.loss_comp] = lossg;
        if (ex) u[0] += h_weight_c(a, i, j, k - 1, 3) - h_weight_c(a, i, j, k, 3) + h_weight_c(a, i, j - 1, k, 4) - h_weight_c(a, i, j, k, 4);
        if (ey) u[1] += h_weight_c(a, i, j, k - 1, 0) - h_weight_c(a, i, j, k, 0) + h_weight_c(a, i - 1, j, k, 5) - h_weight_c(a, i, j, k, 5);
        if (ez) u[2] += h_weight_c(a, i, j - 1, k, 1) - h_weight_c(a, i, j, k, 1) + h_weight_c(a, i - 1, j, k, 2) - h_weight_c(a, i, j, k, 2);
        M[0] = fmad(s, u[0], M[0]);
        M[1] = fmad(s, u[1], M[1]);
        M[2] = fmad(s, u[2], M[2]);
      }
    } else {
      const T *sc = a.sc + id * 6, *isc = a.isc + id * 6;
      T L[3] = {mul(M[0], isc[0]), mul(M[1], isc[1]), mul(M[2], isc[2])};
      if (a.do_e_own) {
        if (ex) {
          if (ys >= 0) {
            T *q = a.m.ex_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
            *q = mul(p.cp[1].b_e[j], fmad(mul(c[2], p.dl[1]), L[0], *q));
          }
          if (zs >= 0) {
            T *q = a.m.ex_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
            *q = mul(p.cp[2].b_e[k], fmad(mul(c[1], p.dl[2]), L[0], *q));
          }
          if (in_j && in_k) L[0] = mul(c[0], L[0]);
        }
        if (ey) {
          if (xs >= 0) {
            T *q = a.m.ey_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
            *q = mul(p.cp[0].b_e[i], fmad(mul(c[4], p.dl[0]), L[1], *q));
          }
          if (zs >= 0) {
            T *q = a.m.ey_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
            *q = mul(p.cp[2].b_e[k], fmad(mul(c[5], p.dl[2]), L[1], *q));
          }
          if (in_i && in_k) L[1] = mul(c[3], L[1]);
        }
        if (ez) {
          if (xs >= 0) {
            T *q = a.m.ez_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
            *q = mul(p.cp[0].b_e[i], fmad(mul(c[8], p.dl[0]), L[2], *q));
          }
          if (ys >= 0) {
            T *q = a.m.ez_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
            *q = mul(p.cp[1].b_e[j], fmad(mul(c[7], p.dl[1]), L[2], *q));
          }
          if (in_i && in_j) L[2] = mul(c[6], L[2]);
        }
      }
      if (a.do_gather) {
        L[a.loss_comp] += lossg;
        if (ex) L[0] += h_weight(a, i, j, k - 1, 3) - h_weight(a, i, j, k, 3) + h_weight(a, i, j - 1, k, 4) - h_weight(a, i, j, k, 4);
        if (ey) L[1] += h_weight(a, i, j, k - 1, 0) - h_weight(a, i, j, k, 0) + h_weight(a, i - 1, j, k, 5) - h_weight(a, i, j, k, 5);
        if (ez) L[2] += h_weight(a, i, j - 1, k, 1) - h_weight(a, i, j, k, 1) + h_weight(a, i - 1, j, k, 2) - h_weight(a, i, j, k, 2);
      }
      M[0] = mul(sc[0], L[0]);
      M[1] = mul(sc[1], L[1]);
      M[2] = mul(sc[2], L[2]);
    }
  }
  if (ex) a.lE[0][b] = M[0];
  if (ey) a.lE[1][b] = M[1];
  if (ez) a.lE[2][b] = M[2];
}

// Marks (mark[i] = 1) the x planes that hold a cell whose table entry has
// nc[entry] set: curl coefficients other than s and -s on some component.
template <typename I>
__global__ void k_adj_mark(const I *idx, Dims d, const uint8_t *nc, int *mark) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z;
  if (k > d.nz || j > d.ny || i > d.nx) return;
  const long long b = static_cast<long long>(i) * d.si + static_cast<long long>(j) * d.sj + k;
  if (nc[static_cast<unsigned>(idx[b])]) mark[i] = 1;
}

template <typename T>
struct FieldPtrs {
  const T *f[6];
};

// The design-box records: E over the box and H over the box grown by one
// cell on the low sides, one slot per step.  With checkpoints every K
// steps, two buffers of K slots: step t goes to slot ((t / K) % 2) K + t % K;
// with K = 0, slot t.
template <typename T>
struct AdjRecords {
  T *recE[3], *recH[3];   // slot 0
  long long nE, nH;       // cells of a slot
  int K;
};

// Copies E(t) and H(t) into the records of step t = *step (the step about
// to run), so that the same launch serves every step of a captured graph.
template <typename T>
__global__ void k_adj_record(FieldPtrs<T> F, Dims d, int lo0, int lo1, int lo2, int n0, int n1, int n2,
                             AdjRecords<T> r, const long long *step) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;   // 0 .. n2 (H box is one larger)
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z;
  if (k > n2 || j > n1 || i > n0) return;
  const long long t = *step;
  const long long slot = r.K > 0 ? ((t / r.K) % 2) * r.K + t % r.K : t;
  T *recE0 = r.recE[0] + slot * r.nE, *recE1 = r.recE[1] + slot * r.nE, *recE2 = r.recE[2] + slot * r.nE;
  T *recH0 = r.recH[0] + slot * r.nH, *recH1 = r.recH[1] + slot * r.nH, *recH2 = r.recH[2] + slot * r.nH;
  // H box cell (i, j, k) is grid cell (lo-1 + i, ...)
  const long long gh = static_cast<long long>(lo0 - 1 + i) * d.si + static_cast<long long>(lo1 - 1 + j) * d.sj + (lo2 - 1 + k);
  const long long h = (static_cast<long long>(i) * (n1 + 1) + j) * (n2 + 1) + k;
  recH0[h] = F.f[3][gh];
  recH1[h] = F.f[4][gh];
  recH2[h] = F.f[5][gh];
  if (i >= 1 && j >= 1 && k >= 1) {
    const long long e = (static_cast<long long>(i - 1) * n1 + (j - 1)) * n2 + (k - 1);
    recE0[e] = F.f[0][gh];
    recE1[e] = F.f[1][gh];
    recE2[e] = F.f[2][gh];
  }
}

// Copies the loss component over the plane after step t = *step - 1 (the
// step that just ran) into its record, row-major over the two other axes,
// when t lies in the loss window [t_begin, t_end); nothing otherwise.
template <typename T>
__global__ void k_adj_plane(const T *f, Dims d, int axis, int index, int lo0, int lo1, int n0, int n1, T *rec,
                            const long long *step, long long t_begin, long long t_end) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const int u = blockIdx.y;
  if (v >= n1 || u >= n0) return;
  const long long t = *step - 1;
  if (t < t_begin || t >= t_end) return;
  rec += (t - t_begin) * n0 * n1;
  int ijk[3];
  ijk[axis] = index;
  ijk[axis == 0 ? 1 : 0] = lo0 + u;
  ijk[axis == 2 ? 1 : 2] = lo1 + v;
  rec[static_cast<long long>(u) * n1 + v] = f[static_cast<long long>(ijk[0]) * d.si + static_cast<long long>(ijk[1]) * d.sj + ijk[2]];
}

}  // namespace xg
