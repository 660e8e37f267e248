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
// the same expression as the general path so both give identical bits.
#pragma once

#include "common.cuh"

namespace xg {

template <typename T, typename I, bool SMEM_TABLE>
__device__ __forceinline__ const T *load_table(const VolParams<T, I> &p, int half, int &ts) {
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

// E update of one cell (fast path when the cell is plain, else the general
// path with walls and CPML).
template <typename T, typename I>
__device__ __forceinline__ void e_cell(const VolParams<T, I> &p, const T *tab, int ts, int i, int j, int k) {
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const unsigned b = static_cast<unsigned>(i) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
  const T *__restrict__ Hx = p.H[0];
  const T *__restrict__ Hy = p.H[1];
  const T *__restrict__ Hz = p.H[2];
  T *__restrict__ Ex = p.E[0];
  T *__restrict__ Ey = p.E[1];
  T *__restrict__ Ez = p.E[2];

  if (!((__ldg(p.flags[0] + i) | __ldg(p.flags[1] + j) | __ldg(p.flags[2] + k)) & kSpecialE)) {
    const T hx = __ldg(Hx + b), hy = __ldg(Hy + b), hz = __ldg(Hz + b);
    const T hx_k = __ldg(Hx + b - 1), hy_k = __ldg(Hy + b - 1);
    const T hx_j = __ldg(Hx + b - usj), hz_j = __ldg(Hz + b - usj);
    const T hy_im1 = __ldg(Hy + b - usi), hz_im1 = __ldg(Hz + b - usi);
    const T *c = tab + static_cast<unsigned>(__ldg(p.idx + b)) * ts;
    const T ex = Ex[b], ey = Ey[b], ez = Ez[b];
    Ex[b] = c[0] * ex + c[1] * (hy - hy_k) + c[2] * (hz - hz_j);
    Ey[b] = c[3] * ey + c[5] * (hx - hx_k) + c[4] * (hz - hz_im1);
    Ez[b] = c[6] * ez + c[7] * (hx - hx_j) + c[8] * (hy - hy_im1);
    return;
  }

  // ---------------- general path: outer walls and CPML slabs -------------
  const T hx = __ldg(Hx + b), hy = __ldg(Hy + b), hz = __ldg(Hz + b);
  const T hx_k = k > 0 ? __ldg(Hx + b - 1) : T(0);
  const T hy_k = k > 0 ? __ldg(Hy + b - 1) : T(0);
  const T hx_j = j > 0 ? __ldg(Hx + b - usj) : T(0);
  const T hz_j = j > 0 ? __ldg(Hz + b - usj) : T(0);
  const T hy_im1 = i > 0 ? __ldg(Hy + b - usi) : T(0);
  const T hz_im1 = i > 0 ? __ldg(Hz + b - usi) : T(0);
  const T *c = tab + static_cast<unsigned>(__ldg(p.idx + b)) * ts;
  const int xs = p.cp[0].n_layers ? p.cp[0].slot_e[i] : -1;
  const int ys = p.cp[1].n_layers ? p.cp[1].slot_e[j] : -1;
  const int zs = p.cp[2].n_layers ? p.cp[2].slot_e[k] : -1;
  const bool in_i = i >= 1 && i < nx, in_j = j >= 1 && j < ny, in_k = k >= 1 && k < nz;
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);

  // ---- Ex (nx, ny+1, nz+1) ----
  if (i < nx) {
    const T d_hz_y = hz - hz_j;   // Hz(j) - Hz(j-1)
    const T d_hy_z = hy - hy_k;   // Hy(k) - Hy(k-1)
    T e = Ex[b];
    bool w = false;
    if (in_j && in_k) {
      T ca = c[1], cb = c[2];
      if (zs >= 0) ca *= p.cp[2].rk_e[k];
      if (ys >= 0) cb *= p.cp[1].rk_e[j];
      e = c[0] * e + ca * d_hy_z + cb * d_hz_y;
      w = true;
    }
    if (ys >= 0) {   // Y slabs: psi_eb of YN/YP, c_psi = cexhz * dy
      T *ps = p.psi.ex_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      const T s = p.cp[1].b_e[j] * (*ps) + p.cp[1].a_e[j] * d_hz_y;
      *ps = s;
      e = e + (c[2] * p.dl[1]) * s;
      w = true;
    }
    if (zs >= 0) {   // Z slabs: psi_ea of ZN/ZP, c_psi = cexhy * dz
      T *ps = p.psi.ex_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      const T s = p.cp[2].b_e[k] * (*ps) + p.cp[2].a_e[k] * d_hy_z;
      *ps = s;
      e = e + (c[1] * p.dl[2]) * s;
      w = true;
    }
    if (w) Ex[b] = e;
  }

  // ---- Ey (nx+1, ny, nz+1) ----
  if (j < ny) {
    const T d_hz_x = hz - hz_im1;  // Hz(i) - Hz(i-1)
    const T d_hx_z = hx - hx_k;    // Hx(k) - Hx(k-1)
    T e = Ey[b];
    bool w = false;
    if (in_i && in_k) {
      T ca = c[5], cb = c[4];      // ceyhx, ceyhz
      if (zs >= 0) ca *= p.cp[2].rk_e[k];
      if (xs >= 0) cb *= p.cp[0].rk_e[i];
      e = c[3] * e + ca * d_hx_z + cb * d_hz_x;
      w = true;
    }
    if (xs >= 0) {   // X slabs: psi_ea of XN/XP, c_psi = ceyhz * dx
      T *ps = p.psi.ey_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      const T s = p.cp[0].b_e[i] * (*ps) + p.cp[0].a_e[i] * d_hz_x;
      *ps = s;
      e = e + (c[4] * p.dl[0]) * s;
      w = true;
    }
    if (zs >= 0) {   // Z slabs: psi_eb of ZN/ZP, c_psi = ceyhx * dz
      T *ps = p.psi.ey_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      const T s = p.cp[2].b_e[k] * (*ps) + p.cp[2].a_e[k] * d_hx_z;
      *ps = s;
      e = e + (c[5] * p.dl[2]) * s;
      w = true;
    }
    if (w) Ey[b] = e;
  }

  // ---- Ez (nx+1, ny+1, nz) ----
  if (k < nz) {
    const T d_hy_x = hy - hy_im1;  // Hy(i) - Hy(i-1)
    const T d_hx_y = hx - hx_j;    // Hx(j) - Hx(j-1)
    T e = Ez[b];
    bool w = false;
    if (in_i && in_j) {
      T ca = c[7], cb = c[8];      // cezhx, cezhy
      if (ys >= 0) ca *= p.cp[1].rk_e[j];
      if (xs >= 0) cb *= p.cp[0].rk_e[i];
      e = c[6] * e + ca * d_hx_y + cb * d_hy_x;
      w = true;
    }
    if (xs >= 0) {   // X slabs: psi_eb of XN/XP, c_psi = cezhy * dx
      T *ps = p.psi.ez_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      const T s = p.cp[0].b_e[i] * (*ps) + p.cp[0].a_e[i] * d_hy_x;
      *ps = s;
      e = e + (c[8] * p.dl[0]) * s;
      w = true;
    }
    if (ys >= 0) {   // Y slabs: psi_ea of YN/YP, c_psi = cezhx * dy
      T *ps = p.psi.ez_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      const T s = p.cp[1].b_e[j] * (*ps) + p.cp[1].a_e[j] * d_hx_y;
      *ps = s;
      e = e + (c[7] * p.dl[1]) * s;
      w = true;
    }
    if (w) Ez[b] = e;
  }
}

// NC plain cells (i0 .. i0+NC-1) of one (j, k) column: every load is issued
// before any store, and the H at i-1 of cell c+1 is cell c's own.
template <typename T, typename I, int NC>
__device__ __forceinline__ void e_fast(const VolParams<T, I> &p, const T *tab, int ts, int i0, int j, int k) {
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const unsigned b0 = static_cast<unsigned>(i0) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
  const T *__restrict__ Hx = p.H[0];
  const T *__restrict__ Hy = p.H[1];
  const T *__restrict__ Hz = p.H[2];
  T *__restrict__ Ex = p.E[0];
  T *__restrict__ Ey = p.E[1];
  T *__restrict__ Ez = p.E[2];
  T hx[NC], hy[NC + 1], hz[NC + 1], hx_k[NC], hy_k[NC], hx_j[NC], hz_j[NC], ex[NC], ey[NC], ez[NC];
  const T *c[NC];
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
    c[q] = tab + static_cast<unsigned>(__ldg(p.idx + b)) * ts;
    ex[q] = Ex[b];
    ey[q] = Ey[b];
    ez[q] = Ez[b];
  }
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    const unsigned b = b0 + q * usi;
    const T *cc = c[q];
    Ex[b] = cc[0] * ex[q] + cc[1] * (hy[q + 1] - hy_k[q]) + cc[2] * (hz[q + 1] - hz_j[q]);
    Ey[b] = cc[3] * ey[q] + cc[5] * (hx[q] - hx_k[q]) + cc[4] * (hz[q + 1] - hz[q]);
    Ez[b] = cc[6] * ez[q] + cc[7] * (hx[q] - hx_j[q]) + cc[8] * (hy[q + 1] - hy[q]);
  }
}

// MINB: minimum resident blocks per SM requested from the register
// allocator (1 = no cap); NC: cells per thread along i.  The autotuner in
// engine.cu picks both (and the block shape) per plan.
template <typename T, typename I, bool SMEM_TABLE, int MINB, int NC>
__global__ void __launch_bounds__(256, MINB) k_update_e(VolParams<T, I> p) {
  int ts;
  const T *tab = load_table<T, I, SMEM_TABLE>(p, 0, ts);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i0 = (blockIdx.z * blockDim.z + threadIdx.z) * NC;
  if (k > p.d.nz || j > p.d.ny || i0 > p.d.nx) return;
  bool plain = !((__ldg(p.flags[1] + j) | __ldg(p.flags[2] + k)) & kSpecialE) && i0 + NC - 1 <= p.d.nx;
#pragma unroll
  for (int q = 0; q < NC; ++q) plain = plain && !(__ldg(p.flags[0] + min(i0 + q, p.d.nx)) & kSpecialE);
  if (plain) {
    e_fast<T, I, NC>(p, tab, ts, i0, j, k);
    return;
  }
#pragma unroll
  for (int q = 0; q < NC; ++q)
    if (i0 + q <= p.d.nx) e_cell<T, I>(p, tab, ts, i0 + q, j, k);
}

// H update of one cell (fast path when the cell is plain).
template <typename T, typename I>
__device__ __forceinline__ void h_cell(const VolParams<T, I> &p, const T *tab, int ts, int i, int j, int k) {
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const unsigned b = static_cast<unsigned>(i) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
  const T *__restrict__ Ex = p.E[0];
  const T *__restrict__ Ey = p.E[1];
  const T *__restrict__ Ez = p.E[2];
  T *__restrict__ Hx = p.H[0];
  T *__restrict__ Hy = p.H[1];
  T *__restrict__ Hz = p.H[2];

  if (!((__ldg(p.flags[0] + i) | __ldg(p.flags[1] + j) | __ldg(p.flags[2] + k)) & kSpecialH)) {
    const T ex = __ldg(Ex + b), ey = __ldg(Ey + b), ez = __ldg(Ez + b);
    const T ey_ip = __ldg(Ey + b + usi), ez_ip = __ldg(Ez + b + usi);
    const T ex_kp = __ldg(Ex + b + 1), ey_kp = __ldg(Ey + b + 1);
    const T ex_jp = __ldg(Ex + b + usj), ez_jp = __ldg(Ez + b + usj);
    const T *c = tab + static_cast<unsigned>(__ldg(p.idx + b)) * ts;
    const T hx = Hx[b], hy = Hy[b], hz = Hz[b];
    Hx[b] = c[0] * hx + c[1] * (ey_kp - ey) + c[2] * (ez_jp - ez);
    Hy[b] = c[3] * hy + c[4] * (ez_ip - ez) + c[5] * (ex_kp - ex);
    Hz[b] = c[6] * hz + c[7] * (ex_jp - ex) + c[8] * (ey_ip - ey);
    return;
  }

  // ---------------- general path: last planes and CPML slabs -------------
  const T ex = __ldg(Ex + b), ey_i = __ldg(Ey + b), ez_i = __ldg(Ez + b);
  const T ey_ip = i < nx ? __ldg(Ey + b + usi) : T(0);
  const T ez_ip = i < nx ? __ldg(Ez + b + usi) : T(0);
  const T ex_kp = k < nz ? __ldg(Ex + b + 1) : T(0);
  const T ey_kp = k < nz ? __ldg(Ey + b + 1) : T(0);
  const T ex_jp = j < ny ? __ldg(Ex + b + usj) : T(0);
  const T ez_jp = j < ny ? __ldg(Ez + b + usj) : T(0);
  const T *c = tab + static_cast<unsigned>(__ldg(p.idx + b)) * ts;
  const int xs = p.cp[0].n_layers ? p.cp[0].slot_h[i] : -1;
  const int ys = p.cp[1].n_layers ? p.cp[1].slot_h[j] : -1;
  const int zs = p.cp[2].n_layers ? p.cp[2].slot_h[k] : -1;
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);

  // ---- Hx (nx+1, ny, nz) ----
  if (j < ny && k < nz) {
    const T d_ey_z = ey_kp - ey_i;   // Ey(k+1) - Ey(k)
    const T d_ez_y = ez_jp - ez_i;   // Ez(j+1) - Ez(j)
    T h = Hx[b];
    bool w = false;
    if (i < nx) {
      T ca = c[1], cb = c[2];        // chxey, chxez
      if (zs >= 0) ca *= p.cp[2].rk_m[k];
      if (ys >= 0) cb *= p.cp[1].rk_m[j];
      h = c[0] * h + ca * d_ey_z + cb * d_ez_y;
      w = true;
    }
    if (ys >= 0) {   // Y slabs: psi_hb of YN/YP, c_psi = chxez * dy
      T *ps = p.psi.hx_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      const T s = p.cp[1].b_m[j] * (*ps) + p.cp[1].a_m[j] * d_ez_y;
      *ps = s;
      h = h + (c[2] * p.dl[1]) * s;
      w = true;
    }
    if (zs >= 0) {   // Z slabs: psi_ha of ZN/ZP, c_psi = chxey * dz
      T *ps = p.psi.hx_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      const T s = p.cp[2].b_m[k] * (*ps) + p.cp[2].a_m[k] * d_ey_z;
      *ps = s;
      h = h + (c[1] * p.dl[2]) * s;
      w = true;
    }
    if (w) Hx[b] = h;
  }

  // ---- Hy (nx, ny+1, nz) ----
  if (i < nx && k < nz) {
    const T d_ez_x = ez_ip - ez_i;   // Ez(i+1) - Ez(i)
    const T d_ex_z = ex_kp - ex;     // Ex(k+1) - Ex(k)
    T h = Hy[b];
    bool w = false;
    if (j < ny) {
      T ca = c[4], cb = c[5];        // chyez, chyex
      if (xs >= 0) ca *= p.cp[0].rk_m[i];
      if (zs >= 0) cb *= p.cp[2].rk_m[k];
      h = c[3] * h + ca * d_ez_x + cb * d_ex_z;
      w = true;
    }
    if (xs >= 0) {   // X slabs: psi_ha of XN/XP, c_psi = chyez * dx
      T *ps = p.psi.hy_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      const T s = p.cp[0].b_m[i] * (*ps) + p.cp[0].a_m[i] * d_ez_x;
      *ps = s;
      h = h + (c[4] * p.dl[0]) * s;
      w = true;
    }
    if (zs >= 0) {   // Z slabs: psi_hb of ZN/ZP, c_psi = chyex * dz
      T *ps = p.psi.hy_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      const T s = p.cp[2].b_m[k] * (*ps) + p.cp[2].a_m[k] * d_ex_z;
      *ps = s;
      h = h + (c[5] * p.dl[2]) * s;
      w = true;
    }
    if (w) Hy[b] = h;
  }

  // ---- Hz (nx, ny, nz+1) ----
  if (i < nx && j < ny) {
    const T d_ex_y = ex_jp - ex;     // Ex(j+1) - Ex(j)
    const T d_ey_x = ey_ip - ey_i;   // Ey(i+1) - Ey(i)
    T h = Hz[b];
    bool w = false;
    if (k < nz) {
      T ca = c[7], cb = c[8];        // chzex, chzey
      if (ys >= 0) ca *= p.cp[1].rk_m[j];
      if (xs >= 0) cb *= p.cp[0].rk_m[i];
      h = c[6] * h + ca * d_ex_y + cb * d_ey_x;
      w = true;
    }
    if (xs >= 0) {   // X slabs: psi_hb of XN/XP, c_psi = chzey * dx
      T *ps = p.psi.hz_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      const T s = p.cp[0].b_m[i] * (*ps) + p.cp[0].a_m[i] * d_ey_x;
      *ps = s;
      h = h + (c[8] * p.dl[0]) * s;
      w = true;
    }
    if (ys >= 0) {   // Y slabs: psi_ha of YN/YP, c_psi = chzex * dy
      T *ps = p.psi.hz_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      const T s = p.cp[1].b_m[j] * (*ps) + p.cp[1].a_m[j] * d_ex_y;
      *ps = s;
      h = h + (c[7] * p.dl[1]) * s;
      w = true;
    }
    if (w) Hz[b] = h;
  }
}

// NC plain cells of one column for H: the E at i+1 of cell c is cell c+1's own.
template <typename T, typename I, int NC>
__device__ __forceinline__ void h_fast(const VolParams<T, I> &p, const T *tab, int ts, int i0, int j, int k) {
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const unsigned b0 = static_cast<unsigned>(i0) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
  const T *__restrict__ Ex = p.E[0];
  const T *__restrict__ Ey = p.E[1];
  const T *__restrict__ Ez = p.E[2];
  T *__restrict__ Hx = p.H[0];
  T *__restrict__ Hy = p.H[1];
  T *__restrict__ Hz = p.H[2];
  T ex[NC], ey[NC + 1], ez[NC + 1], ex_kp[NC], ey_kp[NC], ex_jp[NC], ez_jp[NC], hx[NC], hy[NC], hz[NC];
  const T *c[NC];
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
    c[q] = tab + static_cast<unsigned>(__ldg(p.idx + b)) * ts;
    hx[q] = Hx[b];
    hy[q] = Hy[b];
    hz[q] = Hz[b];
  }
  ey[NC] = __ldg(Ey + b0 + NC * usi);
  ez[NC] = __ldg(Ez + b0 + NC * usi);
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    const unsigned b = b0 + q * usi;
    const T *cc = c[q];
    Hx[b] = cc[0] * hx[q] + cc[1] * (ey_kp[q] - ey[q]) + cc[2] * (ez_jp[q] - ez[q]);
    Hy[b] = cc[3] * hy[q] + cc[4] * (ez[q + 1] - ez[q]) + cc[5] * (ex_kp[q] - ex[q]);
    Hz[b] = cc[6] * hz[q] + cc[7] * (ex_jp[q] - ex[q]) + cc[8] * (ey[q + 1] - ey[q]);
  }
}

template <typename T, typename I, bool SMEM_TABLE, int MINB, int NC>
__global__ void __launch_bounds__(256, MINB) k_update_h(VolParams<T, I> p) {
  int ts;
  const T *tab = load_table<T, I, SMEM_TABLE>(p, 1, ts);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i0 = (blockIdx.z * blockDim.z + threadIdx.z) * NC;
  if (k > p.d.nz || j > p.d.ny || i0 > p.d.nx) return;
  bool plain = !((__ldg(p.flags[1] + j) | __ldg(p.flags[2] + k)) & kSpecialH) && i0 + NC - 1 <= p.d.nx;
#pragma unroll
  for (int q = 0; q < NC; ++q) plain = plain && !(__ldg(p.flags[0] + min(i0 + q, p.d.nx)) & kSpecialH);
  if (plain) {
    h_fast<T, I, NC>(p, tab, ts, i0, j, k);
    return;
  }
#pragma unroll
  for (int q = 0; q < NC; ++q)
    if (i0 + q <= p.d.nx) h_cell<T, I>(p, tab, ts, i0 + q, j, k);
}

}  // namespace xg
