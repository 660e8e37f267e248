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
// choice is made per warp: a warp with any non-plain cell runs the general
// path for all its cells.
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

// One CPML recursion: psi' = b psi + a d (read from pr, written to pw when
// `store`), returns the field term (c dl) psi'.
template <typename T>
__device__ __forceinline__ T psi_step(const T *pr, T *pw, bool store, T b, T a, T d, T c_dl, T f) {
  const T s = fmad(a, d, mul(b, *pr));
  if (store) *pw = s;
  return fmad(c_dl, s, f);
}

// General E update of one cell: outer walls and CPML slabs.  E psi is read
// from pr and, when store_psi, written to pw (SEPARATE_PSI) or back to pr
// (in place).  w[c] reports whether component c was updated.
template <typename T, typename I, bool SEPARATE_PSI>
__device__ __forceinline__ void e_general(const VolParams<T, I> &p, const T *c, int i, int j, int k,
                                          const ECurl<T> &h, const Psi<T> &pr, const Psi<T> &pw_, bool store_psi,
                                          T &ex, T &ey, T &ez, bool w[3]) {
  const Psi<T> &pw = SEPARATE_PSI ? pw_ : pr;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const int xs = p.cp[0].n_layers ? p.cp[0].slot_e[i] : -1;
  const int ys = p.cp[1].n_layers ? p.cp[1].slot_e[j] : -1;
  const int zs = p.cp[2].n_layers ? p.cp[2].slot_e[k] : -1;
  const bool in_i = i >= 1 && i < nx, in_j = j >= 1 && j < ny, in_k = k >= 1 && k < nz;
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);
  w[0] = w[1] = w[2] = false;

  // ---- Ex (nx, ny+1, nz+1) ----
  if (i < nx) {
    const T d_hz_y = h.hz - h.hz_j;   // Hz(j) - Hz(j-1)
    const T d_hy_z = h.hy - h.hy_k;   // Hy(k) - Hy(k-1)
    if (in_j && in_k) {
      T ca = c[1], cb = c[2];
      if (zs >= 0) ca = mul(ca, p.cp[2].rk_e[k]);
      if (ys >= 0) cb = mul(cb, p.cp[1].rk_e[j]);
      ex = yee(c[0], ex, ca, d_hy_z, cb, d_hz_y);
      w[0] = true;
    }
    if (ys >= 0) {   // Y slabs: psi_eb of YN/YP, c_psi = cexhz * dy
      const unsigned o = (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      ex = psi_step(pr.ex_y + o, pw.ex_y + o, store_psi, p.cp[1].b_e[j], p.cp[1].a_e[j], d_hz_y, mul(c[2], p.dl[1]), ex);
      w[0] = true;
    }
    if (zs >= 0) {   // Z slabs: psi_ea of ZN/ZP, c_psi = cexhy * dz
      const unsigned o = (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      ex = psi_step(pr.ex_z + o, pw.ex_z + o, store_psi, p.cp[2].b_e[k], p.cp[2].a_e[k], d_hy_z, mul(c[1], p.dl[2]), ex);
      w[0] = true;
    }
  }

  // ---- Ey (nx+1, ny, nz+1) ----
  if (j < ny) {
    const T d_hz_x = h.hz - h.hz_i;  // Hz(i) - Hz(i-1)
    const T d_hx_z = h.hx - h.hx_k;  // Hx(k) - Hx(k-1)
    if (in_i && in_k) {
      T ca = c[5], cb = c[4];      // ceyhx, ceyhz
      if (zs >= 0) ca = mul(ca, p.cp[2].rk_e[k]);
      if (xs >= 0) cb = mul(cb, p.cp[0].rk_e[i]);
      ey = yee(c[3], ey, ca, d_hx_z, cb, d_hz_x);
      w[1] = true;
    }
    if (xs >= 0) {   // X slabs: psi_ea of XN/XP, c_psi = ceyhz * dx
      const unsigned o = (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      ey = psi_step(pr.ey_x + o, pw.ey_x + o, store_psi, p.cp[0].b_e[i], p.cp[0].a_e[i], d_hz_x, mul(c[4], p.dl[0]), ey);
      w[1] = true;
    }
    if (zs >= 0) {   // Z slabs: psi_eb of ZN/ZP, c_psi = ceyhx * dz
      const unsigned o = (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      ey = psi_step(pr.ey_z + o, pw.ey_z + o, store_psi, p.cp[2].b_e[k], p.cp[2].a_e[k], d_hx_z, mul(c[5], p.dl[2]), ey);
      w[1] = true;
    }
  }

  // ---- Ez (nx+1, ny+1, nz) ----
  if (k < nz) {
    const T d_hy_x = h.hy - h.hy_i;  // Hy(i) - Hy(i-1)
    const T d_hx_y = h.hx - h.hx_j;  // Hx(j) - Hx(j-1)
    if (in_i && in_j) {
      T ca = c[7], cb = c[8];      // cezhx, cezhy
      if (ys >= 0) ca = mul(ca, p.cp[1].rk_e[j]);
      if (xs >= 0) cb = mul(cb, p.cp[0].rk_e[i]);
      ez = yee(c[6], ez, ca, d_hx_y, cb, d_hy_x);
      w[2] = true;
    }
    if (xs >= 0) {   // X slabs: psi_eb of XN/XP, c_psi = cezhy * dx
      const unsigned o = (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      ez = psi_step(pr.ez_x + o, pw.ez_x + o, store_psi, p.cp[0].b_e[i], p.cp[0].a_e[i], d_hy_x, mul(c[8], p.dl[0]), ez);
      w[2] = true;
    }
    if (ys >= 0) {   // Y slabs: psi_ea of YN/YP, c_psi = cezhx * dy
      const unsigned o = (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      ez = psi_step(pr.ez_y + o, pw.ez_y + o, store_psi, p.cp[1].b_e[j], p.cp[1].a_e[j], d_hx_y, mul(c[7], p.dl[1]), ez);
      w[2] = true;
    }
  }
}

// General H update of one cell: last planes and CPML slabs (H psi in place).
template <typename T, typename I>
__device__ __forceinline__ void h_general(const VolParams<T, I> &p, const T *c, int i, int j, int k,
                                          const HCurl<T> &e, T &hx, T &hy, T &hz, bool w[3]) {
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const int xs = p.cp[0].n_layers ? p.cp[0].slot_h[i] : -1;
  const int ys = p.cp[1].n_layers ? p.cp[1].slot_h[j] : -1;
  const int zs = p.cp[2].n_layers ? p.cp[2].slot_h[k] : -1;
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const unsigned nzp = static_cast<unsigned>(p.d.nzp), ny1 = static_cast<unsigned>(ny + 1);
  const Psi<T> &ps = p.psi;
  w[0] = w[1] = w[2] = false;

  // ---- Hx (nx+1, ny, nz) ----
  if (j < ny && k < nz) {
    const T d_ey_z = e.ey_k - e.ey;   // Ey(k+1) - Ey(k)
    const T d_ez_y = e.ez_j - e.ez;   // Ez(j+1) - Ez(j)
    if (i < nx) {
      T ca = c[1], cb = c[2];        // chxey, chxez
      if (zs >= 0) ca = mul(ca, p.cp[2].rk_m[k]);
      if (ys >= 0) cb = mul(cb, p.cp[1].rk_m[j]);
      hx = yee(c[0], hx, ca, d_ey_z, cb, d_ez_y);
      w[0] = true;
    }
    if (ys >= 0) {   // Y slabs: psi_hb of YN/YP, c_psi = chxez * dy
      T *q = ps.hx_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      hx = psi_step(q, q, true, p.cp[1].b_m[j], p.cp[1].a_m[j], d_ez_y, mul(c[2], p.dl[1]), hx);
      w[0] = true;
    }
    if (zs >= 0) {   // Z slabs: psi_ha of ZN/ZP, c_psi = chxey * dz
      T *q = ps.hx_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      hx = psi_step(q, q, true, p.cp[2].b_m[k], p.cp[2].a_m[k], d_ey_z, mul(c[1], p.dl[2]), hx);
      w[0] = true;
    }
  }

  // ---- Hy (nx, ny+1, nz) ----
  if (i < nx && k < nz) {
    const T d_ez_x = e.ez_i - e.ez;   // Ez(i+1) - Ez(i)
    const T d_ex_z = e.ex_k - e.ex;   // Ex(k+1) - Ex(k)
    if (j < ny) {
      T ca = c[4], cb = c[5];        // chyez, chyex
      if (xs >= 0) ca = mul(ca, p.cp[0].rk_m[i]);
      if (zs >= 0) cb = mul(cb, p.cp[2].rk_m[k]);
      hy = yee(c[3], hy, ca, d_ez_x, cb, d_ex_z);
      w[1] = true;
    }
    if (xs >= 0) {   // X slabs: psi_ha of XN/XP, c_psi = chyez * dx
      T *q = ps.hy_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      hy = psi_step(q, q, true, p.cp[0].b_m[i], p.cp[0].a_m[i], d_ez_x, mul(c[4], p.dl[0]), hy);
      w[1] = true;
    }
    if (zs >= 0) {   // Z slabs: psi_hb of ZN/ZP, c_psi = chyex * dz
      T *q = ps.hy_z + (static_cast<unsigned>(i) * ny1 + j) * Lz + zs;
      hy = psi_step(q, q, true, p.cp[2].b_m[k], p.cp[2].a_m[k], d_ex_z, mul(c[5], p.dl[2]), hy);
      w[1] = true;
    }
  }

  // ---- Hz (nx, ny, nz+1) ----
  if (i < nx && j < ny) {
    const T d_ex_y = e.ex_j - e.ex;   // Ex(j+1) - Ex(j)
    const T d_ey_x = e.ey_i - e.ey;   // Ey(i+1) - Ey(i)
    if (k < nz) {
      T ca = c[7], cb = c[8];        // chzex, chzey
      if (ys >= 0) ca = mul(ca, p.cp[1].rk_m[j]);
      if (xs >= 0) cb = mul(cb, p.cp[0].rk_m[i]);
      hz = yee(c[6], hz, ca, d_ex_y, cb, d_ey_x);
      w[2] = true;
    }
    if (xs >= 0) {   // X slabs: psi_hb of XN/XP, c_psi = chzey * dx
      T *q = ps.hz_x + (static_cast<unsigned>(xs) * ny1 + j) * nzp + k;
      hz = psi_step(q, q, true, p.cp[0].b_m[i], p.cp[0].a_m[i], d_ey_x, mul(c[8], p.dl[0]), hz);
      w[2] = true;
    }
    if (ys >= 0) {   // Y slabs: psi_ha of YN/YP, c_psi = chzex * dy
      T *q = ps.hz_y + (static_cast<unsigned>(i) * Ly + ys) * nzp + k;
      hz = psi_step(q, q, true, p.cp[1].b_m[j], p.cp[1].a_m[j], d_ex_y, mul(c[7], p.dl[1]), hz);
      w[2] = true;
    }
  }
}

// Whether cell (i, j, k) is plain for the E update (no outer wall, no CPML
// slab): then e_fast applies.  Indices are clamped to the box.
template <typename T, typename I>
__device__ __forceinline__ bool e_plain_cell(const VolParams<T, I> &p, int i, int j, int k) {
  return !((__ldg(p.flags[0] + min(i, p.d.nx)) | __ldg(p.flags[1] + min(j, p.d.ny)) | __ldg(p.flags[2] + min(k, p.d.nz))) &
           kSpecialE);
}
template <typename T, typename I>
__device__ __forceinline__ bool h_plain_cell(const VolParams<T, I> &p, int i, int j, int k) {
  return !((__ldg(p.flags[0] + min(i, p.d.nx)) | __ldg(p.flags[1] + min(j, p.d.ny)) | __ldg(p.flags[2] + min(k, p.d.nz))) &
           kSpecialH);
}

// E update of one cell by the general path.  It serves any cell: a plain
// cell gets the bits of the fast path (same expressions, no CPML terms).
// The volume kernels decide per warp: a warp whose cells are not all plain
// runs this path for all of them, so that no warp runs both paths.
template <typename T, typename I>
__device__ __forceinline__ void e_cell_general(const VolParams<T, I> &p, const T *tab, int ts, int i, int j, int k) {
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
  h.hx_k = k > 0 ? __ldg(Hx + b - 1) : T(0);
  h.hy_k = k > 0 ? __ldg(Hy + b - 1) : T(0);
  h.hx_j = j > 0 ? __ldg(Hx + b - usj) : T(0);
  h.hz_j = j > 0 ? __ldg(Hz + b - usj) : T(0);
  h.hy_i = i > 0 ? __ldg(Hy + b - usi) : T(0);
  h.hz_i = i > 0 ? __ldg(Hz + b - usi) : T(0);
  const T *c = tab + static_cast<unsigned>(__ldg(p.idx + b)) * ts;
  T ex = Ex[b], ey = Ey[b], ez = Ez[b];
  bool w[3];
  e_general<T, I, false>(p, c, i, j, k, h, p.psi, p.psi, true, ex, ey, ez, w);
  if (w[0]) Ex[b] = ex;
  if (w[1]) Ey[b] = ey;
  if (w[2]) Ez[b] = ez;
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
    const ECurl<T> h{hx[q], hy[q + 1], hz[q + 1], hx_k[q], hy_k[q], hx_j[q], hz_j[q], hy[q], hz[q]};
    e_plain(c[q], h, ex[q], ey[q], ez[q]);
    Ex[b] = ex[q];
    Ey[b] = ey[q];
    Ez[b] = ez[q];
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
  const bool valid = k <= p.d.nz && j <= p.d.ny && i0 <= p.d.nx;
  bool plain = valid && i0 + NC - 1 <= p.d.nx;
#pragma unroll
  for (int q = 0; q < NC; ++q) plain = plain && e_plain_cell(p, i0 + q, j, k);
  // one path per warp (blockDim.x is a multiple of 32: a warp is one row)
  const bool fast = __all_sync(0xffffffffu, plain || !valid);
  if (!valid) return;
  if (fast) {
    e_fast<T, I, NC>(p, tab, ts, i0, j, k);
    return;
  }
#pragma unroll
  for (int q = 0; q < NC; ++q)
    if (i0 + q <= p.d.nx) e_cell_general<T, I>(p, tab, ts, i0 + q, j, k);
}

// H update of one cell by the general path (any cell, as e_cell_general).
template <typename T, typename I>
__device__ __forceinline__ void h_cell_general(const VolParams<T, I> &p, const T *tab, int ts, int i, int j, int k) {
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
  e.ey_i = i < nx ? __ldg(Ey + b + usi) : T(0);
  e.ez_i = i < nx ? __ldg(Ez + b + usi) : T(0);
  e.ex_k = k < nz ? __ldg(Ex + b + 1) : T(0);
  e.ey_k = k < nz ? __ldg(Ey + b + 1) : T(0);
  e.ex_j = j < ny ? __ldg(Ex + b + usj) : T(0);
  e.ez_j = j < ny ? __ldg(Ez + b + usj) : T(0);
  const T *c = tab + static_cast<unsigned>(__ldg(p.idx + b)) * ts;
  T hx = Hx[b], hy = Hy[b], hz = Hz[b];
  bool w[3];
  h_general(p, c, i, j, k, e, hx, hy, hz, w);
  if (w[0]) Hx[b] = hx;
  if (w[1]) Hy[b] = hy;
  if (w[2]) Hz[b] = hz;
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
    const HCurl<T> e{ex[q], ey[q], ez[q], ex_kp[q], ey_kp[q], ex_jp[q], ez_jp[q], ey[q + 1], ez[q + 1]};
    h_plain(c[q], e, hx[q], hy[q], hz[q]);
    Hx[b] = hx[q];
    Hy[b] = hy[q];
    Hz[b] = hz[q];
  }
}

template <typename T, typename I, bool SMEM_TABLE, int MINB, int NC>
__global__ void __launch_bounds__(256, MINB) k_update_h(VolParams<T, I> p) {
  int ts;
  const T *tab = load_table<T, I, SMEM_TABLE>(p, 1, ts);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i0 = (blockIdx.z * blockDim.z + threadIdx.z) * NC;
  const bool valid = k <= p.d.nz && j <= p.d.ny && i0 <= p.d.nx;
  bool plain = valid && i0 + NC - 1 <= p.d.nx;
#pragma unroll
  for (int q = 0; q < NC; ++q) plain = plain && h_plain_cell(p, i0 + q, j, k);
  const bool fast = __all_sync(0xffffffffu, plain || !valid);
  if (!valid) return;
  if (fast) {
    h_fast<T, I, NC>(p, tab, ts, i0, j, k);
    return;
  }
#pragma unroll
  for (int q = 0; q < NC; ++q)
    if (i0 + q <= p.d.nx) h_cell_general<T, I>(p, tab, ts, i0 + q, j, k);
}

}  // namespace xg
