// volume.cuh -- the fused Yee E and H kernels.
//
// One thread per cell (i, j, k) of the (nx+1)(ny+1)(nz+1) box, k on the
// fastest thread axis so that a warp reads 32 contiguous values.  The
// curl operands are read-only during the kernel (H in the E kernel, E in the
// H kernel), so they go through the read-only data path; neighbours along
// k and j hit L1, neighbours along i (another block) hit L2.  Per cell the
// kernel applies, in the reference's order:
//
//   E:  updateE main update          src/simulation/simulation_update.cpp:170-196
//       TFSF3D::updateE faces        src/tfsf/tfsf_3d.cpp:299-411
//       PML::updateE psi recursions  src/boundary/perfect_match_layer.cpp:574-718
//   H:  updateH main update          src/simulation/simulation_update.cpp:84-100
//       TFSF3D::updateH faces        src/tfsf/tfsf_3d.cpp:185-297
//       PML::updateH psi recursions  src/boundary/perfect_match_layer.cpp:434-572
//
// The update coefficients come from the material table (18 per entry,
// FDTDBasicCoff::initCoff, src/fdtd_basic_coff/fdtd_basic_coff.cpp:77-121),
// multiplied by 1/kappa inside CPML slabs (perfect_match_layer.cpp:190-206,
// 342-358).  The CPML's c_psi = coefficient * dl (same lines) is formed from
// the table entry as well.  Main updates skip the outer walls exactly where
// the reference's loops do; psi terms cover the full transverse extent of the
// component, walls included, as the reference's PML loops do.
#pragma once

#include "common.cuh"

namespace xg {

template <typename T>
__device__ __forceinline__ void add_corr(T &v, double corr) {
  v = static_cast<T>(static_cast<double>(v) + corr);
}

// MINB: minimum resident blocks per SM requested from the register
// allocator (1 = no cap); the autotuner in engine.cu picks it per plan.
template <typename T, typename I, bool SMEM_TABLE, int MINB>
__global__ void __launch_bounds__(256, MINB) k_update_e(VolParams<T, I> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const T *tab = p.table;
  int ts = 18;
  if (SMEM_TABLE) {
    T *st = reinterpret_cast<T *>(smem_raw);
    const int nt = blockDim.x * blockDim.y * blockDim.z;
    const int tid = (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x;
    for (int q = tid; q < p.n_mat * 9; q += nt) st[q] = p.table[(q / 9) * 18 + (q % 9)];
    __syncthreads();
    tab = st;
    ts = 9;
  }
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z * blockDim.z + threadIdx.z;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  if (k > nz || j > ny || i > nx) return;
  const long long si = p.d.si, sj = p.d.sj;
  const T *__restrict__ Hx = p.H[0];
  const T *__restrict__ Hy = p.H[1];
  const T *__restrict__ Hz = p.H[2];

  // CPML data for the y and z axes (E-located indices).
  const int ys = p.cp[1].n_layers ? p.cp[1].slot_e[j] : -1;
  const int zs = p.cp[2].n_layers ? p.cp[2].slot_e[k] : -1;
  T by = 0, ay = 0, rky = 1, bz = 0, az = 0, rkz = 1;
  if (ys >= 0) { by = p.cp[1].b_e[j]; ay = p.cp[1].a_e[j]; rky = p.cp[1].rk_e[j]; }
  if (zs >= 0) { bz = p.cp[2].b_e[k]; az = p.cp[2].a_e[k]; rkz = p.cp[2].rk_e[k]; }
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;
  const bool in_j = j >= 1 && j < ny, in_k = k >= 1 && k < nz;

  // TFSF faces (E side) for this column.
  const TfsfDev &tf = p.tf;
  long long t = 0;
  const double *hinc = nullptr;
  if (tf.enabled) {
    t = *p.step;
    hinc = tf.inc + ((t + 1) & 1) * 6 * tf.L;   // incident H of the previous step
  }

  const long long b = static_cast<long long>(i) * si + static_cast<long long>(j) * sj + k;
  {
    const T hx = __ldg(Hx + b), hy = __ldg(Hy + b), hz = __ldg(Hz + b);
    const T hx_k = k > 0 ? __ldg(Hx + b - 1) : T(0);
    const T hy_k = k > 0 ? __ldg(Hy + b - 1) : T(0);
    const T hx_j = j > 0 ? __ldg(Hx + b - sj) : T(0);
    const T hz_j = j > 0 ? __ldg(Hz + b - sj) : T(0);
    const T hy_im1 = i > 0 ? __ldg(Hy + b - si) : T(0);
    const T hz_im1 = i > 0 ? __ldg(Hz + b - si) : T(0);
    const T *c = tab + static_cast<long long>(__ldg(p.idx + b)) * ts;
    const int xs = p.cp[0].n_layers ? p.cp[0].slot_e[i] : -1;
    T bx = 0, ax = 0, rkx = 1;
    if (xs >= 0) { bx = p.cp[0].b_e[i]; ax = p.cp[0].a_e[i]; rkx = p.cp[0].rk_e[i]; }
    const bool in_i = i >= 1 && i < nx;

    // ---- Ex (nx, ny+1, nz+1) ----
    if (i < nx) {
      const T d_hz_y = hz - hz_j;   // Hz(j) - Hz(j-1)
      const T d_hy_z = hy - hy_k;   // Hy(k) - Hy(k-1)
      T e = p.E[0][b];
      bool w = false;
      if (in_j && in_k) {
        T ca = c[1], cb = c[2];
        if (zs >= 0) ca *= rkz;
        if (ys >= 0) cb *= rky;
        e = c[0] * e + ca * d_hy_z + cb * d_hz_y;
        w = true;
      }
      if (tf.enabled) {
        const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
        if ((j == lj || j == rj) && k >= lk && k <= rk && i >= li && i < ri) {
          const int jj = j == lj ? lj - 1 : rj;   // Hz_inc(i, lj-1, k) / Hz_inc(i, rj, k)
          const double pr = tf.ph[0][i - li + 1] + tf.ph[1][jj - lj + 1] + tf.pf[2][k - lk] - 0.5;
          const double v = tf.ca[1] * tfsf_interp(hinc + 5 * tf.L, pr);
          add_corr(e, j == lj ? -v : v);
          w = true;
        }
        if ((k == lk || k == rk) && i >= li && i < ri && j >= lj && j <= rj) {
          const int kk = k == lk ? lk - 1 : rk;   // Hy_inc(i, j, lk-1) / Hy_inc(i, j, rk)
          const double pr = tf.ph[0][i - li + 1] + tf.pf[1][j - lj] + tf.ph[2][kk - lk + 1] - 0.5;
          const double v = tf.ca[2] * tfsf_interp(hinc + 4 * tf.L, pr);
          add_corr(e, k == lk ? v : -v);
          w = true;
        }
      }
      if (ys >= 0) {   // Y slabs: psi_eb of YN/YP, c_psi = cexhz * dy
        T *ps = p.psi.ex_y + (static_cast<long long>(i) * Ly + ys) * p.d.nzp + k;
        const T s = by * (*ps) + ay * d_hz_y;
        *ps = s;
        e = e + (c[2] * p.dl[1]) * s;
        w = true;
      }
      if (zs >= 0) {   // Z slabs: psi_ea of ZN/ZP, c_psi = cexhy * dz
        T *ps = p.psi.ex_z + (static_cast<long long>(i) * (ny + 1) + j) * Lz + zs;
        const T s = bz * (*ps) + az * d_hy_z;
        *ps = s;
        e = e + (c[1] * p.dl[2]) * s;
        w = true;
      }
      if (w) p.E[0][b] = e;
    }

    // ---- Ey (nx+1, ny, nz+1) ----
    if (j < ny) {
      const T d_hz_x = hz - hz_im1;  // Hz(i) - Hz(i-1)
      const T d_hx_z = hx - hx_k;    // Hx(k) - Hx(k-1)
      T e = p.E[1][b];
      bool w = false;
      if (in_i && in_k) {
        T ca = c[5], cb = c[4];      // ceyhx, ceyhz
        if (zs >= 0) ca *= rkz;
        if (xs >= 0) cb *= rkx;
        e = c[3] * e + ca * d_hx_z + cb * d_hz_x;
        w = true;
      }
      if (tf.enabled) {
        const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
        if ((i == li || i == ri) && j >= lj && j < rj && k >= lk && k <= rk) {
          const int ii = i == li ? li - 1 : ri;   // Hz_inc(li-1, j, k) / Hz_inc(ri, j, k)
          const double pr = tf.ph[0][ii - li + 1] + tf.ph[1][j - lj + 1] + tf.pf[2][k - lk] - 0.5;
          const double v = tf.ca[0] * tfsf_interp(hinc + 5 * tf.L, pr);
          add_corr(e, i == li ? v : -v);
          w = true;
        }
        if ((k == lk || k == rk) && i >= li && i <= ri && j >= lj && j < rj) {
          const int kk = k == lk ? lk - 1 : rk;   // Hx_inc(i, j, lk-1) / Hx_inc(i, j, rk)
          const double pr = tf.pf[0][i - li] + tf.ph[1][j - lj + 1] + tf.ph[2][kk - lk + 1] - 0.5;
          const double v = tf.ca[2] * tfsf_interp(hinc + 3 * tf.L, pr);
          add_corr(e, k == lk ? -v : v);
          w = true;
        }
      }
      if (xs >= 0) {   // X slabs: psi_ea of XN/XP, c_psi = ceyhz * dx
        T *ps = p.psi.ey_x + (static_cast<long long>(xs) * (ny + 1) + j) * p.d.nzp + k;
        const T s = bx * (*ps) + ax * d_hz_x;
        *ps = s;
        e = e + (c[4] * p.dl[0]) * s;
        w = true;
      }
      if (zs >= 0) {   // Z slabs: psi_eb of ZN/ZP, c_psi = ceyhx * dz
        T *ps = p.psi.ey_z + (static_cast<long long>(i) * (ny + 1) + j) * Lz + zs;
        const T s = bz * (*ps) + az * d_hx_z;
        *ps = s;
        e = e + (c[5] * p.dl[2]) * s;
        w = true;
      }
      if (w) p.E[1][b] = e;
    }

    // ---- Ez (nx+1, ny+1, nz) ----
    if (k < nz) {
      const T d_hy_x = hy - hy_im1;  // Hy(i) - Hy(i-1)
      const T d_hx_y = hx - hx_j;    // Hx(j) - Hx(j-1)
      T e = p.E[2][b];
      bool w = false;
      if (in_i && in_j) {
        T ca = c[7], cb = c[8];      // cezhx, cezhy
        if (ys >= 0) ca *= rky;
        if (xs >= 0) cb *= rkx;
        e = c[6] * e + ca * d_hx_y + cb * d_hy_x;
        w = true;
      }
      if (tf.enabled) {
        const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
        if ((i == li || i == ri) && j >= lj && j <= rj && k >= lk && k < rk) {
          const int ii = i == li ? li - 1 : ri;   // Hy_inc(li-1, j, k) / Hy_inc(ri, j, k)
          const double pr = tf.ph[0][ii - li + 1] + tf.pf[1][j - lj] + tf.ph[2][k - lk + 1] - 0.5;
          const double v = tf.ca[0] * tfsf_interp(hinc + 4 * tf.L, pr);
          add_corr(e, i == li ? -v : v);
          w = true;
        }
        if ((j == lj || j == rj) && k >= lk && k < rk && i >= li && i <= ri) {
          const int jj = j == lj ? lj - 1 : rj;   // Hx_inc(i, lj-1, k) / Hx_inc(i, rj, k)
          const double pr = tf.pf[0][i - li] + tf.ph[1][jj - lj + 1] + tf.ph[2][k - lk + 1] - 0.5;
          const double v = tf.ca[1] * tfsf_interp(hinc + 3 * tf.L, pr);
          add_corr(e, j == lj ? v : -v);
          w = true;
        }
      }
      if (xs >= 0) {   // X slabs: psi_eb of XN/XP, c_psi = cezhy * dx
        T *ps = p.psi.ez_x + (static_cast<long long>(xs) * (ny + 1) + j) * p.d.nzp + k;
        const T s = bx * (*ps) + ax * d_hy_x;
        *ps = s;
        e = e + (c[8] * p.dl[0]) * s;
        w = true;
      }
      if (ys >= 0) {   // Y slabs: psi_ea of YN/YP, c_psi = cezhx * dy
        T *ps = p.psi.ez_y + (static_cast<long long>(i) * Ly + ys) * p.d.nzp + k;
        const T s = by * (*ps) + ay * d_hx_y;
        *ps = s;
        e = e + (c[7] * p.dl[1]) * s;
        w = true;
      }
      if (w) p.E[2][b] = e;
    }
  }
}

template <typename T, typename I, bool SMEM_TABLE, int MINB>
__global__ void __launch_bounds__(256, MINB) k_update_h(VolParams<T, I> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const T *tab = p.table + 9;
  int ts = 18;
  if (SMEM_TABLE) {
    T *st = reinterpret_cast<T *>(smem_raw);
    const int nt = blockDim.x * blockDim.y * blockDim.z;
    const int tid = (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x;
    for (int q = tid; q < p.n_mat * 9; q += nt) st[q] = p.table[(q / 9) * 18 + 9 + (q % 9)];
    __syncthreads();
    tab = st;
    ts = 9;
  }
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z * blockDim.z + threadIdx.z;
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  if (k > nz || j > ny || i > nx) return;
  const long long si = p.d.si, sj = p.d.sj;
  const T *__restrict__ Ex = p.E[0];
  const T *__restrict__ Ey = p.E[1];
  const T *__restrict__ Ez = p.E[2];

  const int ys = p.cp[1].n_layers ? p.cp[1].slot_h[j] : -1;
  const int zs = p.cp[2].n_layers ? p.cp[2].slot_h[k] : -1;
  T by = 0, ay = 0, rky = 1, bz = 0, az = 0, rkz = 1;
  if (ys >= 0) { by = p.cp[1].b_m[j]; ay = p.cp[1].a_m[j]; rky = p.cp[1].rk_m[j]; }
  if (zs >= 0) { bz = p.cp[2].b_m[k]; az = p.cp[2].a_m[k]; rkz = p.cp[2].rk_m[k]; }
  const int Ly = p.cp[1].n_layers, Lz = p.cp[2].n_layers;

  const TfsfDev &tf = p.tf;
  const double *einc = nullptr;
  if (tf.enabled) einc = tf.inc + ((*p.step) & 1) * 6 * tf.L;   // incident E of this step

  const long long b = static_cast<long long>(i) * si + static_cast<long long>(j) * sj + k;
  {
    const T ex = __ldg(Ex + b), ey_i = __ldg(Ey + b), ez_i = __ldg(Ez + b);
    const T ey_ip = i < nx ? __ldg(Ey + b + si) : T(0);
    const T ez_ip = i < nx ? __ldg(Ez + b + si) : T(0);
    const T ex_kp = k < nz ? __ldg(Ex + b + 1) : T(0);
    const T ey_kp = k < nz ? __ldg(Ey + b + 1) : T(0);
    const T ex_jp = j < ny ? __ldg(Ex + b + sj) : T(0);
    const T ez_jp = j < ny ? __ldg(Ez + b + sj) : T(0);
    const T *c = tab + static_cast<long long>(__ldg(p.idx + b)) * ts;
    const int xs = p.cp[0].n_layers ? p.cp[0].slot_h[i] : -1;
    T bx = 0, ax = 0, rkx = 1;
    if (xs >= 0) { bx = p.cp[0].b_m[i]; ax = p.cp[0].a_m[i]; rkx = p.cp[0].rk_m[i]; }

    // ---- Hx (nx+1, ny, nz) ----
    if (j < ny && k < nz) {
      const T d_ey_z = ey_kp - ey_i;   // Ey(k+1) - Ey(k)
      const T d_ez_y = ez_jp - ez_i;   // Ez(j+1) - Ez(j)
      T h = p.H[0][b];
      bool w = false;
      if (i < nx) {
        T ca = c[1], cb = c[2];        // chxey, chxez
        if (zs >= 0) ca *= rkz;
        if (ys >= 0) cb *= rky;
        h = c[0] * h + ca * d_ey_z + cb * d_ez_y;
        w = true;
      }
      if (tf.enabled) {
        const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
        if ((j == lj - 1 || j == rj) && k >= lk && k < rk && i >= li && i <= ri) {
          const int jj = j == rj ? rj : lj;   // Ez_inc(i, lj, k) / Ez_inc(i, rj, k)
          const double pr = tf.pf[0][i - li] + tf.pf[1][jj - lj] + tf.ph[2][k - lk + 1];
          const double v = tf.cb[1] * tfsf_interp(einc + 2 * tf.L, pr);
          add_corr(h, j == rj ? -v : v);
          w = true;
        }
        if ((k == lk - 1 || k == rk) && i >= li && i <= ri && j >= lj && j < rj) {
          const int kk = k == rk ? rk : lk;   // Ey_inc(i, j, lk) / Ey_inc(i, j, rk)
          const double pr = tf.pf[0][i - li] + tf.ph[1][j - lj + 1] + tf.pf[2][kk - lk];
          const double v = tf.cb[2] * tfsf_interp(einc + 1 * tf.L, pr);
          add_corr(h, k == rk ? v : -v);
          w = true;
        }
      }
      if (ys >= 0) {   // Y slabs: psi_hb of YN/YP, c_psi = chxez * dy
        T *ps = p.psi.hx_y + (static_cast<long long>(i) * Ly + ys) * p.d.nzp + k;
        const T s = by * (*ps) + ay * d_ez_y;
        *ps = s;
        h = h + (c[2] * p.dl[1]) * s;
        w = true;
      }
      if (zs >= 0) {   // Z slabs: psi_ha of ZN/ZP, c_psi = chxey * dz
        T *ps = p.psi.hx_z + (static_cast<long long>(i) * (ny + 1) + j) * Lz + zs;
        const T s = bz * (*ps) + az * d_ey_z;
        *ps = s;
        h = h + (c[1] * p.dl[2]) * s;
        w = true;
      }
      if (w) p.H[0][b] = h;
    }

    // ---- Hy (nx, ny+1, nz) ----
    if (i < nx && k < nz) {
      const T d_ez_x = ez_ip - ez_i;   // Ez(i+1) - Ez(i)
      const T d_ex_z = ex_kp - ex;     // Ex(k+1) - Ex(k)
      T h = p.H[1][b];
      bool w = false;
      if (j < ny) {
        T ca = c[4], cb = c[5];        // chyez, chyex
        if (xs >= 0) ca *= rkx;
        if (zs >= 0) cb *= rkz;
        h = c[3] * h + ca * d_ez_x + cb * d_ex_z;
        w = true;
      }
      if (tf.enabled) {
        const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
        if ((i == li - 1 || i == ri) && j >= lj && j <= rj && k >= lk && k < rk) {
          const int ii = i == ri ? ri : li;   // Ez_inc(li, j, k) / Ez_inc(ri, j, k)
          const double pr = tf.pf[0][ii - li] + tf.pf[1][j - lj] + tf.ph[2][k - lk + 1];
          const double v = tf.cb[0] * tfsf_interp(einc + 2 * tf.L, pr);
          add_corr(h, i == ri ? v : -v);
          w = true;
        }
        if ((k == lk - 1 || k == rk) && i >= li && i < ri && j >= lj && j <= rj) {
          const int kk = k == rk ? rk : lk;   // Ex_inc(i, j, lk) / Ex_inc(i, j, rk)
          const double pr = tf.ph[0][i - li + 1] + tf.pf[1][j - lj] + tf.pf[2][kk - lk];
          const double v = tf.cb[2] * tfsf_interp(einc + 0 * tf.L, pr);
          add_corr(h, k == rk ? -v : v);
          w = true;
        }
      }
      if (xs >= 0) {   // X slabs: psi_ha of XN/XP, c_psi = chyez * dx
        T *ps = p.psi.hy_x + (static_cast<long long>(xs) * (ny + 1) + j) * p.d.nzp + k;
        const T s = bx * (*ps) + ax * d_ez_x;
        *ps = s;
        h = h + (c[4] * p.dl[0]) * s;
        w = true;
      }
      if (zs >= 0) {   // Z slabs: psi_hb of ZN/ZP, c_psi = chyex * dz
        T *ps = p.psi.hy_z + (static_cast<long long>(i) * (ny + 1) + j) * Lz + zs;
        const T s = bz * (*ps) + az * d_ex_z;
        *ps = s;
        h = h + (c[5] * p.dl[2]) * s;
        w = true;
      }
      if (w) p.H[1][b] = h;
    }

    // ---- Hz (nx, ny, nz+1) ----
    if (i < nx && j < ny) {
      const T d_ex_y = ex_jp - ex;     // Ex(j+1) - Ex(j)
      const T d_ey_x = ey_ip - ey_i;   // Ey(i+1) - Ey(i)
      T h = p.H[2][b];
      bool w = false;
      if (k < nz) {
        T ca = c[7], cb = c[8];        // chzex, chzey
        if (ys >= 0) ca *= rky;
        if (xs >= 0) cb *= rkx;
        h = c[6] * h + ca * d_ex_y + cb * d_ey_x;
        w = true;
      }
      if (tf.enabled) {
        const int li = tf.lo[0], ri = tf.hi[0], lj = tf.lo[1], rj = tf.hi[1], lk = tf.lo[2], rk = tf.hi[2];
        if ((i == li - 1 || i == ri) && j >= lj && j < rj && k >= lk && k <= rk) {
          const int ii = i == ri ? ri : li;   // Ey_inc(li, j, k) / Ey_inc(ri, j, k)
          const double pr = tf.pf[0][ii - li] + tf.ph[1][j - lj + 1] + tf.pf[2][k - lk];
          const double v = tf.cb[0] * tfsf_interp(einc + 1 * tf.L, pr);
          add_corr(h, i == ri ? -v : v);
          w = true;
        }
        if ((j == lj - 1 || j == rj) && k >= lk && k <= rk && i >= li && i < ri) {
          const int jj = j == rj ? rj : lj;   // Ex_inc(i, lj, k) / Ex_inc(i, rj, k)
          const double pr = tf.ph[0][i - li + 1] + tf.pf[1][jj - lj] + tf.pf[2][k - lk];
          const double v = tf.cb[1] * tfsf_interp(einc + 0 * tf.L, pr);
          add_corr(h, j == rj ? v : -v);
          w = true;
        }
      }
      if (xs >= 0) {   // X slabs: psi_hb of XN/XP, c_psi = chzey * dx
        T *ps = p.psi.hz_x + (static_cast<long long>(xs) * (ny + 1) + j) * p.d.nzp + k;
        const T s = bx * (*ps) + ax * d_ey_x;
        *ps = s;
        h = h + (c[8] * p.dl[0]) * s;
        w = true;
      }
      if (ys >= 0) {   // Y slabs: psi_ha of YN/YP, c_psi = chzex * dy
        T *ps = p.psi.hz_y + (static_cast<long long>(i) * Ly + ys) * p.d.nzp + k;
        const T s = by * (*ps) + ay * d_ex_y;
        *ps = s;
        h = h + (c[7] * p.dl[1]) * s;
        w = true;
      }
      if (w) p.H[2][b] = h;
    }
  }
}

}  // namespace xg
