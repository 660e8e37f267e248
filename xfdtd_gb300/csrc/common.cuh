// common.cuh -- device-side data layout shared by the engine's kernels.
//
// Fields live in one uniform padded box per component: (nx+1) x (ny+1) x NZP
// with NZP = nz+1 rounded up to 32 (4 on the 2-D grid, nz = 1), i.e. index
// (i*(ny+1) + j)*NZP + k.  Every
// component of the reference (Ex (nx,ny+1,nz+1) ... Hz (nx,ny,nz+1),
// src/simulation/simulation_init.cpp:28-35) fits in that box at the same
// (i, j, k); the cells a component does not have stay zero and are never
// written.  k is the contiguous axis, so a warp reads 128 contiguous bytes
// (FP32) of one row.
#pragma once

#include <cstdint>

namespace xg {

struct Dims {
  int nx, ny, nz;
  int nzp;            // padded row length
  long long sj, si;   // strides of j and i
  long long cells;    // (nx+1)*(ny+1)*nzp
};

// CPML profile along one axis (device copy of xfdtd_cpml_axis).
template <typename T>
struct CpmlAxis {
  int n_layers;
  const int *slot_e, *slot_h;
  const T *b_e, *a_e, *rk_e;
  const T *b_m, *a_m, *rk_m;
};

// TFSF surface data.  inc holds two buffers (step parity) of the projected
// incident arrays ex, ey, ez (aux_len each) and hx, hy, hz (aux_len-1 each,
// stored with stride aux_len).
struct TfsfDev {
  int enabled;
  int two_d;   // TFSF2D (src/tfsf/tfsf_2d.cpp:150-228): Ez on the x and y faces, Hy on the x faces,
               // Hx on the y faces; the z projection tables are zero
  int L;
  int lo[3], hi[3];
  const double *pf[3], *ph[3];
  double ca[3], cb[3];
  const double *inc;   // [2][6][L]
  // the same tables in FP32 (FP32 form): projections, coefficients and the
  // incident arrays (written by the 1-D line beside the FP64 ones)
  const float *pff[3], *phf[3];
  float caf[3], cbf[3];
  const float *incf;   // [2][6][L]
};

// The TFSF tables in the arithmetic of the field precision T: FP64 (the
// reference's) for FP64 fields, FP32 for the FP32 form.
template <typename R>
struct TfsfView {
  const R *pf[3], *ph[3];
  R ca[3], cb[3];
  const R *inc;
};
template <typename T>
__device__ __forceinline__ auto tfsf_view(const TfsfDev &tf) {
  if constexpr (sizeof(T) == 8) {
    return TfsfView<double>{{tf.pf[0], tf.pf[1], tf.pf[2]}, {tf.ph[0], tf.ph[1], tf.ph[2]},
                            {tf.ca[0], tf.ca[1], tf.ca[2]}, {tf.cb[0], tf.cb[1], tf.cb[2]}, tf.inc};
  } else {
    return TfsfView<float>{{tf.pff[0], tf.pff[1], tf.pff[2]}, {tf.phf[0], tf.phf[1], tf.phf[2]},
                           {tf.caf[0], tf.caf[1], tf.caf[2]}, {tf.cbf[0], tf.cbf[1], tf.cbf[2]}, tf.incf};
  }
}

// psi storage: axis X (L, ny+1, nzp), axis Y (nx+1, L, nzp), axis Z (nx+1, ny+1, L).
template <typename T>
struct Psi {
  T *ex_y, *ex_z, *ey_x, *ey_z, *ez_x, *ez_y;   // E recursions
  T *hx_y, *hx_z, *hy_x, *hy_z, *hz_x, *hz_y;   // H recursions
};

// What the volume updates read: fields, material index and table, CPML.
template <typename T, typename I>
struct VolCore {
  Dims d;
  T *E[3];
  T *H[3];
  const I *idx;
  const T *table;      // [n_mat][18], reference coefficient order
  const T *ctable;     // [n_mat][2][4]: compact table (compact_coefs)
  int n_mat;
  CpmlAxis<T> cp[3];
  Psi<T> psi;
  T dl[3];
};

// VolCore plus what the fused sweep and the adjoint also need.
template <typename T, typename I>
struct VolParams : VolCore<T, I> {
  TfsfDev tf;
  const long long *step;
  const uint8_t *flags[3];   // per-axis index flags (kSpecialE / kSpecialH)
};

// Index flags: an index needs the general per-cell path of the E (H) kernel
// when it is an outer wall, lies in a CPML slab or on a TFSF face plane of
// that side; a cell whose three indices carry no flag takes the fast path.
constexpr uint8_t kSpecialE = 1;
constexpr uint8_t kSpecialH = 2;
// An index on a TFSF face plane (lo or hi of that axis): the fused sweep
// applies the TFSF E corrections to cells with this flag on any axis.
constexpr uint8_t kTfsfE = 4;

__device__ __forceinline__ double tfsf_interp(const double *v, double projection) {
  // TFSF3D::getIncident*, src/tfsf/tfsf_3d.cpp:413-483
  const unsigned long long index = static_cast<unsigned long long>(projection);
  const double weight = projection - static_cast<double>(index);
  return (1 - weight) * v[index] + weight * v[index + 1];
}
__device__ __forceinline__ float tfsf_interp(const float *v, float projection) {
  const int index = static_cast<int>(projection);
  const float weight = projection - static_cast<float>(index);
  return (1 - weight) * v[index] + weight * v[index + 1];
}

}  // namespace xg
