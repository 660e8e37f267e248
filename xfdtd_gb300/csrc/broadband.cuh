// broadband.cuh -- the far field of NffftBroadBand (src/nffft/nffft_broadband.cpp)
// from the surface samples of every step.
//
// The engine keeps each step's 24 surface sample arrays (the same face-centre
// values as NffftFd, nffft_sampling in surface.cuh) for all steps.  At the
// end of the run each series x_c(t) (t < T, zero-padded to N = 2T-1 points)
// is transformed by a batched complex FFT (cuFFT), and for each output bin m
// (the fftshifted spectrum, bin frequency taken from linspace(-fs/2, fs/2,
// N) as the reference does, calculateFarField :346-348) the series are
// summed with the phase of their cell's path delay (calculateLNXYZ /
// calculateAuxiliary :374-464):
//   A[m] += ds * exp(i * delay_c * k_m) * X_c[(m + (N+1)/2) mod N]
// into the six auxiliary arrays n_x, n_y, n_z, l_x, l_y, l_z.
#pragma once

#include <cuComplex.h>

#include "common.cuh"

namespace xg {

// One chunk of series of one (face pair, quantity): series b of the chunk
// is cell c0 + b of the face plane; samples at buf[(t * 8 + q) * plane + c].
template <typename T>
__global__ void k_bb_load(const T *buf, int q, long long plane, long long c0, int nb, long long steps, long long n,
                          double2 *out) {
  const long long total = static_cast<long long>(nb) * n;
  for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long b = e / n, t = e - b * n;
    const double v = t < steps ? static_cast<double>(buf[(t * 8 + q) * plane + c0 + b]) : 0.0;
    out[e] = make_double2(v, 0.0);
  }
}

struct BbChunk {
  int group;              // 0 X faces, 1 Y faces, 2 Z faces
  int side;               // 0 the low face, 1 the high face
  long long c0;           // first cell of the chunk
  int nb;                 // series in the chunk
  int du;                 // cells along the plane's fast axis
  double face_coord;      // the face's own axis coordinate minus the centre
  double off_v, off_u;    // slow / fast axis index offsets (lo + 0.5 - centre)
  double ds;
  double dir[3];          // far-field direction (sin t cos p, sin t sin p, cos t)
  double dl[3];           // cell size per axis
  double fs, n;           // sample rate, number of bins
  double pi, c_0;
};

// One block per output bin m: the chunk's series summed with their delay
// phase into acc[m] (a single writer per bin and chunk: deterministic).
__global__ void k_bb_phase_sum(BbChunk c, const double2 *spec, double2 *acc) {
  const long long N = static_cast<long long>(c.n);
  const long long m = blockIdx.x;
  // linspace(-fs/2, fs/2, N) and k = 2 pi f / c0 (nffft_broadband.cpp:346-347)
  const double step = (c.fs / 2 - (-c.fs / 2)) / (c.n - 1);
  const double f = -c.fs / 2 + step * static_cast<double>(m);
  const double k = 2 * c.pi * f / c.c_0;
  const long long src = (m + (N + 1) / 2) % N;   // fftshift, odd N
  double re = 0.0, im = 0.0;
  for (int b = threadIdx.x; b < c.nb; b += blockDim.x) {
    const long long cell = c.c0 + b;
    const double v = static_cast<double>(cell / c.du) + c.off_v, u = static_cast<double>(cell % c.du) + c.off_u;
    // the delay: x_r + y_r + z_r of the face's meshgrid (:383-396)
    double x, y, z;
    if (c.group == 0) x = c.face_coord, y = v, z = u;
    else if (c.group == 1) x = v, y = c.face_coord, z = u;
    else x = v, y = u, z = c.face_coord;
    const double delay = x * c.dir[0] * c.dl[0] + y * c.dir[1] * c.dl[1] + z * c.dir[2] * c.dl[2];
    double s, co;
    sincos(delay * k, &s, &co);
    const double2 X = spec[static_cast<long long>(b) * N + src];
    // ds * phase * X
    const double pr = c.ds * co, pi = c.ds * s;
    re += pr * X.x - pi * X.y;
    im += pr * X.y + pi * X.x;
  }
  __shared__ double sr[256], si[256];
  sr[threadIdx.x] = re;
  si[threadIdx.x] = im;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sr[threadIdx.x] += sr[threadIdx.x + w];
      si[threadIdx.x] += si[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    acc[m].x += sr[0];
    acc[m].y += si[0];
  }
}

}  // namespace xg
