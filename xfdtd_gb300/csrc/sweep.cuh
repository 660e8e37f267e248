// sweep.cuh -- one kernel per step for the E and H volume updates.
//
// The split kernels (volume.cuh) read every field twice per step: the E
// kernel reads E and H and writes E, the H kernel reads E and H again and
// writes H.  The sweep does both in one pass: a block owns a tile of 8 rows
// (j) x 32 cells (k) and marches along i through a chunk of planes.  At
// plane i it computes E(t+1) of plane i, then H(t+1) of plane i-1, which
// needs E(t+1) of planes i-1 and i -- both still in shared memory.  Per cell
// and step the fields cross HBM once each way: 6 reads + 6 writes + the
// material index (12w + 1 bytes instead of 2 (9w + 1)).
//
// A tile's H(t+1) needs E(t+1) one cell beyond the tile on the high j and k
// sides, and E(t+1) there needs H(t) one cell beyond on the low sides: the
// block recomputes that one-cell E halo (and the first plane of the next
// chunk) itself.  So that no block ever reads a value another block has
// already advanced, the sweep reads the state of step t from one set of
// buffers (E, H, E psi) and writes step t+1 to a second set; the engine
// swaps the two after each step.  H psi is only touched by the block that
// owns the cell and is updated in place.
//
// Per cell the arithmetic is that of the split kernels -- the same device
// functions (e_plain / e_general, h_plain / h_general) and the same TFSF E
// correction (tfsf_e_terms / tfsf_e_add, TFSF3D::updateE,
// src/tfsf/tfsf_3d.cpp:299-411) applied to E(t+1) before H uses it -- so the
// sweep and the split kernels give identical bits.  Every owned cell is
// written each step (cells no update touches are copied), so the second
// buffer set always holds the whole state.  Lumped elements are not handled
// here: plans with them run the split kernels.
#pragma once

#include "common.cuh"
#include "surface.cuh"
#include "volume.cuh"

namespace xg {

template <typename T, typename I>
struct SweepParams {
  VolParams<T, I> v;   // state of step t (E, H, E psi read; H psi updated in place)
  T *E2[3], *H2[3];    // E and H of step t+1
  Psi<T> psi2;         // E psi of step t+1 (the H members are unused)
  int chunk;           // planes along i per block
};

constexpr int kSwK = 32;                         // owned tile: 32 cells along k
constexpr int kSwJ = 8;                          //             8 rows along j
constexpr int kHK = kSwK + 2, kHJ = kSwJ + 2;    // H(t) tile: one halo cell on each side
constexpr int kEK = kSwK + 1, kEJ = kSwJ + 1;    // E(t+1) tile: one halo cell on the high side
constexpr int kEHalo = kEK + kSwJ;               // halo E cells: row j0+8 (33) and column k0+32 (8)
constexpr int kSwThreads = kSwK * kSwJ;

// Per thread, the global values of one plane that the sweep needs: up to
// two H(t) tile elements, E(t) and the material index of the thread's own
// cell and (for the first kEHalo threads) of one halo cell.  Loaded one
// plane ahead so that the loads of plane i+1 are in flight while plane i is
// computed.
template <typename T>
struct SweepPlane {
  T h0[3], h1[3];
  T e[3], eh[3];
  unsigned idx, idxh;
  uint8_t fi;   // flags of plane i
};

template <typename T, typename I, int MINB>
__global__ void __launch_bounds__(kSwThreads, MINB) k_sweep(SweepParams<T, I> f) {
  const VolParams<T, I> &p = f.v;
  __shared__ T sH[3][3][kHJ][kHK];   // H(t) of planes i-2 .. i (ring of 3)
  __shared__ T sE[3][3][kEJ][kEK];   // E(t+1) of planes i-2 .. i (ring of 3)
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const int lane = threadIdx.x, row = threadIdx.y, tid = row * kSwK + lane;
  const int k0 = blockIdx.x * kSwK, j0 = blockIdx.y * kSwJ;
  const int ia = blockIdx.z * f.chunk;
  if (ia > nx) return;
  const int ib = min(ia + f.chunk, nx + 1);   // owned planes [ia, ib)
  const double *hinc = p.tf.enabled ? p.tf.inc + (((*p.step) + 1) & 1) * 6 * p.tf.L : nullptr;

  // this thread's H tile elements (tid and tid + 256 of the 10 x 34 tile)
  const int hr0 = tid / kHK, hc0 = tid - hr0 * kHK;
  const int e1 = tid + kSwThreads, hr1 = e1 / kHK, hc1 = e1 - hr1 * kHK;
  const bool has1 = e1 < kHJ * kHK;
  const int hj0 = j0 - 1 + hr0, hk0 = k0 - 1 + hc0, hj1 = j0 - 1 + hr1, hk1 = k0 - 1 + hc1;
  const bool hin0 = hj0 >= 0 && hj0 <= ny && hk0 >= 0 && hk0 <= nz;
  const bool hin1 = has1 && hj1 >= 0 && hj1 <= ny && hk1 >= 0 && hk1 <= nz;
  // the thread's own cell and its halo cell of the E tile
  const int jm = j0 + row, km = k0 + lane;
  const bool min_ = jm <= ny && km <= nz;
  const bool has_h = tid < kEHalo;
  const int rh = tid < kEK ? kSwJ : tid - kEK, ch = tid < kEK ? tid : kSwK;
  const int jh = j0 + rh, kh = k0 + ch;
  const bool hin_ = has_h && jh <= ny && kh <= nz;
  const uint8_t fjk = min_ ? (__ldg(p.flags[1] + jm) | __ldg(p.flags[2] + km)) : 0;
  const uint8_t fjkh = hin_ ? (__ldg(p.flags[1] + jh) | __ldg(p.flags[2] + kh)) : 0;

  auto fetch = [&](int i, SweepPlane<T> &q) {
    const bool pin = i >= 0 && i <= nx;
    const unsigned bi = pin ? static_cast<unsigned>(i) * usi : 0u;
    const unsigned b0 = bi + static_cast<unsigned>(hj0) * usj + hk0, b1 = bi + static_cast<unsigned>(hj1) * usj + hk1;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      q.h0[c] = pin && hin0 ? __ldg(p.H[c] + b0) : T(0);
      q.h1[c] = pin && hin1 ? __ldg(p.H[c] + b1) : T(0);
    }
    const unsigned bm = bi + static_cast<unsigned>(jm) * usj + km, bh = bi + static_cast<unsigned>(jh) * usj + kh;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      q.e[c] = pin && min_ ? __ldg(p.E[c] + bm) : T(0);
      q.eh[c] = pin && hin_ ? __ldg(p.E[c] + bh) : T(0);
    }
    q.idx = pin && min_ ? static_cast<unsigned>(__ldg(p.idx + bm)) : 0u;
    q.idxh = pin && hin_ ? static_cast<unsigned>(__ldg(p.idx + bh)) : 0u;
    q.fi = pin ? __ldg(p.flags[0] + i) : 0;
  };
  auto stash_h = [&](const SweepPlane<T> &q, int s) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      sH[s][c][hr0][hc0] = q.h0[c];
      if (has1) sH[s][c][hr1][hc1] = q.h1[c];
    }
  };

  // E(t+1) of plane i at tile cell (r, c) from E(t) = e; `own`: also store
  // it (and its psi) as the new state
  auto e_update = [&](int i, int r, int c, bool own, const T *eo, unsigned id, uint8_t fl) {
    const int j = j0 + r, k = k0 + c, s = i % 3, sm = (i + 2) % 3;
    T ex = eo[0], ey = eo[1], ez = eo[2];
    const ECurl<T> h{sH[s][0][r + 1][c + 1], sH[s][1][r + 1][c + 1], sH[s][2][r + 1][c + 1],
                     sH[s][0][r + 1][c],     sH[s][1][r + 1][c],     sH[s][0][r][c + 1],
                     sH[s][2][r][c + 1],     sH[sm][1][r + 1][c + 1], sH[sm][2][r + 1][c + 1]};
    const T *cf = p.table + id * 18;
    if (!(fl & kSpecialE)) {
      e_plain(cf, h, ex, ey, ez);
    } else {
      bool w[3];
      e_general<T, I, true>(p, cf, i, j, k, h, p.psi, f.psi2, own, ex, ey, ez, w);
    }
    if ((fl & kTfsfE) && hinc) {
      int t;
      if ((t = tfsf_e_terms<0>(p.tf, i, j, k))) tfsf_e_add<0>(p.tf, hinc, i, j, k, t, ex);
      if ((t = tfsf_e_terms<1>(p.tf, i, j, k))) tfsf_e_add<1>(p.tf, hinc, i, j, k, t, ey);
      if ((t = tfsf_e_terms<2>(p.tf, i, j, k))) tfsf_e_add<2>(p.tf, hinc, i, j, k, t, ez);
    }
    if (own) {
      const unsigned b = static_cast<unsigned>(i) * usi + static_cast<unsigned>(j) * usj + k;
      f.E2[0][b] = ex;
      f.E2[1][b] = ey;
      f.E2[2][b] = ez;
    }
    sE[s][0][r][c] = ex;
    sE[s][1][r][c] = ey;
    sE[s][2][r][c] = ez;
  };
  auto e_zero = [&](int s, int r, int c) {
    sE[s][0][r][c] = T(0);
    sE[s][1][r][c] = T(0);
    sE[s][2][r][c] = T(0);
  };

  // H(t+1) of plane i at owned tile cell (r, c)
  auto h_update = [&](int i, int r, int c, unsigned id, uint8_t fl) {
    const int j = j0 + r, k = k0 + c, s = i % 3, sp = (i + 1) % 3;
    const HCurl<T> e{sE[s][0][r][c],     sE[s][1][r][c],     sE[s][2][r][c],
                     sE[s][0][r][c + 1], sE[s][1][r][c + 1], sE[s][0][r + 1][c],
                     sE[s][2][r + 1][c], sE[sp][1][r][c],    sE[sp][2][r][c]};
    T hx = sH[s][0][r + 1][c + 1], hy = sH[s][1][r + 1][c + 1], hz = sH[s][2][r + 1][c + 1];
    const T *cf = p.table + id * 18 + 9;
    if (!(fl & kSpecialH)) {
      h_plain(cf, e, hx, hy, hz);
    } else {
      bool w[3];
      h_general(p, cf, i, j, k, e, hx, hy, hz, w);
    }
    const unsigned b = static_cast<unsigned>(i) * usi + static_cast<unsigned>(j) * usj + k;
    f.H2[0][b] = hx;
    f.H2[1][b] = hy;
    f.H2[2][b] = hz;
  };

  SweepPlane<T> cur, nxt;
  fetch(ia - 1, nxt);   // H(t) of plane ia-1 (zeros for ia = 0)
  stash_h(nxt, (ia + 2) % 3);
  fetch(ia, cur);
  unsigned idx_prev = 0;   // material index of the own cell on plane i-1
  uint8_t fi_prev = 0;
  for (int i = ia; i <= ib; ++i) {
    const int s = i % 3;
    stash_h(cur, s);
    if (i < ib) fetch(i + 1, nxt);   // in flight while plane i is computed
    __syncthreads();
    if (i <= nx) {
      if (min_) e_update(i, row, lane, i < ib, cur.e, cur.idx, cur.fi | fjk);
      else e_zero(s, row, lane);
      if (has_h) {
        if (hin_) e_update(i, rh, ch, false, cur.eh, cur.idxh, cur.fi | fjkh);
        else e_zero(s, rh, ch);
      }
    } else {   // past the last plane: E(t+1) of plane nx+1 is zero
      T *z = &sE[s][0][0][0];
      for (int e = tid; e < 3 * kEJ * kEK; e += kSwThreads) z[e] = T(0);
    }
    __syncthreads();
    if (i > ia && min_) h_update(i - 1, row, lane, idx_prev, fi_prev | fjk);
    idx_prev = cur.idx;
    fi_prev = cur.fi;
    cur = nxt;
  }
}

}  // namespace xg
