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

#include <type_traits>

#include "common.cuh"
#include "surface.cuh"
#include "tma.cuh"
#include "volume.cuh"

namespace xg {

template <typename T, typename I>
struct SweepParams {
  VolParams<T, I> v;   // state of step t (E, H, E psi read; H psi updated in place)
  T *E2[3], *H2[3];    // E and H of step t+1
  Psi<T> psi2;         // E psi of step t+1 (the H members are unused)
  int chunk;           // planes along i per block
  int *status;         // set to XFDTD_ERR_TIMEOUT if a stage wait gives up
};

constexpr int kSwK = 32;                         // owned tile: 32 cells along k
constexpr int kSwJ = 8;                          //             8 rows along j
constexpr int kHK = kSwK + 2, kHJ = kSwJ + 2;    // H(t) tile: one halo cell on each side
constexpr int kEK = kSwK + 1, kEJ = kSwJ + 1;    // E(t+1) tile: one halo cell on the high side
constexpr int kEHalo = kEK + kSwJ;               // halo E cells: row j0+8 (33) and column k0+32 (8)
constexpr int kSwThreads = kSwK * kSwJ;

// Shared-memory staging.  For each plane the block needs H(t) on its tile
// with a one-cell halo all round (rows j0-1 .. j0+8, columns k0-1 .. k0+32),
// E(t) and the material index on the E tile (rows j0 .. j0+8, columns
// k0 .. k0+32).  One elected thread fetches them with tiled TMA loads
// (cp.async.bulk.tensor) into a ring of kStages plane stages, kStages-2
// planes ahead of the plane being computed; an mbarrier per stage counts
// the bytes in.  Tile rows start on 16-byte boundaries as TMA requires: the
// H rows start at k0-4 (FP32) or k0-2 (FP64), the E and index rows at k0,
// and the boxes are widened to whole 16-byte rows.  Out-of-range parts of a
// box (j or k beyond the grid, plane -1) arrive as zeros.
constexpr int kStages = 4;

__host__ __device__ constexpr int round128(int b) { return (b + 127) / 128 * 128; }

template <typename T, typename I>
struct SweepTiles {
  static constexpr int HW = sizeof(T) == 4 ? 40 : 36;    // H row: columns k0-HOFF-1 ..
  static constexpr int HOFF = sizeof(T) == 4 ? 3 : 1;    // tile column of k0-1, minus 0
  static constexpr int EW = sizeof(T) == 4 ? 36 : 34;    // E row: columns k0 ..
  static constexpr int IW = sizeof(I) == 1 ? 48 : 40;    // index row: columns k0 ..
  static constexpr int H_TILE = round128(kHJ * HW * int(sizeof(T)));
  static constexpr int E_TILE = round128(kEJ * EW * int(sizeof(T)));
  static constexpr int I_TILE = round128(kEJ * IW * int(sizeof(I)));
  static constexpr int STAGE = 3 * H_TILE + 3 * E_TILE + I_TILE;
  static constexpr int SE = round128(2 * 3 * kEJ * kEK * int(sizeof(T)));   // E(t+1) of planes i-1, i
  static constexpr int SMEM = kStages * STAGE + SE + kStages * 8;
  static constexpr unsigned H_BYTES = 3u * kHJ * HW * sizeof(T);
  static constexpr unsigned FULL_BYTES = H_BYTES + 3u * kEJ * EW * sizeof(T) + unsigned(kEJ * IW * sizeof(I));
};

// The tensor maps of one launch: H(t) and E(t) components and the index.
struct SweepMaps {
  CUtensorMap h[3];
  CUtensorMap e[3];
  CUtensorMap idx;
};

// Polls of a stage barrier before the sweep gives up and reports
// XFDTD_ERR_TIMEOUT through the status word.
constexpr int kSweepWaitLimit = 1 << 22;

template <typename T, typename I, int MINB>
__global__ void __launch_bounds__(kSwThreads, MINB) k_sweep(const __grid_constant__ SweepMaps maps, SweepParams<T, I> f) {
  using G = SweepTiles<T, I>;
  const VolParams<T, I> &p = f.v;
  extern __shared__ __align__(128) unsigned char smem[];
  T(*sE)[3][kEJ][kEK] = reinterpret_cast<T(*)[3][kEJ][kEK]>(smem + kStages * G::STAGE);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kStages * G::STAGE + G::SE);
  const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  const int lane = threadIdx.x, row = threadIdx.y, tid = row * kSwK + lane;
  const int k0 = blockIdx.x * kSwK, j0 = blockIdx.y * kSwJ;
  const int ia = blockIdx.z * f.chunk;
  if (ia > nx) return;
  const int ib = min(ia + f.chunk, nx + 1);   // owned planes [ia, ib)
  const int last = min(ib, nx);               // last plane loaded
  const auto hinc = p.tf.enabled ? tfsf_view<T>(p.tf).inc + (((*p.step) + 1) & 1) * 6 * p.tf.L : nullptr;

  // stage of plane q: planes ia-1 .. last in order, kStages in the ring
  auto stage_of = [&](int q) { return (q - ia + 1) % kStages; };
  auto h_tile = [&](int st, int c) { return reinterpret_cast<T *>(smem + st * G::STAGE + c * G::H_TILE); };
  auto e_tile = [&](int st, int c) {
    return reinterpret_cast<T *>(smem + st * G::STAGE + 3 * G::H_TILE + c * G::E_TILE);
  };
  auto i_tile = [&](int st) { return reinterpret_cast<I *>(smem + st * G::STAGE + 3 * G::H_TILE + 3 * G::E_TILE); };
  // H(t) at H-tile cell (r, c), r = j - (j0-1), c = k - (k0-1)
  auto hv = [&](int st, int comp, int r, int c) { return h_tile(st, comp)[r * G::HW + c + G::HOFF]; };

  // thread 0: start the loads of plane q (H only for plane ia-1)
  auto issue = [&](int q) {
    const int st = stage_of(q);
    const bool full = q >= ia;
    mbar_arrive_expect_tx(&bar[st], full ? G::FULL_BYTES : G::H_BYTES);
    for (int c = 0; c < 3; ++c) tma_load_3d(h_tile(st, c), &maps.h[c], k0 - G::HOFF - 1, j0 - 1, q, &bar[st]);
    if (full) {
      for (int c = 0; c < 3; ++c) tma_load_3d(e_tile(st, c), &maps.e[c], k0, j0, q, &bar[st]);
      tma_load_3d(i_tile(st), &maps.idx, k0, j0, q, &bar[st]);
    }
  };

  if (tid == 0) {
    for (int q = 0; q < kStages; ++q) mbar_init(&bar[q], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (ia == 0) {   // plane -1: H(t) = 0, written here instead of loaded
    for (int c = 0; c < 3; ++c)
      for (int e = tid; e < kHJ * G::HW; e += kSwThreads) h_tile(0, c)[e] = T(0);
  }
  if (tid == 0) {
    fence_proxy_async();
    for (int q = max(ia - 1, 0); q <= min(ia + kStages - 2, last); ++q) issue(q);
  }
  unsigned phase = 0;   // bit s: parity of the next completion of stage s
  bool timed_out = false;
  auto wait_plane = [&](int q) {
    const int st = stage_of(q);
    if (!mbar_wait_bounded(&bar[st], (phase >> st) & 1u, kSweepWaitLimit)) timed_out = true;
    phase ^= 1u << st;
  };
  if (ia > 0) wait_plane(ia - 1);
  __syncthreads();   // the zeros of plane -1 are visible

  // this thread's own cell and its halo cell of the E tile
  const int jm = j0 + row, km = k0 + lane;
  const bool min_ = jm <= ny && km <= nz;
  const bool has_h = tid < kEHalo;
  const int rh = tid < kEK ? kSwJ : tid - kEK, ch = tid < kEK ? tid : kSwK;
  const int jh = j0 + rh, kh = k0 + ch;
  const bool hin_ = has_h && jh <= ny && kh <= nz;
  const uint8_t fjk = min_ ? (__ldg(p.flags[1] + jm) | __ldg(p.flags[2] + km)) : 0;
  const uint8_t fjkh = hin_ ? (__ldg(p.flags[1] + jh) | __ldg(p.flags[2] + kh)) : 0;

  // E(t+1) of plane i at E-tile cell (r, c); `own`: also store it (and its
  // psi) as the new state
  auto e_update = [&](auto plain_tile, int i, int r, int c, bool own, uint8_t fl) {
    constexpr bool kPlain = decltype(plain_tile)::value;
    const int j = j0 + r, k = k0 + c, s = i & 1, st = stage_of(i), sm = stage_of(i - 1);
    T ex = e_tile(st, 0)[r * G::EW + c], ey = e_tile(st, 1)[r * G::EW + c], ez = e_tile(st, 2)[r * G::EW + c];
    const ECurl<T> h{hv(st, 0, r + 1, c + 1), hv(st, 1, r + 1, c + 1), hv(st, 2, r + 1, c + 1),
                     hv(st, 0, r + 1, c),     hv(st, 1, r + 1, c),     hv(st, 0, r, c + 1),
                     hv(st, 2, r, c + 1),     hv(sm, 1, r + 1, c + 1), hv(sm, 2, r + 1, c + 1)};
    const T *cf = p.table + static_cast<unsigned>(i_tile(st)[r * G::IW + c]) * 18;
    if (kPlain || !(fl & kSpecialE)) {
      e_plain(cf, h, ex, ey, ez);
    } else {
      bool w[3];
      e_general<T, I, true>(p, cf, i, j, k, h, p.psi, f.psi2, own, ex, ey, ez, w);
    }
    if (!kPlain && (fl & kTfsfE) && hinc) {
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
  auto h_update = [&](auto plain_tile, int i, int r, int c, uint8_t fl) {
    constexpr bool kPlain = decltype(plain_tile)::value;
    const int j = j0 + r, k = k0 + c, s = i & 1, sp = (i + 1) & 1, st = stage_of(i);
    const HCurl<T> e{sE[s][0][r][c],     sE[s][1][r][c],     sE[s][2][r][c],
                     sE[s][0][r][c + 1], sE[s][1][r][c + 1], sE[s][0][r + 1][c],
                     sE[s][2][r + 1][c], sE[sp][1][r][c],    sE[sp][2][r][c]};
    T hx = hv(st, 0, r + 1, c + 1), hy = hv(st, 1, r + 1, c + 1), hz = hv(st, 2, r + 1, c + 1);
    const T *cf = p.table + static_cast<unsigned>(i_tile(st)[r * G::IW + c]) * 18 + 9;
    if (kPlain || !(fl & kSpecialH)) {
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

  // Tiles whose rows and columns carry no wall, CPML or TFSF flag take the
  // plain update on every plane that carries none either (same bits, no
  // general-path code).
  const std::integral_constant<bool, true> plain;
  const std::integral_constant<bool, false> general;
  const bool tile_plain_e = __syncthreads_and(!((fjk | fjkh) & (kSpecialE | kTfsfE)));
  const bool tile_plain_h = __syncthreads_and(!(fjk & kSpecialH));
  for (int i = ia; i <= ib; ++i) {
    const int s = i & 1;
    if (i <= nx) {
      wait_plane(i);
      const uint8_t fi = __ldg(p.flags[0] + i);
      if (tile_plain_e && !(fi & (kSpecialE | kTfsfE))) {
        if (min_) e_update(plain, i, row, lane, i < ib, 0);
        else e_zero(s, row, lane);
        if (has_h) {
          if (hin_) e_update(plain, i, rh, ch, false, 0);
          else e_zero(s, rh, ch);
        }
      } else {
        if (min_) e_update(general, i, row, lane, i < ib, fi | fjk);
        else e_zero(s, row, lane);
        if (has_h) {
          if (hin_) e_update(general, i, rh, ch, false, fi | fjkh);
          else e_zero(s, rh, ch);
        }
      }
    } else {   // past the last plane: E(t+1) of plane nx+1 is zero
      T *z = &sE[s][0][0][0];
      for (int e = tid; e < 3 * kEJ * kEK; e += kSwThreads) z[e] = T(0);
    }
    __syncthreads();
    if (i > ia && min_) {
      const uint8_t fi = __ldg(p.flags[0] + i - 1);
      if (tile_plain_h && !(fi & kSpecialH)) h_update(plain, i - 1, row, lane, 0);
      else h_update(general, i - 1, row, lane, fi | fjk);
    }
    __syncthreads();   // stage of plane i-1 and E(t+1) slot of plane i-1 are free
    if (tid == 0 && i + kStages - 1 <= last) {
      fence_proxy_async();
      issue(i + kStages - 1);
    }
  }
  if (timed_out) atomicExch(f.status, static_cast<int>(4));   // XFDTD_ERR_TIMEOUT
}

}  // namespace xg
