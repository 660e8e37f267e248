// interior_tma.cuh -- the interior E and H kernels with their planes staged
// by TMA.
//
// The one-thread-per-cell interior kernels (volume.cuh) are latency-bound:
// each warp waits for its own loads, and about 80 % of the warp slots
// cannot keep enough bytes in flight to reach the copy bandwidth.  Here a
// block owns a tile of 8 rows (j) x 32 cells (k) of the interior box and
// marches along i through a chunk of planes.  One elected thread fetches
// each plane's tiles with tiled TMA loads (cp.async.bulk.tensor) into a
// ring of STAGES plane stages, STAGES-2 planes ahead of the one being
// updated; an mbarrier per stage counts the bytes in.  The threads read
// the tiles from shared memory, apply the same per-cell arithmetic as the
// fast path (e_plain / h_plain with the same coefficients) and store the
// updated plane straight to global memory.  The material index comes with
// the tiles in the 32-wide launches; the 16-wide z-edge launch reads it with
// plain loads issued before the wait for the plane (its upper tiles start
// after the interior's last k, which need not lie on a 16-byte boundary of
// a 1-byte index).
//
// The tile is KT cells along k by 256 / KT rows along j: 32 x 8 for the
// interior launches, 16 x 16 for the z-edge launch, whose k runs (the CPML
// slabs and walls below and above the interior's k range) are 10 to 16
// cells long.
//
//   E kernel: plane i needs H(i) on rows j0-1 .. j0+J-1 and columns k0-1
//   .. k0+KT-1, H(i-1) on the tile (the previous stage), E(i) on the tile.
//   H kernel: plane i needs E(i) on rows j0 .. j0+J and columns k0 ..
//   k0+KT, E(i+1) on the tile (the next stage), H(i) on the tile.
//
// MODE selects the cells a launch covers:
//   0  the interior box, plain on every axis;
//   1  (wide) every plane and row, i 0 .. nx and j 0 .. ny, over the
//      interior's k range: the CPML slabs and walls on x and y join the
//      interior.  Planes outside the plain x run and rows outside the plain
//      y run take the general path with x, y or both as the special axes
//      (uniform per block plane and per warp, since a warp is one row);
//   2  (z edges) the same planes and rows over the k tiles below and above
//      the interior's k range, with z special too: tiles from k = 0 up to
//      the interior's first k, and from the one after its last k up to nz.
//      Modes 1 and 2 together cover the grid.
// H and E beyond the grid (plane -1, row -1, plane nx+1, row ny+1, k -1)
// arrive as TMA zeros, the values the general path puts there; E at k nz+1
// (inside the row padding) is zeroed by hand, as the general path does.
//
// Tile rows start on 16-byte boundaries as TMA requires: the engine offers
// these kernels only when the interior's k range starts on one, and (for
// modes 1 and 2) when the k after its last does too (interior_tma_setup in
// engine.cu); the rows of the E kernel's H tile start HOFF+1 cells before
// k0, widened to whole 16-byte rows.  Waits on a stage are bounded; a block
// that gives up reports XFDTD_ERR_TIMEOUT through the status word and
// stops.
#pragma once

#include "common.cuh"
#include "surface.cuh"
#include "tma.cuh"
#include "volume.cuh"

namespace xg {

// The TFSF corrections folded into the wide decomposition's launches
// (modes 1 and 2, which together cover every cell): when `on`,
// the cells of the TFSF box's surface get TFSF3D::updateE's (E kernel) or
// updateH's (H kernel) corrections after their update, with the same
// arithmetic as k_tfsf_e / k_tfsf_h (surface.cuh), before the store.  The
// engine turns it on when the wide decomposition runs on its two TMA
// launches and no lumped element's correction would have to come first.
struct TfsfFuse {
  TfsfDev tf;
  const long long *step;
  int on;
};

// Out-of-line calls into the TFSF corrections: only the few warps on the
// box's surface take them, and kept out of line they leave the launch's
// register budget to the per-cell update.
template <typename T>
__device__ __noinline__ void tfsf_e_fused_call(const TfsfDev &tf, const decltype(tfsf_view<T>(tf).inc) hinc, int i,
                                               int j, int k, T &ex, T &ey, T &ez, bool *w) {
  tfsf_e_fused<T>(tf, hinc, i, j, k, ex, ey, ez, w);
}
template <typename T>
__device__ __noinline__ void tfsf_h_cell_call(const TfsfDev &tf, const decltype(tfsf_view<T>(tf).inc) einc, int i,
                                              int j, int k, T &hx, T &hy, T &hz, bool *w) {
  tfsf_h_cell<T>(tf, einc, i, j, k, hx, hy, hz, w);
}

constexpr int kItThreads = 256;
constexpr int kItK = 32;                  // interior launches' tile: 32 cells along k
constexpr int kItKz = 16;                 // z-edge launch's tile: 16 cells along k
constexpr int kItWaitLimit = 1 << 22;     // polls of a stage barrier before giving up

// Tile geometry of a KT-wide tile (J = 256 / KT rows).  E kernel: H rows of
// HW columns starting at k0-HOFF-1, J+1 rows from j0-1; E tiles KT x J from
// (k0, j0).  H kernel: E rows of EW columns starting at k0, J+1 rows from
// j0; H tiles KT x J.  HW and EW are whole 16-byte rows.
template <typename T, typename I, int KT>
struct ItTiles {
  static constexpr int J = kItThreads / KT;
  static constexpr bool IDX = KT == kItK;   // the index tile comes by TMA
  static constexpr int HOFF = sizeof(T) == 4 ? 3 : 1;
  static constexpr int HW = KT == 32 ? (sizeof(T) == 4 ? 40 : 36)    // covers k0-HOFF-1 .. k0+KT-1
                                     : (sizeof(T) == 4 ? 20 : 18);
  static constexpr int EW = KT == 32 ? (sizeof(T) == 4 ? 36 : 34)    // covers k0 .. k0+KT
                                     : (sizeof(T) == 4 ? 20 : 18);
  static constexpr int RND = 128;
  static constexpr int rnd(int b) { return (b + RND - 1) / RND * RND; }
  // E kernel stage: 3 H tiles (halo), 3 E tiles, the index tile
  static constexpr int EH_TILE = rnd((J + 1) * HW * int(sizeof(T)));
  static constexpr int EE_TILE = rnd(J * KT * int(sizeof(T)));
  static constexpr int I_TILE = IDX ? rnd(J * KT * int(sizeof(I))) : 0;
  static constexpr unsigned I_BYTES = IDX ? unsigned(J * KT * sizeof(I)) : 0u;
  static constexpr int E_STAGE = 3 * EH_TILE + 3 * EE_TILE + I_TILE;
  static constexpr unsigned E_HBYTES = 3u * (J + 1) * HW * sizeof(T);
  static constexpr unsigned E_FULL = E_HBYTES + 3u * J * KT * sizeof(T) + I_BYTES;
  // H kernel stage: 3 E tiles (halo), 3 H tiles, the index tile
  static constexpr int HE_TILE = rnd((J + 1) * EW * int(sizeof(T)));
  static constexpr int HH_TILE = EE_TILE;
  static constexpr int H_STAGE = 3 * HE_TILE + 3 * HH_TILE + I_TILE;
  static constexpr unsigned H_EBYTES = 3u * (J + 1) * EW * sizeof(T);
  static constexpr unsigned H_FULL = H_EBYTES + 3u * J * KT * sizeof(T) + I_BYTES;
  template <int STAGES>
  static constexpr int smem_e() { return STAGES * E_STAGE + STAGES * 8; }
  template <int STAGES>
  static constexpr int smem_h() { return STAGES * H_STAGE + STAGES * 8; }
};

// Tensor maps of one launch: a[3] the halo tiles (H for the E kernel, E for
// the H kernel), b[3] the updated side's tiles, the index (32-wide tiles).
struct ItMaps {
  CUtensorMap a[3];
  CUtensorMap b[3];
  CUtensorMap idx;
};

// The block's planes and tile: k0, j0 of the tile, its last k khi, planes
// [ia, ib) of its chunk.  Every tile starts on a 16-byte boundary: the
// interior box's k range starts on one, and mode 2's upper tiles start
// after its last k, whose successor is on one too.
struct ItBlock {
  int k0, khi, j0, ia, ib;
};
template <int MODE, int KT>
__device__ __forceinline__ ItBlock it_block(const InteriorBox &in, int chunk, uint3 bid) {
  ItBlock b;
  const int t = static_cast<int>(bid.x);
  if (MODE == 2) {
    const int nlo = (in.pz_lo + KT - 1) / KT;
    const bool below = t < nlo;
    b.k0 = below ? t * KT : in.pz_hi + 1 + (t - nlo) * KT;
    b.khi = below ? in.pz_lo - 1 : in.hi[2];
  } else {
    b.k0 = in.lo[2] + t * KT;
    b.khi = in.hi[2];
  }
  b.j0 = in.lo[1] + static_cast<int>(bid.y) * (kItThreads / KT);
  b.ia = in.lo[0] + static_cast<int>(bid.z) * chunk;
  b.ib = min(b.ia + chunk, in.hi[0] + 1);
  return b;
}

// The CPML context of plane i for the thread's cells: the row's y and z
// context `cyz` with the x slot and profile values of index i (E half 0,
// H half 1).  Plane i is the same for every thread of the block, so every
// thread loads them, unconditionally (on the plain x planes the slot is
// -1, as no CPML index lies in the plain run, and the profile stays the
// identity).  Loaded only for the cells whose class has the x bit, through
// references into a per-thread context, the x part was lost in the builds
// without the 5-block cap for the cells in both an x and a y slab.
template <typename T, typename I, int MODE>
__device__ __forceinline__ SlabCtx<T> it_plane_ctx(const VolCore<T, I> &p, int half, int i, const SlabCtx<T> &cyz) {
  SlabCtx<T> cx = cyz;
  if constexpr (MODE != 0) {
    const CpmlAxis<T> &ax = p.cp[0];
    const int xs = ax.n_layers ? __ldg((half ? ax.slot_h : ax.slot_e) + i) : -1;
    cx.xs = xs;
    cx.X = half ? axis_coef(xs, ax.b_m, ax.a_m, ax.rk_m, i) : axis_coef(xs, ax.b_e, ax.a_e, ax.rk_e, i);
  }
  return cx;
}

// Stage bookkeeping of one block (thread 0 issues and drains; every thread
// waits).  A wait that gives up marks the block timed out; the block then
// stops, and thread 0 waits (bounded) for the loads it issued before the
// block exits, so that no copy lands in a finished block's shared memory.
//
// The plane waits poll at most `limit` times (kItWaitLimit unless the handle
// lowered it, xfdtd_set_wait_limit; 0 gives up at once, which is how the
// failure path is tested).  The drain of copies in flight always polls up
// to kItWaitLimit.
template <int STAGES>
struct ItRing {
  uint64_t *bar;
  int limit = kItWaitLimit;
  unsigned phase = 0;   // bit s: parity of the next completion of stage s
  bool timed_out = false;
  __device__ bool wait(int st) {
    if (timed_out) return false;
    if (!mbar_wait_bounded(&bar[st], (phase >> st) & 1u, limit)) {
      timed_out = true;
      return false;
    }
    phase ^= 1u << st;
    return true;
  }
};

// The E update of one block: tile `bid` (k tile, j tile, chunk of planes)
// of the launch over box `in`.  `maps` may lie in the launch's parameter
// space or in global memory (the batched launches).
template <typename T, typename I, int STAGES, bool CT, int MODE, int KT, bool TF>
__device__ __forceinline__ void it_e_block(const ItMaps &maps, const VolCore<T, I> &p, const InteriorBox &in,
                                           int chunk, int *status, int wait_limit, const TfsfFuse &fz, uint3 bid) {
  using G = ItTiles<T, I, KT>;
  extern __shared__ __align__(128) unsigned char smem[];
  ItRing<STAGES> ring{reinterpret_cast<uint64_t *>(smem + STAGES * G::E_STAGE), wait_limit};
  const int tid = threadIdx.x, c = tid % KT, r = tid / KT;
  const ItBlock blk = it_block<MODE, KT>(in, chunk, bid);
  if (blk.ia >= blk.ib) return;
  auto stage_of = [&](int q) { return (q - blk.ia + 1) % STAGES; };   // plane ia-1 in stage 0
  auto htile = [&](int st, int comp) { return reinterpret_cast<const T *>(smem + st * G::E_STAGE + comp * G::EH_TILE); };
  auto etile = [&](int st, int comp) {
    return reinterpret_cast<const T *>(smem + st * G::E_STAGE + 3 * G::EH_TILE + comp * G::EE_TILE);
  };
  auto issue = [&](int q) {   // thread 0: the loads of plane q (H only for plane ia-1)
    const int st = stage_of(q);
    const bool full = q >= blk.ia;
    unsigned char *base = smem + st * G::E_STAGE;
    mbar_arrive_expect_tx(&ring.bar[st], full ? G::E_FULL : G::E_HBYTES);
    for (int comp = 0; comp < 3; ++comp)
      tma_load_3d(base + comp * G::EH_TILE, &maps.a[comp], blk.k0 - G::HOFF - 1, blk.j0 - 1, q, &ring.bar[st]);
    if (full) {
      for (int comp = 0; comp < 3; ++comp)
        tma_load_3d(base + 3 * G::EH_TILE + comp * G::EE_TILE, &maps.b[comp], blk.k0, blk.j0, q, &ring.bar[st]);
      if (G::IDX) tma_load_3d(base + 3 * G::EH_TILE + 3 * G::EE_TILE, &maps.idx, blk.k0, blk.j0, q, &ring.bar[st]);
    }
  };
  int issued = blk.ia - 2, waited = blk.ia - 2;   // thread 0: last plane issued, last plane waited
  if (tid == 0) {
    for (int q = 0; q < STAGES; ++q) mbar_init(&ring.bar[q], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    issued = min(blk.ia + STAGES - 2, blk.ib - 1);
    for (int q = blk.ia - 1; q <= issued; ++q) issue(q);
  }
  if (ring.wait(stage_of(blk.ia - 1))) waited = blk.ia - 1;
  const int j = blk.j0 + r, k = blk.k0 + c;
  const bool mine = j <= in.hi[1] && k <= blk.khi;
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  // the CPML context of the thread's row and column, fixed over the planes
  SlabCtx<T> cyz = slab_ctx<T, I, 0>(p, 0, 0, 0, 0);
  const bool yspec = MODE != 0 && (j < in.py_lo || j > in.py_hi);
  if (MODE != 0 && mine) {
    if (yspec) slab_axis(p, 1, 0, j, cyz.ys, cyz.Y);
    if (MODE == 2) slab_axis(p, 2, 0, k, cyz.zs, cyz.Z);
  }
  // the incident H arrays of the previous step (the 1-D line's other buffer)
  const auto hinc = (MODE != 0 && TF) ? tfsf_view<T>(fz.tf).inc + ((*fz.step + 1) & 1) * 6 * fz.tf.L : nullptr;
  for (int i = blk.ia; i < blk.ib; ++i) {
    // a special cell's psi operands, loaded before the wait for the plane
    const int cls = MODE == 0 ? 0 : ((i < in.px_lo || i > in.px_hi) ? 1 : 0) | (yspec ? 2 : 0) | (MODE == 2 ? 4 : 0);
    const SlabCtx<T> cx = it_plane_ctx<T, I, MODE>(p, 0, i, cyz);
    PsiOps<T> ps{};
    if (MODE != 0 && mine && cls != 0) ps = e_psi_load<T, I, 7>(p, cx, i, j, k, p.psi);
    const unsigned b = static_cast<unsigned>(i) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
    const unsigned m_plain = (!G::IDX && mine) ? static_cast<unsigned>(__ldg(p.idx + b)) : 0u;
    if (ring.wait(stage_of(i))) waited = i;
    if (mine && !ring.timed_out) {
      const int st = stage_of(i), sm = stage_of(i - 1);
      auto hv = [&](int s, int comp, int rr, int cc) { return htile(s, comp)[rr * G::HW + cc + G::HOFF]; };
      // H at (j, k), (k-1), (j-1) of plane i and at (j, k) of plane i-1
      ECurl<T> h{hv(st, 0, r + 1, c + 1), hv(st, 1, r + 1, c + 1), hv(st, 2, r + 1, c + 1),
                       hv(st, 0, r + 1, c),     hv(st, 1, r + 1, c),     hv(st, 0, r, c + 1),
                       hv(st, 2, r, c + 1),     hv(sm, 1, r + 1, c + 1), hv(sm, 2, r + 1, c + 1)};
      T ex = etile(st, 0)[r * KT + c], ey = etile(st, 1)[r * KT + c], ez = etile(st, 2)[r * KT + c];
      const unsigned m =
          G::IDX ? static_cast<unsigned>(reinterpret_cast<const I *>(smem + st * G::E_STAGE + 3 * G::EH_TILE +
                                                                     3 * G::EE_TILE)[r * KT + c])
                 : m_plain;
      T cf[9];
      coefs<T, I, CT>(p, p.table, 18, m, 0, cf);
      if (MODE != 2 && cls == 0) {
        e_plain(cf, h, ex, ey, ez);
        if (MODE != 0 && TF && tfsf_on_e_surface(fz.tf, i, j, k)) {
          bool w[3];
          tfsf_e_fused_call<T>(fz.tf, hinc, i, j, k, ex, ey, ez, w);
        }
        p.E[0][b] = ex;
        p.E[1][b] = ey;
        p.E[2][b] = ez;
      } else {
        bool w[3];
        if (MODE == 2) {
          if (k == 0) h.hx_k = h.hy_k = T(0);
          if (cls == 4) e_general_ops<T, I, 4>(p, cf, i, j, k, h, cx, ps, p.psi, true, ex, ey, ez, w);
          else if (cls == 5) e_general_ops<T, I, 5>(p, cf, i, j, k, h, cx, ps, p.psi, true, ex, ey, ez, w);
          else if (cls == 6) e_general_ops<T, I, 6>(p, cf, i, j, k, h, cx, ps, p.psi, true, ex, ey, ez, w);
          else e_general_ops<T, I, 7>(p, cf, i, j, k, h, cx, ps, p.psi, true, ex, ey, ez, w);
        } else if (cls == 1) {
          e_general_ops<T, I, 1>(p, cf, i, j, k, h, cx, ps, p.psi, true, ex, ey, ez, w);
        } else if (cls == 2) {
          e_general_ops<T, I, 2>(p, cf, i, j, k, h, cx, ps, p.psi, true, ex, ey, ez, w);
        } else {
          e_general_ops<T, I, 3>(p, cf, i, j, k, h, cx, ps, p.psi, true, ex, ey, ez, w);
        }
        if (MODE != 0 && TF && tfsf_on_e_surface(fz.tf, i, j, k)) {
          bool wt[3];
          tfsf_e_fused_call<T>(fz.tf, hinc, i, j, k, ex, ey, ez, wt);
          for (int q = 0; q < 3; ++q) w[q] = w[q] || wt[q];
        }
        if (w[0]) p.E[0][b] = ex;
        if (w[1]) p.E[1][b] = ey;
        if (w[2]) p.E[2][b] = ez;
      }
    }
    if (__syncthreads_or(ring.timed_out)) break;   // the stage of plane i-1 is free
    if (tid == 0 && i + STAGES - 1 <= blk.ib - 1) {
      fence_proxy_async();
      issue(i + STAGES - 1);
      issued = i + STAGES - 1;
    }
  }
  if (tid == 0) {
    const bool failed = ring.timed_out;
    ring.timed_out = false;
    ring.limit = kItWaitLimit;
    for (int q = waited + 1; q <= issued; ++q) ring.wait(stage_of(q));   // copies still in flight
    if (failed || ring.timed_out) atomicExch(status, static_cast<int>(4));   // XFDTD_ERR_TIMEOUT
  }
}

// The H update of one block (as it_e_block).
template <typename T, typename I, int STAGES, bool CT, int MODE, int KT, bool TF>
__device__ __forceinline__ void it_h_block(const ItMaps &maps, const VolCore<T, I> &p, const InteriorBox &in,
                                           int chunk, int *status, int wait_limit, const TfsfFuse &fz, uint3 bid) {
  using G = ItTiles<T, I, KT>;
  extern __shared__ __align__(128) unsigned char smem[];
  ItRing<STAGES> ring{reinterpret_cast<uint64_t *>(smem + STAGES * G::H_STAGE), wait_limit};
  const int tid = threadIdx.x, c = tid % KT, r = tid / KT;
  const ItBlock blk = it_block<MODE, KT>(in, chunk, bid);
  if (blk.ia >= blk.ib) return;
  auto stage_of = [&](int q) { return (q - blk.ia) % STAGES; };
  auto etile = [&](int st, int comp) { return reinterpret_cast<const T *>(smem + st * G::H_STAGE + comp * G::HE_TILE); };
  auto htile = [&](int st, int comp) {
    return reinterpret_cast<const T *>(smem + st * G::H_STAGE + 3 * G::HE_TILE + comp * G::HH_TILE);
  };
  auto issue = [&](int q) {   // thread 0: the loads of plane q (E only for plane ib)
    const int st = stage_of(q);
    const bool full = q < blk.ib;
    unsigned char *base = smem + st * G::H_STAGE;
    mbar_arrive_expect_tx(&ring.bar[st], full ? G::H_FULL : G::H_EBYTES);
    for (int comp = 0; comp < 3; ++comp)
      tma_load_3d(base + comp * G::HE_TILE, &maps.a[comp], blk.k0, blk.j0, q, &ring.bar[st]);
    if (full) {
      for (int comp = 0; comp < 3; ++comp)
        tma_load_3d(base + 3 * G::HE_TILE + comp * G::HH_TILE, &maps.b[comp], blk.k0, blk.j0, q, &ring.bar[st]);
      if (G::IDX) tma_load_3d(base + 3 * G::HE_TILE + 3 * G::HH_TILE, &maps.idx, blk.k0, blk.j0, q, &ring.bar[st]);
    }
  };
  int issued = blk.ia - 1, waited = blk.ia - 1;   // thread 0: last plane issued, last plane waited
  if (tid == 0) {
    for (int q = 0; q < STAGES; ++q) mbar_init(&ring.bar[q], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    issued = min(blk.ia + STAGES - 1, blk.ib);
    for (int q = blk.ia; q <= issued; ++q) issue(q);
  }
  if (ring.wait(stage_of(blk.ia))) waited = blk.ia;
  const int j = blk.j0 + r, k = blk.k0 + c;
  const bool mine = j <= in.hi[1] && k <= blk.khi;
  const unsigned usj = static_cast<unsigned>(p.d.sj), usi = static_cast<unsigned>(p.d.si);
  SlabCtx<T> cyz = slab_ctx<T, I, 0>(p, 1, 0, 0, 0);
  const bool yspec = MODE != 0 && (j < in.py_lo || j > in.py_hi);
  if (MODE != 0 && mine) {
    if (yspec) slab_axis(p, 1, 1, j, cyz.ys, cyz.Y);
    if (MODE == 2) slab_axis(p, 2, 1, k, cyz.zs, cyz.Z);
  }
  // the incident E arrays of this step (written by the 1-D line beside the E update)
  const auto einc = (MODE != 0 && TF) ? tfsf_view<T>(fz.tf).inc + (*fz.step & 1) * 6 * fz.tf.L : nullptr;
  for (int i = blk.ia; i < blk.ib; ++i) {
    const int cls = MODE == 0 ? 0 : ((i < in.px_lo || i > in.px_hi) ? 1 : 0) | (yspec ? 2 : 0) | (MODE == 2 ? 4 : 0);
    const SlabCtx<T> cx = it_plane_ctx<T, I, MODE>(p, 1, i, cyz);
    PsiOps<T> pv{};
    if (MODE != 0 && mine && cls != 0) pv = h_psi_load<T, I, 7>(p, cx, i, j, k);
    const unsigned b = static_cast<unsigned>(i) * usi + static_cast<unsigned>(j) * usj + static_cast<unsigned>(k);
    const unsigned m_plain = (!G::IDX && mine) ? static_cast<unsigned>(__ldg(p.idx + b)) : 0u;
    if (ring.wait(stage_of(i + 1))) waited = i + 1;
    if (mine && !ring.timed_out) {
      const int st = stage_of(i), sn = stage_of(i + 1);
      auto ev = [&](int s, int comp, int rr, int cc) { return etile(s, comp)[rr * G::EW + cc]; };
      // E at (j, k), (k+1), (j+1) of plane i and at (j, k) of plane i+1
      HCurl<T> e{ev(st, 0, r, c),     ev(st, 1, r, c),     ev(st, 2, r, c),
                       ev(st, 0, r, c + 1), ev(st, 1, r, c + 1), ev(st, 0, r + 1, c),
                       ev(st, 2, r + 1, c), ev(sn, 1, r, c),     ev(sn, 2, r, c)};
      T hx = htile(st, 0)[r * KT + c], hy = htile(st, 1)[r * KT + c], hz = htile(st, 2)[r * KT + c];
      const unsigned m =
          G::IDX ? static_cast<unsigned>(reinterpret_cast<const I *>(smem + st * G::H_STAGE + 3 * G::HE_TILE +
                                                                     3 * G::HH_TILE)[r * KT + c])
                 : m_plain;
      T cf[9];
      coefs<T, I, CT>(p, p.table + 9, 18, m, 1, cf);
      if (MODE != 2 && cls == 0) {
        h_plain(cf, e, hx, hy, hz);
        if (MODE != 0 && TF && tfsf_h_terms(fz.tf, i, j, k)) {
          bool w[3];
          tfsf_h_cell_call<T>(fz.tf, einc, i, j, k, hx, hy, hz, w);
        }
        p.H[0][b] = hx;
        p.H[1][b] = hy;
        p.H[2][b] = hz;
      } else {
        bool w[3];
        if (MODE == 2) {
          if (k >= p.d.nz) e.ex_k = e.ey_k = T(0);
          if (cls == 4) h_general_ops<T, I, 4>(p, cf, i, j, k, e, cx, pv, hx, hy, hz, w);
          else if (cls == 5) h_general_ops<T, I, 5>(p, cf, i, j, k, e, cx, pv, hx, hy, hz, w);
          else if (cls == 6) h_general_ops<T, I, 6>(p, cf, i, j, k, e, cx, pv, hx, hy, hz, w);
          else h_general_ops<T, I, 7>(p, cf, i, j, k, e, cx, pv, hx, hy, hz, w);
        } else if (cls == 1) {
          h_general_ops<T, I, 1>(p, cf, i, j, k, e, cx, pv, hx, hy, hz, w);
        } else if (cls == 2) {
          h_general_ops<T, I, 2>(p, cf, i, j, k, e, cx, pv, hx, hy, hz, w);
        } else {
          h_general_ops<T, I, 3>(p, cf, i, j, k, e, cx, pv, hx, hy, hz, w);
        }
        if (MODE != 0 && TF && tfsf_h_terms(fz.tf, i, j, k)) {
          bool wt[3];
          tfsf_h_cell_call<T>(fz.tf, einc, i, j, k, hx, hy, hz, wt);
          for (int q = 0; q < 3; ++q) w[q] = w[q] || wt[q];
        }
        if (w[0]) p.H[0][b] = hx;
        if (w[1]) p.H[1][b] = hy;
        if (w[2]) p.H[2][b] = hz;
      }
    }
    if (__syncthreads_or(ring.timed_out)) break;   // the stage of plane i is free
    if (tid == 0 && i + STAGES <= blk.ib) {
      fence_proxy_async();
      issue(i + STAGES);
      issued = i + STAGES;
    }
  }
  if (tid == 0) {
    const bool failed = ring.timed_out;
    ring.timed_out = false;
    ring.limit = kItWaitLimit;
    for (int q = waited + 1; q <= issued; ++q) ring.wait(stage_of(q));
    if (failed || ring.timed_out) atomicExch(status, static_cast<int>(4));   // XFDTD_ERR_TIMEOUT
  }
}

template <typename T, typename I, int STAGES, bool CT, int MODE, int KT = kItK, bool TF = false, int MINB = 1>
__global__ void __launch_bounds__(kItThreads, MINB) k_interior_tma_e(const __grid_constant__ ItMaps maps, VolCore<T, I> p,
                                                                     InteriorBox in, int chunk, int *status,
                                                                     int wait_limit, const __grid_constant__ TfsfFuse fz) {
  it_e_block<T, I, STAGES, CT, MODE, KT, TF>(maps, p, in, chunk, status, wait_limit, fz, blockIdx);
}

template <typename T, typename I, int STAGES, bool CT, int MODE, int KT = kItK, bool TF = false, int MINB = 1>
__global__ void __launch_bounds__(kItThreads, MINB) k_interior_tma_h(const __grid_constant__ ItMaps maps, VolCore<T, I> p,
                                                                     InteriorBox in, int chunk, int *status,
                                                                     int wait_limit, const __grid_constant__ TfsfFuse fz) {
  it_h_block<T, I, STAGES, CT, MODE, KT, TF>(maps, p, in, chunk, status, wait_limit, fz, blockIdx);
}

}  // namespace xg
