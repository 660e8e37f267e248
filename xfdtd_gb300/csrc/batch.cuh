// batch.cuh -- kernels that advance many independent simulations at once.
//
// A batch (engine.cu, xfdtd_batch_*) drives several engine handles of
// different grid sizes.  Each phase of a step is one launch over a work
// list of (simulation, tile) items for all simulations still running, one
// block per item.  The volume phases find a block's member from block
// offsets in the launch's parameters; the surface phases read the item
// from a list and load its simulation's parameters into shared memory.
// Per cell the work is that of the single-simulation kernels (e_fast /
// e_shell_cell, h_fast / h_shell_cell, tfsf_e_surface / tfsf_h_surface,
// nffft_sample / nffft_fold, tfsf_aux_block), so a batched simulation gives
// the same bits as the same simulation run alone.
#pragma once

#include "common.cuh"
#include "interior_tma.cuh"
#include "surface.cuh"
#include "volume.cuh"

namespace xg {

// One work item: simulation `sim`, tile `tile` of that simulation's launch
// grid for the phase (a tile is one 256-thread block of the split kernel).
struct WorkItem {
  int sim;
  int tile;
};

// Copies the parameter struct of simulation `sim` into shared memory (all
// threads; returns after a barrier).
template <typename P>
__device__ __forceinline__ void load_params(P &dst, const P *all, int sim) {
  __syncthreads();   // everyone is done with the previous simulation's copy
  const int *src = reinterpret_cast<const int *>(all + sim);
  int *d = reinterpret_cast<int *>(&dst);
  for (int q = threadIdx.x; q < static_cast<int>(sizeof(P) / sizeof(int)); q += blockDim.x) d[q] = src[q];
  __syncthreads();
}

// Volume update (E or H) of each member as in the single-simulation split
// kernels: interior tiles by the fast path, shell cells by the general path
// specialised per box class.  The members' parameters travel in the
// launch's own parameter space, up to kBatchGroup members per launch (a
// group): read there, as in the single-simulation kernels, they take no
// registers until used.
constexpr int kBatchGroup = 64;
template <typename T, typename I>
struct VolGroup {
  VolCore<T, I> m[kBatchGroup];
};
static_assert(sizeof(VolGroup<double, uint32_t>) <= 30000, "a group's parameters fit one launch");

// Blocks of one volume launch per group member: member q owns blocks
// first[q] .. first[q+1]-1 (none when it has stopped).  The member of a
// block follows from blockIdx and these launch parameters alone, so the
// compiler knows it is the same for the whole block.
struct GroupBlocks {
  int n;                          // members in the group
  unsigned first[kBatchGroup + 1];
};

__device__ __forceinline__ int group_member(const GroupBlocks &gb) {
  int lo = 0, hi = gb.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (blockIdx.x >= gb.first[mid]) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Interior: one block per tile of 32 (k) x 8 (j) cells of one plane i of the
// member's interior box, tiles numbered k-block fastest, then j-block,
// then i, counted from the box's k0, lo[1], lo[0].
template <typename T, typename I, bool E_SIDE, bool CT>
__global__ void __launch_bounds__(256, 8) k_interior_batch(const __grid_constant__ VolGroup<T, I> g,
                                                            const __grid_constant__ GroupBlocks gb,
                                                            const InteriorBox *__restrict__ boxes) {
  const int q = group_member(gb);
  const VolCore<T, I> &p = g.m[q];
  const InteriorBox in = boxes[q];
  const unsigned t = blockIdx.x - gb.first[q];
  const unsigned gx = static_cast<unsigned>((in.hi[2] - in.k0) / 32 + 1), gy = static_cast<unsigned>((in.hi[1] - in.lo[1]) / 8 + 1);
  const unsigned t2 = t / gx;
  const int i = in.lo[0] + static_cast<int>(t2 / gy);
  const int j = in.lo[1] + static_cast<int>(t2 % gy) * 8 + static_cast<int>(threadIdx.x >> 5);
  const int k = in.k0 + static_cast<int>(t % gx) * 32 + static_cast<int>(threadIdx.x & 31);
  if (k < in.lo[2] || k > in.hi[2] || j > in.hi[1]) return;
  if (E_SIDE) e_fast<T, I, 1, CT>(p, p.table, 18, i, j, k);
  else h_fast<T, I, 1, CT>(p, p.table + 9, 18, i, j, k);
}

// Shell: the member's shell blocks (numbered as in the single-simulation
// shell kernel).
template <typename T, typename I, bool E_SIDE, bool CT>
__global__ void __launch_bounds__(256, 6) k_shell_batch(const __grid_constant__ VolGroup<T, I> g,
                                                         const __grid_constant__ GroupBlocks gb,
                                                         const ShellBoxes *__restrict__ shells) {
  const int q = group_member(gb);
  int cls, i, j, k;
  if (!shell_cell(shells[q], blockIdx.x - gb.first[q], cls, i, j, k)) return;
  if (E_SIDE) e_shell_cell<T, I, CT>(g.m[q], cls, i, j, k);
  else h_shell_cell<T, I, CT>(g.m[q], cls, i, j, k);
}

// The wide decomposition's TMA-staged launches (interior_tma.cuh) over the
// members whose grids allow them: MODE 1 every plane and row over the
// member's interior k range, MODE 2 its z edges, with the single-simulation
// launches' tiles and arithmetic, so the same bits.  The block's tile is
// block t of the member's own launch grid (k tiles fastest, then j tiles,
// then chunks of `chunk` planes; grids[q] = k tiles, j tiles).  The
// members' tensor maps lie in global memory, written by the host when the
// batch is made; the thread that issues the copies acquires them first.
template <typename T, typename I, int STAGES, bool CT, int MODE, bool E_SIDE>
__global__ void __launch_bounds__(kItThreads, sizeof(T) == 4 ? 5 : 1) k_tma_batch(const __grid_constant__ VolGroup<T, I> g,
                                                          const __grid_constant__ GroupBlocks gb,
                                                          const ItMaps *__restrict__ maps,
                                                          const InteriorBox *__restrict__ boxes,
                                                          const int2 *__restrict__ grids, int *const *__restrict__ status,
                                                          int chunk) {
  const int q = group_member(gb);
  const unsigned t = blockIdx.x - gb.first[q];
  const int2 gd = grids[q];
  const unsigned nk = static_cast<unsigned>(gd.x), nj = static_cast<unsigned>(gd.y);
  const uint3 bid = make_uint3(t % nk, (t / nk) % nj, t / (nk * nj));
  const ItMaps &m = maps[q];
  if (threadIdx.x == 0) {
    for (int c = 0; c < 3; ++c) {
      fence_tensormap_acquire(&m.a[c]);
      fence_tensormap_acquire(&m.b[c]);
    }
    if (ItTiles<T, I, kItK>::IDX) fence_tensormap_acquire(&m.idx);
  }
  const InteriorBox in = boxes[q];
  const TfsfFuse fz{};
  if (E_SIDE)
    it_e_block<T, I, STAGES, CT, MODE, kItK, false>(m, g.m[q], in, chunk, status[q], kItWaitLimit, fz, bid);
  else
    it_h_block<T, I, STAGES, CT, MODE, kItK, false>(m, g.m[q], in, chunk, status[q], kItWaitLimit, fz, bid);
}

// TFSF E or H corrections: one block per work item, tile = 256 consecutive
// surface cells of the item's simulation.
template <typename T, bool E_SIDE>
__global__ void __launch_bounds__(256) k_tfsf_batch(const TfsfSurfParams<T> *__restrict__ all,
                                                    const WorkItem *__restrict__ items) {
  __shared__ TfsfSurfParams<T> p;
  const WorkItem it = items[blockIdx.x];
  load_params(p, all, it.sim);
  const int q = it.tile * 256 + threadIdx.x;
  if (E_SIDE) tfsf_e_surface(p, q);
  else tfsf_h_surface(p, q);
}

// NF-FF surface samples: one block per work item, tile = (face, 32 x 8
// face block), numbered u-block fastest, then v-block, then face; the grid
// of a simulation is that of k_nffft, given by gu x gv per face (ints 0, 1
// of the tile).
template <typename T>
__global__ void __launch_bounds__(256) k_nffft_batch(const NfParams<T> *__restrict__ all, const int2 *__restrict__ grid,
                                                     const WorkItem *__restrict__ items) {
  __shared__ NfParams<T> p;
  const WorkItem it = items[blockIdx.x];
  load_params(p, all, it.sim);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int2 g = grid[it.sim];
  const int bu = it.tile % g.x, bv = (it.tile / g.x) % g.y, face = it.tile / (g.x * g.y);
  nffft_sample(p, face, bu * 32 + tx, bv * 8 + ty);
}

// NF-FF fold of `count` buffered steps: one block per work item, tile =
// (group, 256 face cells), numbered cell block fastest; per simulation nb
// blocks per group.
template <typename T>
__global__ void __launch_bounds__(256) k_nffft_fold_batch(const NfParams<T> *__restrict__ all, const int *__restrict__ nb,
                                                          const WorkItem *__restrict__ items, int count) {
  __shared__ NfParams<T> p;
  const WorkItem it = items[blockIdx.x];
  load_params(p, all, it.sim);
  const int n = nb[it.sim];
  nffft_fold(p, it.tile / n, static_cast<long long>(it.tile % n) * 256 + threadIdx.x, count, 0);
}

// The 1-D incident lines: one block per listed simulation.
__global__ void __launch_bounds__(512) k_tfsf_aux_batch(const AuxParams *__restrict__ all, const int *__restrict__ sims) {
  __shared__ AuxParams p;
  load_params(p, all, sims[blockIdx.x]);
  tfsf_aux_block(p);
}

// Step counters of the listed simulations.
__global__ void k_advance_batch(long long *const *__restrict__ steps, int n) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) *steps[q] += 1;
}

}  // namespace xg
