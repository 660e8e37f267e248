// engine.cu -- C-ABI of the GB300 FDTD engine (include/xfdtd_cuda.h).
//
// One handle = one simulation = one CUDA stream.  xfdtd_create validates the
// plan on the host, allocates every device buffer once and uploads the
// tables; xfdtd_step enqueues the per-step kernel sequence
//
//   k_tfsf_aux (1 block: 1-D incident line)
//   -> k_update_e (Yee E + CPML E, one thread per cell)
//   -> k_lumped_e (sparse) -> k_tfsf_e (TFSF surface E corrections)
//   -> k_update_h (Yee H + CPML H) -> k_tfsf_h (TFSF surface H corrections)
//   -> k_nffft (surface samples into the batch buffer)
//   -> k_nffft_accumulate (every nf_batch steps: DFT fold of the batch)
//   -> k_probes -> k_advance
//
// which is the order of the reference's loop body
// (src/simulation/simulation_update.cpp:13-35), except that the CPML terms
// are added inside the volume kernels, before the lumped and TFSF
// corrections rather than after them.  The two only meet on cells where a
// TFSF face or a lumped element lies inside a CPML slab, where the same
// terms are added in another order.  The step index lives on the device
// (k_advance bumps it), so a captured CUDA graph of G steps (G a multiple of
// the NF-FF batch) replays for any starting step on a batch boundary.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <dlfcn.h>

#include <algorithm>
#include <chrono>
#include <functional>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/xfdtd_cuda.h"
#include "common.cuh"
#include "adjoint.cuh"
#include "batch.cuh"
#include "broadband.cuh"
#include "surface.cuh"
#include "interior_tma.cuh"
#include "sweep.cuh"
#include "volume.cuh"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEps0 = 8.854187817e-12;
constexpr double kMu0 = 4 * kPi * 1e-7;

struct Err {
  int code;
  std::string msg;
};

#define XCHECK(call)                                                                    \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      throw Err{e_ == cudaErrorMemoryAllocation ? XFDTD_ERR_OOM : XFDTD_ERR_CUDA,       \
                std::string(#call) + ": " + cudaGetErrorString(e_)};                    \
  } while (0)

// Profile entries.  update_e / update_h time the whole E / H volume update
// (its interior and shell kernels, which run concurrently on two streams);
// the *_interior and *_shell entries time each kernel on its own stream.
const char *kKernelNames[] = {"tfsf_aux",         "update_e",       "lumped_e",         "update_h",
                              "nffft",            "probes",         "advance",          "tfsf_e",
                              "tfsf_h",           "nffft_acc",      "sweep_eh",         "update_e_shell",
                              "update_h_shell",   "update_e_interior", "update_h_interior", "snapshots",
                              "dispersive_e"};
constexpr int kNumKernels = 17;

}  // namespace

struct AdjointState;
size_t adjoint_bytes(const xfdtd_handle *h);   // device bytes of the handle's adjoint state

struct xfdtd_handle {
  std::string err;
  int device = 0;
  int precision = XFDTD_FP64;
  int idx_bytes = 1;
  int flags = 0;
  xg::Dims d{};
  long long total = 0;
  long long host_step = 0;   // steps enqueued so far
  size_t esize = 8;
  double dl[3] = {0, 0, 0};
  double dt = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;            // the TFSF 1-D line runs here, forked and joined per step
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // NF-FF sampling beside the TFSF H corrections (its reads lie strictly
  // inside the TFSF box, which the corrections' writes surround)
  bool nf_beside_tfsf = false;
  cudaEvent_t ev_nf_fork = nullptr, ev_nf_join = nullptr;
  // split NF-FF sampling (enqueue_step_t): its stream, fork event, the
  // events after the H half (+ fold) and after the E half, and whether the
  // H half of the last stepped step is still to be taken
  cudaStream_t nfs = nullptr;
  cudaEvent_t ev_nfs_fork = nullptr, ev_nfh = nullptr, ev_nfe = nullptr;
  bool nf_pending = false;
  // the split NF-FF schedule (two sampling halves and the batch folds on
  // nfs, beside the volume updates); else one sampling launch after the H
  // update, with the fold on the main stream.  Chosen by the autotuner.
  bool nf_split = true;
  float nf_sched_ms[2] = {0.f, 0.f};   // trial step time split / one launch (0 = not timed)
  cudaStream_t shell = nullptr;           // the volume shell kernels run here, beside the interior kernels
  cudaEvent_t ev_vfork[2] = {}, ev_vjoin[2] = {};
  std::vector<void *> allocs;
  size_t bytes = 0;
  long long h2d = 0, d2h = 0;   // bytes copied host<->device

  void *F[6] = {};
  void *idx = nullptr;
  void *table = nullptr;
  void *ctable = nullptr;   // compact coefficient table (volume.cuh coefs)
  int n_mat = 0;
  bool smem_table = false;
  size_t smem_bytes = 0;

  // CPML
  int L[3] = {0, 0, 0};
  int *slot_e[3] = {}, *slot_h[3] = {};
  uint8_t *axis_flags[3] = {};  // per-axis fast-path flags
  void *prof[3][6] = {};   // b_e a_e rk_e b_m a_m rk_m (precision T)
  void *psi[12] = {};      // ex_y ex_z ey_x ey_z ez_x ez_y hx_y hx_z hy_x hy_z hz_x hz_y
  size_t psi_bytes[12] = {};

  // TFSF
  bool tfsf = false;
  int aux_len = 0;
  int tf_lo[3] = {}, tf_hi[3] = {};
  double *tf_pf[3] = {}, *tf_ph[3] = {};
  double *tf_state = nullptr, *tf_inc = nullptr, *tf_src = nullptr;
  float *tf_pff[3] = {}, *tf_phf[3] = {}, *tf_incf = nullptr;   // FP32 copies (FP32 form)
  double tf_ca[3] = {}, tf_cb[3] = {}, tf_te[3] = {}, tf_th[3] = {};
  double tf_ceihi = 0, tf_chiei = 0, tf_c1 = 0, tf_c2 = 0;

  // NF-FF
  bool nffft = false;
  int nf = 0, nt = 0, np = 0;
  int nf_lo[3] = {}, nf_hi[3] = {};
  double2 *acc[24] = {};
  long long acc_len[24] = {};
  double2 *phase_j = nullptr, *phase_m = nullptr;
  float2 *phase_jf = nullptr, *phase_mf = nullptr;
  double *ff_theta = nullptr, *ff_phi = nullptr, *ff_k = nullptr;
  double2 *ff_out[8] = {};
  double *ff_power[2] = {};
  long long ff_step = -1;

  // sparse
  int n_inj = 0, n_ind = 0, n_probes = 0, n_waveforms = 0;
  // linear dispersive media: the listed E components, their media (in the
  // field precision) and their recursion state J, previous J, previous E
  int n_disp = 0;
  xg::DispCell *disp_cells = nullptr;
  void *disp_media = nullptr;
  void *disp_j = nullptr, *disp_jp = nullptr, *disp_ep = nullptr;
  double disp_dl = 0;
  xfdtd_injection *inj = nullptr;
  xfdtd_inductor_cell *ind = nullptr;
  double *ind_j = nullptr;
  double *waveforms = nullptr;
  xfdtd_probe_term *terms = nullptr;
  int *probe_off = nullptr;
  double *probe_out = nullptr;
  // field snapshot series (host copies of the descriptors, device table)
  std::vector<xg::SnapDev> snaps;
  xg::SnapDev *d_snaps = nullptr;
  long long snap_cells_max = 0;

  long long *d_step = nullptr;
  int *d_status = nullptr;
  int wait_polls = xg::kItWaitLimit;   // polls of a TMA plane wait before a block gives up
  double create_ms[2] = {0, 0};         // xfdtd_create: allocation and upload; autotuning
  int *d_flag = nullptr;

  // host copies kept for the adjoint: the coefficient table (FP64) and the
  // per-axis index flags
  std::vector<double> table_host;
  std::vector<uint8_t> axis_flags_host[3];
  std::shared_ptr<AdjointState> adj;   // set up by xfdtd_adjoint_forward

  // volume-kernel variants (autotuned)
  int var_e = 1, var_h = 1;   // L1-table variant: valid for every plan
  float tune_ms[2][24] = {};
  float tune_step_ms = 0.f;   // the autotuner's last round: the kept pairing's trial step
  // TMA-staged interior kernels (interior_tma.cuh): offered per side when the
  // interior's k range starts on a 16-byte boundary for fields and index
  bool it_ok[2] = {};
  xg::ItMaps itm[2] = {};     // interior launches (32 x 8 tiles), E and H side
  xg::ItMaps itm_z[2] = {};   // z-edge launch (16 x 16 tiles)
  void *itm_base = nullptr;   // E_x buffer the maps were encoded for
  // split volume update, per side (0 E, 1 H): the plain interior box and
  // the shell around it, with their cell counts; shell register cap
  xg::InteriorBox vin[2] = {};
  // wide decomposition (TMA-staged interior over every plane and row of the
  // interior's k range; the shell keeps the z slabs)
  xg::InteriorBox vin_w[2] = {};
  xg::InteriorBox vin_z[2] = {};   // the z slabs of the wide decomposition as TMA tiles
  xg::ShellBoxes vshell_w[2] = {};
  long long vin_w_cells[2] = {}, vshell_w_cells[2] = {};
  bool wide_ok[2] = {};
  xg::ShellBoxes vshell[2] = {};
  long long vin_cells[2] = {}, vshell_cells[2] = {};
  int shell_var[2] = {0, 0};   // shell-kernel variant per side

  // fused E/H sweep (sweep.cuh): the state of step t+1 goes to the second
  // buffer set, swapped with the first after each step
  bool sweep_ok = false;   // the plan allows the sweep (buffers allocated)
  bool tf_two_d = false;   // TFSF2D: Ez, Hx, Hy corrections on the x and y faces only
  // the TFSF corrections may run inside the wide TMA launch (E, H): the
  // surface lies in its k range and no lumped element corrects E first
  bool tf_fuse_ok[2] = {false, false};
  bool tf_fuse_on[2] = {true, true};   // the autotuner's choice between fused and separate corrections
  float tf_fuse_ms[2][2] = {{0, 0}, {0, 0}};   // its trials: fused, separate (ms per pair)
  bool sweep = false;      // the sweep runs
  int cur_set = 0;         // which buffer set (0: allocated as F, 1: as F2) is current
  CUtensorMap tm_h[2][3], tm_e[2][3], tm_idx;   // TMA maps of both sets and the index
  void *F2[6] = {};
  void *psi2[6] = {};         // E psi of the second set (order of psi[0..5])
  int var_s = 1;
  float sweep_ms[8] = {};

  // graph replay
  cudaGraphExec_t gexec = nullptr;
  int graph_steps = 0;
  long long graph_launches = 0;
  long long launch_count = 0;   // per-step kernels enqueued so far

  // NF-FF batching: surface values of up to nf_batch steps are buffered and
  // folded into the accumulators together
  int nf_batch = 8;
  long long nf_done = 0;        // steps already folded
  void *nf_buf[3] = {};
  int nf_rows = 8;              // rows of the sample buffers: nf_batch, or every step (broadband)
  bool nf_bb = false;           // NffftBroadBand: keep every step's samples, no running DFT
  double bb_theta = 0, bb_phi = 0;

  // profiling
  std::vector<cudaEvent_t> ev_pool;
  struct ProfEntry {
    int id;        // kernel id
    int ev;        // event index of the start (end: ev + 1)
    bool closed;   // end event recorded
  };
  std::vector<ProfEntry> ev_pending;
  double prof_ms[kNumKernels] = {};
  long long prof_n[kNumKernels] = {};

  template <class P>
  P *alloc(size_t count) {
    void *p = nullptr;
    size_t nb = std::max<size_t>(count * sizeof(P), 16);
    XCHECK(cudaMalloc(&p, nb));
    allocs.push_back(p);
    bytes += nb;
    XCHECK(cudaMemsetAsync(p, 0, nb, stream));
    return static_cast<P *>(p);
  }
  void *alloc_bytes(size_t nb) {
    void *p = nullptr;
    nb = std::max<size_t>(nb, 16);
    XCHECK(cudaMalloc(&p, nb));
    allocs.push_back(p);
    bytes += nb;
    XCHECK(cudaMemsetAsync(p, 0, nb, stream));
    return p;
  }
  template <class P>
  P *upload(const P *src, size_t count) {
    P *p = alloc<P>(count);
    if (count) XCHECK(cudaMemcpyAsync(p, src, count * sizeof(P), cudaMemcpyHostToDevice, stream));
    h2d += static_cast<long long>(count * sizeof(P));
    return p;
  }
  // upload doubles, converting to the field precision
  void *upload_real(const double *src, size_t count) {
    if (precision == XFDTD_FP64) return upload<double>(src, count);
    std::vector<float> tmp(count);
    for (size_t q = 0; q < count; ++q) tmp[q] = static_cast<float>(src[q]);
    return upload<float>(tmp.data(), count);
  }
  ~xfdtd_handle() {
    if (gexec) cudaGraphExecDestroy(gexec);
    for (auto e : ev_pool) cudaEventDestroy(e);
    for (void *p : allocs) cudaFree(p);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_nf_fork) cudaEventDestroy(ev_nf_fork);
    if (ev_nf_join) cudaEventDestroy(ev_nf_join);
    if (ev_nfs_fork) cudaEventDestroy(ev_nfs_fork);
    if (ev_nfh) cudaEventDestroy(ev_nfh);
    if (ev_nfe) cudaEventDestroy(ev_nfe);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    if (nfs) cudaStreamDestroy(nfs);
    for (int q = 0; q < 2; ++q) {
      if (ev_vfork[q]) cudaEventDestroy(ev_vfork[q]);
      if (ev_vjoin[q]) cudaEventDestroy(ev_vjoin[q]);
    }
    if (shell) cudaStreamDestroy(shell);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

template <class F>
int guarded(xfdtd_handle *h, F &&fn) {
  try {
    if (h && h->stream) XCHECK(cudaSetDevice(h->device));
    fn();
    return XFDTD_OK;
  } catch (const Err &e) {
    if (h) h->err = e.msg;
    return e.code;
  } catch (const std::exception &e) {
    if (h) h->err = e.what();
    return XFDTD_ERR_INVALID_PLAN;
  }
}

void invalid(const std::string &m) { throw Err{XFDTD_ERR_INVALID_PLAN, m}; }

// Calls f(T{}, I{}) with the field type and material-index type of a handle.
template <class F>
void with_types(int precision, int idx_bytes, F &&f) {
  if (precision == XFDTD_FP64) {
    if (idx_bytes == 1) f(double{}, uint8_t{});
    else if (idx_bytes == 2) f(double{}, uint16_t{});
    else f(double{}, uint32_t{});
  } else {
    if (idx_bytes == 1) f(float{}, uint8_t{});
    else if (idx_bytes == 2) f(float{}, uint16_t{});
    else f(float{}, uint32_t{});
  }
}

// ------------------------------------------------------------ launches ---
void prof_region_begin(xfdtd_handle *h, int id, cudaStream_t st = nullptr) {
  if (!(h->flags & XFDTD_FLAG_PROFILE)) return;
  size_t need = h->ev_pending.size() * 2 + 2;
  while (h->ev_pool.size() < need) {
    cudaEvent_t e;
    XCHECK(cudaEventCreate(&e));
    h->ev_pool.push_back(e);
  }
  int s = static_cast<int>(h->ev_pending.size() * 2);
  XCHECK(cudaEventRecord(h->ev_pool[s], st ? st : h->stream));
  h->ev_pending.push_back({id, s, false});
}
// Ends the innermost open entry (entries nest: an entry opened after another
// closes first).
void prof_end(xfdtd_handle *h, cudaStream_t st = nullptr) {
  if (!(h->flags & XFDTD_FLAG_PROFILE)) return;
  for (auto it = h->ev_pending.rbegin(); it != h->ev_pending.rend(); ++it)
    if (!it->closed) {
      it->closed = true;
      XCHECK(cudaEventRecord(h->ev_pool[it->ev + 1], st ? st : h->stream));
      return;
    }
}
// One kernel launch: counted, and timed under XFDTD_FLAG_PROFILE.
void prof_begin(xfdtd_handle *h, int id, cudaStream_t st = nullptr) {
  h->launch_count += 1;   // every per-step kernel launch passes here
  prof_region_begin(h, id, st);
}
void prof_collect(xfdtd_handle *h) {
  if (h->ev_pending.empty()) return;
  XCHECK(cudaStreamSynchronize(h->stream));
  for (auto &pr : h->ev_pending) {
    float ms = 0;
    XCHECK(cudaEventElapsedTime(&ms, h->ev_pool[pr.ev], h->ev_pool[pr.ev + 1]));
    h->prof_ms[pr.id] += ms;
    h->prof_n[pr.id] += 1;
  }
  h->ev_pending.clear();
}

template <typename T, typename I>
xg::VolParams<T, I> vol_params(xfdtd_handle *h) {
  xg::VolParams<T, I> p{};
  p.d = h->d;
  for (int c = 0; c < 3; ++c) {
    p.E[c] = static_cast<T *>(h->F[c]);
    p.H[c] = static_cast<T *>(h->F[3 + c]);
  }
  p.idx = static_cast<const I *>(h->idx);
  p.table = static_cast<const T *>(h->table);
  p.ctable = static_cast<const T *>(h->ctable);
  p.n_mat = h->n_mat;
  for (int a = 0; a < 3; ++a) {
    p.cp[a].n_layers = h->L[a];
    p.cp[a].slot_e = h->slot_e[a];
    p.cp[a].slot_h = h->slot_h[a];
    p.cp[a].b_e = static_cast<const T *>(h->prof[a][0]);
    p.cp[a].a_e = static_cast<const T *>(h->prof[a][1]);
    p.cp[a].rk_e = static_cast<const T *>(h->prof[a][2]);
    p.cp[a].b_m = static_cast<const T *>(h->prof[a][3]);
    p.cp[a].a_m = static_cast<const T *>(h->prof[a][4]);
    p.cp[a].rk_m = static_cast<const T *>(h->prof[a][5]);
    p.dl[a] = static_cast<T>(h->dl[a]);
  }
  T **ps = reinterpret_cast<T **>(&p.psi);
  for (int q = 0; q < 12; ++q) ps[q] = static_cast<T *>(h->psi[q]);
  p.tf.enabled = h->tfsf ? 1 : 0;
  p.tf.two_d = h->tf_two_d ? 1 : 0;
  p.tf.L = h->aux_len;
  for (int a = 0; a < 3; ++a) {
    p.tf.lo[a] = h->tf_lo[a];
    p.tf.hi[a] = h->tf_hi[a];
    p.tf.pf[a] = h->tf_pf[a];
    p.tf.ph[a] = h->tf_ph[a];
    p.tf.ca[a] = h->tf_ca[a];
    p.tf.cb[a] = h->tf_cb[a];
    p.tf.pff[a] = h->tf_pff[a];
    p.tf.phf[a] = h->tf_phf[a];
    p.tf.caf[a] = static_cast<float>(h->tf_ca[a]);
    p.tf.cbf[a] = static_cast<float>(h->tf_cb[a]);
  }
  p.tf.inc = h->tf_inc;
  p.tf.incf = h->tf_incf;
  p.step = h->d_step;
  for (int a = 0; a < 3; ++a) p.flags[a] = h->axis_flags[a];
  return p;
}

// Volume-kernel variants the autotuner chooses from.  A variant fixes the
// register cap (the minimum number of resident 256-thread blocks per SM
// asked of the register allocator; 1 = none), the block shape (k fastest,
// 32..128 along k for 128..512-byte rows), the cells per thread along i
// (1 or 2) and where the coefficient table lives (shared memory, filled per
// block behind a barrier, or read through L1).  Every variant computes the
// same per-cell arithmetic, so all give identical bits.
struct Variant {
  int minb;
  int bx, by, bz;
  int nc;
  bool smem;
  bool ct;      // coefficients from the compact table (volume.cuh coefs)
  int stages;   // TMA-staged kernel (interior_tma.cuh): ring stages, 0 = not staged
  int chunk;    //   and planes per block
  bool wide;    //   over the wide decomposition (the shell keeps the z slabs only)
};
constexpr Variant kVariants[] = {
    {8, 32, 4, 2, 1, true, false},   {8, 32, 4, 2, 1, false, false}, {8, 32, 8, 1, 1, false, false},
    {8, 64, 4, 1, 1, false, false},  {8, 128, 2, 1, 1, false, false}, {6, 32, 4, 2, 2, false, false},
    {6, 32, 8, 1, 2, false, false},  {6, 64, 4, 1, 2, false, false},  {1, 32, 4, 2, 2, false, false},
    {1, 32, 4, 2, 1, false, false},  {8, 32, 4, 2, 2, false, false},  {6, 32, 4, 2, 1, true, false},
    {8, 32, 4, 2, 1, false, true},   {8, 32, 8, 1, 1, false, true},   {1, 32, 4, 2, 1, false, true},
    {6, 32, 4, 2, 1, true, true},
    {0, 32, 8, 1, 1, false, false, 4, 16}, {0, 32, 8, 1, 1, false, false, 6, 16},
    {0, 32, 8, 1, 1, false, false, 4, 32}, {0, 32, 8, 1, 1, false, true, 4, 16},
    {0, 32, 8, 1, 1, false, false, 4, 16, true}, {0, 32, 8, 1, 1, false, false, 6, 16, true},
    {0, 32, 8, 1, 1, false, true, 4, 16, true},
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);
static_assert(kNumVariants <= 24, "tune_ms holds 24 variants per side");

// A shared-memory-table variant needs the table to fit (smem_table); a
// TMA-staged one an aligned interior on both sides (it_ok), a wide one the
// wide decomposition on both sides too.
bool variant_allowed(const xfdtd_handle *h, const Variant &v) {
  return (!v.smem || h->smem_table) && (!v.stages || (h->it_ok[0] && h->it_ok[1])) &&
         (!v.wide || (h->wide_ok[0] && h->wide_ok[1]));
}

// The decomposition a side runs with its current variant: narrow (the
// interior box and the shell around it) or wide.
bool side_wide(const xfdtd_handle *h, int side) { return kVariants[side == 0 ? h->var_e : h->var_h].wide; }
const xg::InteriorBox &side_interior(const xfdtd_handle *h, int side, bool wide) {
  return wide ? h->vin_w[side] : h->vin[side];
}
const xg::ShellBoxes &side_shell(const xfdtd_handle *h, int side, bool wide) {
  return wide ? h->vshell_w[side] : h->vshell[side];
}
long long side_interior_cells(const xfdtd_handle *h, int side, bool wide) {
  return wide ? h->vin_w_cells[side] : h->vin_cells[side];
}
long long side_shell_cells(const xfdtd_handle *h, int side, bool wide) {
  return wide ? h->vshell_w_cells[side] : h->vshell_cells[side];
}

template <typename T, typename I, bool S, int MB, int NC, bool CT>
void launch_vol_v(xfdtd_handle *h, const xg::VolParams<T, I> &p, bool e_side, const Variant &v) {
  xg::InteriorBox in = h->vin[e_side ? 0 : 1];
  in.k0 = (in.lo[2] / v.bx) * v.bx;   // rows of threads start on the block's k alignment
  const int nk = in.hi[2] - in.k0 + 1, nj = in.hi[1] - in.lo[1] + 1, ni = in.hi[0] - in.lo[0] + 1;
  const int zc = v.bz * NC;
  dim3 block(v.bx, v.by, v.bz);
  dim3 grid((nk + v.bx - 1) / v.bx, (nj + v.by - 1) / v.by, (ni + zc - 1) / zc);
  const size_t smem = S ? h->smem_bytes : 0;
  if (e_side) xg::k_update_e<T, I, S, MB, NC, CT><<<grid, block, smem, h->stream>>>(p, in);
  else xg::k_update_h<T, I, S, MB, NC, CT><<<grid, block, smem, h->stream>>>(p, in);
}


// Shell-kernel variants the autotuner chooses from: register cap (minimum
// resident 256-thread blocks per SM) and table form (compact or full); or,
// for the wide decomposition only, the z-edge TMA launch (interior_tma.cuh
// mode 2) with its ring stages and planes per block.
struct ShellVariant {
  int minb;
  bool ct;
  int stages;   // 0 = the shell kernel
  int chunk;
  int kt;       // tile width along k of the z-edge launch: 32 (x 8 rows) or 16 (x 16 rows)
};
// (8 and 4 planes per block measured slower on the 280^3 dielectric sphere.)
// The z-edge variants with minb 5 cap the launch at 5 blocks per SM (48
// registers a thread).
constexpr ShellVariant kShellVariants[] = {{4, false},           {6, false},           {4, true},
                                           {6, true},            {0, false, 4, 16, 32}, {0, false, 6, 16, 32},
                                           {0, true, 4, 16, 32}, {0, false, 4, 16, 16}, {0, false, 6, 16, 16},
                                           {0, true, 4, 16, 16}, {5, false, 4, 16, 32}, {5, false, 4, 16, 16}};
constexpr int kNumShellVariants = sizeof(kShellVariants) / sizeof(kShellVariants[0]);

// A z-edge TMA variant runs on the wide decomposition only.
bool shell_allowed(const xfdtd_handle *h, const ShellVariant &v, bool wide) {
  return !v.stages || (wide && h->it_ok[0] && h->it_ok[1] && h->wide_ok[0] && h->wide_ok[1]);
}

// Whether the side's TFSF corrections run inside its wide decomposition's
// launches this step: the plan allows it (tf_fuse_ok, set at create), the
// autotuner kept it (tf_fuse_on) and the side runs the wide decomposition
// with the split kernels.
bool tfsf_fused(const xfdtd_handle *h, int side) {
  if (!(h->tfsf && h->tf_fuse_ok[side] && h->tf_fuse_on[side] && !h->sweep && side_wide(h, side))) return false;
  // both launches of the wide decomposition are TMA-staged: the interior
  // launch and, where there are z slabs, the z-edge launch
  return side_shell_cells(h, side, true) == 0 || kShellVariants[h->shell_var[side]].stages != 0;
}


template <typename T, typename I, int MB, bool CT>
void launch_shell_v(xfdtd_handle *h, bool e_side, const xg::ShellBoxes &s, cudaStream_t st) {
  const auto p = vol_params<T, I>(h);
  if (e_side) xg::k_update_e_shell<T, I, MB, CT><<<s.blocks, 256, 0, st>>>(p, s);
  else xg::k_update_h_shell<T, I, MB, CT><<<s.blocks, 256, 0, st>>>(p, s);
}

template <typename T, typename I, int S, bool CT, int MODE, int KT = xg::kItK, int MINB = 1>
void launch_vol_tma(xfdtd_handle *h, const xg::VolParams<T, I> &p, bool e_side, int chunk, cudaStream_t st);

// The shell kernel of one side over the decomposition of its current
// variant (wide: 0 narrow, 1 wide, -1 the current one).
template <typename T, typename I>
void launch_shell(xfdtd_handle *h, bool e_side, int var = -1, cudaStream_t st = nullptr, int wide = -1) {
  const int side = e_side ? 0 : 1;
  const xg::ShellBoxes &s = side_shell(h, side, wide < 0 ? side_wide(h, side) : wide != 0);
  if (s.blocks == 0) return;
  if (var < 0) var = h->shell_var[side];
  const ShellVariant &v = kShellVariants[var];
  if (!st) st = h->stream;
  if (v.stages) {
    if (&s != &h->vshell_w[side]) throw Err{XFDTD_ERR_STATE, "z-edge TMA launch outside the wide decomposition"};
    auto p = vol_params<T, I>(h);
    if (v.minb == 5) {
      if (v.kt == xg::kItKz) launch_vol_tma<T, I, 4, false, 2, xg::kItKz, 5>(h, p, e_side, v.chunk, st);
      else launch_vol_tma<T, I, 4, false, 2, xg::kItK, 5>(h, p, e_side, v.chunk, st);
    } else if (v.kt == xg::kItKz) {
      if (v.stages == 6) launch_vol_tma<T, I, 6, false, 2, xg::kItKz>(h, p, e_side, v.chunk, st);
      else if (v.ct) launch_vol_tma<T, I, 4, true, 2, xg::kItKz>(h, p, e_side, v.chunk, st);
      else launch_vol_tma<T, I, 4, false, 2, xg::kItKz>(h, p, e_side, v.chunk, st);
    } else {
      if (v.stages == 6) launch_vol_tma<T, I, 6, false, 2>(h, p, e_side, v.chunk, st);
      else if (v.ct) launch_vol_tma<T, I, 4, true, 2>(h, p, e_side, v.chunk, st);
      else launch_vol_tma<T, I, 4, false, 2>(h, p, e_side, v.chunk, st);
    }
  } else if (v.minb == 6) {
    if (v.ct) launch_shell_v<T, I, 6, true>(h, e_side, s, st);
    else launch_shell_v<T, I, 6, false>(h, e_side, s, st);
  } else {
    if (v.ct) launch_shell_v<T, I, 4, true>(h, e_side, s, st);
    else launch_shell_v<T, I, 4, false>(h, e_side, s, st);
  }
  XCHECK(cudaGetLastError());
}

// The compact coefficient table (volume.cuh coefs): per material and side
// (E: coefficients 0..8, H: 9..17) c0, c1, c2 and a flag, 0 when the
// side's three components share their coefficients bit for bit in the
// field precision (c0 = c3 = c6, c1 = c4 = c7, c2 = c5 = c8), else 1.
template <typename T>
void *compact_table_t(xfdtd_handle *h, const double *table, int n_mat) {
  std::vector<T> ct(static_cast<size_t>(n_mat) * 8, T(0));
  for (int m = 0; m < n_mat; ++m)
    for (int half = 0; half < 2; ++half) {
      T c[9];
      for (int q = 0; q < 9; ++q) c[q] = static_cast<T>(table[static_cast<size_t>(m) * XFDTD_N_COEFF + 9 * half + q]);
      bool same = true;
      for (int t = 0; t < 3; ++t)
        same = same && std::memcmp(&c[t], &c[t + 3], sizeof(T)) == 0 && std::memcmp(&c[t], &c[t + 6], sizeof(T)) == 0;
      T *o = ct.data() + static_cast<size_t>(m) * 8 + 4 * half;
      o[0] = c[0];
      o[1] = c[1];
      o[2] = c[2];
      o[3] = same ? T(0) : T(1);
    }
  return h->upload<T>(ct.data(), ct.size());
}
void *compact_table(xfdtd_handle *h, const double *table, int n_mat) {
  return h->precision == XFDTD_FP64 ? compact_table_t<double>(h, table, n_mat) : compact_table_t<float>(h, table, n_mat);
}

// Multiply-shift constants for dividing n < 2^31 by d (Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994:
// with l = ceil(log2 d) and sh = 31 + l, m = ceil(2^sh / d) gives
// floor(n / d) = (n m) >> sh for every n < 2^31).
void div_constants(unsigned d, unsigned long long &m, int &sh) {
  int l = 0;
  while ((1ull << l) < d) ++l;
  sh = 31 + l;
  m = ((1ull << sh) + d - 1) / d;
}

// The plain box of one side (kSpecialE, or kSpecialH, clear on all three
// axes: no outer wall, no CPML slab) and the shell around it.  Per axis the
// indices split into the plain run P and the special ones S (below and
// above P).  Along k, P is narrowed to whole 128-byte lines of a row (on
// short rows to 32-byte sectors), so that the rows of every box start on a
// line and the interior kernel's warps each cover one line (the cells it
// gives up are plain cells of the shell, where the general path gives the
// same bits).  The shell is S x P x P, P x S x P, P x P x S (faces, one
// special axis), S x P x S, P x S x S (edges) and S x S x all (edges along
// z with the corners); a box that is S along k numbers the cells below and
// above P of one row together.  Without one contiguous plain run on every
// axis there is no interior and the shell is the whole component box.
void volume_boxes(xfdtd_handle *h, int side) {
  const uint8_t bit = side == 0 ? xg::kSpecialE : xg::kSpecialH;
  const int n[3] = {h->d.nx, h->d.ny, h->d.nz};
  int lo[3], hi[3];
  bool run[3];
  for (int a = 0; a < 3; ++a) {
    const std::vector<uint8_t> &fl = h->axis_flags_host[a];
    lo[a] = 0;
    while (lo[a] <= n[a] && (fl[lo[a]] & bit)) ++lo[a];
    hi[a] = n[a];
    while (hi[a] >= lo[a] && (fl[hi[a]] & bit)) --hi[a];
    run[a] = lo[a] <= hi[a];
    for (int q = lo[a]; q <= hi[a]; ++q)
      if (fl[q] & bit) run[a] = false;
  }
  const int px_lo = lo[0], px_hi = hi[0], py_lo = lo[1], py_hi = hi[1];
  // cut on 128-byte lines, else (a short run) on 32-byte sectors, else not at all
  for (int bytes : {128, 32}) {
    const int q = bytes / static_cast<int>(h->esize);
    const int l = (lo[2] + q - 1) / q * q, u = (hi[2] + 1) / q * q - 1;
    if (l <= u) {
      lo[2] = l;
      hi[2] = u;
      break;
    }
  }
  // the 2-D grid (nz = 1) runs as shell boxes only: their cells are
  // numbered k fastest over the short rows, where an interior launch would
  // give each 32-wide row of threads one cell
  const bool interior = run[0] && run[1] && run[2] && n[2] > 1;
  // ranges per axis: 0 = below the plain run, 1 = the plain run, 2 = above,
  // 3 = all, 4 = below and above (k only: the row's two parts together)
  auto add = [&](xg::ShellBoxes &s, unsigned &blocks, long long &total, int ri, int rj, int rk, int cls) {
    const int r[3] = {ri, rj, rk};
    int r0[3], ext[3], ksplit = 0, kgap = 0;
    for (int a = 0; a < 3; ++a) {
      if (r[a] == 0) r0[a] = 0, ext[a] = lo[a];
      else if (r[a] == 1) r0[a] = lo[a], ext[a] = hi[a] - lo[a] + 1;
      else if (r[a] == 2) r0[a] = hi[a] + 1, ext[a] = n[a] - hi[a];
      else if (r[a] == 3) r0[a] = 0, ext[a] = n[a] + 1;
      else r0[a] = 0, ext[a] = lo[a] + n[a] - hi[a];
      if (ext[a] <= 0) return;
    }
    if (rk == 4) {
      ksplit = lo[2];
      kgap = hi[2] + 1 - lo[2];
    } else {
      ksplit = ext[2];
    }
    if (s.n == xg::kMaxShellBoxes) throw Err{XFDTD_ERR_STATE, "shell box table full"};
    xg::ShellBox &b = s.b[s.n++];
    long long cells = 1;
    for (int a = 0; a < 3; ++a) {
      b.lo[a] = r0[a];
      b.ext[a] = ext[a];
      cells *= ext[a];
    }
    if (cells >= (1ll << 31)) throw Err{XFDTD_ERR_INVALID_PLAN, "CPML shell box above 2^31 cells"};
    b.ksplit = ksplit;
    b.kgap = kgap;
    b.cells = static_cast<unsigned>(cells);
    b.cls = cls;
    div_constants(static_cast<unsigned>(b.ext[2]), b.m2, b.sh2);
    div_constants(static_cast<unsigned>(b.ext[1]), b.m1, b.sh1);
    b.block0 = blocks;
    blocks += static_cast<unsigned>((cells + 255) / 256);
    total += cells;
  };

  // narrow: the interior box P x P x P, the shell around it
  {
    xg::InteriorBox &in = h->vin[side];
    xg::ShellBoxes &s = h->vshell[side];
    s = xg::ShellBoxes{};
    long long total = 0;
    unsigned blocks = 0;
    in = xg::InteriorBox{};
    if (!interior) {
      for (int a = 0; a < 3; ++a) {
        in.lo[a] = 0;
        in.hi[a] = -1;
      }
      add(s, blocks, total, 3, 3, 3, 7);
      h->vin_cells[side] = 0;
    } else {
      for (int a = 0; a < 3; ++a) {
        in.lo[a] = lo[a];
        in.hi[a] = hi[a];
      }
      in.px_lo = in.lo[0], in.px_hi = in.hi[0], in.py_lo = in.lo[1], in.py_hi = in.hi[1];
      in.pz_lo = in.lo[2], in.pz_hi = in.hi[2];
      for (int r : {0, 2}) {
        add(s, blocks, total, r, 1, 1, 1);   // x faces
        add(s, blocks, total, 1, r, 1, 2);   // y faces
      }
      add(s, blocks, total, 1, 1, 4, 4);     // z faces
      for (int r : {0, 2}) {
        add(s, blocks, total, r, 1, 4, 5);   // x-z edges
        add(s, blocks, total, 1, r, 4, 6);   // y-z edges
        for (int q : {0, 2}) add(s, blocks, total, r, q, 3, 7);   // x-y edges with the corners
      }
      h->vin_cells[side] = static_cast<long long>(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
    }
    s.blocks = blocks;
    h->vshell_cells[side] = total;
  }

  // wide (TMA-staged interior only): every plane and row over the interior's
  // k range, the plain x and y runs marking the planes and rows of the fast
  // path; the shell keeps the z slabs, by the x and y class of their rows
  {
    xg::InteriorBox &in = h->vin_w[side];
    xg::ShellBoxes &s = h->vshell_w[side];
    s = xg::ShellBoxes{};
    in = xg::InteriorBox{};
    long long total = 0;
    unsigned blocks = 0;
    h->wide_ok[side] = interior;
    if (interior) {
      in.lo[0] = 0, in.hi[0] = n[0];
      in.lo[1] = 0, in.hi[1] = n[1];
      in.lo[2] = lo[2], in.hi[2] = hi[2];
      in.px_lo = px_lo, in.px_hi = px_hi, in.py_lo = py_lo, in.py_hi = py_hi;
      in.pz_lo = lo[2], in.pz_hi = hi[2];
      // the same cells as the z slabs, for the z-edge TMA launch
      xg::InteriorBox &z = h->vin_z[side];
      z = in;
      z.lo[2] = 0;
      z.hi[2] = n[2];
      add(s, blocks, total, 1, 1, 4, 4);     // z faces
      for (int r : {0, 2}) {
        add(s, blocks, total, r, 1, 4, 5);   // x-z edges
        add(s, blocks, total, 1, r, 4, 6);   // y-z edges
        for (int q : {0, 2}) add(s, blocks, total, r, q, 4, 7);   // corners
      }
      h->vin_w_cells[side] = static_cast<long long>(n[0] + 1) * (n[1] + 1) * (hi[2] - lo[2] + 1);
    }
    s.blocks = blocks;
    h->vshell_w_cells[side] = total;
  }
}

// Fused-sweep variants: register cap (minimum resident 256-thread blocks
// per SM) and planes per block along i.
struct SweepVariant {
  int minb;
  int chunk;
};
constexpr SweepVariant kSweepVariants[] = {{1, 32}, {2, 32}, {3, 32}, {4, 32}, {2, 16}, {4, 16}, {2, 64}, {4, 64}};
constexpr int kNumSweepVariants = sizeof(kSweepVariants) / sizeof(kSweepVariants[0]);

template <typename T, typename I>
void launch_sweep(xfdtd_handle *h, int var = -1) {
  using G = xg::SweepTiles<T, I>;
  if (var < 0) var = h->var_s;
  const SweepVariant &v = kSweepVariants[var];
  xg::SweepParams<T, I> f{};
  f.v = vol_params<T, I>(h);
  for (int c = 0; c < 3; ++c) {
    f.E2[c] = static_cast<T *>(h->F2[c]);
    f.H2[c] = static_cast<T *>(h->F2[3 + c]);
  }
  T **ps = reinterpret_cast<T **>(&f.psi2);
  for (int q = 0; q < 6; ++q) ps[q] = static_cast<T *>(h->psi2[q]);
  f.chunk = v.chunk;
  f.status = h->d_status;
  xg::SweepMaps m;
  for (int c = 0; c < 3; ++c) {
    m.h[c] = h->tm_h[h->cur_set][c];
    m.e[c] = h->tm_e[h->cur_set][c];
  }
  m.idx = h->tm_idx;
  dim3 block(xg::kSwK, xg::kSwJ, 1);
  dim3 grid((h->d.nz + xg::kSwK) / xg::kSwK, (h->d.ny + xg::kSwJ) / xg::kSwJ, (h->d.nx + v.chunk) / v.chunk);
  switch (v.minb) {
    case 1: xg::k_sweep<T, I, 1><<<grid, block, G::SMEM, h->stream>>>(m, f); break;
    case 2: xg::k_sweep<T, I, 2><<<grid, block, G::SMEM, h->stream>>>(m, f); break;
    case 3: xg::k_sweep<T, I, 3><<<grid, block, G::SMEM, h->stream>>>(m, f); break;
    default: xg::k_sweep<T, I, 4><<<grid, block, G::SMEM, h->stream>>>(m, f); break;
  }
  XCHECK(cudaGetLastError());
}

template <typename T, typename I>
void sweep_smem_attr() {
  const int bytes = xg::SweepTiles<T, I>::SMEM;
  XCHECK(cudaFuncSetAttribute(xg::k_sweep<T, I, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  XCHECK(cudaFuncSetAttribute(xg::k_sweep<T, I, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  XCHECK(cudaFuncSetAttribute(xg::k_sweep<T, I, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  XCHECK(cudaFuncSetAttribute(xg::k_sweep<T, I, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

// cuTensorMapEncodeTiled, from the driver through the runtime (no link to libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    XCHECK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !ptr) throw Err{XFDTD_ERR_CUDA, "cuTensorMapEncodeTiled is not available"};
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  }
  return fn;
}

// A 3-D tiled map over one padded field (or index) array: dims (nzp, ny+1,
// nx+1), box (box_x, box_y, 1); out-of-range box parts read as zero.
void encode_map(xfdtd_handle *h, CUtensorMap *m, void *base, CUtensorMapDataType dt, size_t esize, unsigned box_x,
                unsigned box_y) {
  const cuuint64_t dims[3] = {static_cast<cuuint64_t>(h->d.nzp), static_cast<cuuint64_t>(h->d.ny + 1),
                              static_cast<cuuint64_t>(h->d.nx + 1)};
  const cuuint64_t strides[2] = {static_cast<cuuint64_t>(h->d.nzp) * esize,
                                 static_cast<cuuint64_t>(h->d.nzp) * (h->d.ny + 1) * esize};
  const cuuint32_t box[3] = {box_x, box_y, 1};
  const cuuint32_t elem[3] = {1, 1, 1};
  const CUresult r = tensor_map_encoder()(m, dt, 3, base, dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Err{XFDTD_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string(static_cast<int>(r))};
}

template <typename T, typename I>
void sweep_setup(xfdtd_handle *h) {
  using G = xg::SweepTiles<T, I>;
  const CUtensorMapDataType dt = sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  for (int c = 0; c < 3; ++c) {
    encode_map(h, &h->tm_h[0][c], h->F[3 + c], dt, sizeof(T), G::HW, xg::kHJ);
    encode_map(h, &h->tm_h[1][c], h->F2[3 + c], dt, sizeof(T), G::HW, xg::kHJ);
    encode_map(h, &h->tm_e[0][c], h->F[c], dt, sizeof(T), G::EW, xg::kEJ);
    encode_map(h, &h->tm_e[1][c], h->F2[c], dt, sizeof(T), G::EW, xg::kEJ);
  }
  encode_map(h, &h->tm_idx, h->idx, sizeof(I) == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16,
             sizeof(I), G::IW, xg::kEJ);
  sweep_smem_attr<T, I>();
}

// Tensor maps of the TMA-staged interior kernels over the current buffers:
// E kernel H tiles (HW x 9 rows), E and index tiles (32 x 8); H kernel E
// tiles (EW x 9 rows), H and index tiles.
// The maps of the interior launches (32 x 8 tiles: itm) and of the z-edge
// launch (16 x 16 tiles: itm_z).
template <typename T, typename I>
void interior_tma_encode(xfdtd_handle *h) {
  const CUtensorMapDataType dt = sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  const CUtensorMapDataType it = sizeof(I) == 1   ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                 : sizeof(I) == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16
                                                  : CU_TENSOR_MAP_DATA_TYPE_UINT32;
  auto encode = [&](xg::ItMaps *m, auto geom) {
    using G = decltype(geom);
    constexpr unsigned KT = static_cast<unsigned>(xg::kItThreads / G::J);
    for (int c = 0; c < 3; ++c) {
      encode_map(h, &m[0].a[c], h->F[3 + c], dt, sizeof(T), G::HW, G::J + 1);
      encode_map(h, &m[0].b[c], h->F[c], dt, sizeof(T), KT, G::J);
      encode_map(h, &m[1].a[c], h->F[c], dt, sizeof(T), G::EW, G::J + 1);
      encode_map(h, &m[1].b[c], h->F[3 + c], dt, sizeof(T), KT, G::J);
    }
    if (G::IDX)
      for (int side = 0; side < 2; ++side) encode_map(h, &m[side].idx, h->idx, it, sizeof(I), KT, G::J);
  };
  encode(h->itm, xg::ItTiles<T, I, xg::kItK>{});
  encode(h->itm_z, xg::ItTiles<T, I, xg::kItKz>{});
  h->itm_base = h->F[0];
}

// Which sides may run the TMA-staged interior kernels: the interior's first
// k (and, for the E kernel, its H tile's first column) on a 16-byte
// boundary for the fields; for the wide decomposition, the same of its k
// range and of the k after its last (where the z-edge launch's upper tiles
// start).  The material index is read with plain loads.
template <typename T, typename I>
void interior_tma_setup(xfdtd_handle *h) {
  using G = xg::ItTiles<T, I, xg::kItK>;
  using Gz = xg::ItTiles<T, I, xg::kItKz>;
  const int es = static_cast<int>(sizeof(T)), is = static_cast<int>(sizeof(I));
  for (int side = 0; side < 2; ++side) {
    const int k = h->vin[side].lo[2], kh = side == 0 ? k - G::HOFF - 1 : k;
    h->it_ok[side] = h->vin_cells[side] > 0 && kh >= 0 && (k * es) % 16 == 0 && (kh * es) % 16 == 0 &&
                     (k * is) % 16 == 0;
  }
  if (!(h->it_ok[0] && h->it_ok[1])) return;
  interior_tma_encode<T, I>(h);
  auto attr = [](auto kern, int bytes) {
    XCHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  };
  auto attrs = [&](auto mode, auto kt) {
    constexpr int M = decltype(mode)::value;
    constexpr int KT = decltype(kt)::value;
    using GG = xg::ItTiles<T, I, KT>;
    attr(xg::k_interior_tma_e<T, I, 4, false, M, KT>, GG::template smem_e<4>());
    attr(xg::k_interior_tma_e<T, I, 6, false, M, KT>, GG::template smem_e<6>());
    attr(xg::k_interior_tma_e<T, I, 4, true, M, KT>, GG::template smem_e<4>());
    attr(xg::k_interior_tma_h<T, I, 4, false, M, KT>, GG::template smem_h<4>());
    attr(xg::k_interior_tma_h<T, I, 6, false, M, KT>, GG::template smem_h<6>());
    attr(xg::k_interior_tma_h<T, I, 4, true, M, KT>, GG::template smem_h<4>());
    if constexpr (M != 0) {   // the wide decomposition's launches with the TFSF corrections
      attr(xg::k_interior_tma_e<T, I, 4, false, M, KT, true>, GG::template smem_e<4>());
      attr(xg::k_interior_tma_e<T, I, 6, false, M, KT, true>, GG::template smem_e<6>());
      attr(xg::k_interior_tma_e<T, I, 4, true, M, KT, true>, GG::template smem_e<4>());
      attr(xg::k_interior_tma_h<T, I, 4, false, M, KT, true>, GG::template smem_h<4>());
      attr(xg::k_interior_tma_h<T, I, 6, false, M, KT, true>, GG::template smem_h<6>());
      attr(xg::k_interior_tma_h<T, I, 4, true, M, KT, true>, GG::template smem_h<4>());
    }
    if constexpr (M == 1 && sizeof(T) == 4) {   // the wide launches capped at 5 blocks per SM (FP32)
      attr(xg::k_interior_tma_e<T, I, 4, false, M, KT, false, 5>, GG::template smem_e<4>());
      attr(xg::k_interior_tma_h<T, I, 4, false, M, KT, false, 5>, GG::template smem_h<4>());
      attr(xg::k_interior_tma_e<T, I, 4, true, M, KT, false, 5>, GG::template smem_e<4>());
      attr(xg::k_interior_tma_h<T, I, 4, true, M, KT, false, 5>, GG::template smem_h<4>());
      attr(xg::k_interior_tma_e<T, I, 4, false, M, KT, true, 5>, GG::template smem_e<4>());
      attr(xg::k_interior_tma_h<T, I, 4, false, M, KT, true, 5>, GG::template smem_h<4>());
      attr(xg::k_interior_tma_e<T, I, 4, true, M, KT, true, 5>, GG::template smem_e<4>());
      attr(xg::k_interior_tma_h<T, I, 4, true, M, KT, true, 5>, GG::template smem_h<4>());
    }
    if constexpr (M == 2) {   // the capped z-edge launches
      attr(xg::k_interior_tma_e<T, I, 4, false, M, KT, false, 5>, GG::template smem_e<4>());
      attr(xg::k_interior_tma_h<T, I, 4, false, M, KT, false, 5>, GG::template smem_h<4>());
      attr(xg::k_interior_tma_e<T, I, 4, false, M, KT, true, 5>, GG::template smem_e<4>());
      attr(xg::k_interior_tma_h<T, I, 4, false, M, KT, true, 5>, GG::template smem_h<4>());
    }
  };
  attrs(std::integral_constant<int, 0>{}, std::integral_constant<int, xg::kItK>{});
  for (int side = 0; side < 2; ++side) {
    if (!h->wide_ok[side]) continue;
    // the z-edge launch's upper tiles start after the interior's last k
    const int k = h->vin_w[side].lo[2], kh = side == 0 ? k - G::HOFF - 1 : k;
    const int ku = h->vin_w[side].hi[2] + 1, kuh = side == 0 ? ku - Gz::HOFF - 1 : ku;
    if (kh < 0 || (k * es) % 16 || (kh * es) % 16 || (k * is) % 16 || (ku * es) % 16 || (kuh * es) % 16 ||
        (ku * is) % 16)
      h->wide_ok[side] = false;
  }
  if (!(h->wide_ok[0] && h->wide_ok[1])) return;
  attrs(std::integral_constant<int, 1>{}, std::integral_constant<int, xg::kItK>{});
  attrs(std::integral_constant<int, 2>{}, std::integral_constant<int, xg::kItK>{});
  attrs(std::integral_constant<int, 2>{}, std::integral_constant<int, xg::kItKz>{});
}

template <typename T, typename I, int S, bool CT, int MODE, int KT, int MINB>
void launch_vol_tma(xfdtd_handle *h, const xg::VolParams<T, I> &p, bool e_side, int chunk, cudaStream_t st) {
  using G = xg::ItTiles<T, I, KT>;
  if (h->itm_base != h->F[0]) interior_tma_encode<T, I>(h);   // the buffers were swapped
  const int side = e_side ? 0 : 1;
  const xg::InteriorBox in = MODE == 2 ? h->vin_z[side] : side_interior(h, side, MODE == 1);
  const int nj = in.hi[1] - in.lo[1] + 1, ni = in.hi[0] - in.lo[0] + 1;
  const int nkt = MODE == 2 ? (in.pz_lo + KT - 1) / KT + (in.hi[2] - in.pz_hi + KT - 1) / KT
                            : (in.hi[2] - in.lo[2] + KT) / KT;
  dim3 grid(nkt, (nj + G::J - 1) / G::J, (ni + chunk - 1) / chunk);
  const xg::ItMaps *maps = KT == xg::kItKz ? h->itm_z : h->itm;
  xg::TfsfFuse fz{};
  if (MODE != 0 && tfsf_fused(h, side)) {
    fz.tf = p.tf;
    fz.step = h->d_step;
    fz.on = 1;
  }
  const unsigned smem = e_side ? G::template smem_e<S>() : G::template smem_h<S>();
  if constexpr (MODE != 0) {
    // the launches with the TFSF corrections folded in run with the same cap
    constexpr int MB = MINB;
    if (fz.on) {
      if (e_side)
        xg::k_interior_tma_e<T, I, S, CT, MODE, KT, true, MB><<<grid, xg::kItThreads, smem, st>>>(
            maps[0], p, in, chunk, h->d_status, h->wait_polls, fz);
      else
        xg::k_interior_tma_h<T, I, S, CT, MODE, KT, true, MB><<<grid, xg::kItThreads, smem, st>>>(
            maps[1], p, in, chunk, h->d_status, h->wait_polls, fz);
      return;
    }
  }
  if (e_side) {
    xg::k_interior_tma_e<T, I, S, CT, MODE, KT, false, MINB><<<grid, xg::kItThreads, smem, st>>>(
        maps[0], p, in, chunk, h->d_status, h->wait_polls, fz);
  } else {
    xg::k_interior_tma_h<T, I, S, CT, MODE, KT, false, MINB><<<grid, xg::kItThreads, smem, st>>>(
        maps[1], p, in, chunk, h->d_status, h->wait_polls, fz);
  }
}

// After a sweep the second buffer set holds step t+1: make it current.
void swap_state(xfdtd_handle *h) {
  for (int c = 0; c < 6; ++c) std::swap(h->F[c], h->F2[c]);
  for (int q = 0; q < 6; ++q) std::swap(h->psi[q], h->psi2[q]);
  h->cur_set ^= 1;
}

// Interior kernel of one side (nothing when the plan has no interior).
template <typename T, typename I>
void launch_volume(xfdtd_handle *h, bool e_side, int var = -1) {
  if (var < 0) var = e_side ? h->var_e : h->var_h;
  const Variant &v = kVariants[var];
  if (side_interior_cells(h, e_side ? 0 : 1, v.wide) == 0) return;
  auto p = vol_params<T, I>(h);
  if (v.stages) {
    if (v.wide) {
      // FP32: the 4-stage launches capped at 5 resident blocks per SM (48
      // registers, no spills; their shared memory allows 5)
      constexpr int MB = sizeof(T) == 4 ? 5 : 1;
      if (v.stages == 6) launch_vol_tma<T, I, 6, false, 1>(h, p, e_side, v.chunk, h->stream);
      else if (v.ct) launch_vol_tma<T, I, 4, true, 1, xg::kItK, MB>(h, p, e_side, v.chunk, h->stream);
      else launch_vol_tma<T, I, 4, false, 1, xg::kItK, MB>(h, p, e_side, v.chunk, h->stream);
    } else {
      if (v.stages == 6) launch_vol_tma<T, I, 6, false, 0>(h, p, e_side, v.chunk, h->stream);
      else if (v.ct) launch_vol_tma<T, I, 4, true, 0>(h, p, e_side, v.chunk, h->stream);
      else launch_vol_tma<T, I, 4, false, 0>(h, p, e_side, v.chunk, h->stream);
    }
    XCHECK(cudaGetLastError());
    return;
  }
  const int key = (v.ct ? 1000 : 0) + v.minb * 100 + v.nc * 10 + (v.smem ? 1 : 0);
  switch (key) {
    case 811: launch_vol_v<T, I, true, 8, 1, false>(h, p, e_side, v); break;
    case 810: launch_vol_v<T, I, false, 8, 1, false>(h, p, e_side, v); break;
    case 820: launch_vol_v<T, I, false, 8, 2, false>(h, p, e_side, v); break;
    case 620: launch_vol_v<T, I, false, 6, 2, false>(h, p, e_side, v); break;
    case 611: launch_vol_v<T, I, true, 6, 1, false>(h, p, e_side, v); break;
    case 120: launch_vol_v<T, I, false, 1, 2, false>(h, p, e_side, v); break;
    case 110: launch_vol_v<T, I, false, 1, 1, false>(h, p, e_side, v); break;
    case 1810: launch_vol_v<T, I, false, 8, 1, true>(h, p, e_side, v); break;
    case 1110: launch_vol_v<T, I, false, 1, 1, true>(h, p, e_side, v); break;
    case 1611: launch_vol_v<T, I, true, 6, 1, true>(h, p, e_side, v); break;
    default: throw Err{XFDTD_ERR_STATE, "volume-kernel variant without an instantiation"};
  }
  XCHECK(cudaGetLastError());
}

// Opts the shared-memory-table instantiations in to `bytes` of dynamic
// shared memory (needed above 48 KB).
template <typename T, typename I>
void smem_attr(int bytes) {
  XCHECK(cudaFuncSetAttribute(xg::k_update_e<T, I, true, 8, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  XCHECK(cudaFuncSetAttribute(xg::k_update_h<T, I, true, 8, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  XCHECK(cudaFuncSetAttribute(xg::k_update_e<T, I, true, 6, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  XCHECK(cudaFuncSetAttribute(xg::k_update_h<T, I, true, 6, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  XCHECK(cudaFuncSetAttribute(xg::k_update_e<T, I, true, 6, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  XCHECK(cudaFuncSetAttribute(xg::k_update_h<T, I, true, 6, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

template <typename T, typename I>
void volume_pair(xfdtd_handle *h, bool e_side);

// Times every variant of the E and H kernels on the handle's current state
// and keeps the fastest.  Run before the first step, when every field and
// psi is zero: the volume kernels then write zeros back (the TFSF buffers
// they read are zero too), so the trials leave the simulation unchanged.
template <typename T>
xg::TfsfSurfParams<T> tfsf_surf_params(xfdtd_handle *h);

// The TFSF surface corrections of one side as their own launch (k_tfsf_e
// over the E box's surface, k_tfsf_h over the H box's) on the main stream.
template <typename T>
void launch_tfsf_side(xfdtd_handle *h, bool e_side) {
  const auto sp = tfsf_surf_params<T>(h);
  const int d = e_side ? 0 : 1;
  const long long n = xg::surface_count(h->tf_lo[0] - d, h->tf_hi[0], h->tf_lo[1] - d, h->tf_hi[1],
                                        h->tf_lo[2] - d, h->tf_hi[2]);
  if (e_side) xg::k_tfsf_e<T><<<static_cast<unsigned>((n + 255) / 256), 256, 0, h->stream>>>(sp);
  else xg::k_tfsf_h<T><<<static_cast<unsigned>((n + 255) / 256), 256, 0, h->stream>>>(sp);
  XCHECK(cudaGetLastError());
}

// One candidate of the autotuner's last rounds: a side's interior and shell
// variants, whether its TFSF corrections are folded into them, and its time.
struct TuneCand {
  float ms;
  int v, sv;
  bool fold;
};

template <typename T, typename I>
void trial_step(xfdtd_handle *h, bool nf_split = true);

template <typename T, typename I>
void autotune_t(xfdtd_handle *h, int trials) {
  cudaEvent_t a, b;
  XCHECK(cudaEventCreate(&a));
  XCHECK(cudaEventCreate(&b));
  // an update of the all-zero state writes zeros: the trials change nothing
  float best_sweep = 1e30f, best_split = 0.f;
  if (h->sweep_ok) {
    float best = 1e30f;
    for (int v = 0; v < kNumSweepVariants; ++v) {
      launch_sweep<T, I>(h, v);
      XCHECK(cudaEventRecord(a, h->stream));
      for (int r = 0; r < trials; ++r) launch_sweep<T, I>(h, v);
      XCHECK(cudaEventRecord(b, h->stream));
      XCHECK(cudaEventSynchronize(b));
      float ms = 0;
      XCHECK(cudaEventElapsedTime(&ms, a, b));
      h->sweep_ms[v] = ms / trials;
      if (ms < best) {
        best = ms;
        h->var_s = v;
      }
    }
    best_sweep = best / trials;
  }
  const bool forced = h->sweep && (h->flags & XFDTD_FLAG_FUSED_EH);
  const bool was_sweep = h->sweep;
  const long long launches = h->launch_count;
  h->sweep = false;
  auto time_n = [&](auto &&run, int n) {
    run();   // warm-up / module load
    XCHECK(cudaEventRecord(a, h->stream));
    for (int r = 0; r < n; ++r) run();
    XCHECK(cudaEventRecord(b, h->stream));
    XCHECK(cudaEventSynchronize(b));
    float ms = 0;
    XCHECK(cudaEventElapsedTime(&ms, a, b));
    return ms / n;
  };
  auto time_ms = [&](auto &&run) { return time_n(run, trials); };
  std::vector<TuneCand> cands[2];
  for (int side = 0; side < 2 && !forced; ++side) {
    // shell kernel of each decomposition: its fastest variant, timed alone
    int shell_best[2] = {0, 0};
    float shell_alone[2][kNumShellVariants], shell_alone_best[2] = {1e30f, 1e30f};
    for (int w = 0; w < 2; ++w) {
      for (int v = 0; v < kNumShellVariants; ++v) shell_alone[w][v] = 1e30f;
      if (w && !h->wide_ok[side]) continue;
      if (!side_shell_cells(h, side, w != 0)) continue;
      for (int v = 0; v < kNumShellVariants; ++v) {
        if (!shell_allowed(h, kShellVariants[v], w != 0)) continue;
        const float ms = time_ms([&] { launch_shell<T, I>(h, side == 0, v, nullptr, w); });
        shell_alone[w][v] = ms;
        if (ms < shell_alone_best[w]) shell_alone_best[w] = ms, shell_best[w] = v;
      }
    }
    // each interior variant with its decomposition's best shell variant,
    // timed as the step runs them: the pair on two streams
    int &var = side == 0 ? h->var_e : h->var_h;
    float best = 1e30f;
    int best_v = 0;
    for (int v = 0; v < kNumVariants; ++v) {
      if (!variant_allowed(h, kVariants[v])) continue;
      var = v;
      h->shell_var[side] = shell_best[kVariants[v].wide ? 1 : 0];
      const float ms = time_ms([&] { volume_pair<T, I>(h, side == 0); });
      h->tune_ms[side][v] = ms;
      if (ms < best) best = ms, best_v = v;
    }
    // the three fastest interior variants, each with every shell variant
    // its decomposition allows that is within 20 % of the fastest alone
    // (the shell variant fastest alone need not be fastest beside the
    // interior launch), timed again over three times the trials, so that
    // timing noise does not pick the pair
    int top[3] = {-1, -1, -1};
    for (int v = 0; v < kNumVariants; ++v) {
      if (!variant_allowed(h, kVariants[v])) continue;
      for (int q = 0; q < 3; ++q)
        if (top[q] < 0 || h->tune_ms[side][v] < h->tune_ms[side][top[q]]) {
          for (int r = 2; r > q; --r) top[r] = top[r - 1];
          top[q] = v;
          break;
        }
    }
    // Each candidate is timed with this side's TFSF corrections: inside the
    // wide decomposition's TMA launches where it can take them, else as
    // their own launch after the pair, so that the forms compare on the same
    // work.
    best = 1e30f;
    int best_sv = shell_best[kVariants[best_v].wide ? 1 : 0];
    bool best_fold = false;
    std::vector<TuneCand> &cand = cands[side];
    for (int q = 0; q < 3 && top[q] >= 0; ++q) {
      const int v = top[q];
      var = v;
      const bool wide = kVariants[v].wide;
      for (int sv = 0; sv < kNumShellVariants; ++sv) {
        if (!shell_allowed(h, kShellVariants[sv], wide)) continue;
        if (!side_shell_cells(h, side, wide) && sv != shell_best[wide ? 1 : 0]) continue;
        // shell variants more than 20 % slower alone than the fastest are
        // not retried beside the interior launch
        if (side_shell_cells(h, side, wide) && shell_alone[wide ? 1 : 0][sv] > 1.2f * shell_alone_best[wide ? 1 : 0])
          continue;
        h->shell_var[side] = sv;
        for (int fold = 0; fold < 2; ++fold) {
          h->tf_fuse_on[side] = fold != 0;
          if (fold && !tfsf_fused(h, side)) continue;
          const bool apart = h->tfsf && !tfsf_fused(h, side);
          const float ms = time_n([&] {
            volume_pair<T, I>(h, side == 0);
            if (apart) launch_tfsf_side<T>(h, side == 0);
          }, 3 * trials);
          if (fold) h->tf_fuse_ms[side][0] = ms;
          else if (h->tf_fuse_ok[side] && wide) h->tf_fuse_ms[side][1] = ms;
          cand.push_back({ms, v, sv, fold != 0});
          if (ms < best) best = ms, best_v = v, best_sv = sv, best_fold = fold != 0;
        }
      }
    }
    var = best_v;
    h->shell_var[side] = best_sv;
    h->tf_fuse_on[side] = best_fold;
    h->tune_ms[side][best_v] = best;
    best_split += best;
  }
  // Last round: the two fastest candidates of each side, paired, timed as
  // the step runs them (the E side, then the H side, with the NF-FF
  // sampling halves beside them on their stream), twice in turn; the
  // fastest pairing is kept.  Each side's time alone misses how its
  // launches share the GPU with the other side's neighbours and with the
  // sampling stream.
  if (!forced && !cands[0].empty() && !cands[1].empty()) {
    for (auto &c : cands) {
      std::stable_sort(c.begin(), c.end(), [](const TuneCand &x, const TuneCand &y) { return x.ms < y.ms; });
      if (c.size() > 2) c.resize(2);
    }
    auto apply = [&](int side, const TuneCand &c) {
      (side == 0 ? h->var_e : h->var_h) = c.v;
      h->shell_var[side] = c.sv;
      h->tf_fuse_on[side] = c.fold;
    };
    float t[2][2] = {{1e30f, 1e30f}, {1e30f, 1e30f}};
    for (int pass = 0; pass < 2; ++pass)
      for (size_t e = 0; e < cands[0].size(); ++e)
        for (size_t hh = 0; hh < cands[1].size(); ++hh) {
          apply(0, cands[0][e]);
          apply(1, cands[1][hh]);
          t[e][hh] = std::min(t[e][hh], time_n([&] { trial_step<T, I>(h); }, 2 * trials));
        }
    size_t be = 0, bh = 0;
    for (size_t e = 0; e < cands[0].size(); ++e)
      for (size_t hh = 0; hh < cands[1].size(); ++hh)
        if (t[e][hh] < t[be][bh]) be = e, bh = hh;
    apply(0, cands[0][be]);
    apply(1, cands[1][bh]);
    h->tune_step_ms = t[be][bh];
    h->tune_ms[0][cands[0][be].v] = cands[0][be].ms;
    h->tune_ms[1][cands[1][bh].v] = cands[1][bh].ms;
  }
  // The NF-FF schedule: the split sampling halves beside the volume
  // updates, or one sampling launch after the H update (beside the TFSF H
  // corrections where it can), timed with the kept pairing, twice in turn.
  // Beside a bandwidth-bound volume launch the halves can cost it more
  // than they save.
  if (!forced && h->nffft && !h->nf_bb) {
    float ts[2] = {1e30f, 1e30f};
    for (int pass = 0; pass < 2; ++pass)
      for (int sp = 0; sp < 2; ++sp)
        ts[sp] = std::min(ts[sp], time_n([&] { trial_step<T, I>(h, sp == 0); }, 2 * trials));
    h->nf_sched_ms[0] = ts[0];
    h->nf_sched_ms[1] = ts[1];
    h->nf_split = ts[0] <= ts[1];
  }
  h->sweep = was_sweep;
  h->launch_count = launches;
  // without a forcing flag, the faster of the sweep and the split pair
  if (h->sweep_ok && !forced) h->sweep = best_sweep < best_split;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
}

void autotune(xfdtd_handle *h, int trials) {
  if (h->host_step != 0) throw Err{XFDTD_ERR_STATE, "autotuning runs before the first step only"};
  with_types(h->precision, h->idx_bytes, [&](auto t, auto i) {
    autotune_t<decltype(t), decltype(i)>(h, trials);
  });
}

template <typename T>
xg::SparseParams<T> sparse_params(xfdtd_handle *h) {
  xg::SparseParams<T> p{};
  p.d = h->d;
  for (int c = 0; c < 6; ++c) p.F[c] = static_cast<T *>(h->F[c]);
  p.inj = h->inj;
  p.n_inj = h->n_inj;
  p.waveforms = h->waveforms;
  p.ind = h->ind;
  p.ind_j = h->ind_j;
  p.n_ind = h->n_ind;
  p.terms = h->terms;
  p.probe_off = h->probe_off;
  p.n_probes = h->n_probes;
  p.probe_out = h->probe_out;
  p.total = h->total;
  p.step = h->d_step;
  return p;
}

template <typename T>
xg::NfParams<T> nf_params(xfdtd_handle *h) {
  xg::NfParams<T> p{};
  p.d = h->d;
  for (int c = 0; c < 3; ++c) {
    p.E[c] = static_cast<const T *>(h->F[c]);
    p.H[c] = static_cast<const T *>(h->F[3 + c]);
  }
  for (int a = 0; a < 3; ++a) {
    p.lo[a] = h->nf_lo[a];
    p.hi[a] = h->nf_hi[a];
  }
  p.nf = h->nf;
  for (int q = 0; q < 24; ++q) p.acc[q] = h->acc[q];
  p.pj = h->phase_j;
  p.pm = h->phase_m;
  p.pjf = h->phase_jf;
  p.pmf = h->phase_mf;
  p.total = h->total;
  p.step = h->d_step;
  for (int g = 0; g < 3; ++g) p.buf[g] = static_cast<T *>(h->nf_buf[g]);
  p.batch = h->nf_rows;
  return p;
}

// Launch grid of the NF-FF sampling kernel (32 x 8 blocks, one z-slice per face pair).
dim3 nffft_grid(const xfdtd_handle *h) {
  const int bx = h->nf_hi[0] - h->nf_lo[0], by = h->nf_hi[1] - h->nf_lo[1], bz = h->nf_hi[2] - h->nf_lo[2];
  const int u = std::max(bz, by), v = std::max(by, bx);
  return dim3((u + 31) / 32, (v + 7) / 8, 3);
}

// Blocks of 256 face cells per face pair for the NF-FF fold.
long long nffft_fold_blocks(const xfdtd_handle *h) {
  const long long bx = h->nf_hi[0] - h->nf_lo[0], by = h->nf_hi[1] - h->nf_lo[1], bz = h->nf_hi[2] - h->nf_lo[2];
  const long long most = std::max(by * bz, std::max(bx * bz, bx * by));
  return (most + 255) / 256;
}

// The NF-FF samples of step *step - lag (part 0: all, 1: the E half, 2: the
// H half; nffft_sample in surface.cuh).
template <typename T>
void launch_nffft(xfdtd_handle *h, cudaStream_t st = nullptr, int part = 0, int lag = 0) {
  const auto p = nf_params<T>(h);
  xg::k_nffft<T><<<nffft_grid(h), dim3(32, 8, 1), 0, st ? st : h->stream>>>(p, part, lag);
  XCHECK(cudaGetLastError());
}

// Folds `count` buffered NF-FF steps into the accumulators; `lag` = 0 inside
// a step (the device step counter points at the last sampled step), 1 after
// it (the counter has advanced past it).
template <typename T>
void launch_nffft_accumulate(xfdtd_handle *h, int count, int lag, cudaStream_t st = nullptr) {
  const auto p = nf_params<T>(h);
  dim3 grid(static_cast<unsigned>(nffft_fold_blocks(h)), 1, 3);
  xg::k_nffft_accumulate<T><<<grid, 256, 0, st ? st : h->stream>>>(p, count, lag);
  XCHECK(cudaGetLastError());
}

// The split NF-FF sampling leaves the H half of the last stepped step
// pending: the next step takes it (and folds a full batch) on the NF-FF
// stream beside its E update.  Before a read of the accumulators or the far
// field, and before a captured graph is replayed, it is taken here on the
// main stream, with the fold of every step sampled since the last one.
template <typename T>
void nffft_catch_up_t(xfdtd_handle *h) {
  if (h->nf_pending) {
    prof_begin(h, 4);
    launch_nffft<T>(h, h->stream, 2, 1);
    prof_end(h);
    h->nf_pending = false;
  }
  const long long pending = h->host_step - h->nf_done;
  if (pending > 0) {
    prof_begin(h, 9);
    launch_nffft_accumulate<T>(h, static_cast<int>(pending), 1);
    prof_end(h);
    h->nf_done = h->host_step;
  }
}

// Accumulates the NF-FF steps sampled since the last fold (before any read
// of the accumulators or the far field).
void nffft_flush(xfdtd_handle *h) {
  if (!h->nffft || h->nf_bb) return;
  if (h->precision == XFDTD_FP64) nffft_catch_up_t<double>(h);
  else nffft_catch_up_t<float>(h);
}

template <typename T>
xg::TfsfSurfParams<T> tfsf_surf_params(xfdtd_handle *h) {
  xg::TfsfSurfParams<T> p{};
  p.d = h->d;
  for (int c = 0; c < 6; ++c) p.F[c] = static_cast<T *>(h->F[c]);
  p.tf.enabled = 1;
  p.tf.two_d = h->tf_two_d ? 1 : 0;
  p.tf.L = h->aux_len;
  for (int a = 0; a < 3; ++a) {
    p.tf.lo[a] = h->tf_lo[a];
    p.tf.hi[a] = h->tf_hi[a];
    p.tf.pf[a] = h->tf_pf[a];
    p.tf.ph[a] = h->tf_ph[a];
    p.tf.ca[a] = h->tf_ca[a];
    p.tf.cb[a] = h->tf_cb[a];
    p.tf.pff[a] = h->tf_pff[a];
    p.tf.phf[a] = h->tf_phf[a];
    p.tf.caf[a] = static_cast<float>(h->tf_ca[a]);
    p.tf.cbf[a] = static_cast<float>(h->tf_cb[a]);
  }
  p.tf.inc = h->tf_inc;
  p.tf.incf = h->tf_incf;
  p.step = h->d_step;
  return p;
}

xg::AuxParams aux_params(xfdtd_handle *h) {
  xg::AuxParams a{};
  a.L = h->aux_len;
  a.state = h->tf_state;
  a.inc = h->tf_inc;
  a.incf = h->tf_incf;
  a.source = h->tf_src;
  a.ceihi = h->tf_ceihi;
  a.chiei = h->tf_chiei;
  a.c1 = h->tf_c1;
  a.c2 = h->tf_c2;
  for (int q = 0; q < 3; ++q) {
    a.te[q] = h->tf_te[q];
    a.th[q] = h->tf_th[q];
  }
  a.step = h->d_step;
  a.total = h->total;
  a.status = h->d_status;
  return a;
}

// The E (or H) update of one step: the interior kernel on the main stream
// and the shell kernel on the shell stream beside it (they write disjoint
// cells and read only the other field), joined before what follows.
template <typename T, typename I>
void volume_pair(xfdtd_handle *h, bool e_side) {
  const int side = e_side ? 0 : 1;
  const bool wide = side_wide(h, side);
  const bool in = side_interior_cells(h, side, wide) != 0, sh = side_shell_cells(h, side, wide) != 0;
  prof_region_begin(h, e_side ? 1 : 3);
  if (in && sh) {
    XCHECK(cudaEventRecord(h->ev_vfork[side], h->stream));
    XCHECK(cudaStreamWaitEvent(h->shell, h->ev_vfork[side], 0));
    prof_begin(h, e_side ? 11 : 12, h->shell);
    launch_shell<T, I>(h, e_side, -1, h->shell);
    prof_end(h, h->shell);
    XCHECK(cudaEventRecord(h->ev_vjoin[side], h->shell));
  } else if (sh) {
    prof_begin(h, e_side ? 11 : 12);
    launch_shell<T, I>(h, e_side);
    prof_end(h);
  }
  if (in) {
    prof_begin(h, e_side ? 13 : 14);
    launch_volume<T, I>(h, e_side);
    prof_end(h);
  }
  if (in && sh) XCHECK(cudaStreamWaitEvent(h->stream, h->ev_vjoin[side], 0));
  prof_end(h);
}

// The volume work of one step as the step runs it, for the autotuner: the
// E pair and its TFSF corrections (folded or apart), then the H pair and
// its corrections, with the two NF-FF sampling halves on their stream
// beside them.  Nothing else of a step runs: no 1-D incident line, sources,
// fold or step counter.  On the all-zero state before the first step it
// writes zeros where there were zeros (the samples of step 0 are taken
// again, from the fields, by the first step).
template <typename T, typename I>
void trial_step(xfdtd_handle *h, bool nf_split) {
  const bool split = h->nffft && !h->nf_bb && nf_split;
  if (split) {
    XCHECK(cudaEventRecord(h->ev_nfs_fork, h->stream));
    XCHECK(cudaStreamWaitEvent(h->nfs, h->ev_nfs_fork, 0));
    launch_nffft<T>(h, h->nfs, 2, 0);
    XCHECK(cudaEventRecord(h->ev_nfh, h->nfs));
  }
  volume_pair<T, I>(h, true);
  if (h->tfsf && !tfsf_fused(h, 0)) launch_tfsf_side<T>(h, true);
  if (split) {
    XCHECK(cudaEventRecord(h->ev_nfs_fork, h->stream));
    XCHECK(cudaStreamWaitEvent(h->nfs, h->ev_nfs_fork, 0));
    launch_nffft<T>(h, h->nfs, 1, 0);
    XCHECK(cudaEventRecord(h->ev_nfe, h->nfs));
    XCHECK(cudaStreamWaitEvent(h->stream, h->ev_nfh, 0));
  }
  volume_pair<T, I>(h, false);
  // the one-launch schedule: the samples beside the TFSF H corrections on
  // the side stream when their cells are disjoint, else after them
  const bool one = h->nffft && !h->nf_bb && !split;
  const bool beside = one && h->tfsf && h->nf_beside_tfsf;
  if (beside) {
    XCHECK(cudaEventRecord(h->ev_nf_fork, h->stream));
    XCHECK(cudaStreamWaitEvent(h->side, h->ev_nf_fork, 0));
    launch_nffft<T>(h, h->side);
    XCHECK(cudaEventRecord(h->ev_nf_join, h->side));
  }
  if (h->tfsf && !tfsf_fused(h, 1)) launch_tfsf_side<T>(h, false);
  if (beside) XCHECK(cudaStreamWaitEvent(h->stream, h->ev_nf_join, 0));
  else if (one) launch_nffft<T>(h);
  if (split) XCHECK(cudaStreamWaitEvent(h->stream, h->ev_nfe, 0));
}

template <typename T, typename I>
void enqueue_step_t(xfdtd_handle *h, long long s, bool pre) {
  // The NF-FF samples of a step are taken in two halves on their own stream
  // (nfs): the E half beside this step's H update, the H half beside the
  // next step's E update; a full batch is folded there too, after the H half
  // of its last step.  (Broadband NF-FF and the fused sweep keep one launch.)
  const bool split = h->nffft && !h->nf_bb && !h->sweep && h->nf_split;
  bool wait_nfh = false;
  if (h->nffft && !h->nf_bb && h->nf_pending && pre) {
    XCHECK(cudaEventRecord(h->ev_nfs_fork, h->stream));
    XCHECK(cudaStreamWaitEvent(h->nfs, h->ev_nfs_fork, 0));
    prof_begin(h, 4, h->nfs);
    launch_nffft<T>(h, h->nfs, 2, 1);
    prof_end(h, h->nfs);
    if (s % h->nf_batch == 0 && s > h->nf_done) {
      prof_begin(h, 9, h->nfs);
      launch_nffft_accumulate<T>(h, static_cast<int>(s - h->nf_done), 1, h->nfs);
      prof_end(h, h->nfs);
      h->nf_done = s;
    }
    XCHECK(cudaEventRecord(h->ev_nfh, h->nfs));
    h->nf_pending = false;
    wait_nfh = true;
  }
  if (h->tfsf) {
    const xg::AuxParams a = aux_params(h);
    // The 1-D line of step t runs on a side stream, beside the E update: it
    // must follow the E corrections of step t-1 (which read the buffer it
    // writes) and precede the H corrections of step t (joined there).
    XCHECK(cudaEventRecord(h->ev_fork, h->stream));
    XCHECK(cudaStreamWaitEvent(h->side, h->ev_fork, 0));
    prof_begin(h, 0, h->side);
    xg::k_tfsf_aux<<<1, 512, 0, h->side>>>(a);
    XCHECK(cudaGetLastError());
    prof_end(h, h->side);
    XCHECK(cudaEventRecord(h->ev_join, h->side));
  }
  if (h->sweep) {
    prof_begin(h, 10);
    launch_sweep<T, I>(h);
    prof_end(h);
    swap_state(h);
  } else {
    volume_pair<T, I>(h, true);
    if (h->n_disp) {
      xg::DispParams<T> dp{};
      dp.d = h->d;
      for (int c = 0; c < 3; ++c) {
        dp.E[c] = static_cast<T *>(h->F[c]);
        dp.H[c] = static_cast<const T *>(h->F[3 + c]);
      }
      dp.cells = h->disp_cells;
      dp.media = static_cast<const xg::DispMedium<T> *>(h->disp_media);
      dp.j = static_cast<T *>(h->disp_j);
      dp.jp = static_cast<T *>(h->disp_jp);
      dp.ep = static_cast<T *>(h->disp_ep);
      dp.n = h->n_disp;
      dp.dl = static_cast<T>(h->disp_dl);
      dp.dt = static_cast<T>(h->dt);
      prof_begin(h, 16);
      xg::k_dispersive_e<T><<<(h->n_disp + 255) / 256, 256, 0, h->stream>>>(dp);
      XCHECK(cudaGetLastError());
      prof_end(h);
    }
    if (h->n_inj || h->n_ind) {
      auto sp = sparse_params<T>(h);
      int n = std::max(h->n_inj, h->n_ind);
      prof_begin(h, 2);
      xg::k_lumped_e<T><<<(n + 127) / 128, 128, 0, h->stream>>>(sp);
      XCHECK(cudaGetLastError());
      prof_end(h);
    }
    if (h->tfsf && !tfsf_fused(h, 0)) {
      const auto sp = tfsf_surf_params<T>(h);
      const long long n = xg::surface_count(h->tf_lo[0], h->tf_hi[0], h->tf_lo[1], h->tf_hi[1], h->tf_lo[2], h->tf_hi[2]);
      prof_begin(h, 7);
      xg::k_tfsf_e<T><<<static_cast<unsigned>((n + 255) / 256), 256, 0, h->stream>>>(sp);
      XCHECK(cudaGetLastError());
      prof_end(h);
    }
    // E is final for this step: its NF-FF half is taken beside the H update
    if (split) {
      XCHECK(cudaEventRecord(h->ev_nfs_fork, h->stream));
      XCHECK(cudaStreamWaitEvent(h->nfs, h->ev_nfs_fork, 0));
      prof_begin(h, 4, h->nfs);
      launch_nffft<T>(h, h->nfs, 1, 0);
      prof_end(h, h->nfs);
      XCHECK(cudaEventRecord(h->ev_nfe, h->nfs));
    }
    // the H launch that applies the TFSF H corrections reads this step's
    // incident E: the 1-D line joins before it; the H half of the previous
    // step's NF-FF samples must be taken before H changes
    if (h->tfsf && tfsf_fused(h, 1)) XCHECK(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
    if (wait_nfh) XCHECK(cudaStreamWaitEvent(h->stream, h->ev_nfh, 0));
    wait_nfh = false;
    volume_pair<T, I>(h, false);
  }
  if (wait_nfh) XCHECK(cudaStreamWaitEvent(h->stream, h->ev_nfh, 0));
  // NF-FF sampling in one launch (broadband, or the fused sweep) on the side
  // stream beside the TFSF H corrections when their cells are disjoint;
  // joined before the samples are folded
  const bool nf_side = !split && h->nffft && h->tfsf && h->nf_beside_tfsf;
  if (nf_side) {
    XCHECK(cudaEventRecord(h->ev_nf_fork, h->stream));
    XCHECK(cudaStreamWaitEvent(h->side, h->ev_nf_fork, 0));
    prof_begin(h, 4, h->side);
    launch_nffft<T>(h, h->side);
    prof_end(h, h->side);
    XCHECK(cudaEventRecord(h->ev_nf_join, h->side));
  }
  if (h->tfsf && (h->sweep || !tfsf_fused(h, 1))) {
    XCHECK(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
    const auto sp = tfsf_surf_params<T>(h);
    const long long n = xg::surface_count(h->tf_lo[0] - 1, h->tf_hi[0], h->tf_lo[1] - 1, h->tf_hi[1],
                                          h->tf_lo[2] - 1, h->tf_hi[2]);
    prof_begin(h, 8);
    xg::k_tfsf_h<T><<<static_cast<unsigned>((n + 255) / 256), 256, 0, h->stream>>>(sp);
    XCHECK(cudaGetLastError());
    prof_end(h);
  }
  if (h->nffft && !split) {
    if (nf_side) {
      XCHECK(cudaStreamWaitEvent(h->stream, h->ev_nf_join, 0));
    } else {
      prof_begin(h, 4);
      launch_nffft<T>(h);
      prof_end(h);
    }
    if (h->nf_bb) {   // broadband: the samples stay, one row per step
      h->nf_done = s + 1;
    } else if ((s + 1) % h->nf_batch == 0) {   // the batch is full: fold it
      prof_begin(h, 9);
      launch_nffft_accumulate<T>(h, static_cast<int>(s + 1 - h->nf_done), 0);
      prof_end(h);
      h->nf_done = s + 1;
    }
  }
  if (h->n_probes) {
    auto sp = sparse_params<T>(h);
    prof_begin(h, 5);
    xg::k_probes<T><<<(h->n_probes + 127) / 128, 128, 0, h->stream>>>(sp);
    XCHECK(cudaGetLastError());
    prof_end(h);
  }
  if (!h->snaps.empty()) {
    xg::SnapParams<T> sp{};
    sp.d = h->d;
    for (int c = 0; c < 6; ++c) sp.F[c] = static_cast<const T *>(h->F[c]);
    sp.s = h->d_snaps;
    sp.step = h->d_step;
    const unsigned bx = static_cast<unsigned>(std::min<long long>((h->snap_cells_max + 255) / 256, 1024));
    prof_begin(h, 15);
    xg::k_snapshots<T><<<dim3(bx, static_cast<unsigned>(h->snaps.size())), 256, 0, h->stream>>>(sp);
    XCHECK(cudaGetLastError());
    prof_end(h);
  }
  // the E half reads the step counter: it joins before the counter moves
  if (split) {
    XCHECK(cudaStreamWaitEvent(h->stream, h->ev_nfe, 0));
    h->nf_pending = true;
  }
  prof_begin(h, 6);
  xg::k_advance<<<1, 1, 0, h->stream>>>(h->d_step);
  XCHECK(cudaGetLastError());
  prof_end(h);
}

// Enqueues the kernels of step s (s = the step's index, known on the host).
// pre: also take the pending H half of the previous step's NF-FF samples
// (and fold a finished batch) first; a captured graph's first step leaves
// that to a catch-up before the replay.
void enqueue_step(xfdtd_handle *h, long long s, bool pre = true) {
  with_types(h->precision, h->idx_bytes, [&](auto t, auto i) {
    enqueue_step_t<decltype(t), decltype(i)>(h, s, pre);
  });
}

int launches_per_step(const xfdtd_handle *h) {
  const int snap = h->snaps.empty() ? 0 : 1;
  if (h->sweep) return (h->tfsf ? 2 : 0) + 1 + (h->nffft ? 1 : 0) + (h->n_probes ? 1 : 0) + snap + 1;
  int vol = 0;
  for (int side = 0; side < 2; ++side) {
    const bool w = side_wide(h, side);
    vol += (side_interior_cells(h, side, w) ? 1 : 0) + (side_shell_cells(h, side, w) ? 1 : 0);
  }
  const int tf = h->tfsf ? 3 - (tfsf_fused(h, 0) ? 1 : 0) - (tfsf_fused(h, 1) ? 1 : 0) : 0;
  return tf + vol + ((h->n_inj || h->n_ind) ? 1 : 0) + (h->n_disp ? 1 : 0) + (h->nffft ? 1 : 0) +
         (h->n_probes ? 1 : 0) + snap + 1;
}

// Captures g steps starting at a step index that is a multiple of the NF-FF
// batch (g is one too), so that the captured kernel sequence -- including
// the batch folds -- is the same for every replay.
void build_graph(xfdtd_handle *h, int g) {
  cudaGraph_t graph;
  const long long nf_done = h->nf_done, launches = h->launch_count;
  const bool nf_pending = h->nf_pending;
  XCHECK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  for (int s = 0; s < g; ++s) enqueue_step(h, h->host_step + s, s > 0);
  XCHECK(cudaStreamEndCapture(h->stream, &graph));
  h->graph_launches = h->launch_count - launches;
  h->nf_done = nf_done;   // capture only recorded the launches
  h->nf_pending = nf_pending;
  h->launch_count = launches;
  cudaError_t e = cudaGraphInstantiate(&h->gexec, graph, 0);
  cudaGraphDestroy(graph);
  XCHECK(e);
  h->graph_steps = g;
}

void check_status(xfdtd_handle *h) {
  int st = 0;
  XCHECK(cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  XCHECK(cudaStreamSynchronize(h->stream));
  if (st == XFDTD_ERR_TIMEOUT) throw Err{XFDTD_ERR_TIMEOUT, "a bounded device wait gave up (TMA plane stage)"};
  if (st != 0) throw Err{XFDTD_ERR_DEVICE_CHECK, "device status " + std::to_string(st) + " (step index past the plan)"};
}

// component shapes of the reference (simulation_init.cpp:28-35)
void comp_shape(const xfdtd_handle *h, int c, long long s[3]) {
  long long nx = h->d.nx, ny = h->d.ny, nz = h->d.nz;
  const long long t[6][3] = {{nx, ny + 1, nz + 1}, {nx + 1, ny, nz + 1}, {nx + 1, ny + 1, nz},
                             {nx + 1, ny, nz},     {nx, ny + 1, nz},     {nx, ny, nz + 1}};
  for (int a = 0; a < 3; ++a) s[a] = t[c][a];
}

// ----------------------------------------------------------- creation ---
double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void create(const xfdtd_plan_desc *pl, xfdtd_handle *h) {
  const auto t_begin = std::chrono::steady_clock::now();
  // the 3-D grid, or the 2-D grid of the TMz path (nz = 1, simulation_update.cpp:157-168)
  if (pl->nx < 2 || pl->ny < 2 || pl->nz < 1) invalid("grid must have at least 2 cells on x and y and 1 on z");
  if (pl->tfsf.enabled == 2 && pl->nz != 1) invalid("the 2-D plane wave (TFSF2D) needs nz = 1");
  if (pl->nz == 1 && pl->tfsf.enabled == 1) invalid("a 2-D grid (nz = 1) takes the 2-D plane wave (TFSF2D)");
  if (pl->nz == 1 && pl->nffft.enabled) invalid("the 2-D grid (nz = 1) carries no NF-FF box");
  if (pl->precision != XFDTD_FP64 && pl->precision != XFDTD_FP32) invalid("precision must be FP64 or FP32");
  if (pl->index_bytes != 1 && pl->index_bytes != 2 && pl->index_bytes != 4) invalid("index_bytes must be 1, 2 or 4");
  if (pl->n_materials < 1 || (pl->index_bytes < 4 && pl->n_materials > (pl->index_bytes == 1 ? 256 : 65536)))
    invalid("material count does not fit the index width");
  if (!pl->material_index || !pl->coeff_table) invalid("material index and coefficient table are required");
  if (pl->total_steps < 1) invalid("total_steps must be positive");
  if (!(pl->dt > 0)) invalid("dt must be positive");
  if (pl->device < 0) invalid("device ordinal must be >= 0");
  h->device = pl->device;
  XCHECK(cudaSetDevice(pl->device));
  h->precision = pl->precision;
  h->idx_bytes = pl->index_bytes;
  h->flags = pl->flags;
  h->esize = pl->precision == XFDTD_FP64 ? 8 : 4;
  h->total = pl->total_steps;
  h->dt = pl->dt;
  for (int a = 0; a < 3; ++a) h->dl[a] = pl->dl[a];
  if (pl->n_disp_cells < 0 || pl->n_disp_media < 0 || (pl->n_disp_cells && (!pl->disp_cells || !pl->disp_media)))
    invalid("dispersive cells and media are required together");
  h->n_disp = pl->n_disp_cells;
  xg::Dims &d = h->d;
  d.nx = pl->nx;
  d.ny = pl->ny;
  d.nz = pl->nz;
  // rows of whole 128-byte lines; the 2-D grid's rows hold k = 0, 1 and the
  // k = 2 the general path reads past the last E, in 16 (FP32) or 32 bytes
  d.nzp = pl->nz == 1 ? 4 : ((pl->nz + 1) + 31) / 32 * 32;
  d.sj = d.nzp;
  d.si = static_cast<long long>(pl->ny + 1) * d.nzp;
  d.cells = static_cast<long long>(pl->nx + 1) * d.si;
  const long long NX1 = pl->nx + 1, NY1 = pl->ny + 1, NZ1 = pl->nz + 1;

  XCHECK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  XCHECK(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
  XCHECK(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
  XCHECK(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
  XCHECK(cudaEventCreateWithFlags(&h->ev_nf_fork, cudaEventDisableTiming));
  XCHECK(cudaEventCreateWithFlags(&h->ev_nf_join, cudaEventDisableTiming));
  {   // the NF-FF halves at the least priority: their blocks fill the slots the
      // volume launches they run beside leave free (at the greatest priority
      // they went first and held those launches back, 0.424 against 0.400 ms
      // per step on the 280^3 dielectric sphere)
    int lo_prio = 0, hi_prio = 0;
    XCHECK(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
    XCHECK(cudaStreamCreateWithPriority(&h->nfs, cudaStreamNonBlocking, lo_prio));
  }
  XCHECK(cudaEventCreateWithFlags(&h->ev_nfs_fork, cudaEventDisableTiming));
  XCHECK(cudaEventCreateWithFlags(&h->ev_nfh, cudaEventDisableTiming));
  XCHECK(cudaEventCreateWithFlags(&h->ev_nfe, cudaEventDisableTiming));
  {
    // the shell launch is the pair's long pole: its blocks go first as the
    // interior's retire
    int least = 0, greatest = 0;
    XCHECK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    XCHECK(cudaStreamCreateWithPriority(&h->shell, cudaStreamNonBlocking, greatest));
  }
  for (int q = 0; q < 2; ++q) {
    XCHECK(cudaEventCreateWithFlags(&h->ev_vfork[q], cudaEventDisableTiming));
    XCHECK(cudaEventCreateWithFlags(&h->ev_vjoin[q], cudaEventDisableTiming));
  }
  for (int c = 0; c < 6; ++c) h->F[c] = h->alloc_bytes(d.cells * h->esize);

  // material index, repacked into the padded layout
  {
    std::vector<uint8_t> buf(d.cells * pl->index_bytes, 0);
    const uint8_t *src = static_cast<const uint8_t *>(pl->material_index);
    for (long long i = 0; i < NX1; ++i)
      for (long long j = 0; j < NY1; ++j) {
        const uint8_t *row = src + ((i * NY1 + j) * NZ1) * pl->index_bytes;
        if (pl->index_bytes == 4) {
          for (long long k = 0; k < NZ1; ++k) {
            uint32_t v;
            std::memcpy(&v, row + 4 * k, 4);
            if (v >= static_cast<uint32_t>(pl->n_materials)) invalid("material index out of range");
          }
        } else if (pl->index_bytes == 2) {
          const uint16_t *r16 = reinterpret_cast<const uint16_t *>(row);
          for (long long k = 0; k < NZ1; ++k)
            if (r16[k] >= pl->n_materials) invalid("material index out of range");
        } else {
          for (long long k = 0; k < NZ1; ++k)
            if (row[k] >= pl->n_materials) invalid("material index out of range");
        }
        std::memcpy(buf.data() + (i * d.si + j * d.sj) * pl->index_bytes, row, NZ1 * pl->index_bytes);
      }
    h->idx = h->upload<uint8_t>(buf.data(), buf.size());
  }
  h->n_mat = pl->n_materials;
  h->table_host.assign(pl->coeff_table, pl->coeff_table + static_cast<size_t>(pl->n_materials) * XFDTD_N_COEFF);
  h->table = h->upload_real(pl->coeff_table, static_cast<size_t>(pl->n_materials) * XFDTD_N_COEFF);
  h->ctable = compact_table(h, pl->coeff_table, pl->n_materials);
  h->smem_bytes = static_cast<size_t>(pl->n_materials) * 9 * h->esize;
  h->smem_table = h->smem_bytes <= 96 * 1024;
  if (h->smem_table && h->smem_bytes > 48 * 1024) {
    // opt in to more than 48 KB of dynamic shared memory for the table
    int bytes = static_cast<int>(h->smem_bytes);
    with_types(h->precision, h->idx_bytes, [&](auto t, auto i) { smem_attr<decltype(t), decltype(i)>(bytes); });
  }

  // CPML profiles
  const int n_axis[3] = {pl->nx, pl->ny, pl->nz};
  for (int a = 0; a < 3; ++a) {
    const xfdtd_cpml_axis &ca = pl->cpml[a];
    if (ca.n_layers < 0) invalid("negative CPML layer count");
    h->L[a] = ca.n_layers;
    if (ca.n_layers == 0) continue;
    const int n1 = n_axis[a] + 1;
    if (!ca.slot_e || !ca.slot_h || !ca.b_e || !ca.a_e || !ca.rk_e || !ca.b_m || !ca.a_m || !ca.rk_m)
      invalid("CPML axis is missing a profile array");
    for (int q = 0; q < n1; ++q) {
      if (ca.slot_e[q] >= ca.n_layers || ca.slot_h[q] >= ca.n_layers) invalid("CPML slot out of range");
      if (ca.slot_e[q] >= 0 && (q < 1 || q > n_axis[a] - 1)) invalid("CPML E slot on an outer wall");
      if (ca.slot_h[q] >= 0 && q > n_axis[a] - 1) invalid("CPML H slot on the last index");
    }
    h->slot_e[a] = h->upload<int>(ca.slot_e, n1);
    h->slot_h[a] = h->upload<int>(ca.slot_h, n1);
    const double *src[6] = {ca.b_e, ca.a_e, ca.rk_e, ca.b_m, ca.a_m, ca.rk_m};
    for (int q = 0; q < 6; ++q) h->prof[a][q] = h->upload_real(src[q], n1);
  }
  // psi arrays: axis X (L, ny+1, nzp), Y (nx+1, L, nzp), Z (nx+1, ny+1, L)
  {
    const size_t sx = static_cast<size_t>(h->L[0]) * NY1 * d.nzp;
    const size_t sy = static_cast<size_t>(NX1) * h->L[1] * d.nzp;
    const size_t sz = static_cast<size_t>(NX1) * NY1 * h->L[2];
    // order: ex_y ex_z ey_x ey_z ez_x ez_y hx_y hx_z hy_x hy_z hz_x hz_y
    const size_t sizes[12] = {sy, sz, sx, sz, sx, sy, sy, sz, sx, sz, sx, sy};
    for (int q = 0; q < 12; ++q) {
      h->psi[q] = sizes[q] ? h->alloc_bytes(sizes[q] * h->esize) : nullptr;
      h->psi_bytes[q] = sizes[q] * h->esize;
    }
    // the fused sweep, unless the plan asks for the split kernels or has
    // lumped elements (whose E corrections run between the E and H updates)
    h->sweep_ok = !(pl->flags & XFDTD_FLAG_SPLIT_EH) && pl->n_injections == 0 && pl->n_inductor_cells == 0 &&
                  pl->index_bytes < 4 && pl->nz > 1 && pl->n_disp_cells == 0;
    h->sweep = h->sweep_ok && (pl->flags & XFDTD_FLAG_FUSED_EH);
    if (h->sweep_ok) {
      for (int c = 0; c < 6; ++c) h->F2[c] = h->alloc_bytes(d.cells * h->esize);
      for (int q = 0; q < 6; ++q) h->psi2[q] = sizes[q] ? h->alloc_bytes(sizes[q] * h->esize) : nullptr;
    }
  }

  // TFSF
  const xfdtd_tfsf_plan &tp = pl->tfsf;
  if (tp.enabled) {
    h->tfsf = true;
    if (tp.aux_len < 6) invalid("TFSF auxiliary grid too short");
    h->aux_len = tp.aux_len;
    h->tf_two_d = tp.enabled == 2;
    for (int a = 0; a < 3; ++a) {
      if (h->tf_two_d && a == 2) {   // TFSF2D: the box spans the one z cell
        if (tp.lo[2] != 0 || tp.hi[2] != 1) invalid("the 2-D TFSF box spans k = 0 .. 1");
      } else if (tp.lo[a] < 1 || tp.hi[a] <= tp.lo[a] || tp.hi[a] > n_axis[a] - 1) {
        invalid("TFSF box outside the grid");
      }
      h->tf_lo[a] = static_cast<int>(tp.lo[a]);
      h->tf_hi[a] = static_cast<int>(tp.hi[a]);
      const long long bn = tp.hi[a] - tp.lo[a];
      if (!tp.proj_full[a] || !tp.proj_half[a]) invalid("TFSF projection tables are required");
      h->tf_pf[a] = h->upload<double>(tp.proj_full[a], bn + 1);
      h->tf_ph[a] = h->upload<double>(tp.proj_half[a], bn + 2);
      if (pl->precision == XFDTD_FP32) {
        h->tf_pff[a] = static_cast<float *>(h->upload_real(tp.proj_full[a], bn + 1));
        h->tf_phf[a] = static_cast<float *>(h->upload_real(tp.proj_half[a], bn + 2));
      }
      h->tf_ca[a] = tp.ca[a];
      h->tf_cb[a] = tp.cb[a];
      h->tf_te[a] = tp.transform_e[a];
      h->tf_th[a] = tp.transform_h[a];
    }
    // Every interpolation index (a sum of one entry per axis, minus 0.5 for
    // H) must stay inside the 1-D arrays: e_inc has L entries, h_inc L-1.
    double lo_sum = 0, hi_sum = 0;
    for (int a = 0; a < 3; ++a) {
      const long long bn = tp.hi[a] - tp.lo[a];
      double mn = tp.proj_full[a][0], mx = mn;
      for (long long q = 0; q < bn + 1; ++q) { mn = std::min(mn, tp.proj_full[a][q]); mx = std::max(mx, tp.proj_full[a][q]); }
      for (long long q = 0; q < bn + 2; ++q) { mn = std::min(mn, tp.proj_half[a][q]); mx = std::max(mx, tp.proj_half[a][q]); }
      if (!std::isfinite(mn) || !std::isfinite(mx)) invalid("TFSF projection is not finite");
      lo_sum += mn;
      hi_sum += mx;
    }
    if (lo_sum - 0.5 < 0 || std::floor(hi_sum) + 1 > tp.aux_len - 2) invalid("TFSF box does not fit the auxiliary grid");
    h->tf_ceihi = tp.ceihi;
    h->tf_chiei = tp.chiei;
    h->tf_c1 = tp.mur_c1;
    h->tf_c2 = tp.mur_c2;
    if (!tp.source) invalid("TFSF source samples are required");
    h->tf_src = h->upload<double>(tp.source, pl->total_steps);
    h->tf_state = h->alloc<double>(2 * static_cast<size_t>(tp.aux_len) + 1);
    h->tf_inc = h->alloc<double>(2 * 6 * static_cast<size_t>(tp.aux_len));
    if (pl->precision == XFDTD_FP32) h->tf_incf = h->alloc<float>(2 * 6 * static_cast<size_t>(tp.aux_len));
  }

  // NF-FF
  const xfdtd_nffft_plan &np = pl->nffft;
  if (np.enabled == 2) {   // NffftBroadBand: every step's samples, the far field at the end
    h->nffft = true;
    h->nf_bb = true;
    if (np.n_theta != 1 || np.n_phi != 1 || !np.theta || !np.phi) invalid("broadband NF-FF takes one direction");
    h->bb_theta = np.theta[0];
    h->bb_phi = np.phi[0];
    for (int a = 0; a < 3; ++a) {
      if (np.lo[a] < 1 || np.hi[a] <= np.lo[a] || np.hi[a] > n_axis[a] - 1) invalid("NF-FF box outside the grid");
      h->nf_lo[a] = static_cast<int>(np.lo[a]);
      h->nf_hi[a] = static_cast<int>(np.hi[a]);
    }
    const long long bx = np.hi[0] - np.lo[0], by = np.hi[1] - np.lo[1], bz = np.hi[2] - np.lo[2];
    const long long face[3] = {by * bz, bz * bx, bx * by};
    h->nf_rows = static_cast<int>(std::max<long long>(1, pl->total_steps));
    long long bytes = 0;
    for (int g = 0; g < 3; ++g) bytes += static_cast<long long>(h->nf_rows) * 8 * face[g] * h->esize;
    if (bytes > (96ll << 30)) invalid("broadband NF-FF samples above 96 GiB");
    for (int g = 0; g < 3; ++g) h->nf_buf[g] = h->alloc_bytes(static_cast<size_t>(h->nf_rows) * 8 * face[g] * h->esize);
  } else if (np.enabled) {
    h->nffft = true;
    if (np.n_freq < 1) invalid("NF-FF needs at least one frequency");
    h->nf = np.n_freq;
    h->nt = np.n_theta;
    h->np = np.n_phi;
    for (int a = 0; a < 3; ++a) {
      if (np.lo[a] < 1 || np.hi[a] <= np.lo[a] || np.hi[a] > n_axis[a] - 1) invalid("NF-FF box outside the grid");
      h->nf_lo[a] = static_cast<int>(np.lo[a]);
      h->nf_hi[a] = static_cast<int>(np.hi[a]);
    }
    const long long bx = np.hi[0] - np.lo[0], by = np.hi[1] - np.lo[1], bz = np.hi[2] - np.lo[2];
    const long long face[3] = {by * bz, bz * bx, bx * by};
    for (int q = 0; q < 24; ++q) {
      h->acc_len[q] = np.n_freq * face[q / 8];
      h->acc[q] = h->alloc<double2>(h->acc_len[q]);
    }
    for (int g = 0; g < 3; ++g) h->nf_buf[g] = h->alloc_bytes(static_cast<size_t>(h->nf_batch) * 8 * face[g] * h->esize);
    if (!np.phase_j || !np.phase_m || !np.wave_number) invalid("NF-FF phase tables are required");
    h->phase_j = h->upload<double2>(reinterpret_cast<const double2 *>(np.phase_j), np.n_freq * pl->total_steps);
    h->phase_m = h->upload<double2>(reinterpret_cast<const double2 *>(np.phase_m), np.n_freq * pl->total_steps);
    if (h->precision == XFDTD_FP32) {   // FP32 copies for the FP32 form's batch partial sums
      const size_t n2 = static_cast<size_t>(np.n_freq) * pl->total_steps * 2;
      std::vector<float> fj(n2), fm(n2);
      for (size_t q = 0; q < n2; ++q) {
        fj[q] = static_cast<float>(np.phase_j[q]);
        fm[q] = static_cast<float>(np.phase_m[q]);
      }
      h->phase_jf = h->upload<float2>(reinterpret_cast<const float2 *>(fj.data()), n2 / 2);
      h->phase_mf = h->upload<float2>(reinterpret_cast<const float2 *>(fm.data()), n2 / 2);
    }
    h->ff_k = h->upload<double>(np.wave_number, np.n_freq);
    if (np.n_theta > 0 && np.n_phi > 0) {
      h->ff_theta = h->upload<double>(np.theta, np.n_theta);
      h->ff_phi = h->upload<double>(np.phi, np.n_phi);
      const size_t dirs = static_cast<size_t>(np.n_freq) * np.n_theta * np.n_phi;
      for (int q = 0; q < 8; ++q) h->ff_out[q] = h->alloc<double2>(dirs);
      for (int q = 0; q < 2; ++q) h->ff_power[q] = h->alloc<double>(dirs);
    }
  }

  // the NF-FF samples read [lo-1, hi] per axis; the TFSF H corrections write
  // cells on the surface of [lo-1, hi] of the TFSF box
  h->nf_beside_tfsf = h->nffft && h->tfsf;
  for (int a = 0; a < 3 && h->nf_beside_tfsf; ++a)
    if (!(h->nf_lo[a] > h->tf_lo[a] && h->nf_hi[a] < h->tf_hi[a])) h->nf_beside_tfsf = false;

  // sparse work
  h->n_waveforms = pl->n_waveforms;
  if (pl->n_waveforms) h->waveforms = h->upload<double>(pl->waveforms, static_cast<size_t>(pl->n_waveforms) * pl->total_steps);
  auto check_cell = [&](int comp, long long i, long long j, long long k) {
    if (comp < 0 || comp > 5) invalid("bad field component in a sparse entry");
    long long s[3];
    comp_shape(h, comp, s);
    if (i < 0 || j < 0 || k < 0 || i >= s[0] || j >= s[1] || k >= s[2]) invalid("sparse entry outside its component");
  };
  h->n_inj = pl->n_injections;
  if (pl->n_injections) {
    for (int q = 0; q < pl->n_injections; ++q) {
      const auto &c = pl->injections[q];
      check_cell(c.comp, c.i, c.j, c.k);
      if (c.comp > 2) invalid("injections act on E components");
      if (c.waveform < 0 || c.waveform >= pl->n_waveforms) invalid("injection waveform out of range");
    }
    h->inj = h->upload<xfdtd_injection>(pl->injections, pl->n_injections);
  }
  if (h->n_disp) {   // dispersive media (xfdtd_dispersive_medium / _cell)
    if (!(pl->disp_dl > 0)) invalid("dispersive media need the cell size");
    std::vector<xg::DispCell> cells(static_cast<size_t>(h->n_disp));
    for (int q = 0; q < h->n_disp; ++q) {
      const auto &c = pl->disp_cells[q];
      if (c.comp < 0 || c.comp > 2) invalid("dispersive cells are E components");
      check_cell(c.comp, c.i, c.j, c.k);
      if (c.i < 1 && c.comp != 0) invalid("dispersive cell on an outer wall");
      if (c.j < 1 && c.comp != 1) invalid("dispersive cell on an outer wall");
      if (c.k < 1 && c.comp != 2) invalid("dispersive cell on an outer wall");
      if (c.medium < 0 || c.medium >= pl->n_disp_media) invalid("dispersive medium index out of range");
      if (pl->disp_media[c.medium].kind < 1 || pl->disp_media[c.medium].kind > 3) invalid("unknown dispersive medium");
      cells[q] = xg::DispCell{c.i * h->d.si + c.j * h->d.sj + c.k, c.comp, c.medium};
    }
    h->disp_cells = h->upload<xg::DispCell>(cells.data(), cells.size());
    h->disp_dl = pl->disp_dl;
    auto media = [&](auto zero) {
      using R = decltype(zero);
      std::vector<xg::DispMedium<R>> m(static_cast<size_t>(pl->n_disp_media));
      for (int q = 0; q < pl->n_disp_media; ++q) {
        const auto &s0 = pl->disp_media[q];
        m[q] = xg::DispMedium<R>{s0.kind, R(s0.ca), R(s0.cb), R(s0.cc), R(s0.alpha), R(s0.xi), R(s0.gamma), R(s0.k),
                                 R(s0.beta)};
      }
      h->disp_media = h->upload<xg::DispMedium<R>>(m.data(), m.size());
    };
    if (h->precision == XFDTD_FP64) media(0.0);
    else media(0.0f);
    h->disp_j = h->alloc_bytes(static_cast<size_t>(h->n_disp) * h->esize);
    h->disp_jp = h->alloc_bytes(static_cast<size_t>(h->n_disp) * h->esize);
    h->disp_ep = h->alloc_bytes(static_cast<size_t>(h->n_disp) * h->esize);
  }
  h->n_ind = pl->n_inductor_cells;
  if (pl->n_inductor_cells) {
    for (int q = 0; q < pl->n_inductor_cells; ++q) {
      const auto &c = pl->inductor_cells[q];
      check_cell(c.comp, c.i, c.j, c.k);
      if (c.comp > 2) invalid("inductors act on E components");
    }
    h->ind = h->upload<xfdtd_inductor_cell>(pl->inductor_cells, pl->n_inductor_cells);
    h->ind_j = h->alloc<double>(pl->n_inductor_cells);
  }
  h->n_probes = pl->n_probes;
  if (pl->n_probes) {
    std::vector<int> off(pl->n_probes + 1, 0);
    int last = -1;
    for (int q = 0; q < pl->n_probe_terms; ++q) {
      const auto &c = pl->probe_terms[q];
      check_cell(c.comp, c.i, c.j, c.k);
      if (c.probe < last || c.probe >= pl->n_probes) invalid("probe terms must be grouped by probe in order");
      last = c.probe;
      off[c.probe + 1] += 1;
    }
    for (int q = 0; q < pl->n_probes; ++q) off[q + 1] += off[q];
    h->terms = h->upload<xfdtd_probe_term>(pl->probe_terms, std::max(1, pl->n_probe_terms));
    h->probe_off = h->upload<int>(off.data(), off.size());
    h->probe_out = h->alloc<double>(static_cast<size_t>(pl->n_probes) * pl->total_steps);
  }
  if (pl->n_snapshots < 0 || (pl->n_snapshots && !pl->snapshots)) invalid("bad snapshot list");
  if (pl->n_snapshots > 65535) invalid("at most 65535 snapshot series");
  long long snap_bytes = 0;
  for (int q = 0; q < pl->n_snapshots; ++q) {
    const xfdtd_snapshot_desc &sd = pl->snapshots[q];
    if (sd.comp < 0 || sd.comp > 5) invalid("bad field component in a snapshot series");
    if (sd.every < 1) invalid("snapshot interval must be at least 1");
    long long cs[3];
    comp_shape(h, sd.comp, cs);
    xg::SnapDev sv{};
    sv.comp = sd.comp;
    sv.cells = 1;
    for (int a = 0; a < 3; ++a) {
      if (sd.n[a] < 1 || sd.lo[a] < 0 || sd.lo[a] + sd.n[a] > cs[a]) invalid("snapshot box outside its component");
      sv.lo[a] = sd.lo[a];
      sv.n[a] = sd.n[a];
      sv.cells *= sd.n[a];
    }
    sv.every = sd.every;
    sv.last = sd.last;
    sv.n_regular = pl->total_steps > 0 ? (pl->total_steps - 1) / sd.every + 1 : 0;
    const bool extra = sd.last >= 0 && sd.last < pl->total_steps && sd.last % sd.every != 0;
    sv.extra = extra ? 1 : 0;
    sv.n_frames = sv.n_regular + sv.extra;
    snap_bytes += sv.n_frames * sv.cells * static_cast<long long>(h->esize);
    if (snap_bytes > (64ll << 30)) invalid("snapshot frames above 64 GiB");
    sv.frames = h->alloc_bytes(static_cast<size_t>(std::max(1ll, sv.n_frames * sv.cells)) * h->esize);
    h->snap_cells_max = std::max(h->snap_cells_max, sv.cells);
    h->snaps.push_back(sv);
  }
  if (!h->snaps.empty()) h->d_snaps = h->upload<xg::SnapDev>(h->snaps.data(), h->snaps.size());

  // per-axis index flags for the volume kernels' fast path
  for (int a = 0; a < 3; ++a) {
    const int n = n_axis[a];
    std::vector<uint8_t> fl(n + 1, 0);
    for (int q = 0; q <= n; ++q) {
      const bool slab_e = pl->cpml[a].n_layers && pl->cpml[a].slot_e[q] >= 0;
      const bool slab_h = pl->cpml[a].n_layers && pl->cpml[a].slot_h[q] >= 0;
      if (q == 0 || q == n || slab_e) fl[q] |= xg::kSpecialE;
      if (q == n || slab_h) fl[q] |= xg::kSpecialH;
      if (h->tfsf && (q == h->tf_lo[a] || q == h->tf_hi[a])) fl[q] |= xg::kTfsfE;
    }
    h->axis_flags[a] = h->upload<uint8_t>(fl.data(), fl.size());
    h->axis_flags_host[a] = fl;
  }
  volume_boxes(h, 0);
  volume_boxes(h, 1);
  with_types(h->precision, h->idx_bytes, [&](auto t, auto i) { interior_tma_setup<decltype(t), decltype(i)>(h); });

  h->d_step = h->alloc<long long>(1);
  h->d_status = h->alloc<int>(1);
  h->d_flag = h->alloc<int>(1);
  if (h->sweep_ok) {
    if (h->precision == XFDTD_FP64) {
      if (h->idx_bytes == 1) sweep_setup<double, uint8_t>(h);
      else sweep_setup<double, uint16_t>(h);
    } else {
      if (h->idx_bytes == 1) sweep_setup<float, uint8_t>(h);
      else sweep_setup<float, uint16_t>(h);
    }
  }
  // the TFSF corrections inside the wide decomposition's TMA launches (they
  // cover every cell): 3-D plane wave, no lumped element
  if (h->tfsf && !h->tf_two_d && h->n_inj == 0 && h->n_ind == 0 && h->n_disp == 0)
    for (int side = 0; side < 2; ++side) h->tf_fuse_ok[side] = h->wide_ok[side];
  XCHECK(cudaStreamSynchronize(h->stream));
  h->create_ms[0] = ms_since(t_begin);
  const auto t_tune = std::chrono::steady_clock::now();
  if (pl->flags & XFDTD_FLAG_AUTOTUNE) autotune(h, 3);
  h->create_ms[1] = ms_since(t_tune);
}

template <typename T>
void read_comp(xfdtd_handle *h, int comp, double *out, long long len) {
  long long s[3];
  comp_shape(h, comp, s);
  if (len != s[0] * s[1] * s[2]) invalid("length does not match the component shape");
  std::vector<T> buf(h->d.cells);
  XCHECK(cudaMemcpyAsync(buf.data(), h->F[comp], h->d.cells * sizeof(T), cudaMemcpyDeviceToHost, h->stream));
  h->d2h += h->d.cells * static_cast<long long>(sizeof(T));
  XCHECK(cudaStreamSynchronize(h->stream));
  long long o = 0;
  for (long long i = 0; i < s[0]; ++i)
    for (long long j = 0; j < s[1]; ++j)
      for (long long k = 0; k < s[2]; ++k) out[o++] = static_cast<double>(buf[i * h->d.si + j * h->d.sj + k]);
}

template <typename T>
void write_comp(xfdtd_handle *h, int comp, const double *in, long long len) {
  long long s[3];
  comp_shape(h, comp, s);
  if (len != s[0] * s[1] * s[2]) invalid("length does not match the component shape");
  std::vector<T> buf(h->d.cells, T(0));
  long long o = 0;
  for (long long i = 0; i < s[0]; ++i)
    for (long long j = 0; j < s[1]; ++j)
      for (long long k = 0; k < s[2]; ++k) buf[i * h->d.si + j * h->d.sj + k] = static_cast<T>(in[o++]);
  XCHECK(cudaMemcpyAsync(h->F[comp], buf.data(), h->d.cells * sizeof(T), cudaMemcpyHostToDevice, h->stream));
  h->h2d += h->d.cells * static_cast<long long>(sizeof(T));
  XCHECK(cudaStreamSynchronize(h->stream));
}

// cuFFT, loaded when a broadband far field is first asked for (the rest of
// the engine does not need it).
struct CufftApi {
  decltype(&cufftPlanMany) plan_many = nullptr;
  decltype(&cufftExecZ2Z) exec_z2z = nullptr;
  decltype(&cufftSetStream) set_stream = nullptr;
  decltype(&cufftDestroy) destroy = nullptr;
};
const CufftApi &cufft_api() {
  static const CufftApi api = [] {
    CufftApi a;
    void *lib = nullptr;
    for (const char *name : {"libcufft.so.12", "libcufft.so"})
      if (!lib) lib = dlopen(name, RTLD_NOW | RTLD_LOCAL);
    if (!lib) return a;
    a.plan_many = reinterpret_cast<decltype(a.plan_many)>(dlsym(lib, "cufftPlanMany"));
    a.exec_z2z = reinterpret_cast<decltype(a.exec_z2z)>(dlsym(lib, "cufftExecZ2Z"));
    a.set_stream = reinterpret_cast<decltype(a.set_stream)>(dlsym(lib, "cufftSetStream"));
    a.destroy = reinterpret_cast<decltype(a.destroy)>(dlsym(lib, "cufftDestroy"));
    return a;
  }();
  if (!api.plan_many || !api.exec_z2z || !api.set_stream || !api.destroy)
    throw Err{XFDTD_ERR_STATE, "cuFFT (libcufft.so) is not available for the broadband far field"};
  return api;
}

// NffftBroadBand::calculateLNXYZ (nffft_broadband.cpp:351-464): the six
// auxiliary arrays n_x, n_y, n_z, l_x, l_y, l_z over the N = 2T-1 output
// bins, from the samples of every step run so far.
template <typename T>
void broadband_aux(xfdtd_handle *h, std::vector<double2> &out) {
  const CufftApi &fft = cufft_api();
  const long long steps = h->total, N = 2 * steps - 1;
  const int li = h->nf_lo[0], lj = h->nf_lo[1], lk = h->nf_lo[2], ri = h->nf_hi[0], rj = h->nf_hi[1],
            rk = h->nf_hi[2];
  const int ci = li + (ri - li) / 2, cj = lj + (rj - lj) / 2, ck = lk + (rk - lk) / 2;   // GridBox centre
  const long long plane[3] = {static_cast<long long>(rj - lj) * (rk - lk), static_cast<long long>(ri - li) * (rk - lk),
                              static_cast<long long>(ri - li) * (rj - lj)};
  // buffer quantity q % 4 of each face pair -> auxiliary array (0 n_x .. 5 l_z)
  const int target[3][4] = {{1, 2, 4, 5}, {2, 0, 5, 3}, {0, 1, 3, 4}};
  double2 *acc = nullptr, *in = nullptr, *spec = nullptr;
  XCHECK(cudaMalloc(&acc, sizeof(double2) * 6 * N));
  XCHECK(cudaMemsetAsync(acc, 0, sizeof(double2) * 6 * N, h->stream));
  const long long max_plane = std::max({plane[0], plane[1], plane[2]});
  const int chunk = static_cast<int>(std::max<long long>(1, std::min<long long>(max_plane, (256ll << 20) / (N * 16))));
  XCHECK(cudaMalloc(&in, sizeof(double2) * chunk * N));
  XCHECK(cudaMalloc(&spec, sizeof(double2) * chunk * N));
  std::vector<std::pair<int, cufftHandle>> plans;
  auto plan_for = [&](int nb) {
    for (auto &p : plans)
      if (p.first == nb) return p.second;
    cufftHandle ph;
    int n = static_cast<int>(N);
    if (fft.plan_many(&ph, 1, &n, nullptr, 1, n, nullptr, 1, n, CUFFT_Z2Z, nb) != CUFFT_SUCCESS)
      throw Err{XFDTD_ERR_CUDA, "cufftPlanMany failed"};
    fft.set_stream(ph, h->stream);
    plans.push_back({nb, ph});
    return ph;
  };
  try {
    const double eta_dir[3] = {std::sin(h->bb_theta) * std::cos(h->bb_phi), std::sin(h->bb_theta) * std::sin(h->bb_phi),
                               std::cos(h->bb_theta)};
    const bool three_d = rk - lk > 1;
    for (int g = 0; g < (three_d ? 3 : 2); ++g)
      for (int side = 0; side < 2; ++side)
        for (int qq = 0; qq < 4; ++qq) {
          const int q = side * 4 + qq;
          for (long long c0 = 0; c0 < plane[g]; c0 += chunk) {
            const int nb = static_cast<int>(std::min<long long>(chunk, plane[g] - c0));
            const long long elems = static_cast<long long>(nb) * N;
            xg::k_bb_load<T><<<static_cast<unsigned>(std::min<long long>((elems + 255) / 256, 65535)), 256, 0,
                               h->stream>>>(static_cast<const T *>(h->nf_buf[g]), q, plane[g], c0, nb, steps, N, in);
            XCHECK(cudaGetLastError());
            if (fft.exec_z2z(plan_for(nb), reinterpret_cast<cufftDoubleComplex *>(in),
                             reinterpret_cast<cufftDoubleComplex *>(spec), CUFFT_FORWARD) != CUFFT_SUCCESS)
              throw Err{XFDTD_ERR_CUDA, "cufftExecZ2Z failed"};
            xg::BbChunk c{};
            c.group = g;
            c.side = side;
            c.c0 = c0;
            c.nb = nb;
            if (g == 0) {
              c.du = rk - lk;
              c.face_coord = (side ? ri : li) - ci;
              c.off_v = lj + 0.5 - cj;
              c.off_u = lk + 0.5 - ck;
              c.ds = h->dl[1] * h->dl[2];
            } else if (g == 1) {
              c.du = rk - lk;
              c.face_coord = (side ? rj : lj) - cj;
              c.off_v = li + 0.5 - ci;
              c.off_u = lk + 0.5 - ck;
              c.ds = h->dl[0] * h->dl[2];
            } else {
              c.du = rj - lj;
              c.face_coord = (side ? rk : lk) - ck;
              c.off_v = li + 0.5 - ci;
              c.off_u = lj + 0.5 - cj;
              c.ds = h->dl[0] * h->dl[1];
            }
            for (int a = 0; a < 3; ++a) {
              c.dir[a] = eta_dir[a];
              c.dl[a] = h->dl[a];
            }
            c.fs = 1 / h->dt;
            c.n = static_cast<double>(N);
            c.pi = kPi;
            c.c_0 = std::sqrt(1 / (kEps0 * kMu0));   // constant.h C_0
            xg::k_bb_phase_sum<<<static_cast<unsigned>(N), 256, 0, h->stream>>>(c, spec, acc + target[g][qq] * N);
            XCHECK(cudaGetLastError());
          }
        }
    out.resize(static_cast<size_t>(6 * N));
    XCHECK(cudaMemcpyAsync(out.data(), acc, sizeof(double2) * 6 * N, cudaMemcpyDeviceToHost, h->stream));
    XCHECK(cudaStreamSynchronize(h->stream));
  } catch (...) {
    for (auto &p : plans) fft.destroy(p.second);
    cudaFree(acc);
    cudaFree(in);
    cudaFree(spec);
    throw;
  }
  for (auto &p : plans) fft.destroy(p.second);
  cudaFree(acc);
  cudaFree(in);
  cudaFree(spec);
  h->d2h += static_cast<long long>(sizeof(double2)) * 6 * N;
}

void run_far_field(xfdtd_handle *h) {
  if (!h->nffft) throw Err{XFDTD_ERR_STATE, "the plan has no NF-FF box"};
  if (h->nf_bb) throw Err{XFDTD_ERR_STATE, "a broadband NF-FF has its own far field (xfdtd_broadband_far_field)"};
  if (!h->ff_theta) throw Err{XFDTD_ERR_STATE, "the plan has no far-field directions"};
  if (h->ff_step == h->host_step) return;
  nffft_flush(h);
  xg::FarParams p{};
  for (int a = 0; a < 3; ++a) {
    p.lo[a] = h->nf_lo[a];
    p.hi[a] = h->nf_hi[a];
    p.dl[a] = h->dl[a];
  }
  p.nf = h->nf;
  p.nt = h->nt;
  p.np = h->np;
  for (int q = 0; q < 24; ++q) p.acc[q] = h->acc[q];
  p.theta = h->ff_theta;
  p.phi = h->ff_phi;
  p.k = h->ff_k;
  p.eta0 = std::sqrt(kMu0 / kEps0);
  p.pi = kPi;
  for (int q = 0; q < 8; ++q) p.out[q] = h->ff_out[q];
  for (int q = 0; q < 2; ++q) p.power[q] = h->ff_power[q];
  xg::k_far_field<<<h->nf * h->nt * h->np, 256, 0, h->stream>>>(p);
  XCHECK(cudaGetLastError());
  XCHECK(cudaStreamSynchronize(h->stream));
  h->ff_step = h->host_step;
}

void do_steps(xfdtd_handle *h, long long n) {
  if (n < 0) invalid("negative step count");
  if (h->host_step + n > h->total) throw Err{XFDTD_ERR_STATE, "stepping past the plan's total_steps"};
  const bool graph = (h->flags & XFDTD_FLAG_GRAPH) && !(h->flags & XFDTD_FLAG_PROFILE);
  const long long end = h->host_step + n;
  const int B = h->nf_batch;
  // single steps up to a batch boundary, whole graphs, then single steps
  while (h->host_step < end) {
    const bool aligned = h->host_step % B == 0;
    const long long graph_len = h->gexec ? h->graph_steps : 4 * B;
    if (graph && aligned && end - h->host_step >= graph_len) {
      // the graph's steps fold whole batches from its first step on
      nffft_flush(h);
      if (!h->gexec) build_graph(h, static_cast<int>(graph_len));
      XCHECK(cudaGraphLaunch(h->gexec, h->stream));
      h->host_step += h->graph_steps;
      h->launch_count += h->graph_launches;
      if (h->nffft && !h->nf_bb && !h->sweep && h->nf_split) {   // split sampling: the last batch and H half wait
        h->nf_done = h->host_step - B;
        h->nf_pending = true;
      } else if (h->nffft) {
        h->nf_done = h->host_step;
      }
      continue;
    }
    enqueue_step(h, h->host_step);
    h->host_step += 1;
  }
}

}  // namespace

extern "C" {

const char *xfdtd_version(void) { return "xfdtd_gb300 engine 0.1 (sm_103a)"; }

int xfdtd_create(const xfdtd_plan_desc *plan, xfdtd_handle **out) {
  if (!plan || !out) return XFDTD_ERR_INVALID_PLAN;
  std::unique_ptr<xfdtd_handle> h(new xfdtd_handle());
  int rc = guarded(h.get(), [&] { create(plan, h.get()); });
  if (rc != XFDTD_OK) {
    // keep the handle so that the caller can read the message; it holds no work
    *out = h.release();
    return rc;
  }
  *out = h.release();
  return XFDTD_OK;
}

int xfdtd_step(xfdtd_handle *h, int64_t n) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    do_steps(h, n);
    prof_collect(h);
  });
}

int xfdtd_synchronize(xfdtd_handle *h) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    XCHECK(cudaStreamSynchronize(h->stream));
    check_status(h);
  });
}

int xfdtd_step_timed(xfdtd_handle *h, int64_t n, double *ms) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    cudaEvent_t a, b;
    XCHECK(cudaEventCreate(&a));
    XCHECK(cudaEventCreate(&b));
    XCHECK(cudaEventRecord(a, h->stream));
    do_steps(h, n);
    XCHECK(cudaEventRecord(b, h->stream));
    XCHECK(cudaEventSynchronize(b));
    float f = 0;
    XCHECK(cudaEventElapsedTime(&f, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    prof_collect(h);
    if (ms) *ms = f;
  });
}

int xfdtd_current_step(xfdtd_handle *h, int64_t *step) {
  if (!h || !step) return XFDTD_ERR_STATE;
  *step = h->host_step;
  return XFDTD_OK;
}

int xfdtd_read_field(xfdtd_handle *h, int comp, double *out, int64_t len) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (comp < 0 || comp > 5) invalid("component must be 0..5");
    if (h->precision == XFDTD_FP64) read_comp<double>(h, comp, out, len);
    else read_comp<float>(h, comp, out, len);
  });
}

int xfdtd_write_field(xfdtd_handle *h, int comp, const double *in, int64_t len) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (comp < 0 || comp > 5) invalid("component must be 0..5");
    if (h->precision == XFDTD_FP64) write_comp<double>(h, comp, in, len);
    else write_comp<float>(h, comp, in, len);
  });
}

int xfdtd_read_probes(xfdtd_handle *h, double *out, int64_t len) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (len != static_cast<int64_t>(h->n_probes) * h->total) invalid("length must be n_probes * total_steps");
    if (!len) return;
    XCHECK(cudaMemcpyAsync(out, h->probe_out, len * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    h->d2h += len * static_cast<long long>(sizeof(double));
    XCHECK(cudaStreamSynchronize(h->stream));
  });
}

int xfdtd_snapshot_frames(xfdtd_handle *h, int s, int64_t *count, int64_t *steps, int64_t max) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (s < 0 || s >= static_cast<int>(h->snaps.size())) invalid("no such snapshot series");
    const xg::SnapDev &sv = h->snaps[s];
    if (count) *count = sv.n_frames;
    if (steps) {   // step order: the multiples of every, with `last` in its place
      long long f = 0;
      for (long long r = 0; r < sv.n_regular && f < max; ++r) {
        if (sv.extra && r * sv.every > sv.last && (r == 0 || (r - 1) * sv.every < sv.last) && f < max)
          steps[f++] = sv.last;
        if (f < max) steps[f++] = r * sv.every;
      }
      if (sv.extra && (sv.n_regular - 1) * sv.every < sv.last && f < max) steps[f++] = sv.last;
    }
  });
}

int xfdtd_read_snapshot(xfdtd_handle *h, int s, int64_t frame, double *out, int64_t len) {
  if (!h || !out) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (s < 0 || s >= static_cast<int>(h->snaps.size())) invalid("no such snapshot series");
    const xg::SnapDev &sv = h->snaps[s];
    if (frame < 0 || frame >= sv.n_frames) invalid("no such frame");
    if (len != sv.cells) invalid("length must be the series' box cells");
    const char *src = static_cast<const char *>(sv.frames) + static_cast<size_t>(frame * sv.cells) * h->esize;
    if (h->precision == XFDTD_FP64) {
      XCHECK(cudaMemcpyAsync(out, src, len * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      XCHECK(cudaStreamSynchronize(h->stream));
    } else {
      std::vector<float> tmp(static_cast<size_t>(len));
      XCHECK(cudaMemcpyAsync(tmp.data(), src, len * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
      XCHECK(cudaStreamSynchronize(h->stream));
      for (int64_t q = 0; q < len; ++q) out[q] = tmp[static_cast<size_t>(q)];
    }
    h->d2h += static_cast<long long>(len) * static_cast<long long>(h->esize);
  });
}

int xfdtd_broadband_far_field(xfdtd_handle *h, double *out, int64_t len) {
  if (!h || !out) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (!h->nf_bb) invalid("the plan has no broadband NF-FF");
    const long long N = 2 * h->total - 1;
    if (len != 12 * N) invalid("length must be 6 * (2 * total_steps - 1) complex values");
    std::vector<double2> aux;
    if (h->precision == XFDTD_FP64) broadband_aux<double>(h, aux);
    else broadband_aux<float>(h, aux);
    std::memcpy(out, aux.data(), aux.size() * sizeof(double2));
  });
}

int xfdtd_read_nffft(xfdtd_handle *h, int which, double *out, int64_t len) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (!h->nffft || h->nf_bb) throw Err{XFDTD_ERR_STATE, "the plan has no NF-FF running DFT"};
    if (which < 0 || which >= 24) invalid("accumulator index must be 0..23");
    if (len != 2 * h->acc_len[which]) invalid("length must be 2 * n_freq * face cells");
    nffft_flush(h);
    std::vector<double2> buf(h->acc_len[which]);
    XCHECK(cudaMemcpyAsync(buf.data(), h->acc[which], buf.size() * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
    h->d2h += static_cast<long long>(buf.size() * sizeof(double2));
    XCHECK(cudaStreamSynchronize(h->stream));
    if (which / 8 == 1) {  // Y faces: device [n][i][k] -> reference [n][k][i]
      const long long bx = h->nf_hi[0] - h->nf_lo[0], bz = h->nf_hi[2] - h->nf_lo[2];
      for (long long n = 0; n < h->nf; ++n)
        for (long long i = 0; i < bx; ++i)
          for (long long k = 0; k < bz; ++k) {
            const double2 v = buf[(n * bx + i) * bz + k];
            const long long o = (n * bz + k) * bx + i;
            out[2 * o] = v.x;
            out[2 * o + 1] = v.y;
          }
    } else {
      for (size_t q = 0; q < buf.size(); ++q) {
        out[2 * q] = buf[q].x;
        out[2 * q + 1] = buf[q].y;
      }
    }
  });
}

int xfdtd_far_field(xfdtd_handle *h, int which, double *out, int64_t len) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    run_far_field(h);
    const long long dirs = static_cast<long long>(h->nf) * h->nt * h->np;
    if (which >= 0 && which < 8) {
      if (len != 2 * dirs) invalid("length must be 2 * n_freq * n_theta * n_phi");
      XCHECK(cudaMemcpyAsync(out, h->ff_out[which], dirs * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
      h->d2h += dirs * static_cast<long long>(sizeof(double2));
    } else if (which == 8 || which == 9) {
      if (len != dirs) invalid("length must be n_freq * n_theta * n_phi");
      XCHECK(cudaMemcpyAsync(out, h->ff_power[which - 8], dirs * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      h->d2h += dirs * static_cast<long long>(sizeof(double));
    } else {
      invalid("far-field output must be 0..9");
    }
    XCHECK(cudaStreamSynchronize(h->stream));
  });
}

int xfdtd_check_finite(xfdtd_handle *h) {
  if (!h) return XFDTD_ERR_STATE;
  int rc = guarded(h, [&] {
    XCHECK(cudaMemsetAsync(h->d_flag, 0, sizeof(int), h->stream));
    for (int c = 0; c < 6; ++c) {
      if (h->precision == XFDTD_FP64)
        xg::k_finite<double><<<304, 256, 0, h->stream>>>(static_cast<const double *>(h->F[c]), h->d.cells, h->d_flag);
      else
        xg::k_finite<float><<<304, 256, 0, h->stream>>>(static_cast<const float *>(h->F[c]), h->d.cells, h->d_flag);
      XCHECK(cudaGetLastError());
    }
    int flag = 0;
    XCHECK(cudaMemcpyAsync(&flag, h->d_flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    XCHECK(cudaStreamSynchronize(h->stream));
    if (flag) throw Err{XFDTD_ERR_NAN, "non-finite field value"};
  });
  return rc;
}

int xfdtd_profile(xfdtd_handle *h, int max, const char **names, double *ms, int64_t *launches, int *count) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    prof_collect(h);
    int c = 0;
    for (int q = 0; q < kNumKernels && c < max; ++q) {
      if (!h->prof_n[q]) continue;
      if (names) names[c] = kKernelNames[q];
      if (ms) ms[c] = h->prof_ms[q];
      if (launches) launches[c] = h->prof_n[q];
      ++c;
    }
    if (count) *count = c;
  });
}

int xfdtd_profile_reset(xfdtd_handle *h) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    prof_collect(h);
    for (int q = 0; q < kNumKernels; ++q) {
      h->prof_ms[q] = 0;
      h->prof_n[q] = 0;
    }
  });
}

int xfdtd_autotune(xfdtd_handle *h, int trials) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] { autotune(h, trials > 0 ? trials : 3); });
}

int xfdtd_kernel_variants(xfdtd_handle *h, int *n, int *current_e, int *current_h, double *trial_ms) {
  if (!h) return XFDTD_ERR_STATE;
  if (h->sweep) {   // one fused kernel: its variants stand for both sides
    if (n) *n = kNumSweepVariants;
    if (current_e) *current_e = h->var_s;
    if (current_h) *current_h = h->var_s;
    if (trial_ms)
      for (int v = 0; v < kNumSweepVariants; ++v) trial_ms[2 * v] = trial_ms[2 * v + 1] = h->sweep_ms[v];
    return XFDTD_OK;
  }
  if (n) *n = kNumVariants;
  if (current_e) *current_e = h->var_e;
  if (current_h) *current_h = h->var_h;
  if (trial_ms)
    for (int v = 0; v < kNumVariants; ++v) {
      trial_ms[2 * v] = h->tune_ms[0][v];
      trial_ms[2 * v + 1] = h->tune_ms[1][v];
    }
  return XFDTD_OK;
}

int xfdtd_set_kernel_variant(xfdtd_handle *h, int e_variant, int h_variant) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (h->sweep) {
      if (e_variant < 0 || e_variant >= kNumSweepVariants || h_variant != e_variant)
        invalid("fused-sweep variant out of range (E and H variants must be equal)");
      h->var_s = e_variant;
      if (h->gexec) {
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
      }
      return;
    }
    if (e_variant < 0 || e_variant >= kNumVariants || h_variant < 0 || h_variant >= kNumVariants ||
        !variant_allowed(h, kVariants[e_variant]) || !variant_allowed(h, kVariants[h_variant]))
      invalid("kernel variant not available for this precision");
    h->var_e = e_variant;
    h->var_h = h_variant;
    for (int side = 0; side < 2; ++side)   // a z-edge shell variant needs the wide decomposition
      if (!shell_allowed(h, kShellVariants[h->shell_var[side]], side_wide(h, side))) h->shell_var[side] = 0;
    if (h->gexec) {   // the captured graph holds the old launches
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
  });
}

int xfdtd_set_wait_limit(xfdtd_handle *h, int64_t polls) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (polls < 0 || polls > xg::kItWaitLimit) invalid("wait limit out of range (0 .. 2^22 polls)");
    h->wait_polls = static_cast<int>(polls);
    if (h->gexec) {   // the captured graph holds the old launch parameters
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
  });
}

int xfdtd_shell_variants(xfdtd_handle *h, int *n, int *current_e, int *current_h) {
  if (!h) return XFDTD_ERR_STATE;
  if (n) *n = kNumShellVariants;
  if (current_e) *current_e = h->shell_var[0];
  if (current_h) *current_h = h->shell_var[1];
  return XFDTD_OK;
}

int xfdtd_set_shell_variant(xfdtd_handle *h, int e_variant, int h_variant) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (e_variant < 0 || e_variant >= kNumShellVariants || h_variant < 0 || h_variant >= kNumShellVariants)
      invalid("shell-kernel variant out of range");
    if (!shell_allowed(h, kShellVariants[e_variant], side_wide(h, 0)) ||
        !shell_allowed(h, kShellVariants[h_variant], side_wide(h, 1)))
      invalid("shell-kernel variant needs the wide decomposition (a wide kernel variant)");
    h->shell_var[0] = e_variant;
    h->shell_var[1] = h_variant;
    if (h->gexec) {   // the captured graph holds the old launches
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
  });
}

int xfdtd_volume_split(xfdtd_handle *h, int64_t cells[4]) {
  if (!h || !cells) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    for (int side = 0; side < 2; ++side) {
      const bool w = side_wide(h, side);
      cells[2 * side] = side_interior_cells(h, side, w);
      cells[2 * side + 1] = side_shell_cells(h, side, w);
    }
  });
}

int xfdtd_volume_decomposition(xfdtd_handle *h, int wide[2]) {
  if (!h || !wide) return XFDTD_ERR_STATE;
  for (int side = 0; side < 2; ++side) wide[side] = side_wide(h, side) ? 1 : 0;
  return XFDTD_OK;
}

int xfdtd_launch_count(xfdtd_handle *h, int64_t *n) {
  if (!h || !n) return XFDTD_ERR_STATE;
  *n = h->launch_count;
  return XFDTD_OK;
}

int xfdtd_launches_per_step(xfdtd_handle *h, int *n) {
  if (!h || !n) return XFDTD_ERR_STATE;
  *n = launches_per_step(h);
  return XFDTD_OK;
}

int xfdtd_transfer_bytes(xfdtd_handle *h, int64_t *h2d, int64_t *d2h) {
  if (!h) return XFDTD_ERR_STATE;
  if (h2d) *h2d = h->h2d;
  if (d2h) *d2h = h->d2h;
  return XFDTD_OK;
}

int xfdtd_set_tfsf_fusion(xfdtd_handle *h, int e_on, int h_on) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    h->tf_fuse_on[0] = e_on != 0;
    h->tf_fuse_on[1] = h_on != 0;
    if (h->gexec) {   // the captured graph holds the old launches
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
  });
}

int xfdtd_set_nffft_split(xfdtd_handle *h, int on) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    nffft_flush(h);   // no H half left pending across the switch
    h->nf_split = on != 0;
    if (h->gexec) {   // the captured graph holds the old launches
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
  });
}

int xfdtd_nffft_split(xfdtd_handle *h, int *on, float ms[2]) {
  if (!h || !on) return XFDTD_ERR_STATE;
  *on = (h->nffft && !h->nf_bb && h->nf_split) ? 1 : 0;
  if (ms) {
    ms[0] = h->nf_sched_ms[0];
    ms[1] = h->nf_sched_ms[1];
  }
  return XFDTD_OK;
}

int xfdtd_tfsf_fusion(xfdtd_handle *h, int active[2]) {
  if (!h || !active) return XFDTD_ERR_STATE;
  for (int side = 0; side < 2; ++side) active[side] = tfsf_fused(h, side) ? 1 : 0;
  return XFDTD_OK;
}

int xfdtd_create_times(xfdtd_handle *h, double ms[2]) {
  if (!h || !ms) return XFDTD_ERR_STATE;
  ms[0] = h->create_ms[0];
  ms[1] = h->create_ms[1];
  return XFDTD_OK;
}

int xfdtd_device_bytes(xfdtd_handle *h, int64_t *bytes) {
  if (!h || !bytes) return XFDTD_ERR_STATE;
  *bytes = static_cast<int64_t>(h->bytes + adjoint_bytes(h));
  return XFDTD_OK;
}

int xfdtd_index_bytes(xfdtd_handle *h, int *bytes) {
  if (!h || !bytes) return XFDTD_ERR_STATE;
  *bytes = h->idx_bytes;
  return XFDTD_OK;
}

const char *xfdtd_last_error(xfdtd_handle *h) { return h ? h->err.c_str() : "null handle"; }

void xfdtd_destroy(xfdtd_handle *h) {
  if (!h) return;
  if (h->stream) {
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
  }
  delete h;
}

}  // extern "C"

// ================================================================ batch ===
// Many independent handles advanced together (batch.cuh): one launch per
// phase over the (simulation, tile) work list of every member still
// running, the step loop replayed from a CUDA graph per set of running
// members.  Members keep their own buffers and are read through the
// ordinary entry points once the batch has been synchronised.

struct xfdtd_batch {
  std::string err;
  std::vector<xfdtd_handle *> m;
  int device = 0, precision = XFDTD_FP64, idx_bytes = 1, flags = 0;
  int n_sm = 152;
  bool ct = false;   // volume kernels read the compact coefficient table (members with many materials)
  cudaStream_t stream = nullptr;
  cudaStream_t shell = nullptr;   // shell kernels, beside the interior kernels
  cudaEvent_t ev_fork[2] = {}, ev_join[2] = {};
  long long clock = 0;   // steps taken (every member started at step 0)
  long long nf_done = 0;
  long long launches = 0;
  std::vector<void *> allocs;
  // per-member parameter arrays (device), built once
  void *tsurf = nullptr, *nfp = nullptr, *aux = nullptr;
  // volume parameters of each group of up to kBatchGroup members (host
  // bytes of an xg::VolGroup, passed by value to the volume launches)
  std::vector<std::vector<unsigned char>> group_params;
  xg::InteriorBox *vin[2] = {};   // per side: the members' interior boxes (k0 on the 32-cell tile grid)
  xg::ShellBoxes *vshell[2] = {};  // per side: the members' shells
  int2 *nf_grid = nullptr;
  int *nf_nb = nullptr;
  // work lists of the running members (device, sized for all members)
  std::vector<int> running;
  bool lists_ok = false;
  struct VolLists {   // per group and side: blocks of the interior and shell launches
    xg::GroupBlocks in[2] = {}, sh[2] = {};
    xg::GroupBlocks tw[2] = {}, tz[2] = {};   // the TMA-staged wide and z-edge launches
  };
  std::vector<VolLists> vl;
  // members on the wide decomposition's TMA-staged launches (batch.cuh
  // k_tma_batch): per member the flag; per side their tensor maps, the
  // wide (MODE 1) and z-edge (MODE 2) boxes and tile grids (device); the
  // members' status words
  std::vector<char> tma_m;
  int n_tma = 0;
  xg::ItMaps *tmaps[2] = {};
  xg::InteriorBox *tbox[2][2] = {};   // [side][mode - 1]
  int2 *tgrid[2][2] = {};
  std::vector<unsigned> ttiles[2][2];   // host: tiles per member
  int **status_list = nullptr;
  xg::WorkItem *it_te = nullptr, *it_th = nullptr, *it_nf = nullptr, *it_fold = nullptr;
  int n_te = 0, n_th = 0, n_nf = 0, n_fold = 0;
  int *aux_list = nullptr;
  int n_aux = 0;
  long long **step_list = nullptr;
  // graph of kGraphSteps steps for the current running set
  cudaGraphExec_t gexec = nullptr;
  long long graph_launches = 0;

  template <class P>
  P *alloc(size_t count) {
    void *p = nullptr;
    XCHECK(cudaMalloc(&p, std::max<size_t>(count * sizeof(P), 16)));
    allocs.push_back(p);
    return static_cast<P *>(p);
  }
  ~xfdtd_batch() {
    if (gexec) cudaGraphExecDestroy(gexec);
    for (void *p : allocs) cudaFree(p);
    for (int q = 0; q < 2; ++q) {
      if (ev_fork[q]) cudaEventDestroy(ev_fork[q]);
      if (ev_join[q]) cudaEventDestroy(ev_join[q]);
    }
    if (shell) cudaStreamDestroy(shell);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

constexpr int kBatchGraphSteps = 32;   // a multiple of the NF-FF batch
constexpr int kBatchChunk = 16;        // planes per block of the TMA-staged launches

template <typename T, typename I>
void batch_setup(xfdtd_batch *b) {
  const int n = static_cast<int>(b->m.size());
  const int groups = (n + xg::kBatchGroup - 1) / xg::kBatchGroup;
  std::vector<xg::VolGroup<T, I>> vg(groups);
  std::vector<xg::TfsfSurfParams<T>> ts(n);
  std::vector<xg::NfParams<T>> nf(n);
  std::vector<xg::AuxParams> ax(n);
  std::vector<int2> grid(n);
  std::vector<int> nb(n);
  std::vector<xg::InteriorBox> vin[2];
  std::vector<xg::ShellBoxes> vsh[2];
  for (int q = 0; q < n; ++q) {
    xfdtd_handle *h = b->m[q];
    vg[q / xg::kBatchGroup].m[q % xg::kBatchGroup] = vol_params<T, I>(h);
    for (int side = 0; side < 2; ++side) {
      xg::InteriorBox in = h->vin[side];
      in.k0 = in.lo[2] / 32 * 32;
      vin[side].push_back(in);
      vsh[side].push_back(h->vshell[side]);
    }
    if (h->tfsf) {
      ts[q] = tfsf_surf_params<T>(h);
      ax[q] = aux_params(h);
    }
    if (h->nffft) {
      nf[q] = nf_params<T>(h);
      const dim3 g = nffft_grid(h);
      grid[q] = make_int2(static_cast<int>(g.x), static_cast<int>(g.y));
      nb[q] = static_cast<int>(nffft_fold_blocks(h));
    }
  }
  auto up = [&](auto &v) {
    using E = typename std::remove_reference<decltype(v)>::type::value_type;
    E *d = b->alloc<E>(v.size());
    XCHECK(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(E), cudaMemcpyHostToDevice, b->stream));
    return d;
  };
  // the members on the TMA-staged launches, their maps, boxes and tile grids
  b->tma_m.assign(n, 0);
  b->n_tma = 0;
  std::vector<xg::ItMaps> tm[2];
  std::vector<xg::InteriorBox> tb[2][2];
  std::vector<int2> tg[2][2];
  for (int q = 0; q < n; ++q) {
    xfdtd_handle *h = b->m[q];
    // FP32 only, on launches capped at 5 blocks per SM (variant_allowed)
    const bool ok = !(b->flags & XFDTD_FLAG_PLAIN_VOLUME) && sizeof(T) == 4 && h->it_ok[0] && h->it_ok[1] &&
                    h->wide_ok[0] && h->wide_ok[1];
    if (ok && h->itm_base != h->F[0]) interior_tma_encode<T, I>(h);   // maps of the current buffers
    b->tma_m[q] = ok ? 1 : 0;
    b->n_tma += ok ? 1 : 0;
    for (int side = 0; side < 2; ++side) {
      tm[side].push_back(h->itm[side]);
      for (int mode = 1; mode <= 2; ++mode) {
        const xg::InteriorBox in = mode == 2 ? h->vin_z[side] : h->vin_w[side];
        const int nj = in.hi[1] - in.lo[1] + 1, ni = in.hi[0] - in.lo[0] + 1;
        const int K = xg::kItK, J = xg::kItThreads / xg::kItK;
        int nk = mode == 2 ? (in.pz_lo + K - 1) / K + (in.hi[2] - in.pz_hi + K - 1) / K : (in.hi[2] - in.lo[2] + K) / K;
        const bool cells = mode == 2 ? h->vshell_w_cells[side] > 0 : h->vin_w_cells[side] > 0;
        if (!ok || !cells || nj <= 0 || ni <= 0) nk = 0;
        const int gj = nj > 0 ? (nj + J - 1) / J : 0, gi = ni > 0 ? (ni + kBatchChunk - 1) / kBatchChunk : 0;
        tb[side][mode - 1].push_back(in);
        tg[side][mode - 1].push_back(make_int2(std::max(nk, 1), std::max(gj, 1)));
        b->ttiles[side][mode - 1].push_back(static_cast<unsigned>(nk) * gj * gi);
      }
    }
  }
  if (b->n_tma) {   // dynamic shared memory of the TMA-staged launches (above 48 KB in FP64)
    const int se = xg::ItTiles<T, I, xg::kItK>::template smem_e<4>(), sh = xg::ItTiles<T, I, xg::kItK>::template smem_h<4>();
    auto attr = [](auto kern, int bytes) {
      XCHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    };
    attr(xg::k_tma_batch<T, I, 4, false, 1, true>, se);
    attr(xg::k_tma_batch<T, I, 4, false, 2, true>, se);
    attr(xg::k_tma_batch<T, I, 4, true, 1, true>, se);
    attr(xg::k_tma_batch<T, I, 4, true, 2, true>, se);
    attr(xg::k_tma_batch<T, I, 4, false, 1, false>, sh);
    attr(xg::k_tma_batch<T, I, 4, false, 2, false>, sh);
    attr(xg::k_tma_batch<T, I, 4, true, 1, false>, sh);
    attr(xg::k_tma_batch<T, I, 4, true, 2, false>, sh);
  }
  b->group_params.assign(groups, std::vector<unsigned char>(sizeof(xg::VolGroup<T, I>)));
  for (int g = 0; g < groups; ++g) std::memcpy(b->group_params[g].data(), &vg[g], sizeof(xg::VolGroup<T, I>));
  b->vl.assign(groups, xfdtd_batch::VolLists{});
  b->tsurf = up(ts);
  b->nfp = up(nf);
  b->aux = up(ax);
  b->nf_grid = up(grid);
  b->nf_nb = up(nb);
  for (int side = 0; side < 2; ++side) {
    b->vin[side] = up(vin[side]);
    b->vshell[side] = up(vsh[side]);
    b->tmaps[side] = up(tm[side]);
    for (int mode = 0; mode < 2; ++mode) {
      b->tbox[side][mode] = up(tb[side][mode]);
      b->tgrid[side][mode] = up(tg[side][mode]);
    }
  }
  std::vector<int *> st(n);
  for (int q = 0; q < n; ++q) st[q] = b->m[q]->d_status;
  b->status_list = up(st);
  XCHECK(cudaStreamSynchronize(b->stream));   // the host vectors go out of scope
}

// Work lists of the members that have steps left.
void batch_lists(xfdtd_batch *b) {
  std::vector<int> run;
  for (int q = 0; q < static_cast<int>(b->m.size()); ++q)
    if (b->m[q]->host_step < b->m[q]->total) run.push_back(q);
  if (run == b->running && b->lists_ok) return;
  b->running = run;
  if (b->gexec) {
    cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
  }
  const int groups = static_cast<int>(b->vl.size());
  const int nm = static_cast<int>(b->m.size());
  std::vector<char> on(nm, 0);
  for (int q : run) on[q] = 1;
  for (int g = 0; g < groups; ++g)   // volume launches: blocks per member, none for stopped members
    for (int side = 0; side < 2; ++side) {
      xg::GroupBlocks &bi = b->vl[g].in[side], &bs = b->vl[g].sh[side];
      xg::GroupBlocks &tw = b->vl[g].tw[side], &tz = b->vl[g].tz[side];
      bi = xg::GroupBlocks{};
      bs = xg::GroupBlocks{};
      tw = xg::GroupBlocks{};
      tz = xg::GroupBlocks{};
      bi.n = bs.n = tw.n = tz.n = std::min(xg::kBatchGroup, nm - g * xg::kBatchGroup);
      for (int ql = 0; ql < bi.n; ++ql) {
        const int q = g * xg::kBatchGroup + ql;
        const xfdtd_handle *h = b->m[q];
        const bool t = b->tma_m[q] != 0;
        const bool r = on[q] != 0;
        tw.first[ql + 1] = tw.first[ql] + (r && t ? b->ttiles[side][0][q] : 0u);
        tz.first[ql + 1] = tz.first[ql] + (r && t ? b->ttiles[side][1][q] : 0u);
        const xg::InteriorBox &in = h->vin[side];
        unsigned tiles = 0;
        if (r && !t && h->vin_cells[side]) {
          const int k0 = in.lo[2] / 32 * 32;
          tiles = static_cast<unsigned>(((in.hi[2] - k0) / 32 + 1) * ((in.hi[1] - in.lo[1]) / 8 + 1) *
                                        (in.hi[0] - in.lo[0] + 1));
        }
        bi.first[ql + 1] = bi.first[ql] + tiles;
        bs.first[ql + 1] = bs.first[ql] + (r && !t ? h->vshell[side].blocks : 0u);
      }
    }
  std::vector<xg::WorkItem> te, th, nf, fold;
  std::vector<int> aux;
  std::vector<long long *> steps;
  for (int q : run) {
    xfdtd_handle *h = b->m[q];
    if (h->tfsf) {
      aux.push_back(q);
      const long long ne = xg::surface_count(h->tf_lo[0], h->tf_hi[0], h->tf_lo[1], h->tf_hi[1], h->tf_lo[2], h->tf_hi[2]);
      const long long nh = xg::surface_count(h->tf_lo[0] - 1, h->tf_hi[0], h->tf_lo[1] - 1, h->tf_hi[1],
                                             h->tf_lo[2] - 1, h->tf_hi[2]);
      for (long long t = 0; t < (ne + 255) / 256; ++t) te.push_back({q, static_cast<int>(t)});
      for (long long t = 0; t < (nh + 255) / 256; ++t) th.push_back({q, static_cast<int>(t)});
    }
    if (h->nffft) {
      const dim3 g = nffft_grid(h);
      for (long long t = 0; t < static_cast<long long>(g.x) * g.y * 3; ++t) nf.push_back({q, static_cast<int>(t)});
      for (long long t = 0; t < 3 * nffft_fold_blocks(h); ++t) fold.push_back({q, static_cast<int>(t)});
    }
    steps.push_back(h->d_step);
  }
  auto put = [&](auto &v, auto *&dst) {
    using E = typename std::remove_reference<decltype(v)>::type::value_type;
    if (!dst) {   // sized once, for the first (largest) running set
      dst = b->alloc<E>(std::max<size_t>(v.size(), 1));
    }
    if (!v.empty()) XCHECK(cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(E), cudaMemcpyHostToDevice, b->stream));
    return static_cast<int>(v.size());
  };
  b->n_te = put(te, b->it_te);
  b->n_th = put(th, b->it_th);
  b->n_nf = put(nf, b->it_nf);
  b->n_fold = put(fold, b->it_fold);
  b->n_aux = put(aux, b->aux_list);
  put(steps, b->step_list);
  XCHECK(cudaStreamSynchronize(b->stream));
  b->lists_ok = true;
}

template <typename T, typename I>
void batch_enqueue_t(xfdtd_batch *b, long long s) {
  cudaStream_t st = b->stream;
  int launched = 0;
  if (b->n_aux) {
    xg::k_tfsf_aux_batch<<<b->n_aux, 512, 0, st>>>(static_cast<const xg::AuxParams *>(b->aux), b->aux_list);
    ++launched;
  }
  // one side of the volume update: per group of members, the shell kernel
  // on the shell stream beside the interior kernel, joined before what
  // follows
  auto volume = [&](bool e_side) {
    const int side = e_side ? 0 : 1;
    XCHECK(cudaEventRecord(b->ev_fork[side], st));
    XCHECK(cudaStreamWaitEvent(b->shell, b->ev_fork[side], 0));
    for (size_t g = 0; g < b->vl.size(); ++g) {
      const auto &vg = *reinterpret_cast<const xg::VolGroup<T, I> *>(b->group_params[g].data());
      const xfdtd_batch::VolLists &l = b->vl[g];
      const size_t base = g * xg::kBatchGroup;
      const unsigned nsh = l.sh[side].first[l.sh[side].n], nin = l.in[side].first[l.in[side].n];
      const unsigned ntw = l.tw[side].first[l.tw[side].n], ntz = l.tz[side].first[l.tz[side].n];
      const xg::ItMaps *mp = b->tmaps[side] + base;
      int *const *stl = b->status_list + base;
      // the TMA-staged members: the z edges on the shell stream, the wide
      // launch on the main stream
      if (ntz) {
        const xg::InteriorBox *bx = b->tbox[side][1] + base;
        const int2 *gr = b->tgrid[side][1] + base;
        const unsigned sm = e_side ? xg::ItTiles<T, I, xg::kItK>::template smem_e<4>()
                                   : xg::ItTiles<T, I, xg::kItK>::template smem_h<4>();
        if (b->ct) {
          if (e_side) xg::k_tma_batch<T, I, 4, true, 2, true><<<ntz, xg::kItThreads, sm, b->shell>>>(vg, l.tz[side], mp, bx, gr, stl, kBatchChunk);
          else xg::k_tma_batch<T, I, 4, true, 2, false><<<ntz, xg::kItThreads, sm, b->shell>>>(vg, l.tz[side], mp, bx, gr, stl, kBatchChunk);
        } else {
          if (e_side) xg::k_tma_batch<T, I, 4, false, 2, true><<<ntz, xg::kItThreads, sm, b->shell>>>(vg, l.tz[side], mp, bx, gr, stl, kBatchChunk);
          else xg::k_tma_batch<T, I, 4, false, 2, false><<<ntz, xg::kItThreads, sm, b->shell>>>(vg, l.tz[side], mp, bx, gr, stl, kBatchChunk);
        }
        ++launched;
      }
      if (ntw) {
        const xg::InteriorBox *bx = b->tbox[side][0] + base;
        const int2 *gr = b->tgrid[side][0] + base;
        const unsigned sm = e_side ? xg::ItTiles<T, I, xg::kItK>::template smem_e<4>()
                                   : xg::ItTiles<T, I, xg::kItK>::template smem_h<4>();
        if (b->ct) {
          if (e_side) xg::k_tma_batch<T, I, 4, true, 1, true><<<ntw, xg::kItThreads, sm, st>>>(vg, l.tw[side], mp, bx, gr, stl, kBatchChunk);
          else xg::k_tma_batch<T, I, 4, true, 1, false><<<ntw, xg::kItThreads, sm, st>>>(vg, l.tw[side], mp, bx, gr, stl, kBatchChunk);
        } else {
          if (e_side) xg::k_tma_batch<T, I, 4, false, 1, true><<<ntw, xg::kItThreads, sm, st>>>(vg, l.tw[side], mp, bx, gr, stl, kBatchChunk);
          else xg::k_tma_batch<T, I, 4, false, 1, false><<<ntw, xg::kItThreads, sm, st>>>(vg, l.tw[side], mp, bx, gr, stl, kBatchChunk);
        }
        ++launched;
      }
      if (nsh) {
        const xg::ShellBoxes *sb = b->vshell[side] + base;
        if (b->ct) {
          if (e_side) xg::k_shell_batch<T, I, true, true><<<nsh, 256, 0, b->shell>>>(vg, l.sh[side], sb);
          else xg::k_shell_batch<T, I, false, true><<<nsh, 256, 0, b->shell>>>(vg, l.sh[side], sb);
        } else {
          if (e_side) xg::k_shell_batch<T, I, true, false><<<nsh, 256, 0, b->shell>>>(vg, l.sh[side], sb);
          else xg::k_shell_batch<T, I, false, false><<<nsh, 256, 0, b->shell>>>(vg, l.sh[side], sb);
        }
        ++launched;
      }
      if (nin) {
        const xg::InteriorBox *ib = b->vin[side] + base;
        if (b->ct) {
          if (e_side) xg::k_interior_batch<T, I, true, true><<<nin, 256, 0, st>>>(vg, l.in[side], ib);
          else xg::k_interior_batch<T, I, false, true><<<nin, 256, 0, st>>>(vg, l.in[side], ib);
        } else {
          if (e_side) xg::k_interior_batch<T, I, true, false><<<nin, 256, 0, st>>>(vg, l.in[side], ib);
          else xg::k_interior_batch<T, I, false, false><<<nin, 256, 0, st>>>(vg, l.in[side], ib);
        }
        ++launched;
      }
    }
    XCHECK(cudaEventRecord(b->ev_join[side], b->shell));
    XCHECK(cudaStreamWaitEvent(st, b->ev_join[side], 0));
  };
  volume(true);
  const auto *tp = static_cast<const xg::TfsfSurfParams<T> *>(b->tsurf);
  if (b->n_te) {
    xg::k_tfsf_batch<T, true><<<b->n_te, 256, 0, st>>>(tp, b->it_te);
    ++launched;
  }
  volume(false);
  if (b->n_th) {
    xg::k_tfsf_batch<T, false><<<b->n_th, 256, 0, st>>>(tp, b->it_th);
    ++launched;
  }
  const auto *np = static_cast<const xg::NfParams<T> *>(b->nfp);
  if (b->n_nf) {
    xg::k_nffft_batch<T><<<b->n_nf, 256, 0, st>>>(np, b->nf_grid, b->it_nf);
    ++launched;
    if ((s + 1) % xg::kMaxNfBatch == 0) {
      xg::k_nffft_fold_batch<T><<<b->n_fold, 256, 0, st>>>(np, b->nf_nb, b->it_fold,
                                                           static_cast<int>(s + 1 - b->nf_done));
      ++launched;
      b->nf_done = s + 1;
    }
  }
  const int nr = static_cast<int>(b->running.size());
  xg::k_advance_batch<<<(nr + 127) / 128, 128, 0, st>>>(b->step_list, nr);
  ++launched;
  XCHECK(cudaGetLastError());
  b->launches += launched;
}

void batch_enqueue(xfdtd_batch *b, long long s) {
  if (b->precision == XFDTD_FP64) {
    if (b->idx_bytes == 1) batch_enqueue_t<double, uint8_t>(b, s);
    else batch_enqueue_t<double, uint16_t>(b, s);
  } else {
    if (b->idx_bytes == 1) batch_enqueue_t<float, uint8_t>(b, s);
    else batch_enqueue_t<float, uint16_t>(b, s);
  }
}

// Host bookkeeping of the running members after `k` batch steps.
void batch_advance_members(xfdtd_batch *b, long long k) {
  b->clock += k;
  for (int q : b->running) {
    xfdtd_handle *h = b->m[q];
    h->host_step += k;
    if (h->nffft) h->nf_done = b->nf_done;
  }
}

void batch_steps(xfdtd_batch *b, long long n) {
  if (n < 0) invalid("negative step count");
  const bool graph = (b->flags & XFDTD_FLAG_GRAPH) != 0;
  while (n > 0) {
    batch_lists(b);
    if (b->running.empty()) return;
    long long seg = n;   // up to the next member that finishes
    for (int q : b->running) seg = std::min(seg, b->m[q]->total - b->m[q]->host_step);
    const long long end = b->clock + seg;
    while (b->clock < end) {
      if (graph && b->clock % kBatchGraphSteps == 0 && end - b->clock >= kBatchGraphSteps) {
        if (!b->gexec) {
          cudaGraph_t g;
          const long long nf_done = b->nf_done, launches = b->launches;
          XCHECK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
          for (int s = 0; s < kBatchGraphSteps; ++s) batch_enqueue(b, b->clock + s);
          XCHECK(cudaStreamEndCapture(b->stream, &g));
          b->graph_launches = b->launches - launches;
          b->launches = launches;
          b->nf_done = nf_done;
          const cudaError_t e = cudaGraphInstantiate(&b->gexec, g, 0);
          cudaGraphDestroy(g);
          XCHECK(e);
        }
        XCHECK(cudaGraphLaunch(b->gexec, b->stream));
        b->launches += b->graph_launches;
        b->nf_done = b->clock + kBatchGraphSteps;
        batch_advance_members(b, kBatchGraphSteps);
        continue;
      }
      batch_enqueue(b, b->clock);
      batch_advance_members(b, 1);
    }
    n -= seg;
  }
}

int batch_guarded(xfdtd_batch *b, const std::function<void()> &fn) {
  try {
    XCHECK(cudaSetDevice(b->device));
    fn();
    return XFDTD_OK;
  } catch (const Err &e) {
    b->err = e.msg;
    return e.code;
  } catch (const std::exception &e) {
    b->err = e.what();
    return XFDTD_ERR_INVALID_PLAN;
  }
}

}  // namespace

extern "C" {

int xfdtd_batch_create(xfdtd_handle *const *members, int n, int flags, xfdtd_batch **out) {
  if (!out) return XFDTD_ERR_INVALID_PLAN;
  std::unique_ptr<xfdtd_batch> b(new xfdtd_batch());
  b->flags = flags;
  const int rc = [&]() -> int {
    try {
      if (!members || n < 1) invalid("a batch needs at least one member");
      for (int q = 0; q < n; ++q) {
        xfdtd_handle *h = members[q];
        if (!h || !h->stream) invalid("batch member " + std::to_string(q) + " is not a created handle");
        if (q == 0) {
          b->device = h->device;
          b->precision = h->precision;
          b->idx_bytes = h->idx_bytes;
        }
        if (h->device != b->device || h->precision != b->precision || h->idx_bytes != b->idx_bytes)
          invalid("batch members must share device, precision and material-index width");
        if (h->idx_bytes > 2) invalid("batch members must use 1- or 2-byte material indices");
        if (h->host_step != 0) invalid("batch members must not have been stepped");
        if (h->n_inj || h->n_ind || h->n_probes || !h->snaps.empty())
          invalid("batch members may not have lumped elements or monitors");
        if (h->nf_bb) invalid("batch members may not have a broadband NF-FF");
        if (h->d.nz < 2) invalid("batch members must be 3-D grids");
        if (h->n_disp) invalid("batch members may not have dispersive media");
        if (h->d.nx >= 65535 || h->d.ny >= 2040 || h->d.nz >= 8160) invalid("batch member grid too large for the tile numbering");
        for (int r = 0; r < q; ++r)
          if (members[r] == h) invalid("a handle appears twice in the batch");
        // many materials scatter the nine full-table loads per cell: read the compact table
        if (h->n_mat > 16) b->ct = true;
      }
      XCHECK(cudaSetDevice(b->device));
      int sms = 0;
      XCHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
      b->n_sm = sms;
      XCHECK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
      XCHECK(cudaStreamCreateWithFlags(&b->shell, cudaStreamNonBlocking));
      for (int q = 0; q < 2; ++q) {
        XCHECK(cudaEventCreateWithFlags(&b->ev_fork[q], cudaEventDisableTiming));
        XCHECK(cudaEventCreateWithFlags(&b->ev_join[q], cudaEventDisableTiming));
      }
      for (int q = 0; q < n; ++q) {
        xfdtd_handle *h = members[q];
        XCHECK(cudaStreamSynchronize(h->stream));
        if (h->gexec) {   // its own graph will not run again
          cudaGraphExecDestroy(h->gexec);
          h->gexec = nullptr;
        }
        h->sweep = false;   // the batch runs the split kernels on the handle's current buffers
        b->m.push_back(h);
      }
      if (b->precision == XFDTD_FP64) {
        if (b->idx_bytes == 1) batch_setup<double, uint8_t>(b.get());
        else batch_setup<double, uint16_t>(b.get());
      } else {
        if (b->idx_bytes == 1) batch_setup<float, uint8_t>(b.get());
        else batch_setup<float, uint16_t>(b.get());
      }
      return XFDTD_OK;
    } catch (const Err &e) {
      b->err = e.msg;
      return e.code;
    }
  }();
  *out = b.release();
  return rc;
}

int xfdtd_batch_step(xfdtd_batch *b, int64_t n) {
  if (!b) return XFDTD_ERR_STATE;
  return batch_guarded(b, [&] { batch_steps(b, n); });
}

int xfdtd_batch_step_timed(xfdtd_batch *b, int64_t n, double *ms) {
  if (!b) return XFDTD_ERR_STATE;
  return batch_guarded(b, [&] {
    batch_lists(b);   // list uploads stay outside the timed region
    cudaEvent_t e0, e1;
    XCHECK(cudaEventCreate(&e0));
    XCHECK(cudaEventCreate(&e1));
    XCHECK(cudaEventRecord(e0, b->stream));
    batch_steps(b, n);
    XCHECK(cudaEventRecord(e1, b->stream));
    XCHECK(cudaEventSynchronize(e1));
    float f = 0;
    XCHECK(cudaEventElapsedTime(&f, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = f;
  });
}

int xfdtd_batch_synchronize(xfdtd_batch *b) {
  if (!b) return XFDTD_ERR_STATE;
  return batch_guarded(b, [&] {
    XCHECK(cudaStreamSynchronize(b->stream));
    for (xfdtd_handle *h : b->m) check_status(h);
  });
}

int xfdtd_batch_status(xfdtd_batch *b, int *n_running, int64_t *clock, int64_t *launches) {
  if (!b) return XFDTD_ERR_STATE;
  int r = 0;
  for (xfdtd_handle *h : b->m) r += h->host_step < h->total ? 1 : 0;
  if (n_running) *n_running = r;
  if (clock) *clock = b->clock;
  if (launches) *launches = b->launches;
  return XFDTD_OK;
}

int xfdtd_batch_tma_members(xfdtd_batch *b, int *n) {
  if (!b) return XFDTD_ERR_STATE;
  if (n) *n = b->n_tma;
  return XFDTD_OK;
}

const char *xfdtd_batch_last_error(xfdtd_batch *b) { return b ? b->err.c_str() : "null batch"; }

void xfdtd_batch_destroy(xfdtd_batch *b) {
  if (!b) return;
  if (b->stream) {
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
  }
  delete b;
}

}  // extern "C"

// ============================================================== adjoint ===
// Gradient of a field loss with respect to eps_r and sigma of the cells of
// a design box (adjoint.cuh).  xfdtd_adjoint_forward runs the whole step
// loop from step 0 on the split kernels, recording the loss component over
// the loss plane after every step of the loss window and, every K steps, a
// checkpoint of the state (fields, psi, TFSF line).  xfdtd_adjoint_backward
// walks the checkpoint segments from the last to the first: it restores the
// segment's checkpoint, re-runs its K steps recording E and H over the
// design box, then runs the K reverse steps.  With K = 0 the forward pass
// records the design box at every step and the backward pass re-runs
// nothing.

struct AdjointState {
  xfdtd_adjoint_desc d{};
  int dn[3] = {0, 0, 0};                 // design box extent
  long long nE = 0, nH = 0;              // cells of the E and H record boxes
  int pn[2] = {0, 0};                    // loss plane extent
  int K = 0;                             // checkpoint interval (0: record every step)
  int slots = 0;                         // design-record slots
  std::vector<void *> allocs;
  void *recE[3] = {}, *recH[3] = {};     // [slots][box]
  void *plane = nullptr;                 // [window][pn0 * pn1]
  std::vector<void *> ck;                // checkpoints: one block each
  size_t ck_bytes = 0;
  void *lE[3] = {}, *lH[3] = {}, *m[12] = {};
  double *g_eps = nullptr, *g_sig = nullptr, *dtab = nullptr;
  void *sc = nullptr, *isc = nullptr;    // per table entry: s and 1/s of the six components (adjoint.cuh)
  uint8_t *aflags_x = nullptr;           // x-axis flags with kAdjGeneral on the planes that need it
  // the reverse steps run on their own stream, beside the re-run of the
  // segment before on the engine's stream (two record buffers)
  cudaStream_t rs = nullptr;
  cudaEvent_t ev_ready = nullptr, ev_rec[2] = {nullptr, nullptr}, ev_rev[2] = {nullptr, nullptr};
  double loss = 0;
  bool forward_done = false;
  int device = 0;
  size_t bytes = 0;   // device bytes held
  void *alloc(size_t nb) {
    void *p = nullptr;
    nb = std::max<size_t>(nb, 16);
    XCHECK(cudaMalloc(&p, nb));
    allocs.push_back(p);
    bytes += nb;
    return p;
  }
  ~AdjointState() {
    cudaSetDevice(device);
    if (rs) {
      cudaStreamSynchronize(rs);
      cudaStreamDestroy(rs);
    }
    for (cudaEvent_t e : {ev_ready, ev_rec[0], ev_rec[1], ev_rev[0], ev_rev[1]})
      if (e) cudaEventDestroy(e);
    for (void *p : allocs) cudaFree(p);
  }
};

size_t adjoint_bytes(const xfdtd_handle *h) { return h->adj ? h->adj->bytes : 0; }

namespace {

// Bytes of one checkpoint: fields, psi, TFSF line state and both incident buffers.
size_t adj_checkpoint_bytes(const xfdtd_handle *h) {
  size_t b = 6 * static_cast<size_t>(h->d.cells) * h->esize;
  for (int q = 0; q < 12; ++q) b += h->psi_bytes[q];
  if (h->tfsf) b += (2 * static_cast<size_t>(h->aux_len) + 1 + 12 * static_cast<size_t>(h->aux_len)) * sizeof(double) +
                    (h->tf_incf ? 12 * static_cast<size_t>(h->aux_len) * sizeof(float) : 0);
  return b;
}

// Copies the state into (save) or out of (restore) one checkpoint block.
void adj_checkpoint(xfdtd_handle *h, void *block, bool save) {
  unsigned char *p = static_cast<unsigned char *>(block);
  auto io = [&](void *dev, size_t bytes) {
    if (!bytes || !dev) return;
    if (save) XCHECK(cudaMemcpyAsync(p, dev, bytes, cudaMemcpyDeviceToDevice, h->stream));
    else XCHECK(cudaMemcpyAsync(dev, p, bytes, cudaMemcpyDeviceToDevice, h->stream));
    p += bytes;
  };
  for (int c = 0; c < 6; ++c) io(h->F[c], static_cast<size_t>(h->d.cells) * h->esize);
  for (int q = 0; q < 12; ++q) io(h->psi[q], h->psi_bytes[q]);
  if (h->tfsf) {
    io(h->tf_state, (2 * static_cast<size_t>(h->aux_len) + 1) * sizeof(double));
    io(h->tf_inc, 12 * static_cast<size_t>(h->aux_len) * sizeof(double));
    if (h->tf_incf) io(h->tf_incf, 12 * static_cast<size_t>(h->aux_len) * sizeof(float));
  }
}

// The design-box record of the step about to run (its slot from the device
// step counter, adjoint.cuh AdjRecords).
template <typename T>
void adj_record_design(xfdtd_handle *h, AdjointState *a) {
  const int n0 = a->dn[0], n1 = a->dn[1], n2 = a->dn[2];
  xg::AdjRecords<T> r{};
  for (int c = 0; c < 3; ++c) {
    r.recE[c] = static_cast<T *>(a->recE[c]);
    r.recH[c] = static_cast<T *>(a->recH[c]);
  }
  r.nE = a->nE;
  r.nH = a->nH;
  r.K = a->K;
  xg::FieldPtrs<T> fp;
  for (int c = 0; c < 6; ++c) fp.f[c] = static_cast<const T *>(h->F[c]);
  dim3 block(32, 8, 1);
  dim3 grid((n2 + 1 + 31) / 32, (n1 + 1 + 7) / 8, n0 + 1);
  xg::k_adj_record<T><<<grid, block, 0, h->stream>>>(fp, h->d, static_cast<int>(a->d.design_lo[0]),
                                                      static_cast<int>(a->d.design_lo[1]), static_cast<int>(a->d.design_lo[2]),
                                                      n0, n1, n2, r, h->d_step);
  XCHECK(cudaGetLastError());
  ++h->launch_count;
}

// The loss plane's record of the step that just ran, when it lies in the
// loss window.
template <typename T>
void adj_record_plane(xfdtd_handle *h, AdjointState *a) {
  dim3 grid((a->pn[1] + 127) / 128, a->pn[0], 1);
  xg::k_adj_plane<T><<<grid, 128, 0, h->stream>>>(static_cast<const T *>(h->F[a->d.loss_comp]), h->d, a->d.plane_axis,
                                                  static_cast<int>(a->d.plane_index), static_cast<int>(a->d.plane_lo[0]),
                                                  static_cast<int>(a->d.plane_lo[1]), a->pn[0], a->pn[1],
                                                  static_cast<T *>(a->plane), h->d_step, a->d.t_begin, a->d.t_end);
  XCHECK(cudaGetLastError());
  ++h->launch_count;
}

// A captured run of g steps of the adjoint's forward or re-run passes: each
// step with its records (adj_steps).
struct AdjGraph {
  cudaGraphExec_t exec = nullptr;
  long long launches = 0;   // kernel launches in the graph
  ~AdjGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

// Runs the steps [t0, t1) with `each` (one step and the records around it)
// as CUDA graph replays of g steps where the handle replays graphs and the
// step sequence is the same for every step (no NF-FF, no snapshots: their
// host bookkeeping follows the step index; the records take their slots
// from the device step counter), single steps for the rest.  The graph is
// captured on its first use.
template <typename F>
void adj_steps(xfdtd_handle *h, long long t0, long long t1, int g, AdjGraph &gr, F &&each) {
  const bool graph = (h->flags & XFDTD_FLAG_GRAPH) && !(h->flags & XFDTD_FLAG_PROFILE) && !h->nffft &&
                     h->snaps.empty();
  long long t = t0;
  while (t < t1) {
    if (graph && g > 1 && t1 - t >= g) {
      if (!gr.exec) {
        cudaGraph_t cg;
        const long long launches = h->launch_count;
        XCHECK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        for (int s = 0; s < g; ++s) each(t + s);
        XCHECK(cudaStreamEndCapture(h->stream, &cg));
        gr.launches = h->launch_count - launches;
        h->launch_count = launches;
        const cudaError_t e = cudaGraphInstantiate(&gr.exec, cg, 0);
        cudaGraphDestroy(cg);
        XCHECK(e);
      }
      XCHECK(cudaGraphLaunch(gr.exec, h->stream));
      h->launch_count += gr.launches;
      t += g;
      continue;
    }
    each(t);
    ++t;
  }
}

// Steps per captured graph: a divisor of the checkpoint interval K (graphs
// never cross a checkpoint), at most 64; 50 without checkpoints.
int adj_graph_steps(int K) {
  if (K <= 0) return 50;
  int g = std::min(K, 64);
  while (K % g) --g;
  return g;
}

void adj_validate(xfdtd_handle *h, const xfdtd_adjoint_desc *d) {
  if (h->host_step != 0) throw Err{XFDTD_ERR_STATE, "the adjoint forward pass starts at step 0"};
  if (h->n_ind) invalid("the adjoint does not cover inductors (their current is extra state)");
  if (h->n_disp) invalid("the adjoint does not cover dispersive media (their currents are extra state)");
  const int n[3] = {h->d.nx, h->d.ny, h->d.nz};
  for (int a = 0; a < 3; ++a) {
    if (d->design_lo[a] < 1 || d->design_hi[a] <= d->design_lo[a] || d->design_hi[a] > n[a] - 1)
      invalid("design box must lie inside the grid, off the outer walls");
    for (long long q = d->design_lo[a] - 1; q <= d->design_hi[a]; ++q)
      if (h->axis_flags_host[a][q] & (xg::kSpecialE | xg::kSpecialH))
        invalid("design box (and its one-cell rim) must lie outside the CPML");
  }
  if (d->loss_comp < 0 || d->loss_comp > 2) invalid("loss component must be Ex, Ey or Ez");
  if (d->plane_axis < 0 || d->plane_axis > 2) invalid("plane axis must be 0, 1 or 2");
  const int u = d->plane_axis == 0 ? 1 : 0, v = d->plane_axis == 2 ? 1 : 2;
  if (d->plane_index < 0 || d->plane_index > n[d->plane_axis]) invalid("plane index outside the grid");
  if (d->plane_lo[0] < 0 || d->plane_hi[0] <= d->plane_lo[0] || d->plane_hi[0] > n[u] + 1 || d->plane_lo[1] < 0 ||
      d->plane_hi[1] <= d->plane_lo[1] || d->plane_hi[1] > n[v] + 1)
    invalid("plane extent outside the grid");
  if (d->t_begin < 0 || d->t_end <= d->t_begin || d->t_end > h->total) invalid("loss window outside the steps");
  if (d->checkpoint_every < 0) invalid("checkpoint interval must be >= 0");
}

template <typename T>
void adj_forward_t(xfdtd_handle *h, const xfdtd_adjoint_desc *d, double *loss) {
  adj_validate(h, d);
  auto a = std::make_shared<AdjointState>();
  a->device = h->device;
  a->d = *d;
  for (int q = 0; q < 3; ++q) a->dn[q] = static_cast<int>(d->design_hi[q] - d->design_lo[q]);
  a->nE = static_cast<long long>(a->dn[0]) * a->dn[1] * a->dn[2];
  a->nH = static_cast<long long>(a->dn[0] + 1) * (a->dn[1] + 1) * (a->dn[2] + 1);
  a->pn[0] = static_cast<int>(d->plane_hi[0] - d->plane_lo[0]);
  a->pn[1] = static_cast<int>(d->plane_hi[1] - d->plane_lo[1]);
  a->K = d->checkpoint_every;
  const long long T_ = h->total;
  a->slots = a->K > 0 ? 2 * a->K : static_cast<int>(T_);   // two record buffers of K steps each
  for (int c = 0; c < 3; ++c) {
    a->recE[c] = a->alloc(static_cast<size_t>(a->slots) * a->nE * sizeof(T));
    a->recH[c] = a->alloc(static_cast<size_t>(a->slots) * a->nH * sizeof(T));
  }
  const long long win = d->t_end - d->t_begin;
  a->plane = a->alloc(static_cast<size_t>(win) * a->pn[0] * a->pn[1] * sizeof(T));
  if (a->K > 0) {
    a->ck_bytes = adj_checkpoint_bytes(h);
    const long long n_ck = (T_ + a->K - 1) / a->K + 1;   // segment starts and the final state
    for (long long q = 0; q < n_ck; ++q) a->ck.push_back(a->alloc(a->ck_bytes));
  }
  h->sweep = false;   // the adjoint transposes the split kernels' arithmetic
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  // Every step: the design-box record (K = 0), the step, the loss plane's
  // record (a no-op outside the window); as graph replays between
  // checkpoints.
  {
    AdjGraph gr;
    const int g = adj_graph_steps(a->K);
    AdjointState *ap = a.get();
    auto each = [&](long long t) {
      if (ap->K == 0) adj_record_design<T>(h, ap);
      enqueue_step(h, t);
      h->host_step = t + 1;
      adj_record_plane<T>(h, ap);
    };
    const long long span = a->K > 0 ? a->K : T_;
    for (long long t = 0; t < T_; t += span) {
      if (a->K > 0) adj_checkpoint(h, a->ck[t / a->K], true);
      adj_steps(h, t, std::min(T_, t + span), g, gr, each);
    }
    XCHECK(cudaStreamSynchronize(h->stream));   // the graph's last replay before it is destroyed
    h->host_step = T_;
  }
  if (a->K > 0) adj_checkpoint(h, a->ck.back(), true);
  prof_collect(h);
  // loss = sum over the window and the plane of F^2
  std::vector<T> pl(static_cast<size_t>(win) * a->pn[0] * a->pn[1]);
  XCHECK(cudaMemcpyAsync(pl.data(), a->plane, pl.size() * sizeof(T), cudaMemcpyDeviceToHost, h->stream));
  XCHECK(cudaStreamSynchronize(h->stream));
  check_status(h);
  double L = 0;
  for (T v : pl) L += static_cast<double>(v) * static_cast<double>(v);
  a->loss = L;
  a->forward_done = true;
  h->adj = a;
  if (loss) *loss = L;
}

template <typename T, typename I>
void adj_backward_t(xfdtd_handle *h, double *g_eps, double *g_sig) {
  AdjointState *a = h->adj.get();
  if (!a || !a->forward_done || h->host_step != h->total)
    throw Err{XFDTD_ERR_STATE, "run xfdtd_adjoint_forward (to the last step) first"};
  const size_t cells = static_cast<size_t>(h->d.cells);
  for (int c = 0; c < 3; ++c) {
    if (!a->lE[c]) a->lE[c] = a->alloc(cells * sizeof(T));
    if (!a->lH[c]) a->lH[c] = a->alloc(cells * sizeof(T));
    XCHECK(cudaMemsetAsync(a->lE[c], 0, cells * sizeof(T), h->stream));
    XCHECK(cudaMemsetAsync(a->lH[c], 0, cells * sizeof(T), h->stream));
  }
  for (int q = 0; q < 12; ++q)
    if (h->psi_bytes[q]) {
      if (!a->m[q]) a->m[q] = a->alloc(h->psi_bytes[q]);
      XCHECK(cudaMemsetAsync(a->m[q], 0, h->psi_bytes[q], h->stream));
    }
  if (!a->g_eps) {
    a->g_eps = static_cast<double *>(a->alloc(a->nE * sizeof(double)));
    a->g_sig = static_cast<double *>(a->alloc(a->nE * sizeof(double)));
  }
  XCHECK(cudaMemsetAsync(a->g_eps, 0, a->nE * sizeof(double), h->stream));
  XCHECK(cudaMemsetAsync(a->g_sig, 0, a->nE * sizeof(double), h->stream));
  if (!a->dtab) {   // coefficient derivatives per table entry, from the FP64 table
    const double eps0 = kEps0, dt = h->dt;
    std::vector<double> dtab(4 * static_cast<size_t>(h->n_mat), 0.0);
    for (int q = 0; q < h->n_mat; ++q) {
      const double c0 = h->table_host[q * XFDTD_N_COEFF + 0], c1 = h->table_host[q * XFDTD_N_COEFF + 1];
      if (c1 == 0) continue;
      const double D = -2 * dt / (c1 * h->dl[2]);   // cexhy = -2 dt / (D dz)
      const double eps = D * (1 + c0) / 4, sig = D * (1 - c0) / (2 * dt);
      dtab[4 * q + 0] = 4 * eps0 * dt * sig / (D * D);   // dc0 / deps_r
      dtab[4 * q + 1] = -4 * dt * eps / (D * D);         // dc0 / dsigma
      dtab[4 * q + 2] = -2 * eps0 / D;                   // (dc / deps_r) / c
      dtab[4 * q + 3] = -dt / D;                         // (dc / dsigma) / c
    }
    a->dtab = static_cast<double *>(a->alloc(dtab.size() * sizeof(double)));
    XCHECK(cudaMemcpyAsync(a->dtab, dtab.data(), dtab.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    XCHECK(cudaStreamSynchronize(h->stream));
  }

  if (!a->sc) {   // scales of the stored adjoint fields and the planes that need the general path
    const size_t nm = static_cast<size_t>(h->n_mat);
    std::vector<T> sc(6 * nm), isc(6 * nm);
    std::vector<uint8_t> nc(nm, 0);
    for (size_t q = 0; q < nm; ++q)
      for (int side = 0; side < 2; ++side) {
        const double *c = h->table_host.data() + q * XFDTD_N_COEFF + 9 * side;
        T t[9];
        for (int r = 0; r < 9; ++r) t[r] = static_cast<T>(c[r]);
        // the shape the fast path assumes: c0 = c3 = c6, c1 = c4 = c7 = -s, c2 = c5 = c8 = s, s != 0
        const bool fast = t[2] != T(0) && t[1] == -t[2] && t[0] == t[3] && t[0] == t[6] && t[1] == t[4] &&
                           t[1] == t[7] && t[2] == t[5] && t[2] == t[8];
        if (!fast) nc[q] = 1;
        for (int comp = 0; comp < 3; ++comp) {
          const T s = t[2 + 3 * comp] != T(0) ? t[2 + 3 * comp] : T(1);
          sc[6 * q + 3 * side + comp] = s;
          isc[6 * q + 3 * side + comp] = T(1) / s;
        }
      }
    a->sc = a->alloc(sc.size() * sizeof(T));
    a->isc = a->alloc(isc.size() * sizeof(T));
    XCHECK(cudaMemcpyAsync(a->sc, sc.data(), sc.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
    XCHECK(cudaMemcpyAsync(a->isc, isc.data(), isc.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
    const int nx = h->d.nx;
    std::vector<uint8_t> fl = h->axis_flags_host[0];
    if (std::find(nc.begin(), nc.end(), uint8_t(1)) != nc.end()) {
      auto *d_nc = static_cast<uint8_t *>(a->alloc(nm));
      auto *d_mark = static_cast<int *>(a->alloc((nx + 1) * sizeof(int)));
      XCHECK(cudaMemcpyAsync(d_nc, nc.data(), nm, cudaMemcpyHostToDevice, h->stream));
      XCHECK(cudaMemsetAsync(d_mark, 0, (nx + 1) * sizeof(int), h->stream));
      dim3 block(32, 8, 1), grid((h->d.nz + 32) / 32, (h->d.ny + 8) / 8, nx + 1);
      xg::k_adj_mark<I><<<grid, block, 0, h->stream>>>(static_cast<const I *>(h->idx), h->d, d_nc, d_mark);
      XCHECK(cudaGetLastError());
      std::vector<int> mark(nx + 1);
      XCHECK(cudaMemcpyAsync(mark.data(), d_mark, mark.size() * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
      XCHECK(cudaStreamSynchronize(h->stream));
      for (int q = 0; q <= nx; ++q)
        if (mark[q]) fl[q] |= xg::kAdjGeneral;
    }
    a->aflags_x = static_cast<uint8_t *>(a->alloc(fl.size()));
    XCHECK(cudaMemcpyAsync(a->aflags_x, fl.data(), fl.size(), cudaMemcpyHostToDevice, h->stream));
    XCHECK(cudaStreamCreateWithFlags(&a->rs, cudaStreamNonBlocking));
    XCHECK(cudaEventCreateWithFlags(&a->ev_ready, cudaEventDisableTiming));
    for (int q = 0; q < 2; ++q) {
      XCHECK(cudaEventCreateWithFlags(&a->ev_rec[q], cudaEventDisableTiming));
      XCHECK(cudaEventCreateWithFlags(&a->ev_rev[q], cudaEventDisableTiming));
    }
  }

  xg::AdjParams<T, I> p{};
  p.v = vol_params<T, I>(h);
  p.v.flags[0] = a->aflags_x;
  p.sc = static_cast<const T *>(a->sc);
  p.isc = static_cast<const T *>(a->isc);
  for (int c = 0; c < 3; ++c) {
    p.lE[c] = static_cast<T *>(a->lE[c]);
    p.lH[c] = static_cast<T *>(a->lH[c]);
  }
  T **mp = reinterpret_cast<T **>(&p.m);
  for (int q = 0; q < 12; ++q) mp[q] = static_cast<T *>(a->m[q]);
  for (int q = 0; q < 3; ++q) {
    p.dlo[q] = static_cast<int>(a->d.design_lo[q]);
    p.dhi[q] = static_cast<int>(a->d.design_hi[q]);
  }
  p.g_eps = a->g_eps;
  p.g_sig = a->g_sig;
  p.dtab = a->dtab;
  p.loss_comp = a->d.loss_comp;
  p.plane_axis = a->d.plane_axis;
  p.plane_index = static_cast<int>(a->d.plane_index);
  for (int q = 0; q < 2; ++q) {
    p.plo[q] = static_cast<int>(a->d.plane_lo[q]);
    p.phi[q] = static_cast<int>(a->d.plane_hi[q]);
  }
  const long long T_ = h->total;
  // k tiling per kernel (adjoint.cuh adj_k): the k whose gather reaches no
  // special index (k_adj_h: k and k+1; k_adj_e: k and k-1, k >= 1)
  const int nz = h->d.nz;
  auto k_tiles = [&](bool e_side, xg::AdjParams<T, I> &q) {
    const std::vector<uint8_t> &fz = h->axis_flags_host[2];
    const uint8_t bits = xg::kSpecialE | xg::kSpecialH;
    int lo = nz + 1, hi = nz;
    for (int k = 0; k < nz; ++k) {
      const bool ok = e_side ? (k >= 1 && !((fz[k] | fz[k - 1]) & bits)) : !((fz[k] | fz[k + 1]) & bits);
      if (!ok) continue;
      if (lo > nz) lo = k;
      hi = k;
    }
    if (lo > nz) lo = 0, hi = -1;   // no plain k: one range over all k
    q.kp_lo = lo;
    q.kp_hi = hi;
    q.kt_n0 = (lo + 31) / 32;
    q.kt_n1 = (hi - lo + 1 + 31) / 32;
    return static_cast<unsigned>(q.kt_n0 + q.kt_n1 + (nz - hi + 31) / 32);
  };
  xg::AdjParams<T, I> pe = p;
  const unsigned gx_h = k_tiles(false, p), gx_e = k_tiles(true, pe);
  const int kt_e[4] = {pe.kp_lo, pe.kp_hi, pe.kt_n0, pe.kt_n1};
  const int kt_h[4] = {p.kp_lo, p.kp_hi, p.kt_n0, p.kt_n1};
  auto use = [&](const int *kt) {
    p.kp_lo = kt[0];
    p.kp_hi = kt[1];
    p.kt_n0 = kt[2];
    p.kt_n1 = kt[3];
  };
  dim3 block(32, 8, 1);
  dim3 grid_h(gx_h, (h->d.ny + 8) / 8, h->d.nx + 1), grid_e(gx_e, (h->d.ny + 8) / 8, h->d.nx + 1);
  auto plane_of = [&](long long t1) -> const T * {   // loss record of the field after step t1
    if (t1 < a->d.t_begin || t1 >= a->d.t_end) return nullptr;
    return static_cast<const T *>(a->plane) + static_cast<size_t>(t1 - a->d.t_begin) * a->pn[0] * a->pn[1];
  };
  auto set_rec = [&](int slot) {
    for (int c = 0; c < 3; ++c) {
      p.recE[c] = static_cast<const T *>(a->recE[c]) + static_cast<size_t>(slot) * a->nE;
      p.recH[c] = static_cast<const T *>(a->recH[c]) + static_cast<size_t>(slot) * a->nH;
    }
  };
  const long long seg = a->K > 0 ? a->K : T_;
  const long long n_seg = (T_ + seg - 1) / seg;
  // Segment q covers steps [q seg, min(T, (q+1) seg)); with K > 0 its
  // re-run records the design box into buffer q % 2.  The re-run of segment
  // q-1 (engine stream) runs beside the reverse steps of segment q (rs): it
  // waits for the reverse steps of segment q+1, the last reader of its
  // buffer, and the reverse steps of segment q-1 wait for it.
  const bool nffft = h->nffft;
  const int n_probes = h->n_probes;
  h->nffft = false;   // the NF-FF sums and probes of the forward pass are final
  h->n_probes = 0;
  AdjGraph rerun_graph;   // the re-run's steps with their design-box records
  const int rerun_g = adj_graph_steps(a->K);
  auto rerun_each = [&](long long t) {
    adj_record_design<T>(h, a);
    enqueue_step(h, t);
  };
  auto rerun = [&](long long q) {
    const long long s0 = q * seg, s1 = std::min(T_, s0 + seg);
    if (q + 2 < n_seg) XCHECK(cudaStreamWaitEvent(h->stream, a->ev_rev[q % 2], 0));   // reverse(q + 2) done
    adj_checkpoint(h, a->ck[q], false);
    XCHECK(cudaMemcpyAsync(h->d_step, &s0, sizeof(long long), cudaMemcpyHostToDevice, h->stream));
    adj_steps(h, s0, s1, rerun_g, rerun_graph, rerun_each);
    XCHECK(cudaEventRecord(a->ev_rec[q % 2], h->stream));
  };
  XCHECK(cudaEventRecord(a->ev_ready, h->stream));   // zeroed adjoint state, tables, flags
  XCHECK(cudaStreamWaitEvent(a->rs, a->ev_ready, 0));
  if (a->K > 0) rerun(n_seg - 1);
  // the loss gradient of the last step
  p.do_e_own = 0;
  p.do_gather = 1;
  p.plane_rec = plane_of(T_ - 1);
  set_rec(0);
  use(kt_e);
  xg::k_adj_e<T, I><<<grid_e, block, 0, a->rs>>>(p);
  XCHECK(cudaGetLastError());
  for (long long q = n_seg - 1; q >= 0; --q) {
    const long long s0 = q * seg, s1 = std::min(T_, s0 + seg);
    if (a->K > 0) {
      XCHECK(cudaStreamWaitEvent(a->rs, a->ev_rec[q % 2], 0));
      if (q >= 1) rerun(q - 1);
    }
    for (long long t = s1 - 1; t >= s0; --t) {
      use(kt_h);
      xg::k_adj_h<T, I><<<grid_h, block, 0, a->rs>>>(p);
      XCHECK(cudaGetLastError());
      set_rec(static_cast<int>(a->K > 0 ? (q % 2) * a->K + (t - s0) : t));
      p.do_e_own = 1;
      p.do_gather = t >= 1 ? 1 : 0;
      p.plane_rec = t >= 1 ? plane_of(t - 1) : nullptr;
      use(kt_e);
      xg::k_adj_e<T, I><<<grid_e, block, 0, a->rs>>>(p);
      XCHECK(cudaGetLastError());
    }
    XCHECK(cudaEventRecord(a->ev_rev[q % 2], a->rs));
  }
  h->nffft = nffft;
  h->n_probes = n_probes;
  XCHECK(cudaEventRecord(a->ev_ready, a->rs));
  XCHECK(cudaStreamWaitEvent(h->stream, a->ev_ready, 0));
  if (a->K > 0) {   // back to the state after the last step
    adj_checkpoint(h, a->ck.back(), false);
    XCHECK(cudaMemcpyAsync(h->d_step, &T_, sizeof(long long), cudaMemcpyHostToDevice, h->stream));
  }
  XCHECK(cudaMemcpyAsync(g_eps, a->g_eps, a->nE * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  XCHECK(cudaMemcpyAsync(g_sig, a->g_sig, a->nE * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  XCHECK(cudaStreamSynchronize(h->stream));
  check_status(h);
}

}  // namespace

extern "C" {

int xfdtd_adjoint_forward(xfdtd_handle *h, const xfdtd_adjoint_desc *d, double *loss) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (!d) invalid("null adjoint description");
    if (h->precision == XFDTD_FP64) adj_forward_t<double>(h, d, loss);
    else adj_forward_t<float>(h, d, loss);
  });
}

int xfdtd_adjoint_backward(xfdtd_handle *h, double *grad_eps, double *grad_sigma, int64_t len) {
  if (!h) return XFDTD_ERR_STATE;
  return guarded(h, [&] {
    if (!h->adj) throw Err{XFDTD_ERR_STATE, "run xfdtd_adjoint_forward first"};
    if (!grad_eps || !grad_sigma || len != h->adj->nE) invalid("gradient arrays must hold one value per design cell");
    with_types(h->precision, h->idx_bytes, [&](auto t, auto i) {
      adj_backward_t<decltype(t), decltype(i)>(h, grad_eps, grad_sigma);
    });
  });
}

}  // extern "C"
