// nffft_noalloc.cu -- the batched NF-FF running DFT as a stand-alone operator
// that allocates no device memory (xfdtd_nffft_dft_noalloc, xfdtd_cuda.h).
//
// Some callers cannot allocate device memory when they call in: a host
// runtime whose memory manager owns every device allocation (a JVM, Go or
// .NET binding that reserves the GPU up front), a solver that budgets its
// device memory before the run and must not grow it mid-run, or a loop
// where cudaMalloc's implicit device synchronisation is not acceptable.  For
// them the batch of buffered surface samples lives in a fixed file-scope
// device array (kScratchBytes, 64 MiB) instead of memory the engine
// allocates per handle; the array is resident on every GPU that loads this
// library until the process exits.  A plan whose batch does not fit
// (batch x 24 x largest face x element size) is rejected with
// XFDTD_ERR_INVALID_PLAN before any GPU work.
//
// The operator follows NffftFd::update (src/nffft/nffft_fd.cpp:108-203)
// with the face-centre interpolations of EMF
// (src/electromagnetic_field/linear_interpolation_emf.cpp:286-421): each call
// samples the 24 surface currents of one step into slot (step mod batch) of
// the scratch array and, when asked, folds the last `fold_count` sampled
// steps into the caller's FP64 accumulators one step at a time, in step
// order.  The accumulators must start at zero (the caller owns and clears
// them); the scratch needs no clearing, because every slot is written by a
// sample before a fold reads it.  One scratch array serves all calls on a
// device, so calls that overlap in time on that device (different streams
// or threads) race on it: callers serialise them.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/xfdtd_cuda.h"

namespace {

// 64 MiB: a batch of 8 steps fits a largest NF-FF face of 87,381 cells in
// FP32 (295 x 295) or 43,690 cells in FP64 (209 x 209).
constexpr size_t kScratchBytes = 64ull << 20;

static __device__ __align__(256) unsigned char g_nffft_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;

// What the slots of a device's scratch were written with: the batch, the
// box and the element size fix where each step's samples sit.  `first` is
// the earliest step sampled with this layout in an unbroken run of steps
// and `last` the latest; a fold may only reach back to `first`.
struct Layout {
  int batch = 0, esize = 0;
  long long lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  long long first = -1, last = -1;
  bool same(int b, int e, const long long *l, const long long *h) const {
    if (b != batch || e != esize) return false;
    for (int a = 0; a < 3; ++a)
      if (l[a] != lo[a] || h[a] != hi[a]) return false;
    return true;
  }
};

void *g_scratch_ptr[kMaxDevices] = {};
Layout g_layout[kMaxDevices];
std::mutex g_scratch_mu;
thread_local char g_err[256];

int fail(int code, const char *msg) {
  std::strncpy(g_err, msg, sizeof(g_err) - 1);
  g_err[sizeof(g_err) - 1] = '\0';
  return code;
}

// Device address of the scratch array on `dev`, looked up once per device
// with that device current (host code must not use the symbol itself: on
// the host it is only a stand-in).  Leaves `dev` current.
int scratch_on_device(int dev, void **out) {
  if (dev < 0 || dev >= kMaxDevices) return fail(XFDTD_ERR_INVALID_PLAN, "device ordinal out of range");
  if (cudaSetDevice(dev) != cudaSuccess) return fail(XFDTD_ERR_CUDA, "cudaSetDevice failed");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_nffft_scratch);
    if (e != cudaSuccess || !p) return fail(XFDTD_ERR_CUDA, "cudaGetSymbolAddress of the NF-FF scratch failed");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return XFDTD_OK;
}

// Records that `step` is sampled with this layout on `dev` and checks that
// the fold's steps (fold_count of them, ending at `step`) were all sampled
// with it, in an unbroken run.  A call with another batch, box or precision
// starts a new run: the slots written before it hold another layout.
int claim_layout(int dev, int batch, int esize, const long long *lo, const long long *hi, long long step,
                 int fold_count) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  Layout &L = g_layout[dev];
  if (!L.same(batch, esize, lo, hi) || step != L.last + 1) {
    if (fold_count > 1)
      return fail(XFDTD_ERR_INVALID_PLAN,
                  "fold reaches steps not sampled with this batch, box and precision in an unbroken run");
    L.batch = batch;
    L.esize = esize;
    for (int a = 0; a < 3; ++a) L.lo[a] = lo[a], L.hi[a] = hi[a];
    L.first = step;
  } else if (step - fold_count + 1 < L.first) {
    return fail(XFDTD_ERR_INVALID_PLAN,
                "fold reaches steps not sampled with this batch, box and precision in an unbroken run");
  }
  L.last = step;
  return XFDTD_OK;
}

// Makes `dev` current for the launches and puts the caller's device back on
// every exit path.
struct DeviceScope {
  int prev = -1;
  bool changed = false;
  int enter(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) return fail(XFDTD_ERR_CUDA, "cudaGetDevice failed");
    if (prev != dev) {
      if (cudaSetDevice(dev) != cudaSuccess) return fail(XFDTD_ERR_CUDA, "cudaSetDevice failed");
      changed = true;
    }
    return XFDTD_OK;
  }
  ~DeviceScope() {
    if (changed) cudaSetDevice(prev);
  }
};

template <typename T>
struct OpParams {
  const T *f[6];
  long long si[6], sj[6];
  int lo[3], hi[3];
  int nf;
  const double2 *pj, *pm;
  long long total;
  int batch;
  T *buf;                // [batch][24][max_plane]: the scratch array
  long long plane[3];    // X (ny_box*nz_box), Y (nz_box*nx_box), Z (nx_box*ny_box)
  long long max_plane;
  long long step;
  double2 *acc[24];
};

// Face-centre averages are taken in the field precision (FP64 as the
// reference does; FP32 for FP32 fields, whose samples are stored as FP32),
// as the engine's own NF-FF kernel does.
template <typename T>
__device__ __forceinline__ T at(const OpParams<T> &p, int c, int i, int j, int k) {
  return p.f[c][static_cast<long long>(i) * p.si[c] + static_cast<long long>(j) * p.sj[c] + k];
}

// Samples the 24 surface currents of step p.step (reference accumulator
// layout: X faces [j][k], Y faces [k][i], Z faces [i][j]).
template <typename T>
__global__ void k_sample(OpParams<T> p) {
  const long long t = p.step;
  const int li = p.lo[0], lj = p.lo[1], lk = p.lo[2], ri = p.hi[0], rj = p.hi[1], rk = p.hi[2];
  const int face = blockIdx.z;
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = blockIdx.y * blockDim.y + threadIdx.y;
  T val[8];
  const T half = T(0.5), quarter = T(0.25), neg = T(-1);
  long long cell;
  if (face == 0) {   // j in [lj, rj), k in [lk, rk): jy jz my mz (xn), then xp
    const int k = lk + u, j = lj + v;
    if (k >= rk || j >= rj) return;
    val[2] = neg * (half * (at(p, 2, li, j, k) + at(p, 2, li, j + 1, k)));
    val[3] = half * (at(p, 1, li, j, k) + at(p, 1, li, j, k + 1));
    val[0] = quarter * (at(p, 5, li, j, k) + at(p, 5, li, j, k + 1) + at(p, 5, li - 1, j, k) + at(p, 5, li - 1, j, k + 1));
    val[1] = neg * (quarter * (at(p, 4, li, j, k) + at(p, 4, li, j + 1, k) + at(p, 4, li - 1, j, k) + at(p, 4, li - 1, j + 1, k)));
    val[6] = half * (at(p, 2, ri, j, k) + at(p, 2, ri, j + 1, k));
    val[7] = neg * (half * (at(p, 1, ri, j, k) + at(p, 1, ri, j, k + 1)));
    val[4] = neg * (quarter * (at(p, 5, ri, j, k) + at(p, 5, ri, j, k + 1) + at(p, 5, ri - 1, j, k) + at(p, 5, ri - 1, j, k + 1)));
    val[5] = quarter * (at(p, 4, ri, j, k) + at(p, 4, ri, j + 1, k) + at(p, 4, ri - 1, j, k) + at(p, 4, ri - 1, j + 1, k));
    cell = static_cast<long long>(j - lj) * (rk - lk) + (k - lk);
  } else if (face == 1) {   // k in [lk, rk), i in [li, ri): jz jx mz mx (yn), then yp
    const int i = li + u, k = lk + v;
    if (i >= ri || k >= rk) return;
    val[2] = neg * (half * (at(p, 0, i, lj, k) + at(p, 0, i, lj + 1, k)));
    val[3] = half * (at(p, 2, i, lj, k) + at(p, 2, i + 1, lj, k));
    val[0] = quarter * (at(p, 3, i + 1, lj, k) + at(p, 3, i, lj, k) + at(p, 3, i + 1, lj - 1, k) + at(p, 3, i, lj - 1, k));
    val[1] = neg * (quarter * (at(p, 5, i, lj, k) + at(p, 5, i, lj, k + 1) + at(p, 5, i, lj - 1, k) + at(p, 5, i, lj - 1, k + 1)));
    val[6] = half * (at(p, 0, i, rj, k) + at(p, 0, i, rj + 1, k));
    val[7] = neg * (half * (at(p, 2, i, rj, k) + at(p, 2, i + 1, rj, k)));
    val[4] = neg * (quarter * (at(p, 3, i + 1, rj, k) + at(p, 3, i, rj, k) + at(p, 3, i + 1, rj - 1, k) + at(p, 3, i, rj - 1, k)));
    val[5] = quarter * (at(p, 5, i, rj, k) + at(p, 5, i, rj, k + 1) + at(p, 5, i, rj - 1, k) + at(p, 5, i, rj - 1, k + 1));
    cell = static_cast<long long>(k - lk) * (ri - li) + (i - li);
  } else {   // i in [li, ri), j in [lj, rj): jx jy mx my (zn), then zp
    const int j = lj + u, i = li + v;
    if (j >= rj || i >= ri) return;
    val[2] = neg * (half * (at(p, 1, i, j, lk) + at(p, 1, i + 1, j, lk)));
    val[3] = half * (at(p, 0, i, j, lk) + at(p, 0, i, j, lk + 1));
    val[0] = quarter * (at(p, 4, i, j, lk) + at(p, 4, i, j + 1, lk) + at(p, 4, i, j, lk - 1) + at(p, 4, i, j + 1, lk - 1));
    val[1] = neg * (quarter * (at(p, 3, i + 1, j, lk) + at(p, 3, i, j, lk) + at(p, 3, i + 1, j, lk - 1) + at(p, 3, i, j, lk - 1)));
    val[6] = half * (at(p, 1, i, j, rk) + at(p, 1, i + 1, j, rk));
    val[7] = neg * (half * (at(p, 0, i, j, rk) + at(p, 0, i, j, rk + 1)));
    val[4] = neg * (quarter * (at(p, 4, i, j, rk) + at(p, 4, i, j + 1, rk) + at(p, 4, i, j, rk - 1) + at(p, 4, i, j + 1, rk - 1)));
    val[5] = quarter * (at(p, 3, i + 1, j, rk) + at(p, 3, i, j, rk) + at(p, 3, i + 1, j, rk - 1) + at(p, 3, i, j, rk - 1));
    cell = static_cast<long long>(i - li) * (rj - lj) + (j - lj);
  }
  T *b = p.buf + (static_cast<long long>(t % p.batch) * 24 + face * 8) * p.max_plane + cell;
#pragma unroll
  for (int q = 0; q < 8; ++q) b[q * p.max_plane] = val[q];
}

// acc += v[s] * phase[t0 + s] for the `count` steps ending at p.step, the
// engine's fold (k_nffft_accumulate): FP64 samples are added one step at a
// time in step order; FP32 samples are summed over the batch in FP32, with
// the phases rounded to FP32, and the partial sum goes to the FP64
// accumulator.
template <typename T>
__global__ void k_fold(OpParams<T> p, int count) {
  const int face = blockIdx.z;
  const long long cell = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (cell >= p.plane[face]) return;
  const long long t_last = p.step, t0 = t_last - count + 1;
  for (int q = 0; q < 8; ++q) {
    const double2 *ph = ((q % 4) < 2 ? p.pj : p.pm) + t0;   // J terms at (t+1/2) dt, M terms at t dt
    for (int n = 0; n < p.nf; ++n) {
      double2 *a = p.acc[face * 8 + q] + n * p.plane[face] + cell;
      double2 r = *a;
      float2 part = make_float2(0.f, 0.f);
      for (int s = 0; s < count; ++s) {
        const long long t = t0 + s;
        const T v = p.buf[(static_cast<long long>(t % p.batch) * 24 + face * 8 + q) * p.max_plane + cell];
        const double2 f = ph[n * p.total + s];
        if constexpr (sizeof(T) == 8) {
          r.x = fma(v, f.x, r.x);
          r.y = fma(v, f.y, r.y);
        } else {
          part.x = fmaf(v, static_cast<float>(f.x), part.x);
          part.y = fmaf(v, static_cast<float>(f.y), part.y);
        }
      }
      if constexpr (sizeof(T) == 4) {
        r.x += static_cast<double>(part.x);
        r.y += static_cast<double>(part.y);
      }
      *a = r;
    }
  }
}

// Validates the description on the host (no device call before it passes),
// then looks up the scratch and launches.
template <typename T>
int run(const xfdtd_nffft_operator *op) {
  OpParams<T> p{};
  const long long n[3] = {op->nx, op->ny, op->nz};
  // the kernels index planes, rows and columns with int, and the sample
  // launch covers the box's longest edge with 8 rows per block on grid.y
  for (int a = 0; a < 3; ++a)
    if (n[a] < 3 || n[a] > (1ll << 30)) return fail(XFDTD_ERR_INVALID_PLAN, "grid size out of range (3 .. 2^30 cells per axis)");
  for (int a = 0; a < 3; ++a) {
    if (op->lo[a] < 1 || op->hi[a] <= op->lo[a] || op->hi[a] > n[a] - 1)
      return fail(XFDTD_ERR_INVALID_PLAN, "NF-FF box outside the grid");
    p.lo[a] = static_cast<int>(op->lo[a]);
    p.hi[a] = static_cast<int>(op->hi[a]);
  }
  // reference component shapes (simulation_init.cpp:28-35), k contiguous
  const long long shp[6][3] = {{n[0], n[1] + 1, n[2] + 1}, {n[0] + 1, n[1], n[2] + 1}, {n[0] + 1, n[1] + 1, n[2]},
                               {n[0] + 1, n[1], n[2]},     {n[0], n[1] + 1, n[2]},     {n[0], n[1], n[2] + 1}};
  for (int c = 0; c < 6; ++c) {
    if (!op->fields[c]) return fail(XFDTD_ERR_INVALID_PLAN, "a field pointer is null");
    p.f[c] = static_cast<const T *>(op->fields[c]);
    p.sj[c] = shp[c][2];
    p.si[c] = shp[c][1] * shp[c][2];
  }
  const long long bx = p.hi[0] - p.lo[0], by = p.hi[1] - p.lo[1], bz = p.hi[2] - p.lo[2];
  p.plane[0] = by * bz;
  p.plane[1] = bz * bx;
  p.plane[2] = bx * by;
  p.max_plane = p.plane[0] > p.plane[1] ? p.plane[0] : p.plane[1];
  if (p.plane[2] > p.max_plane) p.max_plane = p.plane[2];
  const long long m = bx > by ? (bx > bz ? bx : bz) : (by > bz ? by : bz);
  if (m > 8ll * 65535) return fail(XFDTD_ERR_INVALID_PLAN, "NF-FF box edge above 524,280 cells");
  if (op->batch < 1 || op->n_freq < 1 || op->total_steps < 1 || op->step < 0 || op->step >= op->total_steps)
    return fail(XFDTD_ERR_INVALID_PLAN, "batch, n_freq, total_steps and step must be positive and in range");
  if (op->fold_count < 0 || op->fold_count > op->batch || op->fold_count > op->step + 1)
    return fail(XFDTD_ERR_INVALID_PLAN, "fold_count must be within the batch and the steps taken");
  const unsigned long long need = static_cast<unsigned long long>(op->batch) * 24ull * p.max_plane * sizeof(T);
  if (need > kScratchBytes)
    return fail(XFDTD_ERR_INVALID_PLAN, "NF-FF batch exceeds the 64 MiB allocation-free scratch (batch x 24 x face cells)");
  if (!op->phase_j || !op->phase_m) return fail(XFDTD_ERR_INVALID_PLAN, "phase tables are required");
  for (int q = 0; q < 24; ++q) {
    if (!op->acc[q]) return fail(XFDTD_ERR_INVALID_PLAN, "an accumulator pointer is null");
    p.acc[q] = reinterpret_cast<double2 *>(op->acc[q]);
  }
  p.nf = op->n_freq;
  p.pj = reinterpret_cast<const double2 *>(op->phase_j);
  p.pm = reinterpret_cast<const double2 *>(op->phase_m);
  p.total = op->total_steps;
  p.batch = op->batch;
  p.step = op->step;
  if (op->device < 0 || op->device >= kMaxDevices) return fail(XFDTD_ERR_INVALID_PLAN, "device ordinal out of range");
  void *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    scratch = g_scratch_ptr[op->device];
  }
  if (!scratch) return fail(XFDTD_ERR_STATE, "call xfdtd_nffft_noalloc_setup(device) before the first operator call");
  const long long lo[3] = {op->lo[0], op->lo[1], op->lo[2]}, hi[3] = {op->hi[0], op->hi[1], op->hi[2]};
  int rc = claim_layout(op->device, op->batch, static_cast<int>(sizeof(T)), lo, hi, op->step, op->fold_count);
  if (rc != XFDTD_OK) return rc;
  DeviceScope scope;
  rc = scope.enter(op->device);
  if (rc != XFDTD_OK) return rc;
  p.buf = static_cast<T *>(scratch);
  cudaStream_t st = static_cast<cudaStream_t>(op->stream);
  // face 0 spans (k, j), face 1 (i, k), face 2 (j, i): cover the longest edge on both grid axes
  dim3 block(32, 8, 1);
  dim3 grid(static_cast<unsigned>((m + 31) / 32), static_cast<unsigned>((m + 7) / 8), 3);
  k_sample<T><<<grid, block, 0, st>>>(p);
  if (cudaGetLastError() != cudaSuccess) return fail(XFDTD_ERR_CUDA, "NF-FF sample launch failed");
  if (op->fold_count > 0) {
    dim3 g2(static_cast<unsigned>((p.max_plane + 255) / 256), 1, 3);
    k_fold<T><<<g2, 256, 0, st>>>(p, op->fold_count);
    if (cudaGetLastError() != cudaSuccess) return fail(XFDTD_ERR_CUDA, "NF-FF fold launch failed");
  }
  return XFDTD_OK;
}

}  // namespace

extern "C" {

int xfdtd_nffft_noalloc_setup(int device) {
  void *scratch = nullptr;
  return scratch_on_device(device, &scratch);
}

int xfdtd_nffft_dft_noalloc(const xfdtd_nffft_operator *op) {
  if (!op) return fail(XFDTD_ERR_INVALID_PLAN, "null operator description");
  if (op->precision != XFDTD_FP64 && op->precision != XFDTD_FP32)
    return fail(XFDTD_ERR_INVALID_PLAN, "precision must be FP64 or FP32");
  return op->precision == XFDTD_FP64 ? run<double>(op) : run<float>(op);
}

int64_t xfdtd_nffft_noalloc_max_bytes(void) { return static_cast<int64_t>(kScratchBytes); }

const char *xfdtd_nffft_noalloc_last_error(void) { return g_err; }

}  // extern "C"
