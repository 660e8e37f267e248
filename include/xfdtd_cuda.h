/*
 * xfdtd_cuda.h -- C-ABI of the GB300 FDTD engine (libxfdtd_cuda.so).
 *
 * The engine runs the loop body of the reference's Simulation::run
 * (src/simulation/simulation_update.cpp:9-36) on one GPU:
 *
 *   updateE (:130-197) -> correctE: lumped (:282-290), TFSF3D::updateE
 *   (src/tfsf/tfsf_3d.cpp:299-411) -> PML::updateE
 *   (src/boundary/perfect_match_layer.cpp:574-718) -> updateH (:50-108) ->
 *   TFSF3D::updateIncidentField (tfsf_3d.cpp:153-183) -> TFSF3D::updateH
 *   (:185-297) -> PML::updateH (perfect_match_layer.cpp:434-572) ->
 *   NffftFd::update (src/nffft/nffft_fd.cpp:108-203) -> Monitor::update
 *   (src/monitor/voltage_monitor.cpp:64-97, current_monitor.cpp:70-115)
 *
 * and the far-field integration of NffftFd::calculateFarfield
 * (nffft_fd.cpp:379-556) at the end.  The reference has no FFI; these
 * entry points replace the virtual hooks Simulation calls per step
 * (Boundary::updateE/H, TFSF::updateIncidentField/updateE/updateH,
 * NFFFT::update, LumpedElement::correctE, Monitor::update -- declared in
 * src/include/{boundary/boundary.h:28-52, tfsf/tfsf.h:80-90,
 * nffft/nffft.h:71-75, lumped_element/lumped_element.h:22-30,
 * monitor/monitor.h:31-37}) with one plan built once on the host.
 *
 * The plan is what the reference's init() computes
 * (src/simulation/simulation_init.cpp:10-22), in a compact form: a per-cell
 * material index into a table of the 18 update coefficients of
 * FDTDBasicCoff::initCoff (src/fdtd_basic_coff/fdtd_basic_coff.cpp:77-121)
 * instead of 18 full per-cell arrays; 1-D CPML profiles instead of the
 * per-face c_psi slabs; the TFSF projection tables; the NF-FF phase tables.
 *
 * Conventions.  Grid cells nx, ny, nz include the CPML.  Every field,
 * material-index and coefficient array uses the reference's (i, j, k)
 * indexing, row-major with k fastest.  The handle owns all device memory;
 * host arrays passed in are copied and not retained.  Calls on one handle
 * must be serialised by the caller; distinct handles are independent.
 * Every function returns XFDTD_OK (0) or an XFDTD_ERR_* status, and
 * xfdtd_last_error() gives the message of the last failure on that handle.
 */
#ifndef XFDTD_CUDA_H_
#define XFDTD_CUDA_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  XFDTD_OK = 0,
  XFDTD_ERR_INVALID_PLAN = 1,   /* rejected on the host before any GPU work */
  XFDTD_ERR_CUDA = 2,           /* a CUDA runtime call failed               */
  XFDTD_ERR_OOM = 3,            /* device allocation failed                 */
  XFDTD_ERR_TIMEOUT = 4,        /* a bounded device wait gave up            */
  XFDTD_ERR_NAN = 5,            /* non-finite value found by xfdtd_check_finite */
  XFDTD_ERR_DEVICE_CHECK = 6,   /* a device-side bounds check fired          */
  XFDTD_ERR_STATE = 7           /* call not valid in the handle's state     */
};

enum { XFDTD_FP64 = 0, XFDTD_FP32 = 1 };

/* Plan flags. */
enum {
  XFDTD_FLAG_GRAPH = 1,      /* replay the step loop from a captured CUDA graph */
  XFDTD_FLAG_PROFILE = 2,    /* time every kernel launch with CUDA events        */
  XFDTD_FLAG_AUTOTUNE = 4,   /* pick the volume kernels and their variants by timing at create */
  XFDTD_FLAG_SPLIT_EH = 8,   /* always the separate in-place E and H kernels            */
  XFDTD_FLAG_FUSED_EH = 16,  /* always the fused E/H sweep (unless the plan has lumped
                                elements, which run the split kernels).  With neither
                                flag the autotuner picks the faster of the two, and
                                without autotuning the split kernels run. */
  XFDTD_FLAG_PLAIN_VOLUME = 32  /* xfdtd_batch_create: the one-thread-per-cell volume
                                   kernels for every member, none TMA-staged */
};

/* The 18 coefficients of one table entry, in this order (the reference's
 * names, fdtd_basic_coff.h): cexe cexhy cexhz ceye ceyhz ceyhx ceze cezhx
 * cezhy chxh chxey chxez chyh chyez chyex chzh chzex chzey.  Values are
 * those before the CPML's kappa division (perfect_match_layer.cpp:190-206);
 * the engine applies 1/kappa from the CPML profiles. */
#define XFDTD_N_COEFF 18

/* CPML along one axis: the union of its N and P slabs.  For an E-located
 * index I (0..n) slot_e[I] is the psi layer (0..n_layers-1) or -1 outside
 * the slabs; slot_h likewise for H-located indices.  b/a are the CPML
 * recursion coefficients and rk = 1/kappa of the layer (1 outside). */
typedef struct xfdtd_cpml_axis {
  int32_t n_layers;
  int32_t reserved;
  const int32_t *slot_e, *slot_h;          /* [n+1] */
  const double *b_e, *a_e, *rk_e;          /* [n+1] */
  const double *b_m, *a_m, *rk_m;          /* [n+1] */
} xfdtd_cpml_axis;

/* TFSF3D by the 1-D incident-field array (tfsf_3d.cpp:33-183). */
typedef struct xfdtd_tfsf_plan {
  int32_t enabled;
  int32_t aux_len;                 /* L = ceil(diagonal * ratio_delta) + 5      */
  int64_t lo[3], hi[3];            /* li lj lk, ri rj rk                        */
  const double *proj_full[3];      /* [box_n + 1]                               */
  const double *proj_half[3];      /* [box_n + 2]                               */
  double transform_e[3], transform_h[3];
  double ceihi, chiei;             /* 1-D free-space update coefficients        */
  double mur_c1, mur_c2;           /* second-order Mur ABC at the far end       */
  double ca[3], cb[3];             /* dt/(eps0 d), dt/(mu0 d) per axis          */
  const double *source;            /* [total_steps] e0 * w(t dt)                */
} xfdtd_tfsf_plan;

/* NffftFd (nffft_fd.cpp:17-203, 379-556). */
/* enabled: 1 NffftFd (running DFT at n_freq frequencies, far field over
 * theta x phi); 2 NffftBroadBand (src/nffft/nffft_broadband.cpp: every
 * step's surface samples kept, n_freq and the phase tables unused, theta[0]
 * and phi[0] the one direction). */
typedef struct xfdtd_nffft_plan {
  int32_t enabled;
  int32_t n_freq;
  int64_t lo[3], hi[3];
  const double *phase_j;           /* [n_freq * total_steps] (re, im) pairs    */
  const double *phase_m;           /* [n_freq * total_steps] (re, im) pairs    */
  const double *wave_number;       /* [n_freq]                                 */
  int32_t n_theta, n_phi;
  const double *theta, *phi;
} xfdtd_nffft_plan;

/* E(comp)[i,j,k] += coff * waveform[w][t]  (CurrentSource / VoltageSource
 * ::correctE, current_source.cpp:140-163, voltage_source.cpp:171-194). */
typedef struct xfdtd_injection {
  int32_t comp, waveform;
  int64_t i, j, k;
  double coff;
} xfdtd_injection;

/* E += cecjc * J; J = cjcec * E + J  (Inductor::correctE, inductor.cpp:102-143). */
typedef struct xfdtd_inductor_cell {
  int32_t comp, reserved;
  int64_t i, j, k;
  double cecjc, cjcec;
} xfdtd_inductor_cell;

/* value[probe][t] = sum over the probe's terms of weight * F(comp)[i,j,k]
 * (VoltageMonitor / CurrentMonitor as linear functionals).  Terms of one
 * probe are contiguous and summed in order. */
typedef struct xfdtd_probe_term {
  int32_t probe, comp;
  int64_t i, j, k;
  double weight;
} xfdtd_probe_term;

/* A series of field snapshots, what a MovieMonitor over a
 * TimeDomainFieldMonitor records (src/monitor/movie_monitor.cpp:46-59,
 * src/monitor/field_monitor.cpp:91-122): after each step t with
 * t % every == 0, and after step `last` (-1: none), the values of field
 * component comp (0..5: Ex Ey Ez Hx Hy Hz) over the box lo .. lo+n-1 of
 * the component's array. */
typedef struct xfdtd_snapshot_desc {
  int32_t comp;
  int32_t reserved;
  int64_t lo[3];
  int64_t n[3];
  int64_t every;                   /* >= 1                                      */
  int64_t last;
} xfdtd_snapshot_desc;

/* A linear dispersive medium's E recursion, LorentzMedium /
 * DrudeMedium / DebyMedium::updateE{x,y,z} (src/material/dispersive_material.cpp):
 * kind 1 Lorentz, 2 Drude, 3 Debye, with the coefficients their init
 * computes (Lorentz: ca cb cc alpha xi gamma; Drude and Debye: ca cb k
 * beta).  The reference throws on dispersive objects at Object::init
 * (object.cpp:109-110); the engine runs them. */
typedef struct xfdtd_dispersive_medium {
  int32_t kind;
  int32_t reserved;
  double ca, cb, cc, alpha, xi, gamma;
  double k, beta;
} xfdtd_dispersive_medium;

/* One E component (comp 0..2) at (i, j, k) whose update is its medium's
 * recursion instead of the Yee update; its table entry leaves E as it is. */
typedef struct xfdtd_dispersive_cell {
  int32_t comp;
  int32_t medium;
  int64_t i, j, k;
} xfdtd_dispersive_cell;

typedef struct xfdtd_plan_desc {
  int32_t nx, ny, nz;
  int32_t precision;               /* XFDTD_FP64 or XFDTD_FP32 (fields, psi)    */
  double dt;
  double dl[3];
  int64_t total_steps;
  int32_t flags;                   /* XFDTD_FLAG_*                             */
  int32_t index_bytes;             /* 1 or 2                                   */
  int32_t n_materials;
  int32_t device;                  /* CUDA device ordinal the handle runs on   */
  const void *material_index;      /* [(nx+1)*(ny+1)*(nz+1)]                   */
  const double *coeff_table;       /* [n_materials * XFDTD_N_COEFF]            */
  xfdtd_cpml_axis cpml[3];
  xfdtd_tfsf_plan tfsf;
  xfdtd_nffft_plan nffft;
  int32_t n_waveforms;
  int32_t n_injections;
  const double *waveforms;         /* [n_waveforms * total_steps]              */
  const xfdtd_injection *injections;
  int32_t n_inductor_cells;
  int32_t n_probes;
  const xfdtd_inductor_cell *inductor_cells;
  int32_t n_probe_terms;
  int32_t reserved2;
  const xfdtd_probe_term *probe_terms;
  int32_t n_snapshots;
  int32_t reserved3;
  const xfdtd_snapshot_desc *snapshots;
  int32_t n_disp_media;            /* linear dispersive media (above)         */
  int32_t n_disp_cells;
  const xfdtd_dispersive_medium *disp_media;
  const xfdtd_dispersive_cell *disp_cells;
  double disp_dl;                  /* the uniform cell size of their recursions */
} xfdtd_plan_desc;

typedef struct xfdtd_handle xfdtd_handle;

/* Validates the plan, allocates and uploads everything.  Replaces the
 * per-component init hooks (Boundary::init, TFSF::init, NFFFT::init, ...). */
int xfdtd_create(const xfdtd_plan_desc *plan, xfdtd_handle **out);
/* Enqueues n steps of the loop body on the handle's stream (asynchronous). */
int xfdtd_step(xfdtd_handle *h, int64_t n);
/* Waits for the handle's stream and reports any device-side status. */
int xfdtd_synchronize(xfdtd_handle *h);
/* Enqueues n steps and returns their device time in milliseconds, measured
 * with CUDA events on the handle's stream. */
int xfdtd_step_timed(xfdtd_handle *h, int64_t n, double *ms);
/* Current step index (steps completed). */
int xfdtd_current_step(xfdtd_handle *h, int64_t *step);
/* Field component c (0..5: Ex Ey Ez Hx Hy Hz) in the reference's component
 * shape (Ex (nx,ny+1,nz+1) ... Hz (nx,ny,nz+1)), converted to FP64. */
int xfdtd_read_field(xfdtd_handle *h, int comp, double *out, int64_t len);
int xfdtd_write_field(xfdtd_handle *h, int comp, const double *in, int64_t len);
/* Probe time series [n_probes * total_steps]. */
int xfdtd_read_probes(xfdtd_handle *h, double *out, int64_t len);
/* Frames of snapshot series s (plan order): their number, and the step
 * after which each is taken (steps[f] for f < min(max, count); steps may be
 * null).  A frame holds data once its step has run. */
int xfdtd_snapshot_frames(xfdtd_handle *h, int s, int64_t *count, int64_t *steps, int64_t max);
/* Frame f of snapshot series s, [n0][n1][n2] converted to FP64 (len =
 * n0*n1*n2 of the series' box). */
int xfdtd_read_snapshot(xfdtd_handle *h, int s, int64_t frame, double *out, int64_t len);
/* NF-FF accumulator `which` = face*4 + q (faces XN XP YN YP ZN ZP; X faces
 * jy jz my mz over (ny_box, nz_box); Y faces jz jx mz mx over (nz_box,
 * nx_box); Z faces jx jy mx my over (nx_box, ny_box)), [n_freq][a][b] (re, im). */
int xfdtd_read_nffft(xfdtd_handle *h, int which, double *out, int64_t len);
/* Broadband NF-FF (plan nffft.enabled = 2): the auxiliary arrays n_x, n_y,
 * n_z, l_x, l_y, l_z of NffftBroadBand::calculateLNXYZ
 * (src/nffft/nffft_broadband.cpp:351-464) over the N = 2*total_steps - 1
 * fftshifted bins of linspace(-1/(2 dt), 1/(2 dt), N), as [6][N] (re, im)
 * pairs (len = 12 N), from the samples of the steps run so far.  Uses
 * cuFFT (libcufft), loaded at the first call. */
int xfdtd_broadband_far_field(xfdtd_handle *h, double *out, int64_t len);
/* Far field over (n_freq, n_theta, n_phi): which 0 e_theta 1 e_phi 2 h_theta
 * 3 h_phi 4 n_theta 5 n_phi 6 l_theta 7 l_phi (complex pairs), 8 power_theta
 * 9 power_phi (real) -- the arrays NffftFd::outputData writes. */
int xfdtd_far_field(xfdtd_handle *h, int which, double *out, int64_t len);
/* Scans all fields for NaN / Inf (XFDTD_ERR_NAN if any). */
int xfdtd_check_finite(xfdtd_handle *h);
/* Per-kernel device time accumulated under XFDTD_FLAG_PROFILE:
 * names[i] (static strings), total milliseconds and launch counts. */
int xfdtd_profile(xfdtd_handle *h, int max, const char **names, double *ms, int64_t *launches, int *count);
int xfdtd_profile_reset(xfdtd_handle *h);
/* Times every variant of the volume kernels and keeps the fastest: of the
 * fused E/H sweep (register cap x planes per block), or with
 * XFDTD_FLAG_SPLIT_EH of the E and H updates separately.  A split update is
 * an interior launch and a shell launch on two streams; its variants are
 * the interior launch's (register cap x block shape x cells per thread x
 * table placement and form, or TMA-staged planes over the narrow or the
 * wide decomposition) paired with a shell variant, timed as the pair runs.
 * Only before the first step: the trials run on the all-zero initial state
 * and leave it unchanged.  All variants compute bitwise-identical results. */
int xfdtd_autotune(xfdtd_handle *h, int trials);
/* Number of variants, the ones in use, and the last trial times of the
 * whole update with each (trial_ms[2*v] for E, [2*v+1] for H; 0 where not
 * tried).  A variant of the wide decomposition moves the x and y slabs into
 * the interior launch (see xfdtd_volume_decomposition).  For the fused
 * sweep both sides report the sweep's variant and time, and
 * xfdtd_set_kernel_variant takes the same variant for both. */
int xfdtd_kernel_variants(xfdtd_handle *h, int *n, int *current_e, int *current_h, double *trial_ms);
int xfdtd_set_kernel_variant(xfdtd_handle *h, int e_variant, int h_variant);
/* Variants of the shell launches (walls and CPML slabs): how many, the ones
 * in use for E and H; and fixing them (all give the same bits).  Variants
 * 0-3 are the shell kernel (register cap x table form); 4-6 the z-edge
 * TMA-staged launch in 32 x 8 tiles and 7-9 in 16 x 16 tiles (ring stages
 * x table form), offered
 * with a wide interior variant only
 * (XFDTD_ERR_INVALID_PLAN otherwise). */
int xfdtd_shell_variants(xfdtd_handle *h, int *n, int *current_e, int *current_h);
int xfdtd_set_shell_variant(xfdtd_handle *h, int e_variant, int h_variant);
/* Failure detection of the TMA-staged volume launches.  No counterpart in
 * the reference (a single-threaded CPU loop has no device waits).  Each
 * block of those launches waits on an mbarrier for every plane its loads
 * bring in, polling at most `polls` times (default and maximum 2^22);
 * a block that gives up stops, waits (with the full 2^22 polls) for the
 * copies it issued, and sets XFDTD_ERR_TIMEOUT in the handle's status word,
 * which the next xfdtd_synchronize returns.  The fields are then not
 * advanced consistently and the handle should be destroyed; the device
 * context stays usable.  polls = 0 makes every plane wait give up at once
 * (the failure path's test).  Applies to launches enqueued after the call
 * (a captured step graph is recaptured). */
int xfdtd_set_wait_limit(xfdtd_handle *h, int64_t polls);
/* Cells of the split volume update: cells[0] / [1] the E update's interior
 * (plain on every axis, the interior kernel) and shell (walls and CPML
 * slabs, the shell kernel); cells[2] / [3] the same for H. */
int xfdtd_volume_split(xfdtd_handle *h, int64_t cells[4]);
/* The decomposition each update runs with its current variant: wide[0]
 * (E) and wide[1] (H) are 0 for the narrow one (the interior launch covers
 * the cells plain on every axis, the shell launch the rest) and 1 for the
 * wide one (the interior launch covers every plane and row over the
 * interior's k range, x and y slabs included; the shell launch the z
 * slabs). */
int xfdtd_volume_decomposition(xfdtd_handle *h, int wide[2]);
/* Per-step kernel launches enqueued so far (graph replays included). */
int xfdtd_launch_count(xfdtd_handle *h, int64_t *n);
/* Kernel launches the engine enqueues per step for this plan. */
int xfdtd_launches_per_step(xfdtd_handle *h, int *n);
/* Bytes copied host->device and device->host by the handle so far. */
int xfdtd_transfer_bytes(xfdtd_handle *h, int64_t *h2d, int64_t *d2h);
/* The TFSF surface corrections folded into the wide decomposition's TMA
 * launches.  Where a side runs the wide decomposition on its two TMA
 * launches (the wide interior launch and the z-edge launch) and the plan
 * has no lumped element, those launches apply TFSF3D::updateE's
 * (updateH's) corrections to the cells of the box's surface
 * (src/tfsf/tfsf_3d.cpp:185-411), with the arithmetic of the separate
 * k_tfsf_e / k_tfsf_h launches, and those launches are left out.  The
 * autotuner keeps the faster of the two forms per side; set_tfsf_fusion
 * allows (1) or forbids (0) the folded form, and xfdtd_tfsf_fusion reports
 * whether each side uses it with its current variant.  Both give the same
 * bits.  No counterpart in the reference. */
int xfdtd_set_tfsf_fusion(xfdtd_handle *h, int e_on, int h_on);
int xfdtd_tfsf_fusion(xfdtd_handle *h, int active[2]);
/* The schedule of the NF-FF running DFT's sampling
 * (src/nffft/nffft_fd.cpp:108-203 samples E and H on the Huygens box after
 * every step).  Split (1): the E half of step t's samples runs on its own
 * stream beside step t's H update, the H half beside step t+1's E update,
 * with the fold of each batch of 8 steps.  One launch (0): the samples in
 * one launch after the H update (beside the TFSF H corrections where their
 * cells are disjoint), the fold on the engine's stream.  The autotuner
 * times both with the kept volume kernels and keeps the faster;
 * set_nffft_split fixes one (taking any pending samples first).
 * xfdtd_nffft_split reports the schedule in use and, in ms[2] (may be
 * null), the autotuner's trial step times of the split and one-launch
 * forms (0 when not timed).  Both give the same bits.  No counterpart in
 * the reference. */
int xfdtd_set_nffft_split(xfdtd_handle *h, int on);
int xfdtd_nffft_split(xfdtd_handle *h, int *on, float ms[2]);
/* Wall time of xfdtd_create, in ms: ms[0] validation, device allocation
 * and upload of the tables; ms[1] autotuning (0 without
 * XFDTD_FLAG_AUTOTUNE).  No counterpart in the reference. */
int xfdtd_create_times(xfdtd_handle *h, double ms[2]);
/* Device bytes held by the handle (with its adjoint state, if any). */
int xfdtd_device_bytes(xfdtd_handle *h, int64_t *bytes);
/* Bytes per cell of the plan's material index (1, 2 or 4). */
int xfdtd_index_bytes(xfdtd_handle *h, int *bytes);
const char *xfdtd_last_error(xfdtd_handle *h);
void xfdtd_destroy(xfdtd_handle *h);

/* Version string of the engine build. */
const char *xfdtd_version(void);

/* ---------------------------------------------------------------------
 * Adjoint gradients.  No counterpart in the reference, which has no
 * differentiation: the gradient of the loss
 *   L = sum over steps t in [t_begin, t_end) and over a plane of F(t+1)^2
 * (F = Ex, Ey or Ez after step t) with respect to eps_r and sigma of every
 * cell of a design box, by the discrete adjoint (transpose) of the split
 * E/H update including CPML.  Lumped sources and TFSF injection are
 * affine and do not enter the adjoint; inductors are not supported.  The
 * design box and its one-cell rim must lie outside the CPML.
 * xfdtd_adjoint_forward runs all total_steps from step 0 (the handle must
 * not have been stepped), checkpointing the state every checkpoint_every
 * steps (0: record the design box at every step instead) and returns L.
 * xfdtd_adjoint_backward then returns dL/d eps_r and dL/d sigma per design
 * cell, [i][j][k] over the box (with K > 0 it re-runs each checkpoint
 * segment once; with K = 0 it reads the recorded design box).  Memory: K = 0
 * holds 6 components of the design box per step, K > 0 one full state per
 * checkpoint (xfdtd_device_bytes reports both). */
typedef struct xfdtd_adjoint_desc {
  int64_t design_lo[3], design_hi[3];   /* cells [lo, hi) per axis                    */
  int32_t loss_comp;                    /* 0 Ex, 1 Ey, 2 Ez                            */
  int32_t plane_axis;                   /* axis normal to the loss plane               */
  int64_t plane_index;                  /* its index on that axis                      */
  int64_t plane_lo[2], plane_hi[2];     /* extents on the other two axes, in axis order */
  int64_t t_begin, t_end;               /* loss window (steps)                         */
  int32_t checkpoint_every;             /* K                                           */
  int32_t reserved;
} xfdtd_adjoint_desc;

int xfdtd_adjoint_forward(xfdtd_handle *h, const xfdtd_adjoint_desc *d, double *loss);
int xfdtd_adjoint_backward(xfdtd_handle *h, double *grad_eps, double *grad_sigma, int64_t len);

/* ---------------------------------------------------------------------
 * Batches: many independent simulations of different sizes advanced
 * together.  The reference runs one Simulation at a time
 * (simulation_update.cpp:5-40); a batch runs each phase of the loop body
 * for all of its running members in one launch (the volume phases: an
 * interior and a shell launch per group of up to 64 members, TMA-staged
 * for the members whose grids allow it), and replays
 * the step loop from a CUDA graph (XFDTD_FLAG_GRAPH).  Members
 * are ordinary handles from xfdtd_create -- same device, precision and
 * material-index width, not yet stepped, without lumped elements or
 * monitors; the batch does not own them.  Each member stops at its own
 * total_steps.  A batched member gives the same bits as the same handle
 * stepped alone with XFDTD_FLAG_SPLIT_EH.  After xfdtd_batch_synchronize
 * the members are read with the ordinary entry points (xfdtd_read_field,
 * xfdtd_read_nffft, xfdtd_far_field, ...); they must not be stepped on
 * their own while in a batch. */
typedef struct xfdtd_batch xfdtd_batch;

int xfdtd_batch_create(xfdtd_handle *const *members, int n, int flags, xfdtd_batch **out);
/* Advances every member that has steps left by up to n steps (asynchronous). */
int xfdtd_batch_step(xfdtd_batch *b, int64_t n);
/* The same, returning the device time of the n steps (CUDA events). */
int xfdtd_batch_step_timed(xfdtd_batch *b, int64_t n, double *ms);
int xfdtd_batch_synchronize(xfdtd_batch *b);
/* Members with steps left, batch steps taken, kernel launches enqueued. */
int xfdtd_batch_status(xfdtd_batch *b, int *n_running, int64_t *clock, int64_t *launches);
/* Members whose volume phases run on the TMA-staged launches of the wide
 * decomposition (every member whose grid gives those launches aligned
 * tiles, unless the batch was made with XFDTD_FLAG_PLAIN_VOLUME); the
 * others run the one-thread-per-cell kernels.  No counterpart in the
 * reference. */
int xfdtd_batch_tma_members(xfdtd_batch *b, int *n);
const char *xfdtd_batch_last_error(xfdtd_batch *b);
void xfdtd_batch_destroy(xfdtd_batch *b);

/* ---------------------------------------------------------------------
 * Allocation-free NF-FF running DFT.  No counterpart in the reference: it
 * is NffftFd::update (nffft_fd.cpp:108-203) as a stand-alone operator on
 * caller-owned device arrays for callers that may not allocate device
 * memory during a run (runtimes that own every device allocation,
 * fixed-memory solvers).  The sample batch lives in a static 64 MiB device
 * array (xfdtd_nffft_noalloc_max_bytes()); the functions make no device
 * allocation and call no allocating library.
 *
 * Call xfdtd_nffft_noalloc_setup(device) once per device before the first
 * operator call and before any stream capture begins: it looks up the
 * scratch address and leaves `device` current; an operator call before it
 * returns XFDTD_ERR_STATE.  Each operator call makes op->device current for
 * its launches only and puts the caller's current device back before it
 * returns.  It samples step `step` (fields as they stand after that step's
 * H update) into slot step % batch and, if fold_count > 0, folds steps
 * step-fold_count+1 .. step into acc[].  Those steps must have been
 * sampled through this operator on this device, one call per step in an
 * unbroken run, with the same batch, box and precision: a call that
 * changes any of them, or skips a step, starts a new run, and a fold that
 * reaches back before its run's first step is rejected with
 * XFDTD_ERR_INVALID_PLAN.  The accumulators must start at zero.  The
 * scratch is one array shared by all calls on a device, resident on every
 * device that loads this library: calls that overlap in time on a device
 * race on it, so callers serialise them.  A batch larger than the scratch
 * (batch * 24 * largest face * element size), a grid axis above 2^30
 * cells or a box edge above 524,280 cells is rejected with
 * XFDTD_ERR_INVALID_PLAN before any device call.  Launches are asynchronous
 * on `stream`; errors: xfdtd_nffft_noalloc_last_error(). */
typedef struct xfdtd_nffft_operator {
  int32_t precision;        /* XFDTD_FP64 or XFDTD_FP32: element type of fields */
  int32_t device;           /* CUDA device ordinal the pointers live on         */
  int64_t nx, ny, nz;       /* cells per axis                                   */
  const void *fields[6];    /* Ex Ey Ez Hx Hy Hz, reference component shapes,
                               k contiguous (Ex (nx,ny+1,nz+1) ... Hz (nx,ny,nz+1)) */
  int64_t lo[3], hi[3];     /* NF-FF box: cells [lo, hi) per axis, lo >= 1      */
  int32_t n_freq;
  int32_t batch;            /* sample slots (1..), fold_count <= batch          */
  int64_t total_steps;      /* length of the phase tables                        */
  int64_t step;             /* step being sampled, 0 <= step < total_steps       */
  int32_t fold_count;       /* steps to fold after sampling (0 = none)          */
  int32_t reserved;
  const double *phase_j;    /* [n_freq][total_steps] (re, im): dt e^{-j w (t+1/2) dt} */
  const double *phase_m;    /* [n_freq][total_steps] (re, im): dt e^{-j w t dt}       */
  double *acc[24];          /* [n_freq][a][b] (re, im), layout of xfdtd_read_nffft;
                               16-byte aligned, like the phase tables       */
  void *stream;             /* cudaStream_t (NULL: legacy default stream)       */
} xfdtd_nffft_operator;

int xfdtd_nffft_noalloc_setup(int device);
int xfdtd_nffft_dft_noalloc(const xfdtd_nffft_operator *op);
int64_t xfdtd_nffft_noalloc_max_bytes(void);
const char *xfdtd_nffft_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* XFDTD_CUDA_H_ */
