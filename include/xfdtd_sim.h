/*
 * xfdtd_sim.h -- scene-level C-ABI of libxfdtd.so (the C++ Simulation API
 * behind plain C entry points), for callers in other languages.
 *
 * The reference has no FFI; a binding of its C++ API would construct
 * Object / PML / TFSF3D / NffftFd / lumped elements / monitors and call
 * Simulation::run (src/simulation/simulation_update.cpp:5-40).  These entry
 * points do exactly that from an xfdtd_scene_desc (xfdtd_scene.h) and then
 * expose what the reference writes at the end of a run: field snapshots
 * (EMF getters), monitor time series (Monitor::outputData), the NF-FF
 * accumulators and far field (NffftFd::outputData) and the incident-wave
 * DFT (TFSF::getIncidentWaveFourierTransform, src/tfsf/tfsf.cpp:63-66).
 *
 * Status codes are those of xfdtd_cuda.h; setup errors the reference throws
 * as std::runtime_error / std::out_of_range come back as
 * XFDTD_ERR_INVALID_PLAN with the message in xfdtd_sim_last_error().
 */
#ifndef XFDTD_SIM_H_
#define XFDTD_SIM_H_

#include <stdint.h>

#include "xfdtd_cuda.h"
#include "xfdtd_scene.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xfdtd_sim xfdtd_sim;

/* Bits 8..15 of the flags of xfdtd_sim_create carry the CUDA device ordinal. */
#define XFDTD_SIM_DEVICE_SHIFT 8

/* Builds the Simulation and its engine plan for total_steps steps.
 * precision: XFDTD_FP64 or XFDTD_FP32; flags: XFDTD_FLAG_* |
 * (device << XFDTD_SIM_DEVICE_SHIFT).  On failure *out is still set (when
 * non-null) so that xfdtd_sim_last_error can be read; it must then be
 * destroyed. */
int xfdtd_sim_create(const xfdtd_scene_desc *scene, int64_t total_steps, int precision, int flags, xfdtd_sim **out);
int xfdtd_sim_step(xfdtd_sim *s, int64_t n);
int xfdtd_sim_info(xfdtd_sim *s, int64_t out_n[3], double *out_dt, int64_t *out_step);
int xfdtd_sim_read_field(xfdtd_sim *s, int comp, double *out, int64_t len);
int xfdtd_sim_write_field(xfdtd_sim *s, int comp, const double *in, int64_t len);
int xfdtd_sim_read_monitor(xfdtd_sim *s, int index, double *out, int64_t len);
/* A field monitor (TimeDomainFieldMonitor, or a MovieMonitor over one):
 * its box (first index lo and shape, in the component's array), its number
 * of frames and their steps (steps[f] for f < min(max, n_frames); may be
 * null).  A plain field monitor has one frame,
 * the current field, step -1; a movie monitor's frames are those of
 * MovieMonitor::update (src/monitor/movie_monitor.cpp:46-59). */
int xfdtd_sim_field_monitor(xfdtd_sim *s, int index, int64_t lo[3], int64_t shape[3], int64_t *n_frames,
                            int64_t *steps, int64_t max);
/* Frame `frame` of field monitor `index`, [n0][n1][n2]. */
int xfdtd_sim_read_field_monitor(xfdtd_sim *s, int index, int64_t frame, double *out, int64_t len);
int xfdtd_sim_read_nffft(xfdtd_sim *s, int which, double *out, int64_t len);
/* Far field: for an NffftFd over (n_freq, n_theta, n_phi), which 0 e_theta
 * 1 e_phi 2 h_theta 3 h_phi 4 n_theta 5 n_phi 6 l_theta 7 l_phi (complex
 * pairs), 8 power_theta 9 power_phi (real).  For an NffftBroadBand the same
 * arrays over its N = 2*total_steps - 1 bins, and 10 the bins' frequencies
 * (NffftBroadBand::calculateFarField, src/nffft/nffft_broadband.cpp:343-371). */
int xfdtd_sim_far_field(xfdtd_sim *s, int which, double *out, int64_t len);
int xfdtd_sim_incident_dft(xfdtd_sim *s, const double *freqs, int n, double *out);
/* Output directory (and file name) of monitor `index`; with index -1 the
 * NF-FF's output directory, with -2 the network's output path: the
 * constructors' output_dir_path / output_file_name / output_path
 * arguments, which the scene description does not carry.  An empty
 * directory writes nothing. */
int xfdtd_sim_set_output(xfdtd_sim *s, int index, const char *dir, const char *file);
/* The network's S-parameters (Network::outputData's arithmetic,
 * src/network/network.cpp:40-52) from the monitor series recorded so far:
 * their keys (10 * j + i for port indices j and activated i, ascending;
 * keys[q] for q < min(max, count)) and the number of frequencies. */
int xfdtd_sim_s_parameters(xfdtd_sim *s, int32_t *keys, int64_t max, int64_t *count, int64_t *n_freq);
/* S-parameter `key` over the network's frequencies, (re, im) pairs. */
int xfdtd_sim_read_s_parameter(xfdtd_sim *s, int key, double *out, int64_t len);
/* Writes the reference's .npy outputs (NF-FF into its output directory,
 * monitors and the network into theirs). */
int xfdtd_sim_output(xfdtd_sim *s);
/* The engine handle behind the simulation (for timing and profiling). */
xfdtd_handle *xfdtd_sim_engine(xfdtd_sim *s);
const char *xfdtd_sim_last_error(xfdtd_sim *s);
void xfdtd_sim_destroy(xfdtd_sim *s);

#ifdef __cplusplus
}
#endif

#endif /* XFDTD_SIM_H_ */
