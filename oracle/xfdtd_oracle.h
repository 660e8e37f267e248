/*
 * xfdtd_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement, in plain C++17 FP64, of the reference XFDTD time-stepping
 * path (Mrwatermolen/XFDTD).  It is the oracle the GPU engine is compared
 * with; nothing in the product links or calls it.  Only the tests, the smoke
 * check and the benchmark's CPU-baseline leg load it.
 *
 * Parity status: the reference itself cannot be compiled here (it needs
 * xtensor, xtensor-blas, xtensor-fftw, FFTW3, BLAS and LAPACK, none of which
 * is installed), and its own test suite holds no golden vectors for this path
 * (its one assertion test, test/test_grid.cpp, checks grid counts and sizes).
 * The restatement is pinned against that grid test, against analytic facts
 * (TFSF leakage, CPML reflection, Mie-series RCS of a PEC sphere within the
 * ~1 dB the reference's readme reports), and otherwise follows the reference
 * line by line, citing file:line in xfdtd_oracle.cpp.
 */
#ifndef XFDTD_ORACLE_H_
#define XFDTD_ORACLE_H_

#include <stdint.h>

#include "../include/xfdtd_scene.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_sim oracle_sim;

/* Builds the scene exactly as Simulation::init does
 * (src/simulation/simulation_init.cpp:10-22).  0 on success. */
int oracle_sim_create(const xfdtd_scene_desc *scene, int64_t total_steps, oracle_sim **out);
/* Runs n iterations of the loop body of Simulation::run
 * (src/simulation/simulation_update.cpp:9-36). */
int oracle_sim_step(oracle_sim *sim, int64_t n);
/* Grid cells per axis (CPML included), dt and the current step. */
int oracle_sim_info(oracle_sim *sim, int64_t out_n[3], double *out_dt, int64_t *out_step);
/* Copies a field component in the reference's own shape (XFDTD_EX..HZ):
 * Ex (nx,ny+1,nz+1), Ey (nx+1,ny,nz+1), Ez (nx+1,ny+1,nz),
 * Hx (nx+1,ny,nz), Hy (nx,ny+1,nz), Hz (nx,ny,nz+1). */
int oracle_sim_read_field(oracle_sim *sim, int comp, double *out, int64_t len);
/* Overwrites a field component (same shapes); for single-step tests. */
int oracle_sim_write_field(oracle_sim *sim, int comp, const double *in, int64_t len);
/* Monitor time series [total_steps]. */
int oracle_sim_read_monitor(oracle_sim *sim, int index, double *out, int64_t len);
/* A field monitor (TimeDomainFieldMonitor, or a MovieMonitor over one,
 * src/monitor/field_monitor.cpp, movie_monitor.cpp): its view of the
 * component (lo, shape), its frames so far and their steps (a plain field
 * monitor: one frame, the current field, step -1). */
int oracle_sim_field_monitor(oracle_sim *sim, int index, int64_t lo[3], int64_t shape[3], int64_t *n_frames,
                             int64_t *steps, int64_t max);
int oracle_sim_read_field_monitor(oracle_sim *sim, int index, int64_t frame, double *out, int64_t len);
/* NF-FF running-DFT accumulators, complex as (re, im) pairs.  which = face*4+q,
 * faces XN,XP,YN,YP,ZN,ZP; q: X faces jy,jz,my,mz; Y faces jz,jx,mz,mx;
 * Z faces jx,jy,mx,my (nffft_fd.cpp:117-203). */
int oracle_sim_read_nffft(oracle_sim *sim, int which, double *out, int64_t len);
/* Far field (NffftFd::calculateFarfield, nffft_fd.cpp:379-421).  which:
 * 0 e_theta, 1 e_phi, 2 h_theta, 3 h_phi, 4 n_theta, 5 n_phi, 6 l_theta,
 * 7 l_phi (complex [nf][nt][np]); 8 power_theta, 9 power_phi (real). */
int oracle_sim_far_field(oracle_sim *sim, int which, double *out, int64_t len);
/* dt * sum_t e0*w[t] exp(-i 2 pi f t dt)  (util/dft.h:11-27 over the TFSF
 * waveform samples), complex pairs. */
int oracle_sim_incident_dft(oracle_sim *sim, const double *freqs, int n, double *out);
/* Update coefficient arrays after CPML init, in the component shapes.
 * which: 0 cexe 1 cexhy 2 cexhz 3 ceye 4 ceyhz 5 ceyhx 6 ceze 7 cezhx 8 cezhy
 *        9 chxh 10 chxey 11 chxez 12 chyh 13 chyez 14 chyex 15 chzh 16 chzex 17 chzey */
int oracle_sim_read_coeff(oracle_sim *sim, int which, double *out, int64_t len);
/* OpenMP threads for the volume loops (results do not depend on it). */
int oracle_set_threads(int n);
const char *oracle_last_error(void);
void oracle_sim_destroy(oracle_sim *sim);

/* Reference test/test_grid.cpp, restated: builds a GridSpace from one cube
 * and reports nx,ny,nz and the node-size arrays.  out_sizes receives
 * e_size_x[nx], e_size_y[ny], e_size_z[nz], h_size_x[nx+1], h_size_y[ny+1],
 * h_size_z[nz+1] back to back. */
int oracle_grid_from_cube(const double point[3], const double size[3], double dl,
                          int64_t out_n[3], double *out_sizes, int64_t len);

#ifdef __cplusplus
}
#endif

#endif /* XFDTD_ORACLE_H_ */
