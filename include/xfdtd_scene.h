/*
 * xfdtd_scene.h -- plain-C description of an XFDTD scene.
 *
 * This is the data a caller hands to the scene-level C-ABI (xfdtd_sim_*,
 * declared in xfdtd_sim.h).  It carries exactly what the reference's C++
 * constructors take, field for field, so that a foreign-language binding can
 * build the same simulation the reference builds from C++:
 *
 *   Object(name, Shape, Material)          src/include/object/object.h:17-20
 *   Sphere / Cube / Cylinder               src/include/shape/{sphere,cube,cylinder}.h
 *   Material(name, float eps_r, float mu_r, sigma_e, sigma_m)
 *                                          src/include/material/material.h:16-17
 *   ThinWire(name, Cylinder)               src/include/object/thin_wire.h
 *   PML(Orientation, thickness, order=4, sigma_ratio=1, alpha_min=0,
 *       alpha_max=0.05, kappa_max=10)      src/include/boundary/perfect_match_layer.h:33-35
 *   TFSF3D(dx, dy, dz, e0, theta, phi, psi, Waveform)
 *                                          src/include/tfsf/tfsf_3d.h:10-12
 *   NffftFd(dx, dy, dz, frequencies, theta, phi, path)
 *                                          src/include/nffft/nffft_fd.h:39-50
 *   CurrentSource / VoltageSource(Cube, Orientation, R, Waveform),
 *   Resistor / Capacitor / Inductor(Cube, Axis, value)
 *                                          src/include/lumped_element/ (all)
 *   VoltageMonitor / CurrentMonitor(Cube, Orientation, dir, file)
 *                                          src/include/monitor/ (all)
 *   Simulation(cell_size, ..., float cfl)  src/include/simulation/simulation.h:27-66
 *
 * One addition has no reference counterpart: a voxel material raster
 * (`voxel_*`), for heterogeneous media with one material per cell.  Its
 * meaning is that of one 1-cell Cube Object per voxel, appended after all
 * other objects in raster order (last writer wins, as in Object::init,
 * src/object/object.cpp:53-73).
 *
 * All arrays are borrowed for the duration of the call that receives the
 * description; nothing is retained.
 */
#ifndef XFDTD_SCENE_H_
#define XFDTD_SCENE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Orientation, src/include/util/type_define.h:15 (same order). */
enum { XFDTD_XN = 0, XFDTD_XP = 1, XFDTD_YN = 2, XFDTD_YP = 3, XFDTD_ZN = 4, XFDTD_ZP = 5 };
/* Axis, src/include/util/type_define.h:16 (same order). */
enum { XFDTD_AXIS_X = 0, XFDTD_AXIS_Y = 1, XFDTD_AXIS_Z = 2 };

enum { XFDTD_SHAPE_CUBE = 0, XFDTD_SHAPE_SPHERE = 1, XFDTD_SHAPE_CYLINDER = 2 };
enum { XFDTD_OBJECT_PLAIN = 0, XFDTD_OBJECT_THIN_WIRE = 1 };
enum {
  XFDTD_WAVE_GAUSSIAN = 0,       /* GaussianWaveform(amplitude, tau, t0)            */
  XFDTD_WAVE_COS_GAUSSIAN = 1,   /* CosineModulatedGaussianWaveform(A, tau, t0, f)  */
  XFDTD_WAVE_SINUSOIDAL = 2,     /* SinusoidalWaveform(A, f, phase)                 */
  XFDTD_WAVE_CUSTOM = 3          /* CustomWaveform(A, std::function<double(double)>) */
};
enum {
  XFDTD_LUMPED_CURRENT_SOURCE = 0,
  XFDTD_LUMPED_VOLTAGE_SOURCE = 1,
  XFDTD_LUMPED_RESISTOR = 2,
  XFDTD_LUMPED_CAPACITOR = 3,
  XFDTD_LUMPED_INDUCTOR = 4
};
enum { XFDTD_MONITOR_VOLTAGE = 0, XFDTD_MONITOR_CURRENT = 1, XFDTD_MONITOR_FIELD = 2 };

/* Field components in the order of EMF's getters. */
enum { XFDTD_EX = 0, XFDTD_EY = 1, XFDTD_EZ = 2, XFDTD_HX = 3, XFDTD_HY = 4, XFDTD_HZ = 5 };

typedef struct xfdtd_shape_desc {
  int32_t kind;      /* XFDTD_SHAPE_*                                   */
  int32_t axis;      /* cylinder axis (XFDTD_AXIS_*)                     */
  double point[3];   /* cube: corner; sphere / cylinder: centre          */
  double size[3];    /* cube: edge lengths                               */
  double radius;     /* sphere / cylinder                                */
  double height;     /* cylinder                                         */
} xfdtd_shape_desc;

/* dispersion: 0 for a plain Material.  The reference's linear dispersive
 * media (src/include/material/dispersive_material.h) take their E update
 * from the auxiliary-differential-equation recursions of their
 * updateEx/Ey/Ez (src/material/dispersive_material.cpp), with eps_r = mu_r
 * = 1 and the conductivities in sigma_e, sigma_m:
 *   1 LorentzMedium(eps_s, eps_inf, omega_p, nv)  p = {eps_s, eps_inf, omega_p, nv}
 *   2 DrudeMedium(eps_inf, omega_p, nv)           p = {eps_inf, omega_p, nv, 0}
 *   3 DebyMedium(eps_s, eps_inf, tau)             p = {eps_s, eps_inf, tau, 0}
 * The reference throws on them at Object::init (object.cpp:109-110); here
 * they run, as objects outside the CPML. */
enum {
  XFDTD_DISPERSION_NONE = 0,
  XFDTD_DISPERSION_LORENTZ = 1,
  XFDTD_DISPERSION_DRUDE = 2,
  XFDTD_DISPERSION_DEBYE = 3
};

/* xfdtd_material_desc.flags: eps_r exact.  A plain (non-dispersive)
 * material whose relative permittivity is p[0] in double, not the float
 * eps_r field (the reference's Material ctor takes eps_r as float).  For a
 * gradient check by finite differences, whose step (1e-4) a float eps_r
 * would round away.  No counterpart in the reference. */
#define XFDTD_MATERIAL_EXACT_EPS 1

typedef struct xfdtd_material_desc {
  float eps_r;       /* float, as in the reference's Material ctor       */
  float mu_r;
  double sigma_e;    /* S/m; a PEC is sigma_e = 1e10                     */
  double sigma_m;
  int32_t dispersion;   /* XFDTD_DISPERSION_*                            */
  int32_t flags;        /* XFDTD_MATERIAL_EXACT_EPS or 0                 */
  double p[4];          /* the dispersive medium's parameters (above);   */
                        /* p[0] = eps_r with XFDTD_MATERIAL_EXACT_EPS    */
} xfdtd_material_desc;

typedef struct xfdtd_object_desc {
  int32_t kind;      /* XFDTD_OBJECT_*; a thin wire needs a cylinder     */
  int32_t reserved;
  xfdtd_shape_desc shape;
  xfdtd_material_desc material;
} xfdtd_object_desc;

/* A custom waveform is sampled on the host through this callback. */
typedef double (*xfdtd_waveform_fn)(double t, void *ctx);

typedef struct xfdtd_waveform_desc {
  int32_t kind;      /* XFDTD_WAVE_*                                     */
  int32_t reserved;
  double amplitude;
  double tau;
  double t0;
  double frequency;  /* modulation / sinusoid frequency                  */
  double phase;
  xfdtd_waveform_fn fn;  /* XFDTD_WAVE_CUSTOM only                       */
  void *ctx;
} xfdtd_waveform_desc;

typedef struct xfdtd_pml_desc {
  int32_t orientation;  /* XFDTD_XN .. XFDTD_ZP                          */
  int32_t thickness;    /* cells                                         */
  int32_t order;        /* default 4                                     */
  int32_t reserved;
  double sigma_ratio;   /* default 1                                     */
  double alpha_min;     /* default 0                                     */
  double alpha_max;     /* default 0.05                                  */
  double kappa_max;     /* default 10                                    */
} xfdtd_pml_desc;

/* enabled: 1 TFSF3D(distance x, y, z, e0, theta, phi, psi, waveform);
 * 2 TFSF2D(distance x, y, phi, e0, waveform) (src/include/tfsf/tfsf_2d.h:8-10)
 * on a 2-D grid (nz = 1): theta = pi / 2, psi = 0, distance[2] = 0. */
typedef struct xfdtd_tfsf_desc {
  int32_t enabled;
  int32_t reserved;
  int64_t distance[3];  /* cells from the domain edge (CPML included)    */
  double e0;
  double theta;
  double phi;
  double psi;
  xfdtd_waveform_desc waveform;
} xfdtd_tfsf_desc;

/* enabled: 1 NffftFd(dx, dy, dz, frequencies, theta, phi, path); 2
 * NffftBroadBand(dx, dy, dz, theta[0], phi[0], path)
 * (src/include/nffft/nffft_broadband.h), frequencies unused. */
typedef struct xfdtd_nffft_desc {
  int32_t enabled;
  int32_t n_freq;
  int64_t distance[3];
  int32_t n_theta;
  int32_t n_phi;
  const double *frequencies;  /* [n_freq]  Hz      */
  const double *theta;        /* [n_theta] radians */
  const double *phi;          /* [n_phi]   radians */
} xfdtd_nffft_desc;

typedef struct xfdtd_lumped_desc {
  int32_t kind;         /* XFDTD_LUMPED_*                                 */
  int32_t orientation;  /* sources: XFDTD_XN..ZP; R/C/L: XFDTD_AXIS_*     */
  double value;         /* resistance (ohm), capacitance (F), inductance (H) */
  double point[3];      /* cube corner                                    */
  double size[3];       /* cube size                                      */
  xfdtd_waveform_desc waveform;  /* sources only                          */
} xfdtd_lumped_desc;

typedef struct xfdtd_monitor_desc {
  int32_t kind;         /* XFDTD_MONITOR_*                                */
  int32_t orientation;  /* XFDTD_XN .. XFDTD_ZP                           */
  double point[3];
  double size[3];
  /* XFDTD_MONITOR_FIELD: TimeDomainFieldMonitor(cube, plane_type,
   * component, ...) (src/include/monitor/field_monitor.h); with
   * plot_step > 0 wrapped in MovieMonitor(monitor, total_time_steps,
   * plot_step) (src/include/monitor/movie_monitor.h).                    */
  int32_t component;    /* EMComponent: 0 EX .. 5 HZ                       */
  int32_t plane_type;   /* PlaneType: 0 XY, 1 YZ, 2 ZX                     */
  int64_t plot_step;
  int64_t total_time_steps;
} xfdtd_monitor_desc;

/* Port(index, impedance, is_activated_source, voltage, current)
 * (src/include/network/port.h): its voltage and current monitors are
 * indices into the scene's monitor list. */
typedef struct xfdtd_port_desc {
  int32_t index;
  int32_t is_activated_source;
  double impedance_re, impedance_im;
  int32_t voltage_monitor;
  int32_t current_monitor;
} xfdtd_port_desc;

typedef struct xfdtd_scene_desc {
  double cell_size;     /* dx = dy = dz                                   */
  float cfl;            /* float, as in Simulation(..., float cfl)        */
  int32_t n_objects;
  const xfdtd_object_desc *objects;
  int32_t n_pml;
  int32_t n_lumped;
  const xfdtd_pml_desc *pml;
  const xfdtd_lumped_desc *lumped;
  int32_t n_monitors;
  int32_t n_voxel_materials;
  const xfdtd_monitor_desc *monitors;
  xfdtd_tfsf_desc tfsf;
  xfdtd_nffft_desc nffft;
  /* Optional voxel raster: [nx*ny*nz] material indices (row-major, z
   * fastest) into voxel_materials, applied after all objects.  The grid
   * size it must match is the one the objects and PML layers produce.    */
  const xfdtd_material_desc *voxel_materials;
  const void *voxel_index;      /* uint16_t, or uint32_t when voxel_index_bytes = 4 */
  int64_t voxel_shape[3];
  int32_t voxel_index_bytes;    /* 2 (or 0, meaning 2) or 4                      */
  int32_t reserved3;
  /* Optional Network(ports, frequencies, output_path)
   * (src/include/network/network.h): n_ports = 0 for none.              */
  int32_t n_ports;
  int32_t n_network_freqs;
  const xfdtd_port_desc *ports;
  const double *network_freqs;
} xfdtd_scene_desc;

#ifdef __cplusplus
}
#endif

#endif /* XFDTD_SCENE_H_ */
