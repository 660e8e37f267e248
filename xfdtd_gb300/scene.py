"""ctypes mirror of include/xfdtd_scene.h and Python classes that follow the
reference's C++ scene API (Mrwatermolen/XFDTD), so that a Python caller
composes a simulation the way the reference's examples do:

    objects = [Object("domain", Cube(...), Material("air", 1, 1, 0, 0)),
               Object("scatter", Sphere((0, 0, 0), r), Material.create_pec())]
    boundaries = [PML(XN, 8), PML(XP, 8), ...]
    tfsf = TFSF3D(12, 12, 12, 1.0, 0, 0, 0, GaussianWaveform(1, tau, t0))
    nffft = NffftFd(14, 14, 14, [1e9], theta, [0.0], "out")
    scene = Scene(dl, objects, boundaries, tfsf=tfsf, nffft=nffft, cfl=0.98)

Class names, constructor argument order and defaults are those of the
reference headers (cited per class).  `Scene.desc()` lowers the composition
to the plain-C `xfdtd_scene_desc` every scene-level entry point takes.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

# Orientation / Axis, src/include/util/type_define.h:15-16
XN, XP, YN, YP, ZN, ZP = range(6)
AXIS_X, AXIS_Y, AXIS_Z = range(3)
EX, EY, EZ, HX, HY, HZ = range(6)

SHAPE_CUBE, SHAPE_SPHERE, SHAPE_CYLINDER = range(3)
OBJECT_PLAIN, OBJECT_THIN_WIRE = range(2)
WAVE_GAUSSIAN, WAVE_COS_GAUSSIAN, WAVE_SINUSOIDAL, WAVE_CUSTOM = range(4)
LUMPED_CURRENT_SOURCE, LUMPED_VOLTAGE_SOURCE, LUMPED_RESISTOR, LUMPED_CAPACITOR, LUMPED_INDUCTOR = range(5)
MONITOR_VOLTAGE, MONITOR_CURRENT, MONITOR_FIELD = range(3)

# src/include/util/constant.h:10-29
PI = math.pi
EPSILON_0 = 8.854187817e-12
MU_0 = 4 * PI * 1e-7
C_0 = math.sqrt(1 / (EPSILON_0 * MU_0))
ETA_0 = math.sqrt(MU_0 / EPSILON_0)


# ------------------------------------------------------------ C structs ---
class ShapeDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("axis", C.c_int32), ("point", C.c_double * 3),
                ("size", C.c_double * 3), ("radius", C.c_double), ("height", C.c_double)]


class MaterialDesc(C.Structure):
    _fields_ = [("eps_r", C.c_float), ("mu_r", C.c_float), ("sigma_e", C.c_double),
                ("sigma_m", C.c_double), ("dispersion", C.c_int32), ("flags", C.c_int32),
                ("p", C.c_double * 4)]


MATERIAL_EXACT_EPS = 1


DISPERSION_NONE, DISPERSION_LORENTZ, DISPERSION_DRUDE, DISPERSION_DEBYE = 0, 1, 2, 3


class ObjectDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("shape", ShapeDesc),
                ("material", MaterialDesc)]


WAVEFORM_FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)


class WaveformDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("amplitude", C.c_double),
                ("tau", C.c_double), ("t0", C.c_double), ("frequency", C.c_double),
                ("phase", C.c_double), ("fn", WAVEFORM_FN), ("ctx", C.c_void_p)]


class PMLDesc(C.Structure):
    _fields_ = [("orientation", C.c_int32), ("thickness", C.c_int32), ("order", C.c_int32),
                ("reserved", C.c_int32), ("sigma_ratio", C.c_double), ("alpha_min", C.c_double),
                ("alpha_max", C.c_double), ("kappa_max", C.c_double)]


class TFSFDesc(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("reserved", C.c_int32), ("distance", C.c_int64 * 3),
                ("e0", C.c_double), ("theta", C.c_double), ("phi", C.c_double),
                ("psi", C.c_double), ("waveform", WaveformDesc)]


class NFFFTDesc(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("n_freq", C.c_int32), ("distance", C.c_int64 * 3),
                ("n_theta", C.c_int32), ("n_phi", C.c_int32),
                ("frequencies", C.POINTER(C.c_double)), ("theta", C.POINTER(C.c_double)),
                ("phi", C.POINTER(C.c_double))]


class LumpedDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("orientation", C.c_int32), ("value", C.c_double),
                ("point", C.c_double * 3), ("size", C.c_double * 3), ("waveform", WaveformDesc)]


class MonitorDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("orientation", C.c_int32), ("point", C.c_double * 3),
                ("size", C.c_double * 3), ("component", C.c_int32), ("plane_type", C.c_int32),
                ("plot_step", C.c_int64), ("total_time_steps", C.c_int64)]


class PortDesc(C.Structure):
    _fields_ = [("index", C.c_int32), ("is_activated_source", C.c_int32), ("impedance_re", C.c_double),
                ("impedance_im", C.c_double), ("voltage_monitor", C.c_int32), ("current_monitor", C.c_int32)]


class SceneDesc(C.Structure):
    _fields_ = [("cell_size", C.c_double), ("cfl", C.c_float),
                ("n_objects", C.c_int32), ("objects", C.POINTER(ObjectDesc)),
                ("n_pml", C.c_int32), ("n_lumped", C.c_int32),
                ("pml", C.POINTER(PMLDesc)), ("lumped", C.POINTER(LumpedDesc)),
                ("n_monitors", C.c_int32), ("n_voxel_materials", C.c_int32),
                ("monitors", C.POINTER(MonitorDesc)),
                ("tfsf", TFSFDesc), ("nffft", NFFFTDesc),
                ("voxel_materials", C.POINTER(MaterialDesc)),
                ("voxel_index", C.c_void_p),
                ("voxel_shape", C.c_int64 * 3),
                ("voxel_index_bytes", C.c_int32), ("reserved3", C.c_int32),
                ("n_ports", C.c_int32), ("n_network_freqs", C.c_int32),
                ("ports", C.POINTER(PortDesc)), ("network_freqs", C.POINTER(C.c_double))]


# ---------------------------------------------------------------- shapes ---
@dataclass
class Cube:
    """Cube(point, size), src/include/shape/cube.h."""
    point: Sequence[float]
    size: Sequence[float]

    def desc(self) -> ShapeDesc:
        d = ShapeDesc()
        d.kind = SHAPE_CUBE
        d.point[:] = list(map(float, self.point))
        d.size[:] = list(map(float, self.size))
        return d


@dataclass
class Sphere:
    """Sphere(center, radius), src/include/shape/sphere.h."""
    center: Sequence[float]
    radius: float

    def desc(self) -> ShapeDesc:
        d = ShapeDesc()
        d.kind = SHAPE_SPHERE
        d.point[:] = list(map(float, self.center))
        d.radius = float(self.radius)
        return d


@dataclass
class Cylinder:
    """Cylinder(axis, center, radius, height), src/include/shape/cylinder.h."""
    axis: int
    center: Sequence[float]
    radius: float
    height: float

    def desc(self) -> ShapeDesc:
        d = ShapeDesc()
        d.kind = SHAPE_CYLINDER
        d.axis = int(self.axis)
        d.point[:] = list(map(float, self.center))
        d.radius = float(self.radius)
        d.height = float(self.height)
        return d


@dataclass
class Material:
    """Material(name, float eps_r, float mu_r, sigma_e, sigma_m),
    src/include/material/material.h:16-17 (eps_r and mu_r are float there)."""
    name: str
    eps_r: float
    mu_r: float
    sigma_e: float
    sigma_m: float
    # keep eps_r in double (XFDTD_MATERIAL_EXACT_EPS; the reference's ctor
    # takes it as float): for finite-difference gradient checks
    exact_eps: bool = False

    @staticmethod
    def create_air(name: str = "XFDTD_AIR") -> "Material":  # material.cpp:28-30
        return Material(name, 1, 1, 0, 0)

    @staticmethod
    def create_pec() -> "Material":  # material.cpp:32-34
        return Material("XFDTD_PEC", 1, 1, 1e10, 0)

    def desc(self) -> MaterialDesc:
        d = MaterialDesc()
        d.eps_r, d.mu_r = float(self.eps_r), float(self.mu_r)
        d.sigma_e, d.sigma_m = float(self.sigma_e), float(self.sigma_m)
        if self.exact_eps:
            d.flags = MATERIAL_EXACT_EPS
            d.p[0] = float(self.eps_r)
        return d


class LorentzMedium(Material):
    """LorentzMedium(name, eps_s, eps_inf, omega_p, nv, sigma_e=0, sigma_m=0),
    src/include/material/dispersive_material.h:58-73: a Lorentz pole pair of
    strength eps_s - eps_inf at omega_p, damping nv; eps_r = mu_r = 1."""

    def __init__(self, name, eps_s, eps_inf, omega_p, nv, sigma_e=0.0, sigma_m=0.0):
        super().__init__(name, 1, 1, sigma_e, sigma_m)
        self.kind, self.params = DISPERSION_LORENTZ, (eps_s, eps_inf, omega_p, nv)

    def desc(self) -> MaterialDesc:
        d = super().desc()
        d.dispersion = self.kind
        d.p[:] = [float(v) for v in self.params]
        return d


class DrudeMedium(LorentzMedium):
    """DrudeMedium(name, eps_inf, omega_p, nv, sigma_e=0, sigma_m=0),
    dispersive_material.h:106-118."""

    def __init__(self, name, eps_inf, omega_p, nv, sigma_e=0.0, sigma_m=0.0):
        Material.__init__(self, name, 1, 1, sigma_e, sigma_m)
        self.kind, self.params = DISPERSION_DRUDE, (eps_inf, omega_p, nv, 0.0)


class DebyMedium(LorentzMedium):
    """DebyMedium(name, eps_s, eps_inf, tau, sigma_e=0, sigma_m=0),
    dispersive_material.h:138-141 (the reference's spelling)."""

    def __init__(self, name, eps_s, eps_inf, tau, sigma_e=0.0, sigma_m=0.0):
        Material.__init__(self, name, 1, 1, sigma_e, sigma_m)
        self.kind, self.params = DISPERSION_DEBYE, (eps_s, eps_inf, tau, 0.0)


@dataclass
class Object:
    """Object(name, shape, material), src/include/object/object.h:17-20."""
    name: str
    shape: object
    material: Material

    def desc(self) -> ObjectDesc:
        d = ObjectDesc()
        d.kind = OBJECT_PLAIN
        d.shape = self.shape.desc()
        d.material = self.material.desc()
        return d


@dataclass
class ThinWire:
    """ThinWire(name, Cylinder), src/include/object/thin_wire.h."""
    name: str
    shape: Cylinder

    def desc(self) -> ObjectDesc:
        d = ObjectDesc()
        d.kind = OBJECT_THIN_WIRE
        d.shape = self.shape.desc()
        d.material = Material.create_air("placeholder_wire").desc()
        return d


@dataclass
class PML:
    """PML(orientation, thickness, order=4, sigma_ratio=1, alpha_min=0,
    alpha_max=0.05, kappa_max=10), src/include/boundary/perfect_match_layer.h:33-35."""
    orientation: int
    thickness: int
    order: int = 4
    sigma_ratio: float = 1.0
    alpha_min: float = 0.0
    alpha_max: float = 0.05
    kappa_max: float = 10.0

    def desc(self) -> PMLDesc:
        d = PMLDesc()
        d.orientation, d.thickness, d.order = int(self.orientation), int(self.thickness), int(self.order)
        d.sigma_ratio, d.alpha_min = float(self.sigma_ratio), float(self.alpha_min)
        d.alpha_max, d.kappa_max = float(self.alpha_max), float(self.kappa_max)
        return d


# -------------------------------------------------------------- waveforms ---
class Waveform:
    kind = -1

    def desc(self) -> WaveformDesc:
        raise NotImplementedError

    def value_by_time(self, t: np.ndarray) -> np.ndarray:
        raise NotImplementedError


class GaussianWaveform(Waveform):
    """GaussianWaveform(amplitude, tau, t_0) or (tau, t_0),
    src/waveform/gaussian_waveform.cpp:18-24: A*exp(-((t-t0)/tau)^2)."""
    kind = WAVE_GAUSSIAN

    def __init__(self, *args):
        if len(args) == 2:
            self.amplitude, (self.tau, self.t0) = 1.0, args
        else:
            self.amplitude, self.tau, self.t0 = args

    def desc(self) -> WaveformDesc:
        d = WaveformDesc()
        d.kind, d.amplitude, d.tau, d.t0 = self.kind, self.amplitude, self.tau, self.t0
        return d

    def value_by_time(self, t):
        return self.amplitude * np.exp(-(((np.asarray(t) - self.t0) / self.tau) ** 2))


class CosineModulatedGaussianWaveform(Waveform):
    """(amplitude, tau, t_0, f) or (tau, t_0, f),
    src/waveform/cosine_modulated_gaussian_waveform.cpp:24-35."""
    kind = WAVE_COS_GAUSSIAN

    def __init__(self, *args):
        if len(args) == 3:
            self.amplitude, (self.tau, self.t0, self.frequency) = 1.0, args
        else:
            self.amplitude, self.tau, self.t0, self.frequency = args

    def desc(self) -> WaveformDesc:
        d = WaveformDesc()
        d.kind, d.amplitude, d.tau, d.t0, d.frequency = (self.kind, self.amplitude, self.tau,
                                                         self.t0, self.frequency)
        return d

    def value_by_time(self, t):
        t = np.asarray(t)
        return (self.amplitude * np.cos(2 * PI * self.frequency * (t - self.t0))
                * np.exp(-(((t - self.t0) / self.tau) ** 2)))


class SinusoidalWaveform(Waveform):
    """(amplitude, frequency, phase) or (frequency, phase), src/waveform/sinusoidal_waveform.cpp."""
    kind = WAVE_SINUSOIDAL

    def __init__(self, *args):
        if len(args) == 2:
            self.amplitude, (self.frequency, self.phase) = 1.0, args
        else:
            self.amplitude, self.frequency, self.phase = args

    def desc(self) -> WaveformDesc:
        d = WaveformDesc()
        d.kind, d.amplitude, d.frequency, d.phase = self.kind, self.amplitude, self.frequency, self.phase
        return d

    def value_by_time(self, t):
        return self.amplitude * np.sin(2 * PI * self.frequency * np.asarray(t) + self.phase)


class CustomWaveform(Waveform):
    """CustomWaveform(amplitude, f), src/waveform/custom_waveform.cpp:13-23.
    `f` is sampled on the host through a C callback."""
    kind = WAVE_CUSTOM

    def __init__(self, amplitude: float, f: Callable[[float], float]):
        self.amplitude = float(amplitude)
        self.f = f
        self._cb = WAVEFORM_FN(lambda t, ctx: float(self.f(t)))

    def desc(self) -> WaveformDesc:
        d = WaveformDesc()
        d.kind, d.amplitude = self.kind, self.amplitude
        d.fn = self._cb
        return d

    def value_by_time(self, t):
        return self.amplitude * np.vectorize(self.f)(np.asarray(t, dtype=float))


def gaussian_modulated_sine(f0: float, tau: float, t0: float) -> Callable[[float], float]:
    """sin(2 pi f0 (t - t0)) * exp(-((t - t0)/tau)^2), used through CustomWaveform."""
    def f(t: float) -> float:
        return math.sin(2 * PI * f0 * (t - t0)) * math.exp(-(((t - t0) / tau) ** 2))
    return f


# --------------------------------------------------- TFSF / NF-FF / lumped ---
@dataclass
class TFSF3D:
    """TFSF3D(distance_x, distance_y, distance_z, e_0, theta, phi, psi, waveform),
    src/include/tfsf/tfsf_3d.h:10-12."""
    distance_x: int
    distance_y: int
    distance_z: int
    e_0: float
    theta: float
    phi: float
    psi: float
    waveform: Waveform

    def desc(self) -> TFSFDesc:
        d = TFSFDesc()
        d.enabled = 1
        d.distance[:] = [int(self.distance_x), int(self.distance_y), int(self.distance_z)]
        d.e0, d.theta, d.phi, d.psi = float(self.e_0), float(self.theta), float(self.phi), float(self.psi)
        d.waveform = self.waveform.desc()
        return d


@dataclass
class TFSF2D:
    """TFSF2D(distance_x, distance_y, phi_inc, ez_i0, waveform),
    src/include/tfsf/tfsf_2d.h:8-10: the plane wave of the 2-D (nz = 1)
    TMz grid, travelling in the x-y plane at angle phi_inc with Ez
    polarisation.  It is the TFSF base with theta = pi / 2, psi = 0 and no
    z offset (src/tfsf/tfsf_2d.cpp:8-10)."""
    distance_x: int
    distance_y: int
    phi: float
    e_0: float
    waveform: Waveform

    def desc(self) -> TFSFDesc:
        d = TFSFDesc()
        d.enabled = 2
        d.distance[:] = [int(self.distance_x), int(self.distance_y), 0]
        d.e0, d.theta, d.phi, d.psi = float(self.e_0), math.pi / 2, float(self.phi), 0.0
        d.waveform = self.waveform.desc()
        return d


@dataclass
class NffftFd:
    """NffftFd(distance_x, distance_y, distance_z, frequencies, theta, phi,
    output_dir_path), src/include/nffft/nffft_fd.h:39-50."""
    distance_x: int
    distance_y: int
    distance_z: int
    frequencies: Sequence[float]
    theta: Sequence[float]
    phi: Sequence[float]
    output_dir_path: str = ""

    def arrays(self):
        return (np.ascontiguousarray(np.atleast_1d(self.frequencies), dtype=np.float64),
                np.ascontiguousarray(np.atleast_1d(self.theta), dtype=np.float64),
                np.ascontiguousarray(np.atleast_1d(self.phi), dtype=np.float64))


@dataclass
class NffftBroadBand:
    """NffftBroadBand(distance_x, distance_y, distance_z, theta, phi,
    output_dir_path), src/include/nffft/nffft_broadband.h:9-12: the far
    field in one direction over the whole band of the run."""
    distance_x: int
    distance_y: int
    distance_z: int
    theta: float
    phi: float
    output_dir_path: str = ""

    def arrays(self):
        return (np.zeros(0, dtype=np.float64), np.array([float(self.theta)]), np.array([float(self.phi)]))


@dataclass
class _Lumped:
    cube: Cube
    orientation: int
    value: float
    waveform: Optional[Waveform] = None
    kind: int = -1

    def desc(self) -> LumpedDesc:
        d = LumpedDesc()
        d.kind, d.orientation, d.value = self.kind, int(self.orientation), float(self.value)
        d.point[:] = list(map(float, self.cube.point))
        d.size[:] = list(map(float, self.cube.size))
        if self.waveform is not None:
            d.waveform = self.waveform.desc()
        return d


def CurrentSource(cube: Cube, orientation: int, resistance: float, waveform: Waveform) -> _Lumped:
    """CurrentSource(cube, orientation, resistance, waveform), src/lumped_element/current_source.cpp:5-16."""
    return _Lumped(cube, orientation, resistance, waveform, LUMPED_CURRENT_SOURCE)


def VoltageSource(cube: Cube, orientation: int, resistance: float, waveform: Waveform) -> _Lumped:
    """VoltageSource(cube, orientation, resistance, waveform), src/lumped_element/voltage_source.cpp:15-26."""
    return _Lumped(cube, orientation, resistance, waveform, LUMPED_VOLTAGE_SOURCE)


def Resistor(cube: Cube, axis: int, resistance: float) -> _Lumped:
    """Resistor(cube, axis, resistance), src/lumped_element/resistor.cpp."""
    return _Lumped(cube, axis, resistance, None, LUMPED_RESISTOR)


def Capacitor(cube: Cube, axis: int, capacitance: float) -> _Lumped:
    """Capacitor(cube, axis, capacitance), src/lumped_element/capacitor.cpp."""
    return _Lumped(cube, axis, capacitance, None, LUMPED_CAPACITOR)


def Inductor(cube: Cube, axis: int, inductance: float) -> _Lumped:
    """Inductor(cube, axis, inductance), src/lumped_element/inductor.cpp."""
    return _Lumped(cube, axis, inductance, None, LUMPED_INDUCTOR)


@dataclass
class _Monitor:
    cube: Cube
    orientation: int
    output_dir_path: str = ""
    output_file_name: str = ""
    kind: int = -1
    component: int = 0       # field monitors: EMComponent
    plane_type: int = 0      #                 PlaneType
    plot_step: int = 0       # movie monitors: frame interval (0: not a movie)
    total_time_steps: int = 0

    def desc(self) -> MonitorDesc:
        d = MonitorDesc()
        d.kind, d.orientation = self.kind, int(self.orientation)
        d.point[:] = list(map(float, self.cube.point))
        d.size[:] = list(map(float, self.cube.size))
        d.component, d.plane_type = int(self.component), int(self.plane_type)
        d.plot_step, d.total_time_steps = int(self.plot_step), int(self.total_time_steps)
        return d


def VoltageMonitor(cube: Cube, orientation: int, output_dir_path: str = "", output_file_name: str = "") -> _Monitor:
    """VoltageMonitor(cube, orientation, dir, file), src/monitor/voltage_monitor.cpp:11-18."""
    return _Monitor(cube, orientation, output_dir_path, output_file_name, MONITOR_VOLTAGE)


def CurrentMonitor(cube: Cube, orientation: int, output_dir_path: str = "", output_file_name: str = "") -> _Monitor:
    """CurrentMonitor(cube, orientation, dir, file), src/monitor/current_monitor.cpp:9-16."""
    return _Monitor(cube, orientation, output_dir_path, output_file_name, MONITOR_CURRENT)


# EMComponent (src/include/electromagnetic_field/electromagnetic_field.h:8)
EX, EY, EZ, HX, HY, HZ = range(6)
# PlaneType (src/include/util/type_define.h:30)
PLANE_XY, PLANE_YZ, PLANE_ZX = range(3)


def TimeDomainFieldMonitor(cube: Cube, plane_type: int, component: int, output_dir_path: str = "",
                           output_file_name: str = "") -> _Monitor:
    """TimeDomainFieldMonitor(cube, plane_type, component, dir, file),
    src/monitor/field_monitor.cpp:15-24: the component over the cube's grid
    box after the last step (a 3-D .npy at output)."""
    return _Monitor(cube, 0, output_dir_path, output_file_name, MONITOR_FIELD, int(component), int(plane_type))


def MovieMonitor(monitor: _Monitor, total_time_steps: int, plot_step: int = 30) -> _Monitor:
    """MovieMonitor(monitor, total_time_steps, plot_step=30),
    src/monitor/movie_monitor.cpp:6-10, over a TimeDomainFieldMonitor: a
    frame after every step t with t % plot_step == 0 and after step
    total_time_steps - 1 (NNNN.npy files in the field monitor's directory
    at output)."""
    if monitor.kind != MONITOR_FIELD:
        raise ValueError("a MovieMonitor runs over a TimeDomainFieldMonitor")
    if plot_step < 1:
        raise ValueError("plot_step must be at least 1")
    return _Monitor(monitor.cube, 0, monitor.output_dir_path, monitor.output_file_name, MONITOR_FIELD,
                    monitor.component, monitor.plane_type, int(plot_step), int(total_time_steps))


@dataclass
class Port:
    """Port(index, impedance, is_activated_source, voltage, current),
    src/network/port.cpp:10-17; voltage and current are the scene's
    VoltageMonitor and CurrentMonitor objects (they must be in
    Scene.monitors)."""
    index: int
    impedance: complex
    is_activated_source: bool
    voltage: _Monitor
    current: _Monitor


@dataclass
class Network:
    """Network(ports, frequencies, output_path), src/network/network.cpp:10-14."""
    ports: List[Port]
    frequencies: Sequence[float]
    output_path: str = ""


# ----------------------------------------------------------------- scene ---
@dataclass
class Scene:
    """Everything Simulation(cell_size, objects, ..., cfl) is built from
    (src/include/simulation/simulation.h:27-66), plus an optional voxel
    material raster for heterogeneous media."""
    cell_size: float
    objects: List[object] = field(default_factory=list)
    boundaries: List[PML] = field(default_factory=list)
    tfsf: Optional[object] = None   # TFSF3D or TFSF2D
    nffft: Optional[object] = None   # NffftFd or NffftBroadBand
    lumped_elements: List[_Lumped] = field(default_factory=list)
    monitors: List[_Monitor] = field(default_factory=list)
    cfl: float = 0.99
    voxel_materials: Optional[List[Material]] = None
    voxel_index: Optional[np.ndarray] = None  # (nx, ny, nz) material numbers
    network: Optional[Network] = None

    def desc(self) -> SceneDesc:
        """Builds the C description.  The returned struct keeps its arrays
        alive through `_keep`; hold it for as long as the call needs it."""
        d = SceneDesc()
        keep = []
        d.cell_size = float(self.cell_size)
        d.cfl = float(self.cfl)
        objs = (ObjectDesc * max(1, len(self.objects)))(*[o.desc() for o in self.objects])
        d.n_objects, d.objects = len(self.objects), objs
        pml = (PMLDesc * max(1, len(self.boundaries)))(*[b.desc() for b in self.boundaries])
        d.n_pml, d.pml = len(self.boundaries), pml
        lum = (LumpedDesc * max(1, len(self.lumped_elements)))(*[l.desc() for l in self.lumped_elements])
        d.n_lumped, d.lumped = len(self.lumped_elements), lum
        mon = (MonitorDesc * max(1, len(self.monitors)))(*[m.desc() for m in self.monitors])
        d.n_monitors, d.monitors = len(self.monitors), mon
        keep += [objs, pml, lum, mon]
        if self.tfsf is not None:
            d.tfsf = self.tfsf.desc()
            keep.append(self.tfsf.waveform)
        if self.nffft is not None:
            f, t, p = self.nffft.arrays()
            keep += [f, t, p]
            d.nffft.enabled = 2 if isinstance(self.nffft, NffftBroadBand) else 1
            d.nffft.distance[:] = [int(self.nffft.distance_x), int(self.nffft.distance_y),
                                   int(self.nffft.distance_z)]
            d.nffft.n_freq, d.nffft.n_theta, d.nffft.n_phi = len(f), len(t), len(p)
            dp = C.POINTER(C.c_double)
            d.nffft.frequencies = f.ctypes.data_as(dp)
            d.nffft.theta = t.ctypes.data_as(dp)
            d.nffft.phi = p.ctypes.data_as(dp)
        for l in self.lumped_elements:
            if l.waveform is not None:
                keep.append(l.waveform)
        if self.voxel_index is not None:
            wide = len(self.voxel_materials) > 65536
            vi = np.ascontiguousarray(self.voxel_index, dtype=np.uint32 if wide else np.uint16)
            vm = (MaterialDesc * len(self.voxel_materials))(*[m.desc() for m in self.voxel_materials])
            keep += [vi, vm]
            d.voxel_index = vi.ctypes.data
            d.voxel_index_bytes = 4 if wide else 2
            d.voxel_materials = vm
            d.n_voxel_materials = len(self.voxel_materials)
            d.voxel_shape[:] = list(vi.shape)
        if self.network is not None and self.network.ports:
            def mon_index(m):
                for q, x in enumerate(self.monitors):
                    if x is m:
                        return q
                raise ValueError("a port's monitors must be in Scene.monitors")
            ports = (PortDesc * len(self.network.ports))()
            for q, p in enumerate(self.network.ports):
                z = complex(p.impedance)
                ports[q].index, ports[q].is_activated_source = int(p.index), int(bool(p.is_activated_source))
                ports[q].impedance_re, ports[q].impedance_im = z.real, z.imag
                ports[q].voltage_monitor, ports[q].current_monitor = mon_index(p.voltage), mon_index(p.current)
            fr = np.ascontiguousarray(self.network.frequencies, dtype=np.float64)
            keep += [ports, fr]
            d.n_ports, d.ports = len(self.network.ports), ports
            d.n_network_freqs = fr.size
            d.network_freqs = fr.ctypes.data_as(C.POINTER(C.c_double))
        d._keep = keep
        return d


def field_shape(comp: int, n) -> tuple:
    """Reference array shape of a field component (simulation_init.cpp:28-35)."""
    nx, ny, nz = (int(v) for v in n)
    return [(nx, ny + 1, nz + 1), (nx + 1, ny, nz + 1), (nx + 1, ny + 1, nz),
            (nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)][comp]


def nffft_face_shape(which: int, box) -> tuple:
    """Accumulator shape (without the frequency axis) of NF-FF array `which`
    (face*4 + q; X faces (ny,nz), Y faces (nz,nx), Z faces (nx,ny))."""
    bx, by, bz = box
    face = which // 4
    return [(by, bz), (by, bz), (bz, bx), (bz, bx), (bx, by), (bx, by)][face]
