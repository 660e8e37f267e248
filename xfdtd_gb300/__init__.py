"""xfdtd_gb300 -- GB300-native engine for the XFDTD (Mrwatermolen/XFDTD)
time-stepping hot path: Yee E/H with CPML, TFSF plane-wave injection, the
NF-FF running DFT and far-field integration, lumped elements, thin wires and
probes, as hand-written CUDA for sm_103a behind a C-ABI.

Python binding of the scene-level C-ABI (include/xfdtd_sim.h) and of the
engine's timing / profiling entry points (include/xfdtd_cuda.h).  There is
no CPU fallback: if the native libraries are missing or no GPU is present,
every call that would run the engine raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import scene
from .scene import (  # noqa: F401  (re-exported: the reference's scene API)
    AXIS_X, AXIS_Y, AXIS_Z, EX, EY, EZ, HX, HY, HZ, XN, XP, YN, YP, ZN, ZP,
    Capacitor, CosineModulatedGaussianWaveform, CurrentMonitor, CurrentSource, Cube,
    CustomWaveform, Cylinder, DebyMedium, DrudeMedium, GaussianWaveform, Inductor, LorentzMedium, Material, NffftFd, Object, PML,
    Resistor, Scene, SinusoidalWaveform, Sphere, TFSF2D, TFSF3D, ThinWire, VoltageMonitor,
    VoltageSource,
)

FP64, FP32 = 0, 1
FLAG_GRAPH, FLAG_PROFILE, FLAG_AUTOTUNE, FLAG_SPLIT_EH, FLAG_FUSED_EH = 1, 2, 4, 8, 16
FLAG_PLAIN_VOLUME = 32
STATUS = {0: "ok", 1: "invalid plan", 2: "CUDA error", 3: "out of device memory", 4: "timeout",
          5: "non-finite value", 6: "device check", 7: "bad state"}

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_DIR = os.path.join(_HERE, "_lib")
_cuda = None
_host = None


class EngineError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def build(force: bool = False) -> None:
    """Compiles the native libraries in-tree (see native_build.py)."""
    from . import native_build
    native_build.build(force=force)


def libs():
    """Loads libxfdtd_cuda.so and libxfdtd.so (raises if they are not built)."""
    global _cuda, _host
    if _host is None:
        cuda_path = os.path.join(_LIB_DIR, "libxfdtd_cuda.so")
        host_path = os.path.join(_LIB_DIR, "libxfdtd.so")
        if not (os.path.exists(cuda_path) and os.path.exists(host_path)):
            raise ImportError("xfdtd_gb300 native libraries are not built; run xfdtd_gb300.build()")
        cu = C.CDLL(cuda_path, mode=C.RTLD_GLOBAL)
        ho = C.CDLL(host_path)
        P = C.POINTER
        dp = P(C.c_double)
        ho.xfdtd_sim_create.argtypes = [P(scene.SceneDesc), C.c_int64, C.c_int, C.c_int, P(C.c_void_p)]
        ho.xfdtd_sim_step.argtypes = [C.c_void_p, C.c_int64]
        ho.xfdtd_sim_info.argtypes = [C.c_void_p, P(C.c_int64), dp, P(C.c_int64)]
        for fn in ("xfdtd_sim_read_field", "xfdtd_sim_read_monitor", "xfdtd_sim_read_nffft", "xfdtd_sim_far_field"):
            getattr(ho, fn).argtypes = [C.c_void_p, C.c_int, dp, C.c_int64]
        ho.xfdtd_sim_write_field.argtypes = [C.c_void_p, C.c_int, dp, C.c_int64]
        ho.xfdtd_sim_field_monitor.argtypes = [C.c_void_p, C.c_int, P(C.c_int64), P(C.c_int64), P(C.c_int64),
                                               P(C.c_int64), C.c_int64]
        ho.xfdtd_sim_read_field_monitor.argtypes = [C.c_void_p, C.c_int, C.c_int64, dp, C.c_int64]
        ho.xfdtd_sim_incident_dft.argtypes = [C.c_void_p, dp, C.c_int, dp]
        ho.xfdtd_sim_output.argtypes = [C.c_void_p]
        ho.xfdtd_sim_set_output.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_char_p]
        ho.xfdtd_sim_s_parameters.argtypes = [C.c_void_p, P(C.c_int32), C.c_int64, P(C.c_int64), P(C.c_int64)]
        ho.xfdtd_sim_read_s_parameter.argtypes = [C.c_void_p, C.c_int, dp, C.c_int64]
        ho.xfdtd_sim_engine.argtypes = [C.c_void_p]
        ho.xfdtd_sim_engine.restype = C.c_void_p
        ho.xfdtd_sim_last_error.argtypes = [C.c_void_p]
        ho.xfdtd_sim_last_error.restype = C.c_char_p
        ho.xfdtd_sim_destroy.argtypes = [C.c_void_p]
        cu.xfdtd_step_timed.argtypes = [C.c_void_p, C.c_int64, dp]
        cu.xfdtd_step.argtypes = [C.c_void_p, C.c_int64]
        cu.xfdtd_synchronize.argtypes = [C.c_void_p]
        cu.xfdtd_check_finite.argtypes = [C.c_void_p]
        cu.xfdtd_profile.argtypes = [C.c_void_p, C.c_int, P(C.c_char_p), dp, P(C.c_int64), P(C.c_int)]
        cu.xfdtd_profile_reset.argtypes = [C.c_void_p]
        cu.xfdtd_launches_per_step.argtypes = [C.c_void_p, P(C.c_int)]
        cu.xfdtd_device_bytes.argtypes = [C.c_void_p, P(C.c_int64)]
        cu.xfdtd_index_bytes.argtypes = [C.c_void_p, P(C.c_int)]
        cu.xfdtd_transfer_bytes.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64)]
        cu.xfdtd_launch_count.argtypes = [C.c_void_p, P(C.c_int64)]
        cu.xfdtd_autotune.argtypes = [C.c_void_p, C.c_int]
        cu.xfdtd_kernel_variants.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int), dp]
        cu.xfdtd_set_kernel_variant.argtypes = [C.c_void_p, C.c_int, C.c_int]
        cu.xfdtd_volume_split.argtypes = [C.c_void_p, P(C.c_int64)]
        cu.xfdtd_volume_decomposition.argtypes = [C.c_void_p, P(C.c_int)]
        cu.xfdtd_shell_variants.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int)]
        cu.xfdtd_set_shell_variant.argtypes = [C.c_void_p, C.c_int, C.c_int]
        cu.xfdtd_set_wait_limit.argtypes = [C.c_void_p, C.c_int64]
        cu.xfdtd_create_times.argtypes = [C.c_void_p, dp]
        cu.xfdtd_set_tfsf_fusion.argtypes = [C.c_void_p, C.c_int, C.c_int]
        cu.xfdtd_tfsf_fusion.argtypes = [C.c_void_p, P(C.c_int)]
        cu.xfdtd_set_nffft_split.argtypes = [C.c_void_p, C.c_int]
        cu.xfdtd_nffft_split.argtypes = [C.c_void_p, P(C.c_int), P(C.c_float)]
        cu.xfdtd_last_error.argtypes = [C.c_void_p]
        cu.xfdtd_last_error.restype = C.c_char_p
        cu.xfdtd_version.restype = C.c_char_p
        cu.xfdtd_adjoint_forward.argtypes = [C.c_void_p, P(AdjointDesc), dp]
        cu.xfdtd_adjoint_backward.argtypes = [C.c_void_p, dp, dp, C.c_int64]
        cu.xfdtd_batch_create.argtypes = [P(C.c_void_p), C.c_int, C.c_int, P(C.c_void_p)]
        cu.xfdtd_batch_step.argtypes = [C.c_void_p, C.c_int64]
        cu.xfdtd_batch_step_timed.argtypes = [C.c_void_p, C.c_int64, dp]
        cu.xfdtd_batch_synchronize.argtypes = [C.c_void_p]
        cu.xfdtd_batch_status.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int64), P(C.c_int64)]
        cu.xfdtd_batch_tma_members.argtypes = [C.c_void_p, P(C.c_int)]
        cu.xfdtd_batch_last_error.argtypes = [C.c_void_p]
        cu.xfdtd_batch_last_error.restype = C.c_char_p
        cu.xfdtd_batch_destroy.argtypes = [C.c_void_p]
        _cuda, _host = cu, ho
    return _cuda, _host


class AdjointDesc(C.Structure):
    """ctypes mirror of xfdtd_adjoint_desc (include/xfdtd_cuda.h)."""
    _fields_ = [("design_lo", C.c_int64 * 3), ("design_hi", C.c_int64 * 3),
                ("loss_comp", C.c_int32), ("plane_axis", C.c_int32), ("plane_index", C.c_int64),
                ("plane_lo", C.c_int64 * 2), ("plane_hi", C.c_int64 * 2),
                ("t_begin", C.c_int64), ("t_end", C.c_int64),
                ("checkpoint_every", C.c_int32), ("reserved", C.c_int32)]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Simulation:
    """One simulation on the GPU engine, built from a `scene.Scene`.

    precision: "fp64" (the reference's arithmetic) or "fp32" (fields and CPML
    state in FP32; TFSF 1-D grid, NF-FF accumulation and far-field
    integration stay FP64).  fused: True = one E/H sweep kernel per step,
    False = separate E and H kernels, None = the autotuner picks the faster;
    all give identical bits.
    """

    def __init__(self, sc: "scene.Scene", total_steps: int, precision: str = "fp64", graph: bool = True,
                 profile: bool = False, device: int = 0, autotune: bool = True, fused=None):
        self.scene = sc
        self.total_steps = int(total_steps)
        self.precision = precision
        cu, ho = libs()
        self._desc = sc.desc()
        prec = FP64 if precision == "fp64" else FP32
        flags = ((FLAG_GRAPH if graph else 0) | (FLAG_PROFILE if profile else 0)
                 | (FLAG_AUTOTUNE if autotune else 0) | ({True: FLAG_FUSED_EH, False: FLAG_SPLIT_EH, None: 0}[fused]) | (int(device) << 8))
        h = C.c_void_p()
        rc = ho.xfdtd_sim_create(C.byref(self._desc), self.total_steps, prec, flags, C.byref(h))
        self.h = h
        if rc != 0:
            msg = ho.xfdtd_sim_last_error(h).decode() if h.value else "no handle"
            ho.xfdtd_sim_destroy(h)
            self.h = None
            raise EngineError(rc, msg)
        n = (C.c_int64 * 3)()
        dt = C.c_double()
        ho.xfdtd_sim_info(self.h, n, C.byref(dt), None)
        self.n = tuple(int(v) for v in n)
        self.dt = dt.value
        self.engine = C.c_void_p(ho.xfdtd_sim_engine(self.h))
        # output directories the scene description does not carry
        if sc.nffft is not None and sc.nffft.output_dir_path:
            self._check(ho.xfdtd_sim_set_output(self.h, -1, sc.nffft.output_dir_path.encode(), None))
        if sc.network is not None and sc.network.ports and sc.network.output_path:
            self._check(ho.xfdtd_sim_set_output(self.h, -2, sc.network.output_path.encode(), None))
        for q, m in enumerate(sc.monitors):
            if m.output_dir_path:
                self._check(ho.xfdtd_sim_set_output(self.h, q, m.output_dir_path.encode(),
                                                    (m.output_file_name or "").encode()))

    def close(self):
        if getattr(self, "h", None):
            libs()[1].xfdtd_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc: int):
        if rc != 0:
            raise EngineError(rc, libs()[1].xfdtd_sim_last_error(self.h).decode())

    def _check_engine(self, rc: int):
        if rc != 0:
            raise EngineError(rc, libs()[0].xfdtd_last_error(self.engine).decode())

    @property
    def step_index(self) -> int:
        st = C.c_int64()
        libs()[1].xfdtd_sim_info(self.h, None, None, C.byref(st))
        return st.value

    def step(self, n: int = 1):
        self._check(libs()[1].xfdtd_sim_step(self.h, int(n)))

    def step_timed(self, n: int) -> float:
        """Enqueues n steps; returns their device time in ms (CUDA events)."""
        ms = C.c_double()
        self._check_engine(libs()[0].xfdtd_step_timed(self.engine, int(n), C.byref(ms)))
        return ms.value

    def synchronize(self):
        self._check_engine(libs()[0].xfdtd_synchronize(self.engine))

    def check_finite(self):
        self._check_engine(libs()[0].xfdtd_check_finite(self.engine))

    def read_field(self, comp: int) -> np.ndarray:
        out = np.empty(scene.field_shape(comp, self.n), dtype=np.float64)
        self._check(libs()[1].xfdtd_sim_read_field(self.h, comp, _dp(out), out.size))
        return out

    def write_field(self, comp: int, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self._check(libs()[1].xfdtd_sim_write_field(self.h, comp, _dp(a), a.size))

    def read_monitor(self, index: int) -> np.ndarray:
        out = np.empty(self.total_steps, dtype=np.float64)
        self._check(libs()[1].xfdtd_sim_read_monitor(self.h, index, _dp(out), out.size))
        return out

    def s_parameters(self) -> dict:
        """The network's S-parameters {10 j + i: complex array over its
        frequencies} from the monitor series recorded so far
        (src/network/network.cpp:40-52)."""
        n, nf = C.c_int64(), C.c_int64()
        self._check(libs()[1].xfdtd_sim_s_parameters(self.h, None, 0, C.byref(n), C.byref(nf)))
        keys = (C.c_int32 * max(1, n.value))()
        self._check(libs()[1].xfdtd_sim_s_parameters(self.h, keys, n.value, C.byref(n), C.byref(nf)))
        out = {}
        for q in range(n.value):
            buf = np.empty(2 * nf.value, dtype=np.float64)
            self._check(libs()[1].xfdtd_sim_read_s_parameter(self.h, int(keys[q]), _dp(buf), buf.size))
            out[int(keys[q])] = buf[0::2] + 1j * buf[1::2]
        return out

    def field_monitor_frames(self, index: int):
        """Box of field (or movie) monitor `index` in its component's array
        (first index, shape) and the steps of its frames (-1: a field
        monitor's one frame, the current field)."""
        lo, shape = (C.c_int64 * 3)(), (C.c_int64 * 3)()
        n = C.c_int64()
        self._check(libs()[1].xfdtd_sim_field_monitor(self.h, index, lo, shape, C.byref(n), None, 0))
        steps = (C.c_int64 * max(1, n.value))()
        self._check(libs()[1].xfdtd_sim_field_monitor(self.h, index, lo, shape, C.byref(n), steps, n.value))
        return tuple(lo), tuple(shape), [steps[f] for f in range(n.value)]

    def read_field_monitor(self, index: int, frame: int = 0) -> np.ndarray:
        """Frame `frame` of field (or movie) monitor `index`."""
        _, shape, _ = self.field_monitor_frames(index)
        out = np.empty(shape, dtype=np.float64)
        self._check(libs()[1].xfdtd_sim_read_field_monitor(self.h, index, int(frame), _dp(out), out.size))
        return out

    def nffft_box(self):
        nf = self.scene.nffft
        return (self.n[0] - 2 * nf.distance_x, self.n[1] - 2 * nf.distance_y, self.n[2] - 2 * nf.distance_z)

    def read_nffft(self, which: int) -> np.ndarray:
        nfreq = len(np.atleast_1d(self.scene.nffft.frequencies))
        shp = (nfreq,) + scene.nffft_face_shape(which, self.nffft_box())
        out = np.empty(shp + (2,), dtype=np.float64)
        self._check(libs()[1].xfdtd_sim_read_nffft(self.h, which, _dp(out), out.size))
        return out[..., 0] + 1j * out[..., 1]

    def far_field(self, which: int) -> np.ndarray:
        """NffftFd: array `which` (0 e_theta .. 7 l_phi complex, 8/9 power)
        over (frequency, theta, phi).  NffftBroadBand: the same arrays over
        its 2T-1 bins, and 10 the bins' frequencies."""
        if isinstance(self.scene.nffft, scene.NffftBroadBand):
            nb = 2 * self.total_steps - 1
            if which < 8:
                out = np.empty((nb, 2), dtype=np.float64)
                self._check(libs()[1].xfdtd_sim_far_field(self.h, which, _dp(out), out.size))
                return out[:, 0] + 1j * out[:, 1]
            out = np.empty(nb, dtype=np.float64)
            self._check(libs()[1].xfdtd_sim_far_field(self.h, which, _dp(out), out.size))
            return out
        f, t, p = self.scene.nffft.arrays()
        shp = (len(f), len(t), len(p))
        if which < 8:
            out = np.empty(shp + (2,), dtype=np.float64)
            self._check(libs()[1].xfdtd_sim_far_field(self.h, which, _dp(out), out.size))
            return out[..., 0] + 1j * out[..., 1]
        out = np.empty(shp, dtype=np.float64)
        self._check(libs()[1].xfdtd_sim_far_field(self.h, which, _dp(out), out.size))
        return out

    def incident_dft(self, freqs) -> np.ndarray:
        f = np.ascontiguousarray(np.atleast_1d(freqs), dtype=np.float64)
        out = np.empty((len(f), 2), dtype=np.float64)
        self._check(libs()[1].xfdtd_sim_incident_dft(self.h, _dp(f), len(f), _dp(out)))
        return out[:, 0] + 1j * out[:, 1]

    def rcs_db(self) -> np.ndarray:
        et, ep = self.far_field(0), self.far_field(1)
        f, _, _ = self.scene.nffft.arrays()
        inc = self.incident_dft(f)
        sigma = 4 * np.pi * (np.abs(et) ** 2 + np.abs(ep) ** 2) / (np.abs(inc)[:, None, None] ** 2)
        return 10 * np.log10(sigma)

    def output(self):
        self._check(libs()[1].xfdtd_sim_output(self.h))

    def profile(self) -> dict:
        """Per-kernel device time (ms) and launches recorded under profile=True."""
        names = (C.c_char_p * 32)()
        ms = (C.c_double * 32)()
        cnt = (C.c_int64 * 32)()
        n = C.c_int()
        self._check_engine(libs()[0].xfdtd_profile(self.engine, 32, names, ms, cnt, C.byref(n)))
        return {names[i].decode(): (ms[i], int(cnt[i])) for i in range(n.value)}

    def profile_reset(self):
        self._check_engine(libs()[0].xfdtd_profile_reset(self.engine))

    def launch_count(self) -> int:
        """Per-step kernel launches the engine has enqueued so far."""
        n = C.c_int64()
        self._check_engine(libs()[0].xfdtd_launch_count(self.engine, C.byref(n)))
        return n.value

    def launches_per_step(self) -> int:
        n = C.c_int()
        self._check_engine(libs()[0].xfdtd_launches_per_step(self.engine, C.byref(n)))
        return n.value

    def adjoint_forward(self, design_lo, design_hi, plane_axis: int, plane_index: int, plane_lo, plane_hi,
                        t_begin: int, t_end: int, loss_comp: int = 2, checkpoint_every: int = 100) -> float:
        """Runs every step from step 0 for an adjoint gradient (the forward
        half of the forward/backward pair) and returns the loss: the sum,
        over the steps t_begin .. t_end-1 and the plane plane_axis =
        plane_index (extents plane_lo .. plane_hi on the other two axes), of
        the squared field component loss_comp (0 Ex, 1 Ey, 2 Ez) after each
        step.  Cell indices are grid indices (CPML included).  The state is
        checkpointed every checkpoint_every steps (0: the design box
        [design_lo, design_hi) is recorded at every step instead)."""
        d = AdjointDesc()
        d.design_lo[:] = [int(v) for v in design_lo]
        d.design_hi[:] = [int(v) for v in design_hi]
        d.loss_comp, d.plane_axis, d.plane_index = int(loss_comp), int(plane_axis), int(plane_index)
        d.plane_lo[:] = [int(v) for v in plane_lo]
        d.plane_hi[:] = [int(v) for v in plane_hi]
        d.t_begin, d.t_end, d.checkpoint_every = int(t_begin), int(t_end), int(checkpoint_every)
        self._adj_shape = tuple(int(b) - int(a) for a, b in zip(design_lo, design_hi))
        loss = C.c_double()
        self._check_engine(libs()[0].xfdtd_adjoint_forward(self.engine, C.byref(d), C.byref(loss)))
        return loss.value

    def adjoint_backward(self):
        """dL/d eps_r and dL/d sigma of every design cell (arrays over the
        design box), by the discrete adjoint of the step loop."""
        ge = np.empty(self._adj_shape, dtype=np.float64)
        gs = np.empty(self._adj_shape, dtype=np.float64)
        self._check_engine(libs()[0].xfdtd_adjoint_backward(self.engine, _dp(ge), _dp(gs), ge.size))
        return ge, gs

    def kernel_variants(self) -> dict:
        """Volume-kernel variant in use for E and H and the autotuner's trial
        times (ms per launch; 0 = not tried for this precision)."""
        n, ce, ch = C.c_int(), C.c_int(), C.c_int()
        ms = (C.c_double * 64)()
        self._check_engine(libs()[0].xfdtd_kernel_variants(self.engine, C.byref(n), C.byref(ce), C.byref(ch), ms))
        return {"e": ce.value, "h": ch.value, "n": n.value,
                "trials_e": [ms[2 * v] for v in range(n.value)], "trials_h": [ms[2 * v + 1] for v in range(n.value)]}

    def set_kernel_variant(self, e_variant: int, h_variant: int):
        self._check_engine(libs()[0].xfdtd_set_kernel_variant(self.engine, int(e_variant), int(h_variant)))

    def shell_variants(self) -> dict:
        """Number of shell-kernel variants and the ones in use for E and H."""
        n, ce, ch = C.c_int(), C.c_int(), C.c_int()
        self._check_engine(libs()[0].xfdtd_shell_variants(self.engine, C.byref(n), C.byref(ce), C.byref(ch)))
        return {"n": n.value, "e": ce.value, "h": ch.value}

    def set_shell_variant(self, e_variant: int, h_variant: int):
        self._check_engine(libs()[0].xfdtd_set_shell_variant(self.engine, int(e_variant), int(h_variant)))

    def create_times(self) -> dict:
        """Wall time of the engine's create, ms: allocation and upload of the
        plan's tables, and autotuning."""
        ms = (C.c_double * 2)()
        self._check_engine(libs()[0].xfdtd_create_times(self.engine, ms))
        return {"alloc_upload_ms": ms[0], "autotune_ms": ms[1]}

    def set_tfsf_fusion(self, e_on: bool, h_on: bool):
        """Allow or forbid the TFSF corrections inside the wide TMA launches."""
        self._check_engine(libs()[0].xfdtd_set_tfsf_fusion(self.engine, int(bool(e_on)), int(bool(h_on))))

    def tfsf_fusion(self) -> tuple:
        """Whether the E and H updates apply the TFSF corrections in their
        wide launch with the current variants."""
        a = (C.c_int * 2)()
        self._check_engine(libs()[0].xfdtd_tfsf_fusion(self.engine, a))
        return bool(a[0]), bool(a[1])

    def set_nffft_split(self, on: bool):
        """Fix the NF-FF sampling schedule: split halves beside the volume
        updates (True) or one launch after the H update (False)."""
        self._check_engine(libs()[0].xfdtd_set_nffft_split(self.engine, int(bool(on))))

    def nffft_split(self) -> dict:
        """The NF-FF sampling schedule in use and the autotuner's trial step
        times of the split and one-launch forms (ms; 0 = not timed)."""
        on = C.c_int()
        ms = (C.c_float * 2)()
        self._check_engine(libs()[0].xfdtd_nffft_split(self.engine, C.byref(on), ms))
        return {"split": bool(on.value), "trial_ms_split": ms[0], "trial_ms_one_launch": ms[1]}

    def set_wait_limit(self, polls: int):
        """Polls of each TMA plane wait before a block gives up and reports a
        timeout (default and maximum 2^22; 0 gives up at once)."""
        self._check_engine(libs()[0].xfdtd_set_wait_limit(self.engine, int(polls)))

    def volume_split(self) -> dict:
        """Cells of the interior and shell launches of the E and H updates,
        and whether each update runs the wide decomposition (x and y slabs
        in the interior launch, z slabs in the shell launch) or the narrow
        one (plain cells in the interior launch, walls and slabs in the
        shell launch)."""
        c = (C.c_int64 * 4)()
        self._check_engine(libs()[0].xfdtd_volume_split(self.engine, c))
        w = (C.c_int * 2)()
        self._check_engine(libs()[0].xfdtd_volume_decomposition(self.engine, w))
        return {"e_interior": c[0], "e_shell": c[1], "h_interior": c[2], "h_shell": c[3],
                "e_wide": bool(w[0]), "h_wide": bool(w[1])}

    def transfer_bytes(self):
        """(host->device, device->host) bytes the engine has copied so far."""
        a, b = C.c_int64(), C.c_int64()
        self._check_engine(libs()[0].xfdtd_transfer_bytes(self.engine, C.byref(a), C.byref(b)))
        return a.value, b.value

    def device_bytes(self) -> int:
        b = C.c_int64()
        self._check_engine(libs()[0].xfdtd_device_bytes(self.engine, C.byref(b)))
        return b.value

    def index_bytes(self) -> int:
        """Bytes per cell of the material index (1, 2 or 4)."""
        b = C.c_int()
        self._check_engine(libs()[0].xfdtd_index_bytes(self.engine, C.byref(b)))
        return b.value


def version() -> str:
    return libs()[0].xfdtd_version().decode()


class Batch:
    """Several simulations of different sizes advanced together
    (xfdtd_batch_*): one launch per phase over a work list of every member
    still running, the step loop replayed from a CUDA graph.  Members are
    `Simulation`s created with fused=False, not yet stepped, without lumped
    elements or monitors; each stops at its own total_steps.  Read them with
    their own methods after `synchronize()`.  The volume phases run on the
    TMA-staged launches for the members whose grids allow them, unless
    `plain` (every member on the one-thread-per-cell kernels)."""

    def __init__(self, members: list, graph: bool = True, plain: bool = False):
        cu, _ = libs()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.engine.value for m in self.members])
        b = C.c_void_p()
        flags = (FLAG_GRAPH if graph else 0) | (FLAG_PLAIN_VOLUME if plain else 0)
        rc = cu.xfdtd_batch_create(arr, len(self.members), flags, C.byref(b))
        self.b = b
        if rc != 0:
            msg = cu.xfdtd_batch_last_error(b).decode()
            cu.xfdtd_batch_destroy(b)
            self.b = None
            raise EngineError(rc, msg)

    def _check(self, rc):
        if rc != 0:
            raise EngineError(rc, libs()[0].xfdtd_batch_last_error(self.b).decode())

    def step(self, n: int):
        self._check(libs()[0].xfdtd_batch_step(self.b, int(n)))

    def step_timed(self, n: int) -> float:
        ms = C.c_double()
        self._check(libs()[0].xfdtd_batch_step_timed(self.b, int(n), C.byref(ms)))
        return ms.value

    def synchronize(self):
        self._check(libs()[0].xfdtd_batch_synchronize(self.b))

    def status(self) -> dict:
        r, clock, launches = C.c_int(), C.c_int64(), C.c_int64()
        self._check(libs()[0].xfdtd_batch_status(self.b, C.byref(r), C.byref(clock), C.byref(launches)))
        return {"running": r.value, "clock": clock.value, "launches": launches.value}

    def tma_members(self) -> int:
        """Members on the TMA-staged volume launches (the rest run the
        one-thread-per-cell kernels)."""
        n = C.c_int()
        self._check(libs()[0].xfdtd_batch_tma_members(self.b, C.byref(n)))
        return n.value

    def __del__(self):
        if getattr(self, "b", None) and _cuda is not None:
            _cuda.xfdtd_batch_destroy(self.b)
            self.b = None
