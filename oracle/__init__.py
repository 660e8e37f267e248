"""TEST INFRASTRUCTURE ONLY -- the CPU oracle the GPU engine is tested against.

ctypes binding of the FP64 CPU restatement of the reference XFDTD step loop
(oracle/xfdtd_oracle.cpp).  Only the tests, the smoke check and the
benchmark's CPU-baseline leg use it; the product never imports it.

Parity status: pinned against the reference's one assertion test
(test/test_grid.cpp, restated in tests/test_oracle.py) and against analytic
checks (TFSF leakage, CPML reflection, PEC-sphere RCS against a Mie series).
The reference itself cannot be built here (xtensor, xtensor-blas,
xtensor-fftw, FFTW3, BLAS, LAPACK are absent), so no output of the reference
binary pins it further.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from xfdtd_gb300 import scene as S

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build() -> str:
    """Compiles the oracle with its Makefile (a few seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        P = C.POINTER
        L.oracle_sim_create.argtypes = [P(S.SceneDesc), C.c_int64, P(C.c_void_p)]
        L.oracle_sim_step.argtypes = [C.c_void_p, C.c_int64]
        L.oracle_sim_info.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_double), P(C.c_int64)]
        for fn in ("oracle_sim_read_field", "oracle_sim_read_monitor", "oracle_sim_read_nffft",
                   "oracle_sim_far_field", "oracle_sim_read_coeff"):
            getattr(L, fn).argtypes = [C.c_void_p, C.c_int, P(C.c_double), C.c_int64]
        L.oracle_sim_write_field.argtypes = [C.c_void_p, C.c_int, P(C.c_double), C.c_int64]
        L.oracle_sim_field_monitor.argtypes = [C.c_void_p, C.c_int, P(C.c_int64), P(C.c_int64), P(C.c_int64),
                                               P(C.c_int64), C.c_int64]
        L.oracle_sim_read_field_monitor.argtypes = [C.c_void_p, C.c_int, C.c_int64, P(C.c_double), C.c_int64]
        L.oracle_sim_incident_dft.argtypes = [C.c_void_p, P(C.c_double), C.c_int, P(C.c_double)]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_sim_destroy.argtypes = [C.c_void_p]
        L.oracle_grid_from_cube.argtypes = [P(C.c_double), P(C.c_double), C.c_double, P(C.c_int64),
                                            P(C.c_double), C.c_int64]
        _lib = L
    return _lib


def _check(rc: int):
    if rc != 0:
        raise RuntimeError(lib().oracle_last_error().decode())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(int(n))


class OracleSim:
    """One simulation on the CPU oracle (FP64, reference-faithful)."""

    def __init__(self, scene: S.Scene, total_steps: int):
        self.scene = scene
        self.total_steps = int(total_steps)
        self._desc = scene.desc()
        h = C.c_void_p()
        _check(lib().oracle_sim_create(C.byref(self._desc), self.total_steps, C.byref(h)))
        self.h = h
        n = (C.c_int64 * 3)()
        dt = C.c_double()
        st = C.c_int64()
        _check(lib().oracle_sim_info(self.h, n, C.byref(dt), C.byref(st)))
        self.n = tuple(int(v) for v in n)
        self.dt = dt.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_sim_destroy(self.h)
            self.h = None

    @property
    def step_index(self) -> int:
        st = C.c_int64()
        _check(lib().oracle_sim_info(self.h, None, None, C.byref(st)))
        return st.value

    def step(self, n: int = 1):
        _check(lib().oracle_sim_step(self.h, int(n)))

    def read_field(self, comp: int) -> np.ndarray:
        out = np.empty(S.field_shape(comp, self.n), dtype=np.float64)
        _check(lib().oracle_sim_read_field(self.h, comp, _dp(out), out.size))
        return out

    def write_field(self, comp: int, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        _check(lib().oracle_sim_write_field(self.h, comp, _dp(a), a.size))

    def read_coeff(self, which: int) -> np.ndarray:
        comp = [0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5][which]
        out = np.empty(S.field_shape(comp, self.n), dtype=np.float64)
        _check(lib().oracle_sim_read_coeff(self.h, which, _dp(out), out.size))
        return out

    def read_monitor(self, index: int) -> np.ndarray:
        out = np.empty(self.total_steps, dtype=np.float64)
        _check(lib().oracle_sim_read_monitor(self.h, index, _dp(out), out.size))
        return out

    def field_monitor_frames(self, index: int):
        """(lo, shape, frame steps) of field or movie monitor `index`."""
        lo, shape = (C.c_int64 * 3)(), (C.c_int64 * 3)()
        n = C.c_int64()
        _check(lib().oracle_sim_field_monitor(self.h, index, lo, shape, C.byref(n), None, 0))
        steps = (C.c_int64 * max(1, n.value))()
        _check(lib().oracle_sim_field_monitor(self.h, index, lo, shape, C.byref(n), steps, n.value))
        return tuple(lo), tuple(shape), [steps[f] for f in range(n.value)]

    def read_field_monitor(self, index: int, frame: int = 0) -> np.ndarray:
        _, shape, _ = self.field_monitor_frames(index)
        out = np.empty(shape, dtype=np.float64)
        _check(lib().oracle_sim_read_field_monitor(self.h, index, int(frame), _dp(out), out.size))
        return out

    def nffft_box(self):
        nf = self.scene.nffft
        return (self.n[0] - 2 * nf.distance_x, self.n[1] - 2 * nf.distance_y, self.n[2] - 2 * nf.distance_z)

    def read_nffft(self, which: int) -> np.ndarray:
        nfreq = len(np.atleast_1d(self.scene.nffft.frequencies))
        shp = (nfreq,) + S.nffft_face_shape(which, self.nffft_box())
        out = np.empty(shp + (2,), dtype=np.float64)
        _check(lib().oracle_sim_read_nffft(self.h, which, _dp(out), out.size))
        return out[..., 0] + 1j * out[..., 1]

    def far_field(self, which: int) -> np.ndarray:
        if type(self.scene.nffft).__name__ == "NffftBroadBand":   # over the 2T-1 bins; 10 = frequencies
            nb = 2 * self.total_steps - 1
            if which < 8:
                out = np.empty((nb, 2), dtype=np.float64)
                _check(lib().oracle_sim_far_field(self.h, which, _dp(out), out.size))
                return out[:, 0] + 1j * out[:, 1]
            out = np.empty(nb, dtype=np.float64)
            _check(lib().oracle_sim_far_field(self.h, which, _dp(out), out.size))
            return out
        f, t, p = self.scene.nffft.arrays()
        shp = (len(f), len(t), len(p))
        if which < 8:
            out = np.empty(shp + (2,), dtype=np.float64)
            _check(lib().oracle_sim_far_field(self.h, which, _dp(out), out.size))
            return out[..., 0] + 1j * out[..., 1]
        out = np.empty(shp, dtype=np.float64)
        _check(lib().oracle_sim_far_field(self.h, which, _dp(out), out.size))
        return out

    def incident_dft(self, freqs) -> np.ndarray:
        f = np.ascontiguousarray(np.atleast_1d(freqs), dtype=np.float64)
        out = np.empty((len(f), 2), dtype=np.float64)
        _check(lib().oracle_sim_incident_dft(self.h, _dp(f), len(f), _dp(out)))
        return out[:, 0] + 1j * out[:, 1]

    def rcs_db(self) -> np.ndarray:
        """10 log10(4 pi (|E_theta|^2 + |E_phi|^2) / |E_inc(f)|^2), [nf, nt, np]."""
        et, ep = self.far_field(0), self.far_field(1)
        f, _, _ = self.scene.nffft.arrays()
        inc = self.incident_dft(f)
        sigma = 4 * np.pi * (np.abs(et) ** 2 + np.abs(ep) ** 2) / (np.abs(inc)[:, None, None] ** 2)
        return 10 * np.log10(sigma)


def grid_from_cube(point, size, dl):
    """Restated GridSpace of test/test_grid.cpp for one cube."""
    p = np.ascontiguousarray(point, dtype=np.float64)
    s = np.ascontiguousarray(size, dtype=np.float64)
    n = (C.c_int64 * 3)()
    out = np.empty(4096, dtype=np.float64)
    _check(lib().oracle_grid_from_cube(_dp(p), _dp(s), float(dl), n, _dp(out), out.size))
    nx, ny, nz = (int(v) for v in n)
    o = 0
    res = {}
    for name, cnt in (("esx", nx), ("esy", ny), ("esz", nz), ("hsx", nx + 1), ("hsy", ny + 1), ("hsz", nz + 1)):
        res[name] = out[o:o + cnt].copy()
        o += cnt
    return (nx, ny, nz), res
