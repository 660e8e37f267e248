"""The C-ABI libraries build, load and export every entry point that
include/*.h declares (no GPU needed: nothing here launches a kernel)."""
import ctypes as C
import os
import re

import pytest

import xfdtd_gb300 as X
from xfdtd_gb300 import scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xfdtd_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def libs():
    X.build()
    return X.libs()


def test_engine_exports_every_declared_symbol(libs):
    cu, _ = libs
    names = _declared("xfdtd_cuda.h")
    assert len(names) >= 18
    for n in names:
        assert hasattr(cu, n), n


def test_scene_lib_exports_every_declared_symbol(libs):
    _, ho = libs
    names = _declared("xfdtd_sim.h")
    assert len(names) >= 13
    for n in names:
        assert hasattr(ho, n), n


def test_version_string(libs):
    assert "sm_103a" in X.version()


def test_null_and_invalid_plans_are_rejected_on_the_host(libs):
    cu, _ = libs
    cu.xfdtd_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    h = C.c_void_p()
    assert cu.xfdtd_create(None, C.byref(h)) == 1
    # a plan with a 1-cell axis is refused before any CUDA call
    plan = (C.c_char * 4096)()
    C.memmove(plan, (C.c_int32 * 3)(1, 8, 8), 12)
    rc = cu.xfdtd_create(C.addressof(plan), C.byref(h))
    assert rc == 1
    assert b"at least 2 cells" in cu.xfdtd_last_error(h)
    cu.xfdtd_destroy.argtypes = [C.c_void_p]
    cu.xfdtd_destroy(h)


def test_scene_errors_surface_as_exceptions(libs):
    sc = S.Scene(1e-3, [S.Object("o", S.Sphere([0, 0, 0], 1e-3), S.Material("m", 1, 1, 0, 0))])
    sc.objects.append(S.ThinWire("w", S.Cylinder(S.AXIS_Z, [0, 0, 0], 0.9e-3, 1e-3)))
    with pytest.raises(X.EngineError, match="not enough thin"):
        X.Simulation(sc, 10)


def test_plan_struct_layout_matches_header():
    """The ctypes mirror of xfdtd_scene.h has the C layout (sizes checked
    against a compiled probe of the header)."""
    import subprocess
    import tempfile
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "xfdtd_scene.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(xfdtd_scene_desc), sizeof(xfdtd_object_desc),
         sizeof(xfdtd_waveform_desc), sizeof(xfdtd_pml_desc), sizeof(xfdtd_tfsf_desc),
         sizeof(xfdtd_nffft_desc), sizeof(xfdtd_lumped_desc), sizeof(xfdtd_monitor_desc),
         sizeof(xfdtd_port_desc));
  printf("%zu %zu %zu\n", sizeof(xfdtd_material_desc), offsetof(xfdtd_material_desc, dispersion),
         offsetof(xfdtd_material_desc, p));
  printf("%zu %zu %zu %zu %zu %zu %zu\n", offsetof(xfdtd_monitor_desc, component),
         offsetof(xfdtd_monitor_desc, plot_step), offsetof(xfdtd_monitor_desc, total_time_steps),
         offsetof(xfdtd_scene_desc, n_ports), offsetof(xfdtd_scene_desc, ports),
         offsetof(xfdtd_scene_desc, network_freqs), offsetof(xfdtd_port_desc, voltage_monitor));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        sizes = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    mine = [C.sizeof(t) for t in (S.SceneDesc, S.ObjectDesc, S.WaveformDesc, S.PMLDesc, S.TFSFDesc,
                                  S.NFFFTDesc, S.LumpedDesc, S.MonitorDesc, S.PortDesc)]
    mine += [C.sizeof(S.MaterialDesc), S.MaterialDesc.dispersion.offset, S.MaterialDesc.p.offset]
    mine += [S.MonitorDesc.component.offset, S.MonitorDesc.plot_step.offset, S.MonitorDesc.total_time_steps.offset,
             S.SceneDesc.n_ports.offset, S.SceneDesc.ports.offset, S.SceneDesc.network_freqs.offset,
             S.PortDesc.voltage_monitor.offset]
    assert sizes == mine


def test_scene_desc_carries_field_monitors_network_and_broadband():
    """The scene description of the field and movie monitors, the network
    (ports name their monitors by list index) and the broadband NF-FF."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import scenes
    sc, st = scenes.field_monitors(steps=30)
    d = sc.desc()
    kinds = [d.monitors[q].kind for q in range(d.n_monitors)]
    assert kinds == [S.MONITOR_VOLTAGE, S.MONITOR_FIELD, S.MONITOR_FIELD, S.MONITOR_FIELD, S.MONITOR_VOLTAGE]
    movie = d.monitors[1]
    assert (movie.component, movie.plane_type, movie.plot_step, movie.total_time_steps) == (S.EZ, S.PLANE_XY, 6, 30)
    plain = d.monitors[2]
    assert (plain.component, plain.plane_type, plain.plot_step) == (S.HY, S.PLANE_YZ, 0)
    assert d.monitors[3].total_time_steps == 27 and d.monitors[3].plot_step == 7
    with pytest.raises(ValueError):
        S.MovieMonitor(sc.monitors[0], 10)   # only over a field monitor
    sc, st = scenes.two_port(steps=40)
    d = sc.desc()
    assert d.n_ports == 2 and d.n_network_freqs == 4
    assert [(d.ports[q].voltage_monitor, d.ports[q].current_monitor) for q in range(2)] == [(0, 2), (3, 4)]
    assert d.ports[1].impedance_re == 100.0 and d.ports[1].impedance_im == 5.0 and d.ports[0].is_activated_source == 1
    assert [d.network_freqs[q] for q in range(4)] == [1e9, 3e9, 6e9, 9e9]
    sc.network.ports[0].voltage = S.VoltageMonitor(S.Cube([0, 0, 0], [1, 1, 1]), S.ZP)   # not in the list
    with pytest.raises(ValueError):
        sc.desc()
    from xfdtd_gb300 import configs
    sc, _ = configs.pec_sphere_rcs(scale=2, steps=20)
    sc.nffft = S.NffftBroadBand(4, 5, 6, 0.3, 0.7)
    d = sc.desc()
    assert d.nffft.enabled == 2 and d.nffft.n_theta == 1 and d.nffft.n_phi == 1 and d.nffft.n_freq == 0
    assert (d.nffft.theta[0], d.nffft.phi[0]) == (0.3, 0.7) and list(d.nffft.distance) == [4, 5, 6]


def test_batch_rejects_empty_member_list_on_the_host(libs):
    cu, _ = libs
    cu.xfdtd_batch_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    cu.xfdtd_batch_last_error.argtypes = [C.c_void_p]
    cu.xfdtd_batch_last_error.restype = C.c_char_p
    cu.xfdtd_batch_destroy.argtypes = [C.c_void_p]
    b = C.c_void_p()
    assert cu.xfdtd_batch_create(None, 0, 0, C.byref(b)) == 1
    assert b"at least one member" in cu.xfdtd_batch_last_error(b)
    cu.xfdtd_batch_destroy(b)
    members = (C.c_void_p * 2)(None, None)
    assert cu.xfdtd_batch_create(members, 2, 0, C.byref(b)) == 1
    assert b"not a created handle" in cu.xfdtd_batch_last_error(b)
    cu.xfdtd_batch_destroy(b)
