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
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(xfdtd_scene_desc), sizeof(xfdtd_object_desc),
         sizeof(xfdtd_waveform_desc), sizeof(xfdtd_pml_desc), sizeof(xfdtd_tfsf_desc),
         sizeof(xfdtd_nffft_desc), sizeof(xfdtd_lumped_desc), sizeof(xfdtd_monitor_desc));
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
                                  S.NFFFTDesc, S.LumpedDesc, S.MonitorDesc)]
    assert sizes == mine


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
