"""The C++ drop-in: drivers written against the reference's C++ API compile
against xfdtd_gb300/host/include/xfdtd/xfdtd.h, link to libxfdtd.so and run
on the GPU engine.

* tests/drivers/pec_sphere_bistatic_rcs.cpp, a driver in the reference's
  style (the scene of examples/3d_pec_sphere_bistatic_rcs.cpp), compiles
  and links here; on a GPU it runs the example's 500 steps and its .npy
  outputs match the FP64 oracle within 1e-10 (FP32: RCS within 0.05 dB).
* Where the reference's sources are mounted, its own example
  examples/3d_pec_sphere_bistatic_rcs.cpp, with the three edits the
  integration notes name (one include for the reference's headers,
  xt::xarray<double> -> std::vector<double>, xt::linspace ->
  xfdtd::linspace), compiles and links too.  It is edited into a temporary
  directory, never into the repository.
"""
import math
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import xfdtd_gb300 as X
from xfdtd_gb300 import scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "drivers", "pec_sphere_bistatic_rcs.cpp")
REFERENCE_EXAMPLE = "/root/reference/examples/3d_pec_sphere_bistatic_rcs.cpp"


def _compile(src, exe, extra_inc=()):
    X.build()
    lib = os.path.join(ROOT, "xfdtd_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O1", src, "-I", os.path.join(ROOT, "xfdtd_gb300", "host", "include"),
           "-I", os.path.join(ROOT, "include")]
    for d in extra_inc:
        cmd += ["-I", d]
    cmd += ["-L", lib, "-lxfdtd", f"-Wl,-rpath,{lib}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_driver_compiles_and_links():
    with tempfile.TemporaryDirectory() as d:
        _compile(DRIVER, os.path.join(d, "drv"))


def _edit_reference_example(text):
    """The three documented edits."""
    lines = []
    included = False
    for line in text.splitlines():
        m = re.match(r'\s*#include\s+"([^"]+)"', line)
        if m and m.group(1) != "helper.h":
            if not included:
                lines.append("#include <xfdtd/xfdtd.h>")
                included = True
            continue
        lines.append(line)
    out = "\n".join(lines) + "\n"
    out = out.replace("xt::xarray<double>", "std::vector<double>")
    out = out.replace("xt::linspace", "xfdtd::linspace")
    return out


@pytest.mark.skipif(not os.path.exists(REFERENCE_EXAMPLE), reason="the reference's sources are not mounted here")
def test_reference_example_compiles_with_the_documented_edits():
    with open(REFERENCE_EXAMPLE) as f:
        text = f.read()
    edited = _edit_reference_example(text)
    assert "xt::" not in edited
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "example.cpp")
        with open(src, "w") as f:
            f.write(edited)
        _compile(src, os.path.join(d, "example"), extra_inc=[os.path.dirname(REFERENCE_EXAMPLE)])


def _scene():
    """The driver's scene, built with the Python mirror for the oracle."""
    dl = 7.5e-3
    corner, extent = -40 * dl, 80 * dl
    objects = [S.Object("domain", S.Cube([corner] * 3, [extent] * 3), S.Material("air", 1, 1, 0, 0)),
               S.Object("scatter", S.Sphere([0, 0, 0], 0.1), S.Material("pec", 1, 1, 1e10, 0))]
    boundaries = [S.PML(o, 12) for o in (S.XN, S.XP, S.YN, S.YP, S.ZN, S.ZP)]
    tau = 20 * dl / 6e8
    tfsf = S.TFSF3D(27, 27, 27, 1.0, 0.0, 0.0, 0.0, S.GaussianWaveform(1.0, tau, 4.5 * tau))
    step = math.pi / 180
    theta = np.array([0.0 + i * step for i in range(180)])
    nffft = S.NffftFd(17, 17, 17, [1e9], theta, [0.0], "")
    return S.Scene(dl, objects, boundaries, tfsf=tfsf, nffft=nffft, cfl=1.0)


@pytest.mark.gpu
def test_driver_runs_and_matches_the_oracle(tmp_path):
    import oracle as O
    steps = 500
    exe = str(tmp_path / "drv")
    _compile(DRIVER, exe)
    out64, out32 = tmp_path / "fp64", tmp_path / "fp32"
    for out, extra in ((out64, []), (out32, ["fp32"])):
        r = subprocess.run([exe, str(out), str(steps)] + extra, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
    sc = _scene()
    o = O.OracleSim(sc, steps)
    o.step(steps)
    names = ["e_theta", "e_phi", "h_theta", "h_phi", "n_theta", "n_phi", "l_theta", "l_phi", "power_theta",
             "power_phi"]
    for w, name in enumerate(names):
        got = np.load(out64 / f"{name}.npy")
        want = o.far_field(w)
        assert got.shape == want.shape, (name, got.shape, want.shape)
        scale = np.abs(want).max()
        assert scale > 0
        assert np.abs(got - want).max() / scale <= 1e-10, name
    assert np.array_equal(np.load(out64 / "theta.npy"), sc.nffft.theta)
    # FP32 form: RCS (from the written far field and the oracle's incident DFT) within 0.05 dB
    inc = o.incident_dft([1e9])
    rcs = lambda et, ep: 10 * np.log10(4 * np.pi * (np.abs(et) ** 2 + np.abs(ep) ** 2) / np.abs(inc[0]) ** 2)
    want = rcs(o.far_field(0), o.far_field(1))
    got = rcs(np.load(out32 / "e_theta.npy"), np.load(out32 / "e_phi.npy"))
    assert np.abs(got - want).max() < 0.05
