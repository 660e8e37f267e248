"""Pins the CPU oracle (FP64 restatement of the reference) before the GPU
engine is tested against it.

* test/test_grid.cpp of the reference, restated: uniform GridSpace counts
  and node sizes for seeded random cubes.
* Analytic facts of the reference's algorithm: exact TFSF cancellation for
  normal incidence, CPML absorption, and the PEC-sphere bistatic RCS against
  a Mie series within the ~1 dB the reference's readme reports
  (readme.md: "average error of 1dB").
* Committed golden vectors (tests/golden, made by make_golden.py).
"""
import math
import os

import numpy as np
import pytest

import mie
import oracle as O
import scenes
from xfdtd_gb300 import configs
from xfdtd_gb300 import scene as S

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _threads():
    O.set_threads(min(8, os.cpu_count() or 1))


def test_grid_space_matches_reference_test_grid():
    """test/test_grid.cpp:12-91: for random cubes with dl = size/20 the grid
    has 20 cells per axis and every node size equals dl within 10 eps."""
    rng = np.random.default_rng(20240)
    for _ in range(10):
        origin = rng.uniform(0, 1, 3)
        size_x = rng.uniform(0, 1)
        dl = size_x / 20.0
        n, sizes = O.grid_from_cube(origin, [size_x] * 3, dl)
        assert n == (20, 20, 20)
        for key in ("esx", "esy", "esz"):
            assert np.all(np.abs(sizes[key] - dl) <= 10 * np.finfo(float).eps), key
        for key in ("hsx", "hsy", "hsz"):
            assert sizes[key].shape == (21,)
            assert np.all(np.abs(sizes[key] - dl) <= 10 * np.finfo(float).eps), key


def test_2d_grid_time_step_and_tfsf2d_cancellation():
    """The 2-D (nz = 1) TMz path: a zero-thickness domain gives nz = 1 and
    the 2-D time step cfl / (c0 sqrt(1/dx^2 + 1/dy^2))
    (fdtd_basic_coff.cpp:19-21, 348-351); TFSF2D at phi = pi / 4 with
    dx = dy leaves the scattered-field region empty to rounding (the
    1-D line's numerical dispersion matches the grid's along the diagonal),
    carries the plane wave (|Ez| ~ e0) inside the box, and the TE
    components stay exactly zero."""
    sc, st = configs.cylinder_2d(scale=5, steps=200)
    sc.objects = sc.objects[:1]
    o = O.OracleSim(sc, st)
    assert o.n == (90, 80, 1)
    dx = sc.cell_size
    want_dt = float(np.float32(0.8)) / (S.C_0 * math.sqrt(2.0 / (dx * dx)))
    assert o.dt == pytest.approx(want_dt, rel=1e-15)
    o.step(st)
    ez = o.read_field(S.EZ)[:, :, 0]
    d = sc.tfsf.distance_x
    inside = np.abs(ez[d + 2:-d - 2, d + 2:-d - 2]).max()
    m = ez.copy()
    m[d - 1:-d + 1, d - 1:-d + 1] = 0
    assert 0.9 < inside < 1.1, inside
    assert np.abs(m).max() < 1e-12 * inside
    for c in (S.EX, S.EY, S.HZ):
        assert not np.any(o.read_field(c)), c


@pytest.mark.parametrize("kind", ["lorentz", "drude", "debye"])
def test_dispersive_media_reduce_to_the_plain_dielectric(kind):
    """The linear dispersive media's E recursions
    (src/material/dispersive_material.cpp) with no pole (Lorentz omega_p =
    0, Drude omega_p = 0, Debye eps_s = eps_inf) give the fields of a plain
    sphere of eps_r = eps_inf (to rounding: the recursions group the terms
    otherwise); with a pole they differ from it."""
    sc, st = scenes.dispersive(kind, steps=120, limit=True)
    o = O.OracleSim(sc, st)
    o.step(st)
    sc_p, _ = scenes.dispersive(kind, steps=120, limit=True)
    sc_p.objects[1] = S.Object("p", sc_p.objects[1].shape, S.Material("p", 2.5, 1, 0.01, 0))
    p = O.OracleSim(sc_p, st)
    p.step(st)
    scale = max(np.abs(p.read_field(c)).max() for c in range(3))
    for c in range(6):
        assert np.abs(o.read_field(c) - p.read_field(c)).max() <= 1e-12 * scale, c
    sc_d, _ = scenes.dispersive(kind, steps=120)
    d = O.OracleSim(sc_d, st)
    d.step(st)
    assert np.abs(d.read_field(S.EX) - p.read_field(S.EX)).max() > 1e-3 * scale
    assert all(np.isfinite(d.read_field(c)).all() for c in range(6))


def test_exact_eps_material():
    """A material with its eps_r kept in double (XFDTD_MATERIAL_EXACT_EPS)
    gives the float material's fields when the value is a float, and moves
    them when it is not (the float ctor would round 2.5 + 1e-7 to 2.5)."""
    def fields(mat):
        sc, st = scenes.dispersive("lorentz", steps=60, limit=True)
        sc.objects[1] = S.Object("p", sc.objects[1].shape, mat)
        o = O.OracleSim(sc, st)
        o.step(st)
        return [o.read_field(c) for c in range(6)]
    f = fields(S.Material("p", 2.5, 1, 0.01, 0))
    e = fields(S.Material("p", 2.5, 1, 0.01, 0, exact_eps=True))
    assert all(np.array_equal(a, b) for a, b in zip(f, e))
    assert float(np.float32(2.5 + 1e-7)) == 2.5
    d = fields(S.Material("p", 2.5 + 1e-7, 1, 0.01, 0, exact_eps=True))
    assert max(np.abs(a - b).max() for a, b in zip(f, d)) > 0


def test_tfsf_normal_incidence_cancels_outside_box():
    sc, _ = configs.pec_sphere_rcs(scale=2, steps=260)
    sc.objects = sc.objects[:1]
    o = O.OracleSim(sc, 260)
    inside = outside = 0.0
    d = sc.tfsf.distance_x
    for _ in range(13):
        o.step(20)
        ex = o.read_field(S.EX)
        inside = max(inside, np.abs(ex[d + 1:-d - 1, d + 1:-d - 1, d + 1:-d - 1]).max())
        m = ex.copy()
        m[d - 1:-d + 1, d - 1:-d + 1, d - 1:-d + 1] = 0
        outside = max(outside, np.abs(m).max())
    assert inside > 0.99
    assert outside < 1e-12 * inside


def test_tfsf_oblique_incidence_leakage_small():
    sc, st = scenes.oblique(steps=220)
    sc.objects = sc.objects[:1]
    o = O.OracleSim(sc, st)
    o.step(st)
    ey = o.read_field(S.EY)
    d = sc.tfsf.distance_x
    m = ey.copy()
    m[d - 1:-d + 1, d - 1:-d + 1, d - 1:-d + 1] = 0
    # the 1-D auxiliary grid does not match the 3-D grid's dispersion exactly:
    # a leakage of a few percent of the incident amplitude is the method's own
    assert np.abs(m).max() < 0.05 * sc.tfsf.e_0


def test_cpml_absorbs_outgoing_wave():
    """A soft point source radiates in a box with a CPML of T cells 12 cells
    away; a probe 8 cells out is compared with the same probe in a box 40
    cells wide, over the window before that box's own walls answer.  The
    reflection falls with T (about -21, -30, -41 dB for T = 6, 10, 16 with
    the reference's default CPML parameters)."""
    def run(half, t_pml, steps=150):
        dl = 1e-3
        objects = [S.Object("air", S.Cube([-half * dl] * 3, [2 * half * dl] * 3), S.Material("air", 1, 1, 0, 0))]
        src = S.CurrentSource(S.Cube([0, 0, 0], [dl, dl, dl]), S.ZP, 1e30,
                              S.CustomWaveform(1.0, S.gaussian_modulated_sine(30e9, 15e-12, 60e-12)))
        mon = S.VoltageMonitor(S.Cube([8 * dl, 0, 0], [dl, dl, dl]), S.ZP)
        sc = S.Scene(dl, objects, [S.PML(o_, t_pml) for o_ in range(6)], lumped_elements=[src], monitors=[mon])
        o = O.OracleSim(sc, steps)
        o.step(steps)
        return o.read_monitor(0)
    big = run(40, 10)
    refl = {}
    for t_pml in (6, 10, 16):
        small = run(12, t_pml)
        refl[t_pml] = 20 * math.log10(np.abs(small - big).max() / np.abs(big).max())
    assert refl[10] < -25
    assert refl[16] < refl[10] < refl[6]
    assert refl[6] - refl[16] > 15


def test_pec_sphere_rcs_against_mie():
    sc, st = configs.pec_sphere_rcs()
    o = O.OracleSim(sc, st)
    o.step(st)
    rcs = o.rcs_db()[0, :, 0]
    theta = np.linspace(0, 2 * np.pi, 361)
    th = np.where(theta > np.pi, 2 * np.pi - theta, theta)
    se, _ = mie.pec_sphere_rcs(0.05, 1e9, th)
    err = np.abs(rcs - 10 * np.log10(se))
    assert err.mean() < 1.5, err.mean()   # the reference reports ~1 dB on average
    assert err.max() < 3.0


def test_broadband_backscatter_against_mie():
    """The NffftBroadBand restatement (nffft_broadband.cpp) pinned by
    physics: the PEC sphere's monostatic RCS from its far field at theta =
    pi, 4 pi (|E_theta|^2 + |E_phi|^2) dt^2 / |E_inc(f)|^2 (the transform
    carries no dt; the incident DFT does), within 1 dB of the Mie series at
    every bin from 0.5 to 1.4 GHz (the sphere is 10 staircased cells in
    radius)."""
    sc, st = configs.pec_sphere_rcs(scale=1, steps=500)
    nf = sc.nffft
    sc.nffft = S.NffftBroadBand(nf.distance_x, nf.distance_y, nf.distance_z, math.pi, 0.0)
    o = O.OracleSim(sc, st)
    o.step(st)
    f = o.far_field(10)
    sel = np.nonzero((f >= 0.5e9) & (f <= 1.4e9))[0]
    assert len(sel) >= 8
    et, ep = o.far_field(0)[sel], o.far_field(1)[sel]
    inc = o.incident_dft(f[sel])
    sigma = 4 * np.pi * (np.abs(et * o.dt) ** 2 + np.abs(ep * o.dt) ** 2) / np.abs(inc) ** 2
    for fq, sg in zip(f[sel], sigma):
        se, _ = mie.pec_sphere_rcs(0.05, fq, np.array([np.pi]))
        assert abs(10 * np.log10(sg) - 10 * np.log10(se[0])) < 1.0, fq


@pytest.mark.parametrize("name", sorted(scenes.SCENES))
def test_oracle_matches_golden(name):
    path = os.path.join(GOLDEN, f"{name}.npz")
    g = np.load(path)
    sc, _ = scenes.SCENES[name]()
    steps = int(g["steps"])
    o = O.OracleSim(sc, steps)
    o.step(steps)
    for c in range(6):
        f = o.read_field(c)
        np.testing.assert_allclose(f.sum(axis=(1, 2)), g[f"f{c}_xsum"], rtol=1e-12, atol=1e-300)
        np.testing.assert_allclose(f[f.shape[0] // 2], g[f"f{c}_slice"], rtol=1e-12, atol=1e-30)
    for m in range(len(sc.monitors)):
        np.testing.assert_allclose(o.read_monitor(m), g[f"m{m}"], rtol=1e-12, atol=1e-30)
    if sc.nffft is not None:
        for w in (0, 1, 8):
            np.testing.assert_allclose(o.far_field(w), g[f"ff{w}"], rtol=1e-10, atol=1e-30)


@pytest.mark.parametrize("name", sorted(scenes.OUTPUT_SCENES))
def test_oracle_output_formats_match_golden(name):
    """Every frame of the field and movie monitors and the broadband far
    field against their golden vectors."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    sc, _ = scenes.OUTPUT_SCENES[name]()
    steps = int(g["steps"])
    o = O.OracleSim(sc, steps)
    o.step(steps)
    for m, mon in enumerate(sc.monitors):
        if mon.kind != S.MONITOR_FIELD:
            continue
        _, _, frames = o.field_monitor_frames(m)
        assert frames == list(g[f"steps{m}"])
        for f in range(len(frames)):
            np.testing.assert_allclose(o.read_field_monitor(m, f), g[f"mon{m}_{f}"], rtol=1e-12, atol=1e-30)
    if sc.nffft is not None:
        for w in (0, 1, 8, 10):
            np.testing.assert_allclose(o.far_field(w), g[f"ff{w}"], rtol=1e-10, atol=1e-30)


def test_scene_description_round_trip():
    sc, st = scenes.lumped(steps=3)
    d = sc.desc()
    assert d.n_objects == 1 and d.n_pml == 6 and d.n_lumped == 5 and d.n_monitors == 5
    assert abs(d.cfl - 0.99) < 1e-7
    o = O.OracleSim(sc, st)
    assert o.n == (36, 36, 36)


def test_oracle_rejects_bad_scenes():
    sc, st = scenes.pec_sphere()
    sc.objects.append(S.ThinWire("fat", S.Cylinder(S.AXIS_Z, [0, 0, 0], 0.01, 0.05)))
    with pytest.raises(RuntimeError, match="not enough thin"):
        O.OracleSim(sc, st)
    sc2, _ = scenes.pec_sphere()
    with pytest.raises(RuntimeError):
        O.OracleSim(sc2, 0)


def test_oracle_field_and_movie_monitors():
    """TimeDomainFieldMonitor / MovieMonitor restated (field_monitor.cpp,
    movie_monitor.cpp:46-59): a movie frame after every step t with
    t % plot_step == 0 and after its last step, each the component's view
    of the field after that step; a plain field monitor is the view of the
    current field.  Checked against the oracle's own fields stepped one
    step at a time."""
    sc, st = scenes.field_monitors(steps=24)
    o = O.OracleSim(sc, st)
    o.step(st)
    ref = O.OracleSim(sc, st)
    views = {}
    for t in range(st):
        ref.step(1)
        for m in (1, 2, 3):
            lo, shape, _ = o.field_monitor_frames(m)
            c = sc.monitors[m].component
            f = ref.read_field(c)
            views[(m, t)] = f[lo[0]:lo[0] + shape[0], lo[1]:lo[1] + shape[1], lo[2]:lo[2] + shape[2]]
    lo, shape, steps = o.field_monitor_frames(1)
    assert steps == [0, 6, 12, 18, 23] and shape[2] == 1 and lo[2] > 0
    for f, t in enumerate(steps):
        assert np.array_equal(o.read_field_monitor(1, f), views[(1, t)])
    _, _, steps = o.field_monitor_frames(3)
    # total_time_steps 21: its last step, 20, falls between plot steps, and
    # the plot steps go on after it
    assert steps == [0, 7, 14, 20, 21]
    for f, t in enumerate(steps):
        assert np.array_equal(o.read_field_monitor(3, f), views[(3, t)])
    _, shape, steps = o.field_monitor_frames(2)
    assert steps == [-1] and shape[0] == 1
    assert np.array_equal(o.read_field_monitor(2, 0), views[(2, st - 1)])
    # the voltage monitors keep their time series around the field monitors
    assert np.abs(o.read_monitor(0)).max() > 0 and np.abs(o.read_monitor(4)).max() > 0


def test_oracle_field_monitor_rejects_thick_plane():
    """An XY field monitor more than one cell thick in z is an error
    (field_monitor.cpp:35-38)."""
    sc, st = scenes.field_monitors(steps=4)
    dl = sc.cell_size
    sc.monitors = [S.TimeDomainFieldMonitor(S.Cube([0, 0, 2 * dl], [4 * dl, 4 * dl, 3 * dl]), S.PLANE_XY, S.EX)]
    with pytest.raises(RuntimeError):
        O.OracleSim(sc, st)
