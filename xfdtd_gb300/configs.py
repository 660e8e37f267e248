"""Seeded synthetic scenes with the shapes of the benchmark configurations.

Every builder returns (Scene, total_steps).  `scale` shrinks the interior
(cell counts are divided by it, CPML and TFSF / NF-FF offsets are kept) so
that the same scene family can be run at sizes the CPU oracle finishes in
seconds.

  pec_sphere_rcs      3-D PEC sphere bistatic RCS: 40^3 interior + 8-cell
                      CPML (56^3), dx = 5 mm, sphere r = 10 cells, TFSF 4
                      cells inside the CPML, x-polarised +z Gaussian
                      (tau = 30 dt, t0 = 4.5 tau), dt = 0.98 x CFL, 800
                      steps, NF-FF 2 cells inside the TFSF box at 1 GHz,
                      361 angles over the phi = 0 great circle.
  dielectric_sphere   256^3 interior + 12-cell CPML (280^3), dx = 2 mm,
                      eps_r = 4 sphere of radius 60 cells, tau = 40 dt,
                      2000 steps, NF-FF at 1, 2, 3 GHz, 181 angles in the
                      phi = 0 and phi = 90 deg planes.
  heterogeneous       512x512x384 + 10-cell CPML, dx = 1 mm, per-voxel
                      material from a 256-entry table (eps_r U[1,6] as
                      float, sigma U[0, 0.01] S/m; seeds 1001/1002), soft
                      z-directed point current source at the centre
                      (Gaussian-modulated sine, f0 = 10 GHz, 5 GHz
                      bandwidth), 64 Ez probes at seeded cells (seed 1003),
                      1000 steps.
  batched_scatterers  64 uneven dielectric-sphere problems (interior 32 ..
                      160 cells per axis, 8-cell CPML, 500 .. 1500 steps),
                      run together as one batch.
"""
from __future__ import annotations

import math

import numpy as np

from . import scene as S


def cfl_dt(dl: float, cfl: float) -> float:
    """dt of FDTDBasicCoff::calculateDeltaT (fdtd_basic_coff.cpp:342-346) for
    a cubic cell; cfl passes through float as in Simulation(..., float cfl)."""
    c = float(np.float32(cfl))
    return c / (S.C_0 * math.sqrt(3.0 / (dl * dl)))


def _six_pml(t: int):
    return [S.PML(o, t) for o in (S.XN, S.XP, S.YN, S.YP, S.ZN, S.ZP)]


def pec_sphere_rcs(scale: int = 1, steps: int = 800):
    dl = 5e-3
    half = 20 // scale
    cpml = 8
    objects = [
        S.Object("domain", S.Cube([-half * dl] * 3, [2 * half * dl] * 3), S.Material("air", 1, 1, 0, 0)),
        S.Object("scatter", S.Sphere([0, 0, 0], (10 // scale) * dl), S.Material("pec", 1, 1, 1e10, 0)),
    ]
    dt = cfl_dt(dl, 0.98)
    tau = 30 * dt
    t0 = 4.5 * tau
    d_tfsf = cpml + 4
    tfsf = S.TFSF3D(d_tfsf, d_tfsf, d_tfsf, 1.0, 0.0, 0.0, 0.0, S.GaussianWaveform(1.0, tau, t0))
    theta = np.linspace(0.0, 2 * math.pi, 361)
    nffft = S.NffftFd(d_tfsf + 2, d_tfsf + 2, d_tfsf + 2, [1e9], theta, [0.0], "pec_sphere_rcs")
    sc = S.Scene(dl, objects, _six_pml(cpml), tfsf=tfsf, nffft=nffft, cfl=0.98)
    return sc, steps


def dielectric_sphere(scale: int = 1, steps: int = 2000, n_theta: int = 181):
    dl = 2e-3
    half = 128 // scale
    cpml = 12
    objects = [
        S.Object("domain", S.Cube([-half * dl] * 3, [2 * half * dl] * 3), S.Material("air", 1, 1, 0, 0)),
        S.Object("sphere", S.Sphere([0, 0, 0], (60 // scale) * dl), S.Material("dielectric", 4.0, 1, 0, 0)),
    ]
    dt = cfl_dt(dl, 0.98)
    tau = 40 * dt
    t0 = 4.5 * tau
    d_tfsf = cpml + 4
    tfsf = S.TFSF3D(d_tfsf, d_tfsf, d_tfsf, 1.0, 0.0, 0.0, 0.0, S.GaussianWaveform(1.0, tau, t0))
    theta = np.linspace(0.0, math.pi, n_theta)
    nffft = S.NffftFd(d_tfsf + 2, d_tfsf + 2, d_tfsf + 2, [1e9, 2e9, 3e9], theta, [0.0, math.pi / 2],
                      "dielectric_sphere")
    sc = S.Scene(dl, objects, _six_pml(cpml), tfsf=tfsf, nffft=nffft, cfl=0.98)
    return sc, steps


def heterogeneous(scale: int = 1, steps: int = 1000, n_probes: int = 64):
    dl = 1e-3
    cpml = 10
    interior = (512 // scale, 512 // scale, 384 // scale)
    n = tuple(v + 2 * cpml for v in interior)
    objects = [S.Object("domain", S.Cube([0.0, 0.0, 0.0], [v * dl for v in interior]),
                        S.Material("air", 1, 1, 0, 0))]
    rng_t = np.random.default_rng(1001)
    eps = rng_t.uniform(1.0, 6.0, 256).astype(np.float32)
    sig = rng_t.uniform(0.0, 0.01, 256)
    mats = [S.Material(f"m{i}", float(eps[i]), 1.0, float(sig[i]), 0.0) for i in range(256)]
    rng_v = np.random.default_rng(1002)
    voxel = rng_v.integers(0, 256, size=n, dtype=np.uint16)
    dt = cfl_dt(dl, 0.99)
    f0 = 10e9
    tau = 2.0 / (math.pi * 5e9)
    t0 = 4.5 * tau
    src_cell = [v // 2 for v in interior]
    src = S.CurrentSource(S.Cube([c * dl for c in src_cell], [dl, dl, dl]), S.ZP, 1e30,
                          S.CustomWaveform(1.0, S.gaussian_modulated_sine(f0, tau, t0)))
    rng_p = np.random.default_rng(1003)
    probes = []
    for _ in range(n_probes):
        c = [int(rng_p.integers(0, v)) for v in interior]
        probes.append(S.VoltageMonitor(S.Cube([q * dl for q in c], [dl, dl, dl]), S.ZP))
    sc = S.Scene(dl, objects, _six_pml(cpml), lumped_elements=[src], monitors=probes, cfl=0.99,
                 voxel_materials=mats, voxel_index=voxel)
    del dt
    return sc, steps


def batched_scatterers(n: int = 64, scale: int = 1, seed0: int = 4000, n_theta: int = 19):
    """`n` independent scatterer problems with uneven grids (problem i seeded
    with seed0 + i): interior dims uniform in 32 .. 160 cells per axis,
    8-cell CPML, dx = 2 mm, a dielectric sphere of radius 20-40 % of the
    smallest dimension with eps_r uniform in [2, 8] (as float) at the
    centre, TFSF 4 cells inside the CPML (x-polarised +z Gaussian, tau =
    30 dt, t0 = 4.5 tau), NF-FF 6 cells inside the CPML at 1 GHz, steps
    uniform in 500 .. 1500.  Returns a list of (Scene, total_steps); `scale`
    divides the interior dims and the steps."""
    dl = 2e-3
    cpml = 8
    out = []
    for i in range(n):
        rng = np.random.default_rng(seed0 + i)
        dims = [int(v) // scale for v in rng.integers(32, 161, size=3)]
        radius = float(rng.uniform(0.2, 0.4)) * min(dims)
        eps = float(np.float32(rng.uniform(2.0, 8.0)))
        steps = int(rng.integers(500, 1501)) // scale
        objects = [
            S.Object("domain", S.Cube([0.0, 0.0, 0.0], [v * dl for v in dims]), S.Material("air", 1, 1, 0, 0)),
            S.Object("sphere", S.Sphere([v * dl / 2 for v in dims], radius * dl), S.Material("d", eps, 1, 0, 0)),
        ]
        dt = cfl_dt(dl, 0.98)
        tau = 30 * dt
        tfsf = S.TFSF3D(cpml + 4, cpml + 4, cpml + 4, 1.0, 0.0, 0.0, 0.0, S.GaussianWaveform(1.0, tau, 4.5 * tau))
        nffft = S.NffftFd(cpml + 6, cpml + 6, cpml + 6, [1e9], np.linspace(0.0, math.pi, n_theta), [0.0],
                          f"batched_{i}")
        out.append((S.Scene(dl, objects, _six_pml(cpml), tfsf=tfsf, nffft=nffft, cfl=0.98), steps))
    return out


def adjoint_dipole(scale: int = 1, steps: int = 2000, seed: int = 5001):
    """Adjoint-gradient problem: 160 x 160 x 96 interior + 10-cell CPML,
    dx = 50 nm, a z-directed soft point current source (Gaussian-modulated
    sine, f0 = c0 / (12 dx), bandwidth f0 / 2) 20 cells below a 64 x 64 x 32
    design region whose eps_r is 2.5 + U[-0.5, 0.5] clamped to [1, 4]
    (seed 5001), loss plane 20 cells above it.  `scale` divides every
    length in cells and the step count.  Returns (Scene, total_steps, spec)
    with spec = the design box, loss plane and window in grid indices."""
    dl = 50e-9
    cpml = 10
    interior = (160 // scale, 160 // scale, 96 // scale)
    dsz = (64 // scale, 64 // scale, 32 // scale)
    gap = 20 // scale
    steps = steps // scale
    n = tuple(v + 2 * cpml for v in interior)
    lo = (cpml + (interior[0] - dsz[0]) // 2, cpml + (interior[1] - dsz[1]) // 2, cpml + (interior[2] - dsz[2]) // 2)
    hi = tuple(a + b for a, b in zip(lo, dsz))
    rng = np.random.default_rng(seed)
    eps = np.clip(2.5 + rng.uniform(-0.5, 0.5, size=dsz), 1.0, 4.0).astype(np.float32)
    mats = [S.Material("air", 1.0, 1.0, 0.0, 0.0)] + [S.Material("d", float(e), 1.0, 0.0, 0.0) for e in eps.ravel()]
    voxel = np.zeros(n, dtype=np.uint32)
    voxel[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] = (1 + np.arange(eps.size, dtype=np.uint32)).reshape(dsz)
    objects = [S.Object("domain", S.Cube([0.0, 0.0, 0.0], [v * dl for v in interior]), S.Material("air", 1, 1, 0, 0))]
    f0 = S.C_0 / (12 * dl)
    tau = 2.0 / (math.pi * 0.5 * f0)
    t0 = 4.5 * tau
    src_cell = ((lo[0] + hi[0]) // 2 - cpml, (lo[1] + hi[1]) // 2 - cpml, lo[2] - gap - cpml)
    src = S.CurrentSource(S.Cube([c * dl for c in src_cell], [dl, dl, dl]), S.ZP, 1e30,
                          S.CustomWaveform(1.0, S.gaussian_modulated_sine(f0, tau, t0)))
    sc = S.Scene(dl, objects, _six_pml(cpml), lumped_elements=[src], cfl=0.98,
                 voxel_materials=mats, voxel_index=voxel)
    spec = {"design_lo": lo, "design_hi": hi, "plane_axis": 2, "plane_index": hi[2] + gap,
            "plane_lo": (lo[0], lo[1]), "plane_hi": (hi[0], hi[1]),
            "t_begin": steps - steps // 5, "t_end": steps, "loss_comp": 2,
            "checkpoint_every": 100 // scale, "eps": eps}
    return sc, steps, spec


def cylinder_2d(scale: int = 1, steps: int = 1400, pec: bool = True):
    """The reference's 2-D example (examples/2d_cylinder_scatter.cpp:29-98):
    a 350 x 300-cell TMz grid (nz = 1) plus a 10-cell CPML on the four x and
    y faces, dx = (c / 20 GHz) / 20, a cylinder of radius 0.03 m (40 cells)
    along z at the centre (PEC as sigma = 1e24, or eps_r = 3 with `pec`
    False), TFSF2D 50 cells from the domain edge at phi = pi / 4 with a
    cosine-modulated Gaussian (12 GHz, tau = 1.7 / 8 GHz, t0 = 0.8 tau),
    cfl 0.8, 1400 steps.  `scale` divides the cell counts, the radius in
    cells and the TFSF offset beyond the CPML."""
    dx = (3e8 / 20e9) / 20
    nx, ny = 350 // scale, 300 // scale
    pml = 10
    tau = 1.7 / (20e9 - 12e9)
    t0 = 0.8 * tau
    radius = (0.03 / dx) // scale * dx
    objects = [
        S.Object("free_space", S.Cube([0.0, 0.0, 0.0], [nx * dx, ny * dx, 0.0]), S.Material("air", 1, 1, 0, 0)),
        S.Object("objectA", S.Cylinder(S.AXIS_Z, [nx * 0.5 * dx, ny * 0.5 * dx, 0.0], radius, 0.0),
                 S.Material("pec", 1, 1, 1e24, 0) if pec else S.Material("d", 3.0, 1, 0, 0)),
    ]
    boundaries = [S.PML(o, pml) for o in (S.XN, S.XP, S.YN, S.YP)]
    d_tfsf = pml + max(40 // scale, 4)
    tfsf = S.TFSF2D(d_tfsf, d_tfsf, math.pi * 0.25, 1.0, S.CosineModulatedGaussianWaveform(1.0, tau, t0, 12e9))
    return S.Scene(dx, objects, boundaries, tfsf=tfsf, cfl=0.8), steps


CONFIGS = {
    "pec_sphere_rcs": pec_sphere_rcs,
    "dielectric_sphere": dielectric_sphere,
    "heterogeneous": heterogeneous,
}
