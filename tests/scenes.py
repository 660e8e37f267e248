"""Small seeded scenes shared by the CPU and GPU tests (test utility).

Each builder returns (Scene, steps) at a size the CPU oracle runs in seconds.
"""
import math

import numpy as np

from xfdtd_gb300 import configs
from xfdtd_gb300 import scene as S


def pec_sphere(scale=2, steps=300):
    return configs.pec_sphere_rcs(scale=scale, steps=steps)


def dielectric(scale=8, steps=300):
    return configs.dielectric_sphere(scale=scale, steps=steps, n_theta=19)


def heterogeneous(scale=16, steps=150, n_probes=8):
    return configs.heterogeneous(scale=scale, steps=steps, n_probes=n_probes)


def oblique(steps=250):
    """Dielectric sphere lit by an oblique plane wave (theta 30, phi 45, psi 60 deg)."""
    dl = 5e-3
    half = 12
    objects = [
        S.Object("domain", S.Cube([-half * dl] * 3, [2 * half * dl] * 3), S.Material("air", 1, 1, 0, 0)),
        S.Object("ball", S.Sphere([0.3 * dl, -0.2 * dl, 0.1 * dl], 5.5 * dl), S.Material("d", 3.5, 1.0, 0.02, 0.0)),
    ]
    dt = configs.cfl_dt(dl, 0.98)
    tau = 20 * dt
    tfsf = S.TFSF3D(10, 10, 10, 2.0, math.pi / 6, math.pi / 4, math.pi / 3,
                    S.GaussianWaveform(1.0, tau, 4.5 * tau))
    nffft = S.NffftFd(12, 12, 12, [2e9, 5e9], np.linspace(0, math.pi, 13), [0.0, 1.0], "oblique")
    boundaries = [S.PML(o, 6) for o in (S.XN, S.XP, S.YN, S.YP, S.ZN, S.ZP)]
    return S.Scene(dl, objects, boundaries, tfsf=tfsf, nffft=nffft, cfl=0.98), steps


def partial_pml(steps=200):
    """CPML on three faces only (the others stay PEC walls), asymmetric grid,
    cube and cylinder objects, non-default CPML parameters."""
    dl = 4e-3
    objects = [
        S.Object("domain", S.Cube([0, 0, 0], [20 * dl, 26 * dl, 17 * dl]), S.Material("air", 1, 1, 0, 0)),
        S.Object("block", S.Cube([5 * dl, 6 * dl, 4 * dl], [4 * dl, 7 * dl, 5 * dl]), S.Material("b", 2.2, 1.3, 0.05, 10.0)),
        S.Object("rod", S.Cylinder(S.AXIS_Y, [12 * dl, 13 * dl, 9 * dl], 2.6 * dl, 14 * dl),
                 S.Material("r", 5.0, 1.0, 0.0, 0.0)),
    ]
    boundaries = [S.PML(S.XN, 5, 3, 0.8, 0.01, 0.1, 6.0), S.PML(S.YP, 7), S.PML(S.ZN, 4, 2, 1.2, 0.0, 0.03, 12.0)]
    src = S.CurrentSource(S.Cube([10 * dl, 12 * dl, 8 * dl], [dl, dl, dl]), S.ZP, 50.0,
                          S.CosineModulatedGaussianWaveform(1e-3, 40e-12, 160e-12, 6e9))
    mons = [S.VoltageMonitor(S.Cube([14 * dl, 15 * dl, 6 * dl], [dl, dl, 3 * dl]), S.ZP),
            S.VoltageMonitor(S.Cube([8 * dl, 18 * dl, 10 * dl], [2 * dl, dl, dl]), S.XN)]
    return S.Scene(dl, objects, boundaries, lumped_elements=[src], monitors=mons, cfl=0.95), steps


def lumped(steps=300):
    """Voltage source, resistor, capacitor, inductor and current source in a
    CPML box, with voltage and current monitors."""
    dl = 1e-3
    objects = [S.Object("domain", S.Cube([0, 0, 0], [24 * dl, 24 * dl, 24 * dl]), S.Material("air", 1, 1, 0, 0))]
    boundaries = [S.PML(o, 6) for o in (S.XN, S.XP, S.YN, S.YP, S.ZN, S.ZP)]
    tau = 30e-12
    le = [
        S.VoltageSource(S.Cube([10 * dl, 10 * dl, 10 * dl], [dl, dl, 2 * dl]), S.ZP, 50.0,
                        S.GaussianWaveform(1.0, tau, 4.5 * tau)),
        S.Resistor(S.Cube([14 * dl, 10 * dl, 10 * dl], [dl, dl, 2 * dl]), S.AXIS_Z, 100.0),
        S.Capacitor(S.Cube([10 * dl, 14 * dl, 10 * dl], [2 * dl, dl, dl]), S.AXIS_X, 1e-12),
        S.Inductor(S.Cube([13 * dl, 14 * dl, 12 * dl], [dl, dl, 2 * dl]), S.AXIS_Z, 2e-9),
        S.CurrentSource(S.Cube([6 * dl, 16 * dl, 8 * dl], [2 * dl, 2 * dl, dl]), S.ZN, 1e3,
                        S.SinusoidalWaveform(1e-3, 8e9, 0.3)),
    ]
    mons = [
        S.VoltageMonitor(S.Cube([10 * dl, 10 * dl, 10 * dl], [dl, dl, 2 * dl]), S.ZP),
        S.VoltageMonitor(S.Cube([14 * dl, 10 * dl, 10 * dl], [dl, dl, 2 * dl]), S.ZN),
        S.CurrentMonitor(S.Cube([10 * dl, 10 * dl, 11 * dl], [dl, dl, 0]), S.ZP),
        S.CurrentMonitor(S.Cube([13 * dl, 14 * dl, 13 * dl], [dl, dl, 0]), S.ZN),
        S.CurrentMonitor(S.Cube([11 * dl, 14 * dl, 10 * dl], [0, dl, dl]), S.XP),
    ]
    return S.Scene(dl, objects, boundaries, lumped_elements=le, monitors=mons, cfl=0.99), steps


def thin_wire(steps=300):
    """A z-directed half-wave-style thin-wire dipole fed by a voltage source
    across its gap (the reference's examples/thin_wire.cpp layout), plus x-
    and y-directed wires (ThinWire, src/object/thin_wire.cpp)."""
    dl = 2e-3
    objects = [
        S.Object("domain", S.Cube([-12 * dl] * 3, [24 * dl] * 3), S.Material("air", 1, 1, 0, 0)),
        S.ThinWire("arm0", S.Cylinder(S.AXIS_Z, [0, 0, 4.5 * dl], 0.1 * dl, 7 * dl)),
        S.ThinWire("arm1", S.Cylinder(S.AXIS_Z, [0, 0, -4.5 * dl], 0.1 * dl, 7 * dl)),
        S.ThinWire("wx", S.Cylinder(S.AXIS_X, [0, 5 * dl, 5 * dl], 0.2 * dl, 8 * dl)),
        S.ThinWire("wy", S.Cylinder(S.AXIS_Y, [-5 * dl, 0, -4 * dl], 0.15 * dl, 6 * dl)),
    ]
    boundaries = [S.PML(o, 6) for o in (S.XN, S.XP, S.YN, S.YP, S.ZN, S.ZP)]
    tau = 40e-12
    le = [S.VoltageSource(S.Cube([0, 0, -dl], [dl, dl, 2 * dl]), S.ZP, 50.0, S.GaussianWaveform(1.0, tau, 4.5 * tau))]
    mons = [S.VoltageMonitor(S.Cube([0, 0, -dl], [dl, dl, 2 * dl]), S.ZP),
            S.CurrentMonitor(S.Cube([0, 0, 0], [dl, dl, dl]), S.ZP)]
    return S.Scene(dl, objects, boundaries, lumped_elements=le, monitors=mons, cfl=0.99), steps


def _boxed(dims, dl, boundaries, steps, cfl=0.97):
    """A box of `dims` cells with a dielectric block, a lossy cube and a
    soft current source off the centre, and one voltage monitor."""
    objects = [
        S.Object("domain", S.Cube([0, 0, 0], [v * dl for v in dims]), S.Material("air", 1, 1, 0, 0)),
        S.Object("block", S.Cube([v * dl * 0.3 for v in dims], [max(1, v // 3) * dl for v in dims]),
                 S.Material("b", 3.0, 1.0, 0.0, 0.0)),
        S.Object("lossy", S.Cube([v * dl * 0.6 for v in dims], [max(1, v // 5) * dl for v in dims]),
                 S.Material("l", 1.5, 1.2, 0.2, 0.0)),
    ]
    c = [max(1, int(v * 0.45)) for v in dims]
    src = S.CurrentSource(S.Cube([q * dl for q in c], [dl, dl, dl]), S.ZP, 1e3,
                          S.CosineModulatedGaussianWaveform(1e-3, 30e-12, 120e-12, 8e9))
    mon = S.VoltageMonitor(S.Cube([(q + 1) * dl for q in c], [dl, dl, dl]), S.ZP)
    return S.Scene(dl, objects, boundaries, lumped_elements=[src], monitors=[mon], cfl=cfl), steps


def field_monitors(steps=40):
    """A boxed scene (CPML on every face, a soft source) with field
    monitors between its voltage monitors: a movie of Ez on an XY plane
    (plot step 6), a plain Hy monitor on a YZ plane, a movie of Hx on a ZX
    plane whose own total_time_steps ends before the run does (its extra
    last frame falls between plot steps), and a second voltage monitor."""
    dl = 2e-3
    dims = (14, 12, 16)
    sc, _ = _boxed(dims, dl, _six(4), steps)
    ez = S.TimeDomainFieldMonitor(S.Cube([0, 0, 7 * dl], [dims[0] * dl, dims[1] * dl, 0]), S.PLANE_XY, S.EZ)
    hy = S.TimeDomainFieldMonitor(S.Cube([6 * dl, 2 * dl, 3 * dl], [0, 8 * dl, 9 * dl]), S.PLANE_YZ, S.HY)
    hx = S.TimeDomainFieldMonitor(S.Cube([dl, 5 * dl, 0], [10 * dl, 0, 12 * dl]), S.PLANE_ZX, S.HX)
    v2 = S.VoltageMonitor(S.Cube([4 * dl, 4 * dl, 4 * dl], [dl, dl, 2 * dl]), S.ZP)
    sc.monitors = [sc.monitors[0], S.MovieMonitor(ez, steps, 6), hy, S.MovieMonitor(hx, steps - 3, 7), v2]
    return sc, steps


def two_port(steps=160):
    """A boxed scene with a two-port network (Port, Network;
    src/network/port.cpp, network.cpp): port 1 at the soft current source,
    port 2 across the box, each a voltage monitor and a current monitor
    around it; S-parameters at four frequencies."""
    dl = 2e-3
    dims = (16, 14, 12)
    sc, _ = _boxed(dims, dl, _six(4), steps)
    c = [max(1, int(v * 0.45)) for v in dims]   # the source cell of _boxed
    v1 = S.VoltageMonitor(S.Cube([q * dl for q in c], [dl, dl, dl]), S.ZP)
    c1 = S.CurrentMonitor(S.Cube([q * dl for q in c], [dl, dl, dl]), S.ZP)
    far = [c[0] + 5, c[1] - 3, c[2]]
    v2 = S.VoltageMonitor(S.Cube([q * dl for q in far], [dl, dl, 2 * dl]), S.ZP)
    c2 = S.CurrentMonitor(S.Cube([q * dl for q in far], [dl, dl, dl]), S.ZP)
    sc.monitors = [v1, sc.monitors[0], c1, v2, c2]
    ports = [S.Port(1, 50.0, True, v1, c1), S.Port(2, 100.0 + 5.0j, False, v2, c2)]
    sc.network = S.Network(ports, [1e9, 3e9, 6e9, 9e9])
    return sc, steps


def broadband(steps=80):
    """The small PEC-sphere scene with an NffftBroadBand in an oblique
    direction in place of its NffftFd."""
    sc, _ = configs.pec_sphere_rcs(scale=2, steps=steps)
    nf = sc.nffft
    sc.nffft = S.NffftBroadBand(nf.distance_x, nf.distance_y, nf.distance_z, 0.3, 0.7)
    return sc, steps


def _six(t):
    return [S.PML(o, t) for o in (S.XN, S.XP, S.YN, S.YP, S.ZN, S.ZP)]


def tiny_box(steps=120):
    """10 x 9 x 8 cells inside a 4-cell CPML on every face: plain runs of 1-2
    cells per axis, too short for the interior's line cut."""
    return _boxed((10, 9, 8), 2e-3, _six(4), steps)


def pec_box(steps=150):
    """No CPML: PEC walls only, odd extents (23 x 18 x 37)."""
    return _boxed((23, 18, 37), 2e-3, [], steps)


def long_z(steps=120):
    """A long z axis (14 x 12 x 90 + 5-cell CPML): several 128-byte lines per
    row, so the interior's k range is cut on lines."""
    return _boxed((14, 12, 90), 2e-3, _six(5), steps)


def one_sided(steps=150):
    """CPML on XP and ZN only, 21 x 26 x 40: the interior touches the walls on
    the other faces."""
    return _boxed((21, 26, 40), 2e-3, [S.PML(S.XP, 6), S.PML(S.ZN, 9)], steps)


# Scenes for the volume split (interior box and CPML/wall shell), compared
# against the oracle at test time (no golden fixtures).
SPLIT_SCENES = {
    "tiny_box": tiny_box,
    "pec_box": pec_box,
    "long_z": long_z,
    "one_sided": one_sided,
}


# scenes of the output formats (field and movie monitors, the broadband NF-FF),
# with golden vectors of their own
OUTPUT_SCENES = {
    "field_monitors": field_monitors,
    "broadband": broadband,
}


def rel_err(a, b):
    """max |a - b| / max |b| (0 when both vanish)."""
    a = np.asarray(a)
    b = np.asarray(b)
    scale = np.abs(b).max()
    if scale == 0:
        return float(np.abs(a).max())
    return float(np.abs(a - b).max() / scale)


def dispersive(kind="drude", steps=200, limit=False):
    """The dielectric-sphere scene at 1/8 scale with a dispersive sphere:
    Lorentz (eps_s 4, eps_inf 2, pole at 3e10 rad/s, damping 1e9 1/s),
    Drude (eps_inf 1.5, plasma 5e10 rad/s, collisions 2e9 1/s) or Debye
    (eps_s 6, eps_inf 2.5, tau 20 ps), with sigma_e 0.01 S/m.  limit=True
    takes each medium's parameters to the plain dielectric eps_r = 2.5
    (no pole, no plasma, eps_s = eps_inf), which the E recursion must then
    reproduce."""
    sc, st = dielectric(steps=steps)
    if kind == "lorentz":
        m = S.LorentzMedium("l", 2.5 if limit else 4.0, 2.5 if limit else 2.0, 0.0 if limit else 3e10, 1e9, 0.01)
    elif kind == "drude":
        m = S.DrudeMedium("d", 2.5 if limit else 1.5, 0.0 if limit else 5e10, 2e9, 0.01)
    else:
        m = S.DebyMedium("b", 2.5 if limit else 6.0, 2.5, 20e-12, 0.01)
    sc.objects[1] = S.Object(sc.objects[1].name, sc.objects[1].shape, m)
    return sc, st


def cylinder_2d(steps=300):
    """The 2-D (nz = 1) TMz cylinder scatter of the reference's example at a
    fifth of its size: 70 x 60 cells + 10-cell CPML on x and y, PEC
    cylinder, TFSF2D at phi = pi / 4."""
    return configs.cylinder_2d(scale=5, steps=steps)


SCENES = {
    "cylinder_2d": cylinder_2d,
    "pec_sphere": pec_sphere,
    "dielectric": dielectric,
    "heterogeneous": heterogeneous,
    "oblique": oblique,
    "partial_pml": partial_pml,
    "lumped": lumped,
    "thin_wire": thin_wire,
}
