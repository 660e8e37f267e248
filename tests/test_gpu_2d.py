"""The 2-D (nz = 1) TMz path against the FP64 CPU oracle, through the
C-ABI: Simulation::updateE's 2-D branch (src/simulation/simulation_update.cpp:157-168),
the 3-D updateH with nz = 1, the CPML on the four x and y faces, the 2-D
time step and TFSF2D (src/tfsf/tfsf_2d.cpp).

Tolerance for FP64: 1e-10 of the largest |oracle| value of the field (E or
H) an array belongs to; Ex, Ey and Hz stay exactly zero on both sides.  The
FP32 form's error is bounded and printed."""
import numpy as np
import pytest

import oracle as O
import scenes
import xfdtd_gb300 as X
from xfdtd_gb300 import configs
from xfdtd_gb300 import scene as S

TOL = 1e-10


def _compare(g, o, tol):
    worst = 0.0
    for side in ((S.EX, S.EY, S.EZ), (S.HX, S.HY, S.HZ)):
        arrs = [(g.read_field(c), o.read_field(c)) for c in side]
        scale = max(float(np.abs(b).max()) for _, b in arrs)
        assert scale > 0
        for c, (a, b) in zip(side, arrs):
            e = float(np.abs(a - b).max()) / scale
            assert e <= tol, f"component {c}: rel err {e:.3e}"
            worst = max(worst, e)
    for c in (S.EX, S.EY, S.HZ):
        assert not np.any(g.read_field(c)), c
    return worst


@pytest.mark.gpu
@pytest.mark.parametrize("pec", [True, False])
def test_2d_cylinder_scatter_full_size(pec):
    """The reference's 2-D example at its full size (370 x 320 cells, 1400
    steps): PEC cylinder (sigma = 1e24) and a dielectric one."""
    sc, st = configs.cylinder_2d(steps=1400, pec=pec)
    o = O.OracleSim(sc, st)
    o.step(st)
    g = X.Simulation(sc, st, precision="fp64")
    assert g.n == o.n == (370, 320, 1)
    assert g.dt == o.dt
    g.step(st)
    e64 = _compare(g, o, TOL)
    g32 = X.Simulation(sc, st, precision="fp32")
    g32.step(st)
    e32 = _compare(g32, o, 1e-4)
    print(f"2-D cylinder (pec={pec}): FP64 {e64:.2e}, FP32 {e32:.2e}")


@pytest.mark.gpu
def test_2d_steps_in_pieces_and_graph_replay_are_bitwise_equal():
    sc, st = scenes.cylinder_2d(steps=150)
    a = X.Simulation(sc, st, graph=True)
    b = X.Simulation(sc, st, graph=False)
    a.step(70)
    a.step(80)
    b.step(st)
    for c in range(6):
        assert np.array_equal(a.read_field(c), b.read_field(c)), c


@pytest.mark.gpu
def test_2d_from_random_fields():
    """Seeded random Ez, Hx, Hy in every cell (walls and CPML included), a
    few steps: the per-cell update and the CPML recursions alone."""
    sc, _ = scenes.cylinder_2d(steps=6)
    o = O.OracleSim(sc, 6)
    g = X.Simulation(sc, 6)
    rng = np.random.default_rng(21)
    for c in (S.EZ, S.HX, S.HY):
        a = rng.standard_normal(S.field_shape(c, o.n))
        o.write_field(c, a)
        g.write_field(c, a)
    o.step(6)
    g.step(6)
    _compare(g, o, 1e-13)


def test_2d_plans_are_checked_on_the_host():
    """A 3-D plane wave on a 2-D grid, TFSF2D on a 3-D grid and an NF-FF box
    on a 2-D grid are refused before any device work."""
    X.build()
    sc, st = scenes.cylinder_2d(steps=5)
    sc.tfsf = S.TFSF3D(14, 14, 0, 1.0, 0.0, 0.0, 0.0, sc.tfsf.waveform)
    with pytest.raises(X.EngineError, match="TFSF2D"):
        X.Simulation(sc, st)
    sc3, st3 = scenes.pec_sphere(steps=5)
    sc3.tfsf = S.TFSF2D(12, 12, 0.3, 1.0, sc3.tfsf.waveform)
    with pytest.raises(X.EngineError, match="2-D grid"):
        X.Simulation(sc3, st3)
    sc, st = scenes.cylinder_2d(steps=5)
    sc.nffft = S.NffftFd(16, 16, 0, [1e9], [0.0], [0.0], "")
    with pytest.raises(X.EngineError, match="NF-FF"):
        X.Simulation(sc, st)
