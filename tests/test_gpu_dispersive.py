"""Linear dispersive media (Lorentz, Drude, Debye) on the GPU engine against
the FP64 CPU oracle, through the C-ABI.

The reference's dispersive media (src/include/material/dispersive_material.h)
take their E update from the recursions of LorentzMedium / DrudeMedium /
DebyMedium::updateE{x,y,z} (src/material/dispersive_material.cpp), run in
place of the Yee E update for the cells of a dispersive object
(Simulation::updateEWithDispersiveMaterial, simulation_update.cpp:221-280).
The reference throws on them at Object::init (object.cpp:109-110); the
oracle restates the recursions as written, and the engine runs them as a
sparse launch after the E update over those cells.

Tolerance: the FP64 form within 1e-10 of the largest |oracle| value of
the field (E or H) an array belongs to; the FP32 form's relative L2 error
below 1e-4."""
import numpy as np
import pytest

import oracle as O
import scenes
import xfdtd_gb300 as X
from xfdtd_gb300 import scene as S

TOL = 1e-10


def _compare(g, o):
    worst, l2 = 0.0, 0.0
    for side in ((0, 1, 2), (3, 4, 5)):
        arrs = [(g.read_field(c), o.read_field(c)) for c in side]
        scale = max(float(np.abs(b).max()) for _, b in arrs)
        norm = np.sqrt(sum(float(np.linalg.norm(b)) ** 2 for _, b in arrs))
        for a, b in arrs:
            worst = max(worst, float(np.abs(a - b).max()) / scale)
            l2 = max(l2, float(np.linalg.norm(a - b)) / norm)
    return worst, l2


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["lorentz", "drude", "debye"])
def test_dispersive_sphere_against_oracle(kind):
    """A dispersive sphere lit by the TFSF plane wave, 200 steps: fields and
    the NF-FF accumulators of the FP64 form against the oracle; the FP32
    form's field error."""
    sc, st = scenes.dispersive(kind, steps=200)
    o = O.OracleSim(sc, st)
    o.step(st)
    g = X.Simulation(sc, st, precision="fp64")
    g.step(st)
    worst, _ = _compare(g, o)
    assert worst <= TOL, (kind, worst)
    nf = max(scenes.rel_err(g.read_nffft(w), o.read_nffft(w)) for w in (0, 5, 9, 14, 18, 23))
    assert nf <= TOL, (kind, nf)
    g32 = X.Simulation(sc, st, precision="fp32")
    g32.step(st)
    _, l2 = _compare(g32, o)
    assert l2 < 1e-4, (kind, l2)


@pytest.mark.gpu
def test_dispersive_graph_replay_and_pieces_are_bitwise_equal():
    sc, st = scenes.dispersive("lorentz", steps=100)
    a = X.Simulation(sc, st, graph=True)
    b = X.Simulation(sc, st, graph=False)
    a.step(37)
    a.step(63)
    b.step(st)
    for c in range(6):
        assert np.array_equal(a.read_field(c), b.read_field(c)), c


def test_dispersive_plans_are_checked_on_the_host():
    """A lumped element inside a dispersive medium and a dispersive object
    on a 2-D grid are refused before any device work.  (The CPML lies
    outside every object's box, so an object cannot reach into it.)"""
    X.build()
    sc, st = scenes.dispersive("drude", steps=5)
    dl = sc.cell_size
    sc.lumped_elements = [S.CurrentSource(S.Cube([0, 0, 0], [dl, dl, dl]), S.ZP, 50.0,
                                          S.GaussianWaveform(1.0, 1e-11, 4e-11))]
    with pytest.raises(X.EngineError, match="dispersive medium"):
        X.Simulation(sc, st)
    sc, st = scenes.cylinder_2d(steps=5)
    sc.objects[1] = S.Object("c", sc.objects[1].shape, S.DebyMedium("b", 6.0, 2.5, 20e-12))
    with pytest.raises(X.EngineError, match="dx == dy == dz"):
        X.Simulation(sc, st)
