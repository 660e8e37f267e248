"""Batches (xfdtd_batch_*): many simulations of different sizes advanced
with one launch per phase.  A batched member must give exactly the bits of
the same simulation stepped alone with the split kernels."""
import numpy as np
import pytest

import xfdtd_gb300 as X
from xfdtd_gb300 import configs

pytestmark = pytest.mark.gpu


def _problems(n, steps):
    out = []
    for q, (sc, _) in enumerate(configs.batched_scatterers(n=n, scale=2, seed0=4100)):
        out.append((sc, steps[q % len(steps)]))
    return out


@pytest.mark.parametrize("precision,graph", [("fp64", True), ("fp32", True), ("fp32", False)])
def test_batch_matches_members_stepped_alone(precision, graph):
    probs = _problems(5, [45, 70, 33, 70, 58])
    members = [X.Simulation(sc, st, precision=precision, fused=False, autotune=False) for sc, st in probs]
    alone = [X.Simulation(sc, st, precision=precision, fused=False, autotune=False) for sc, st in probs]
    b = X.Batch(members, graph=graph)
    b.step(30)
    assert b.status()["running"] == 5
    b.step(100)   # every member stops at its own total
    b.synchronize()
    st = b.status()
    assert st["running"] == 0 and st["clock"] == 70
    for (sc, steps), m, a in zip(probs, members, alone):
        a.step(steps)
        for c in range(6):
            assert np.array_equal(m.read_field(c), a.read_field(c)), (steps, c)
        for w in (0, 5, 11, 19):
            assert np.array_equal(m.read_nffft(w), a.read_nffft(w)), (steps, w)
        assert np.array_equal(m.far_field(0), a.far_field(0))


def test_batch_rejects_bad_members():
    probs = _problems(2, [20])
    a = X.Simulation(probs[0][0], 20, precision="fp32", fused=False)
    b = X.Simulation(probs[1][0], 20, precision="fp64", fused=False)
    with pytest.raises(X.EngineError, match="precision"):
        X.Batch([a, b])
    a.step(1)
    c = X.Simulation(probs[1][0], 20, precision="fp32", fused=False)
    with pytest.raises(X.EngineError, match="stepped"):
        X.Batch([a, c])
    with pytest.raises(X.EngineError, match="twice"):
        X.Batch([c, c])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_tma_launches_match_plain_and_alone(precision):
    """Members whose grids allow the wide decomposition's TMA-staged launches
    run them inside the batch (batch.cuh k_tma_batch); the others run the
    one-thread-per-cell kernels in the same phases.  Both give the bits of
    the member stepped alone, and of the batch with every member on the
    plain kernels."""
    probs = [(sc, 40 + 9 * q) for q, (sc, _) in enumerate(configs.batched_scatterers(n=4, seed0=4200))]
    probs += _problems(2, [44, 31])   # half-size members
    runs = {}
    for plain in (False, True):
        members = [X.Simulation(sc, st, precision=precision, fused=False, autotune=False) for sc, st in probs]
        b = X.Batch(members, graph=True, plain=plain)
        if plain or precision == "fp64":   # the TMA-staged launches run in FP32 only
            assert b.tma_members() == 0
        else:
            assert b.tma_members() >= 1
        b.step(100)
        b.synchronize()
        runs[plain] = [[m.read_field(c) for c in range(6)] + [m.read_nffft(w) for w in (0, 7, 13, 22)]
                       for m in members]
        del b
    for q, (sc, st) in enumerate(probs):
        a = X.Simulation(sc, st, precision=precision, fused=False, autotune=False)
        a.step(st)
        alone = [a.read_field(c) for c in range(6)] + [a.read_nffft(w) for w in (0, 7, 13, 22)]
        for x, y, z in zip(runs[False][q], runs[True][q], alone):
            assert np.array_equal(x, z), q
            assert np.array_equal(y, z), q
