"""Failure detection on the GPU path, in forms that fault, trap or hang no
GPU: a non-finite value written into a field from the host, and bounded
device waits made to run out by a wait limit of zero polls.

The reference has no counterpart (a single-threaded CPU loop); these test
the engine's own status paths: xfdtd_check_finite (XFDTD_ERR_NAN) and the
status word of the TMA-staged volume launches (XFDTD_ERR_TIMEOUT)."""
import numpy as np
import pytest

import scenes
import xfdtd_gb300 as X

# TMA-staged interior variants: narrow decomposition (16) and wide (20),
# z-edge TMA shell variant (4)
NARROW_TMA, WIDE_TMA, ZEDGE_TMA = 16, 20, 4


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_non_finite_value_from_the_host_is_caught(precision, bad):
    """check_finite passes on the stepped fields, then raises
    XFDTD_ERR_NAN once one cell of one component is non-finite; stepping
    carries the value into its neighbours, and it is still caught."""
    sc, st = scenes.dielectric(steps=12)
    g = X.Simulation(sc, st, precision=precision, graph=False)
    g.step(4)
    g.check_finite()
    comp = 4   # Hy
    a = g.read_field(comp)
    idx = tuple(s // 2 for s in a.shape)
    a[idx] = bad
    g.write_field(comp, a)
    with pytest.raises(X.EngineError) as ei:
        g.check_finite()
    assert ei.value.status == 5
    g.step(3)
    with pytest.raises(X.EngineError) as ei:
        g.check_finite()
    assert ei.value.status == 5
    g.synchronize()


def _tma_sim(sc, st, precision, wide):
    g = X.Simulation(sc, st, precision=precision, autotune=False, fused=False, graph=False)
    try:
        if wide:
            g.set_kernel_variant(WIDE_TMA, WIDE_TMA)
            g.set_shell_variant(ZEDGE_TMA, ZEDGE_TMA)
        else:
            g.set_kernel_variant(NARROW_TMA, NARROW_TMA)
    except X.EngineError:
        return None
    return g


@pytest.mark.gpu
@pytest.mark.parametrize("wide", [False, True])
def test_plane_wait_timeout_is_reported_and_the_context_survives(wide):
    """With a wait limit of zero polls every block of the TMA-staged volume
    launches gives up on its first plane, drains the copies it issued and
    reports XFDTD_ERR_TIMEOUT, which synchronize returns.  The context stays
    usable: a fresh handle on the same device then steps to the bits of a
    handle that never timed out."""
    # the wide launches need a grid whose k range lies on 16-byte boundaries
    # for the fields and the 1-byte index (88^3 cells)
    sc, st = scenes.dielectric(scale=4 if wide else 8, steps=10)
    ran = 0
    for precision in ("fp32", "fp64"):
        bad = _tma_sim(sc, st, precision, wide)
        if bad is None:
            continue   # this grid's k range offers no TMA variant in this precision
        ran += 1
        bad.set_wait_limit(0)
        bad.step(2)
        with pytest.raises(X.EngineError) as ei:
            bad.synchronize()
        assert ei.value.status == 4, ei.value
        bad.close()
        ref = X.Simulation(sc, st, precision=precision, autotune=False, fused=False, graph=False)
        ref.step(st)
        want = [ref.read_field(c) for c in range(6)]
        good = _tma_sim(sc, st, precision, wide)
        good.step(st)
        good.synchronize()
        for c in range(6):
            assert np.array_equal(good.read_field(c), want[c]), (precision, wide, c)
    assert ran >= 1
