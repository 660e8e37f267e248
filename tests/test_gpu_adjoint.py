"""Adjoint gradients (xfdtd_adjoint_forward / _backward) against central
finite differences: of the engine's own FP64 forward pass, and of the CPU
oracle's (the reference's arithmetic), on reduced-size versions of the
dipole / design-region problem."""
import copy

import numpy as np
import pytest

import oracle as O
import xfdtd_gb300 as X
from xfdtd_gb300 import configs
from xfdtd_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _spec_args(spec, k=None):
    a = {q: spec[q] for q in ("design_lo", "design_hi", "plane_axis", "plane_index", "plane_lo", "plane_hi",
                              "t_begin", "t_end", "loss_comp", "checkpoint_every")}
    if k is not None:
        a["checkpoint_every"] = k
    return a


def _with_material(sc, spec, cell, eps=None, sigma=None):
    """The scene with the design voxel `cell` (design-box coordinates) given
    a new eps_r (set in double, bypassing the float Material ctor) / sigma;
    returns (scene, the eps_r / sigma used)."""
    sc2 = copy.copy(sc)
    sc2.voxel_materials = list(sc.voxel_materials)
    dsz = tuple(b - a for a, b in zip(spec["design_lo"], spec["design_hi"]))
    q = 1 + int(np.ravel_multi_index(cell, dsz))
    m = sc.voxel_materials[q]
    e = float(eps) if eps is not None else m.eps_r
    s = sigma if sigma is not None else m.sigma_e
    sc2.voxel_materials[q] = S.Material("d", e, 1.0, s, 0.0, exact_eps=True)
    return sc2, (e if eps is not None else s)


def _loss(sc, st, spec, precision="fp64"):
    g = X.Simulation(sc, st, precision=precision, fused=False, autotune=False)
    return g.adjoint_forward(**_spec_args(spec, 0))


CELLS = [(3, 4, 2), (8, 8, 4), (12, 5, 6), (15, 15, 7)]


@pytest.fixture(scope="module")
def problem():
    sc, st, spec = configs.adjoint_dipole(scale=4)
    g = X.Simulation(sc, st, precision="fp64", fused=False, autotune=False)
    loss = g.adjoint_forward(**_spec_args(spec))
    ge, gs = g.adjoint_backward()
    return sc, st, spec, loss, ge, gs


def test_adjoint_eps_gradient_matches_fd_fp64(problem):
    sc, st, spec, loss, ge, _ = problem
    assert loss > 0
    for cell in CELLS:
        e0 = float(spec["eps"][cell])
        sp, ep = _with_material(sc, spec, cell, eps=e0 + 1e-3)
        sm, em = _with_material(sc, spec, cell, eps=e0 - 1e-3)
        fd = (_loss(sp, st, spec) - _loss(sm, st, spec)) / (ep - em)
        assert abs(ge[cell] - fd) <= 1e-5 * abs(fd) + 1e-12 * abs(loss), (cell, ge[cell], fd)


def test_adjoint_sigma_gradient_matches_fd_fp64(problem):
    """sigma enters through sigma dt / eps (~1e-9 per S/m here): the loss is
    linear in sigma over +-1 S/m, and smaller steps only add the FP64
    rounding of the loss (1e-16 of ~5e11) to the difference."""
    sc, st, spec, loss, _, gs = problem
    for cell in CELLS[:2]:
        h = 1.0
        sp, _ = _with_material(sc, spec, cell, sigma=h)
        sm, _ = _with_material(sc, spec, cell, sigma=-h)
        fd = (_loss(sp, st, spec) - _loss(sm, st, spec)) / (2 * h)
        assert abs(gs[cell] - fd) <= 1e-6 * abs(fd), (cell, gs[cell], fd)


def test_checkpointing_does_not_change_the_gradient(problem):
    """Recording every step (K = 0) and re-running checkpoint segments give
    the same bits: the re-run repeats the forward pass exactly."""
    sc, st, spec, loss, ge, gs = problem
    g = X.Simulation(sc, st, precision="fp64", fused=False, autotune=False)
    assert g.adjoint_forward(**_spec_args(spec, 0)) == loss
    ge0, gs0 = g.adjoint_backward()
    assert np.array_equal(ge0, ge) and np.array_equal(gs0, gs)
    # the handle is back at the last step with the forward pass's fields
    f = X.Simulation(sc, st, precision="fp64", fused=False, autotune=False)
    f.step(st)
    h = X.Simulation(sc, st, precision="fp64", fused=False, autotune=False)
    h.adjoint_forward(**_spec_args(spec, 25))
    h.adjoint_backward()
    for c in range(6):
        assert np.array_equal(h.read_field(c), f.read_field(c))


def test_fp32_adjoint_tracks_fp64_fd(problem):
    """The FP32 form's gradient (FP32 forward and reverse passes, FP64
    gradient sums) against the FP64 finite differences."""
    sc, st, spec, loss, ge64, _ = problem
    g = X.Simulation(sc, st, precision="fp32", fused=False, autotune=False)
    g.adjoint_forward(**_spec_args(spec))
    ge, _ = g.adjoint_backward()
    scale = np.abs(ge64).max()
    for cell in CELLS:
        assert abs(ge[cell] - ge64[cell]) <= 1e-3 * scale, (cell, ge[cell], ge64[cell])


def _oracle_loss(sc, st, spec):
    o = O.OracleSim(sc, st)
    lo, hi = spec["design_lo"], spec["design_hi"]
    L = 0.0
    ax, idx = spec["plane_axis"], spec["plane_index"]
    (u0, v0), (u1, v1) = spec["plane_lo"], spec["plane_hi"]
    for t in range(st):
        o.step(1)
        if spec["t_begin"] <= t < spec["t_end"]:
            f = o.read_field(spec["loss_comp"])
            sl = [slice(None)] * 3
            sl[ax] = idx
            plane = f[tuple(sl)][u0:u1, v0:v1]
            L += float(np.sum(plane * plane))
    del lo, hi
    return L


def test_adjoint_matches_fd_of_the_cpu_oracle():
    """Central differences of the CPU oracle (the reference's FP64
    arithmetic) at two design voxels of a small problem."""
    O.set_threads(8)
    sc, st, spec = configs.adjoint_dipole(scale=8)
    g = X.Simulation(sc, st, precision="fp64", fused=False, autotune=False)
    loss = g.adjoint_forward(**_spec_args(spec))
    ge, _ = g.adjoint_backward()
    assert abs(_oracle_loss(sc, st, spec) - loss) <= 1e-9 * loss
    for cell in [(2, 3, 1), (5, 4, 2)]:
        e0 = float(spec["eps"][cell])
        sp, ep = _with_material(sc, spec, cell, eps=e0 + 1e-3)
        sm, em = _with_material(sc, spec, cell, eps=e0 - 1e-3)
        fd = (_oracle_loss(sp, st, spec) - _oracle_loss(sm, st, spec)) / (ep - em)
        assert abs(ge[cell] - fd) <= 1e-5 * abs(fd) + 1e-12 * loss, (cell, ge[cell], fd)
