"""The allocation-free NF-FF operator (xfdtd_nffft_dft_noalloc) through the
C-ABI, against the engine's own NF-FF accumulation (xfdtd_read_nffft).

The operator keeps its sample batch in a static device array, so this file
is collected last: its GPU test must pass on a device where the other tests
already ran (stale scratch contents) as well as alone."""
import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

import scenes
import xfdtd_gb300 as X
from xfdtd_gb300 import scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class NffftOperator(C.Structure):
    """ctypes mirror of xfdtd_nffft_operator (include/xfdtd_cuda.h)."""
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32),
                ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
                ("fields", C.c_void_p * 6),
                ("lo", C.c_int64 * 3), ("hi", C.c_int64 * 3),
                ("n_freq", C.c_int32), ("batch", C.c_int32),
                ("total_steps", C.c_int64), ("step", C.c_int64),
                ("fold_count", C.c_int32), ("reserved", C.c_int32),
                ("phase_j", C.c_void_p), ("phase_m", C.c_void_p),
                ("acc", C.c_void_p * 24), ("stream", C.c_void_p)]


def _lib():
    X.build()
    cu, _ = X.libs()
    cu.xfdtd_nffft_dft_noalloc.argtypes = [C.POINTER(NffftOperator)]
    cu.xfdtd_nffft_noalloc_setup.argtypes = [C.c_int]
    cu.xfdtd_nffft_noalloc_max_bytes.restype = C.c_int64
    cu.xfdtd_nffft_noalloc_last_error.restype = C.c_char_p
    return cu


def test_operator_struct_layout_matches_header():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "xfdtd_cuda.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(xfdtd_nffft_operator), offsetof(xfdtd_nffft_operator, phase_j),
         offsetof(xfdtd_nffft_operator, acc), offsetof(xfdtd_nffft_operator, stream));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        got = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [C.sizeof(NffftOperator), NffftOperator.phase_j.offset,
                   NffftOperator.acc.offset, NffftOperator.stream.offset]


def _valid_op(batch=8):
    op = NffftOperator()
    op.precision, op.device = 0, 0
    op.nx = op.ny = op.nz = 40
    for c in range(6):
        op.fields[c] = 4096
    op.lo[:] = [5, 5, 5]
    op.hi[:] = [35, 35, 35]
    op.n_freq, op.batch, op.total_steps, op.step, op.fold_count = 1, batch, 100, 7, 8
    op.phase_j = op.phase_m = 4096
    for q in range(24):
        op.acc[q] = 4096
    return op


def test_oversized_and_invalid_descriptions_are_rejected_on_the_host():
    """Rejected before any device call: these run without a GPU."""
    cu = _lib()
    assert cu.xfdtd_nffft_noalloc_max_bytes() == 64 << 20
    assert cu.xfdtd_nffft_dft_noalloc(None) == 1
    # 30 x 30 faces: 24 * 900 * 8 B per step; 400 slots need 69 MB > 64 MiB
    op = _valid_op(batch=400)
    op.fold_count = 0
    assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 1
    assert b"64 MiB" in cu.xfdtd_nffft_noalloc_last_error()
    op = _valid_op()
    op.hi[2] = 40   # the face interpolation reads index hi: hi <= n - 1
    assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 1
    op = _valid_op()
    op.fold_count = 9   # more than the batch holds
    assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 1
    op = _valid_op()
    op.step = 3         # folds steps that were never sampled
    assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 1
    op = _valid_op()
    op.acc[5] = None
    assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 1


def test_out_of_range_grids_and_boxes_are_rejected_on_the_host():
    """A grid axis above 2^30 cells or a box edge above the sample launch's
    reach (8 x 65535 rows) is rejected before any device call."""
    cu = _lib()
    op = _valid_op()
    op.nz = (1 << 30) + 1
    assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 1
    assert b"grid size" in cu.xfdtd_nffft_noalloc_last_error()
    op = _valid_op()
    op.nx = 600000
    op.lo[0], op.hi[0] = 1, 599999
    assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 1
    assert b"box edge" in cu.xfdtd_nffft_noalloc_last_error()


def test_operator_call_before_setup_is_refused():
    """In a fresh process, a valid description without the per-device
    set-up is refused (XFDTD_ERR_STATE) before any device call."""
    code = f"""
import ctypes as C, sys
sys.path.insert(0, {ROOT!r}); sys.path.insert(0, {os.path.join(ROOT, 'tests')!r})
import test_zz_no_alloc as T
cu = T._lib()
op = T._valid_op()
rc = cu.xfdtd_nffft_dft_noalloc(C.byref(op))
print(rc, cu.xfdtd_nffft_noalloc_last_error().decode())
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rc, msg = r.stdout.strip().split(" ", 1)
    assert int(rc) == 7 and "setup" in msg


def _operator_case(precision, st, folds_at):
    """Engine stepped from seeded random fields for `st` steps; after each
    step the operator samples the same fields (copied into caller-owned
    device arrays) and folds the steps given by folds_at[step].  Returns the
    engine, the operator description and its accumulators."""
    import torch
    cu = _lib()
    assert cu.xfdtd_nffft_noalloc_setup(0) == 0
    sc, _ = scenes.dielectric(steps=st)
    g = X.Simulation(sc, st, precision=precision, graph=False)
    rng = np.random.default_rng(11)
    for c in range(6):
        g.write_field(c, rng.standard_normal(S.field_shape(c, g.n)))
    dtype = torch.float64 if precision == "fp64" else torch.float32
    dev = torch.device("cuda:0")
    fields = [torch.empty(S.field_shape(c, g.n), dtype=dtype, device=dev) for c in range(6)]
    freqs = np.atleast_1d(np.asarray(sc.nffft.frequencies, dtype=np.float64))
    t = np.arange(st, dtype=np.float64)
    w = 2.0 * np.pi
    pj = g.dt * np.exp(-1j * w * (freqs[:, None] * (t[None, :] + 0.5) * g.dt))
    pm = g.dt * np.exp(-1j * w * (freqs[:, None] * t[None, :] * g.dt))
    phase_j = torch.from_numpy(np.ascontiguousarray(np.stack([pj.real, pj.imag], -1))).to(dev)
    phase_m = torch.from_numpy(np.ascontiguousarray(np.stack([pm.real, pm.imag], -1))).to(dev)
    box = g.nffft_box()
    acc = [torch.zeros((len(freqs),) + S.nffft_face_shape(q, box) + (2,), dtype=torch.float64, device=dev)
           for q in range(24)]
    nf = sc.nffft
    op = NffftOperator()
    op.precision = 0 if precision == "fp64" else 1
    op.device = 0
    op.nx, op.ny, op.nz = g.n
    for c in range(6):
        op.fields[c] = fields[c].data_ptr()
    op.lo[:] = [nf.distance_x, nf.distance_y, nf.distance_z]
    op.hi[:] = [g.n[0] - nf.distance_x, g.n[1] - nf.distance_y, g.n[2] - nf.distance_z]
    op.n_freq, op.total_steps = len(freqs), st
    op.phase_j, op.phase_m = phase_j.data_ptr(), phase_m.data_ptr()
    for q in range(24):
        op.acc[q] = acc[q].data_ptr()
    op.stream = torch.cuda.current_stream(dev).cuda_stream
    return cu, g, op, fields, acc, dtype


def _compare(g, acc, tol, tag):
    import torch
    torch.cuda.synchronize()
    for q in range(24):
        want = g.read_nffft(q)
        a = acc[q].cpu().numpy()
        got = a[..., 0] + 1j * a[..., 1]
        assert np.abs(want).max() > 0, q
        e = scenes.rel_err(got, want)
        assert e <= tol, (tag, q, e)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_partial_and_wrapping_folds(precision):
    """A batch of 5 slots over 16 steps, folded at uneven points: folds of 3,
    4, 1, 5 and 3 steps, two of them wrapping from the last slot back to
    slot 0.  After the last fold the accumulators equal the engine's (FP64:
    1e-12; FP32: 1e-4, since the operator's FP32 partial sums group the
    steps differently from the engine's batches of 8).  Then a fold after a
    change of batch, and a fold across a skipped step, are refused."""
    import torch
    st, batch = 16, 5
    folds = {2: 3, 6: 4, 7: 1, 12: 5, 15: 3}
    cu, g, op, fields, acc, dtype = _operator_case(precision, st, folds)
    op.batch = batch
    for s in range(st):
        g.step(1)
        for c in range(6):
            fields[c].copy_(torch.from_numpy(g.read_field(c)).to(dtype))
        op.step = s
        op.fold_count = folds.get(s, 0)
        rc = cu.xfdtd_nffft_dft_noalloc(C.byref(op))
        assert rc == 0, cu.xfdtd_nffft_noalloc_last_error()
    assert torch.cuda.current_device() == 0
    _compare(g, acc, 1e-12 if precision == "fp64" else 1e-4, precision)
    # another batch: the slots hold the old layout, a fold over them is refused
    op.batch, op.step, op.fold_count = 4, 15, 2
    assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 1
    assert b"unbroken run" in cu.xfdtd_nffft_noalloc_last_error()
    # a fresh run of batch 4 from step 3; skipping step 5 breaks it
    for s, fc in ((3, 0), (4, 2)):
        op.step, op.fold_count = s, fc
        assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 0, cu.xfdtd_nffft_noalloc_last_error()
    op.step, op.fold_count = 6, 2
    assert cu.xfdtd_nffft_dft_noalloc(C.byref(op)) == 1
    torch.cuda.synchronize()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_operator_matches_engine_accumulators(precision):
    """From seeded random fields, the engine steps 16 times; after every step
    the operator samples the same fields (copied into caller-owned device
    arrays) and folds each batch of 8.  After each of the two folds in a row
    its accumulators equal the engine's within 1e-12 relative (the phase
    tables here come from numpy, the engine's from the C++ host)."""
    import torch
    cu = _lib()
    assert cu.xfdtd_nffft_noalloc_setup(0) == 0
    sc, _ = scenes.dielectric(steps=16)
    st, batch = 16, 8
    g = X.Simulation(sc, st, precision=precision, graph=False)
    rng = np.random.default_rng(11)
    for c in range(6):
        g.write_field(c, rng.standard_normal(S.field_shape(c, g.n)))
    dtype = torch.float64 if precision == "fp64" else torch.float32
    dev = torch.device("cuda:0")
    fields = [torch.empty(S.field_shape(c, g.n), dtype=dtype, device=dev) for c in range(6)]
    freqs = np.atleast_1d(np.asarray(sc.nffft.frequencies, dtype=np.float64))
    t = np.arange(st, dtype=np.float64)
    w = 2.0 * np.pi
    pj = g.dt * np.exp(-1j * w * (freqs[:, None] * (t[None, :] + 0.5) * g.dt))
    pm = g.dt * np.exp(-1j * w * (freqs[:, None] * t[None, :] * g.dt))
    phase_j = torch.from_numpy(np.ascontiguousarray(np.stack([pj.real, pj.imag], -1))).to(dev)
    phase_m = torch.from_numpy(np.ascontiguousarray(np.stack([pm.real, pm.imag], -1))).to(dev)
    box = g.nffft_box()
    acc = [torch.zeros((len(freqs),) + S.nffft_face_shape(q, box) + (2,), dtype=torch.float64, device=dev)
           for q in range(24)]
    nf = sc.nffft
    op = NffftOperator()
    op.precision = 0 if precision == "fp64" else 1
    op.device = 0
    op.nx, op.ny, op.nz = g.n
    for c in range(6):
        op.fields[c] = fields[c].data_ptr()
    op.lo[:] = [nf.distance_x, nf.distance_y, nf.distance_z]
    op.hi[:] = [g.n[0] - nf.distance_x, g.n[1] - nf.distance_y, g.n[2] - nf.distance_z]
    op.n_freq, op.batch, op.total_steps = len(freqs), batch, st
    op.phase_j, op.phase_m = phase_j.data_ptr(), phase_m.data_ptr()
    for q in range(24):
        op.acc[q] = acc[q].data_ptr()
    stream = torch.cuda.current_stream(dev)
    op.stream = stream.cuda_stream
    folds = 0
    for s in range(st):
        g.step(1)
        for c in range(6):
            fields[c].copy_(torch.from_numpy(g.read_field(c)).to(dtype))
        op.step = s
        op.fold_count = batch if (s + 1) % batch == 0 else 0
        rc = cu.xfdtd_nffft_dft_noalloc(C.byref(op))
        assert rc == 0, cu.xfdtd_nffft_noalloc_last_error()
        if op.fold_count:
            folds += 1
            torch.cuda.synchronize(dev)
            for q in range(24):
                want = g.read_nffft(q)
                a = acc[q].cpu().numpy()
                got = a[..., 0] + 1j * a[..., 1]
                assert np.abs(want).max() > 0, q
                e = scenes.rel_err(got, want)
                assert e <= 1e-12, (precision, folds, q, e)
    assert folds == 2
