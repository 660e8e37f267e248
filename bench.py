"""Benchmark of the FDTD step loop on GB300: Mcell-updates/s and the HBM
roofline fraction of the dominant kernel, beside the CPU oracle.

Workload (the headline): the bandwidth-bound heterogeneous medium, the
largest benchmark configuration -- 512 x 512 x 384 interior plus a 10-cell
CPML per face (532 x 532 x 404 = 114,341,696 cells), dx = 1 mm, voxel
materials drawn from a seeded 256-entry table (eps_r U[1, 6], sigma
U[0, 0.01] S/m), a z-directed soft point current source at the centre
(Gaussian-modulated sine, f0 = 10 GHz, 5 GHz bandwidth), Ez probes at 64
seeded cells, 1000 steps -- in its FP32 form (fields and CPML in FP32,
probe series copied out in FP32), the form the configuration names, with
the FP64 oracle as the check.  Synthetic inputs of that shape (there is no
dataset).  Each field component (456 MB) is far larger than the 129 MB L2,
so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one time step of the loop body over the whole grid.  value =
(cells x steps x ranks) / max-over-ranks device time of the K timed steps
(CUDA events on the engine's stream).  e2e = the same metric over the
configuration's whole job (1000 steps) through the public API -- host scene
-> plan lowering -> device allocation and upload -> autotuning -> steps ->
probe series copied back to the host -- wall clock, with each phase's time.
With --gpus N > 1 (torchrun), every rank runs an independent replica of the
workload (the path has no exchange).

The same line carries the FP64 form of the headline (the reference's
arithmetic: its e2e against the reference arm is the precision-matched
ratio), the dielectric-sphere configuration (280^3 cells, TFSF, NF-FF and
RCS) in FP32 and FP64, the batched and the adjoint forms, each with its own
roofline and (where it is a whole job) end-to-end figures, and the FP32
forms' errors against the FP64 forms on the same jobs.  GPU clocks are
sampled by nvidia-smi over the whole run.

--impl reference times the reference's algorithm on the host cores: the
reference cannot be built here (xtensor, xtensor-blas, xtensor-fftw, FFTW3,
BLAS and LAPACK are absent), so its line restates it -- the FP64 CPU oracle
(oracle/), all host threads, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from xfdtd_gb300 import configs  # noqa: E402
from xfdtd_gb300 import scene as S  # noqa: E402

WORKLOAD = ("heterogeneous medium: 512 x 512 x 384 interior + 10-cell CPML (532 x 532 x 404 cells), dx 1 mm, "
            "voxel materials from a seeded 256-entry table (eps_r U[1,6], sigma U[0,0.01] S/m), z-directed soft "
            "point current source (Gaussian-modulated sine, 10 GHz, 5 GHz bandwidth), 64 Ez probes")
METRIC = "Mcell-updates/s"
UNIT = "Mcell-updates/s"


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class _Group:
    """torch.distributed plumbing for N > 1 (barrier and max-reduce only)."""

    def __init__(self, world, local):
        self.world = world
        self.torch = None
        if world > 1:
            import torch
            import torch.distributed as dist
            self.torch = torch
            self.dist = dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            if torch.cuda.is_available():
                torch.cuda.set_device(local)
                dist.init_process_group("nccl")
                self.dev = torch.device("cuda", local)
            else:
                dist.init_process_group("gloo")
                self.dev = torch.device("cpu")

    def barrier(self):
        if self.torch is not None:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.torch is None:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.torch is not None:
            self.dist.destroy_process_group()


def aggregate_value(cells: int, steps: int, world: int, max_ms: float) -> float:
    """Whole-job Mcell-updates/s: every rank advances its own replica."""
    return cells * steps * world / (max_ms / 1e3) / 1e6


# ----------------------------------------------------------------- clocks ---
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[3][q].lower() == "active"})
        loaded = [r for r in rows if r[2] > 300] or rows
        return {"sm_mhz": statistics.median(r[0] for r in loaded), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# --------------------------------------------------------------- roofline ---
# Entries timed on their own streams, concurrently with the main stream's:
# the TFSF 1-D line, the NF-FF sampling and batch folds (the E half of a
# step's samples beside its H update, the H half and the folds beside the
# next step's E update), and the two kernels of each volume update (whose
# main-stream entry, update_e / update_h, spans both).
GRAPH_STEPS = 32        # steps per captured CUDA graph (4 NF-FF batches of 8)
PROFILE_STEPS = 400     # steps of the profiled pass behind the kernel times

SIDE_STREAM_KERNELS = ("tfsf_aux", "nffft", "nffft_acc", "update_e_interior", "update_e_shell",
                       "update_h_interior", "update_h_shell")

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one E and
# one H update on this workload in the wide decomposition, keyed by (entry,
# precision, grid, wide): the wide interior launch plus the z-edge launch,
# one ncu capture of each in step 13 of
# python -m xfdtd_gb300.run --config dielectric_sphere --steps 24 --precision fp32 --no-graph --volume split
#     --no-autotune --kernel-variant 20,20 --shell-variant 5,5
# E: 535.4 + 193.0 MB (interior) + 219.8 + 40.7 MB (z edges); H: 504.4 + 190.5 + 187.7 + 34.3 MB.
#
# The heterogeneous medium (532 x 532 x 404, 2-byte material index), its
# autotuned variants (E: wide compact-table interior 22 + z-edge launch 6;
# H: narrow TMA interior 19 + shell kernel 3), one ncu capture of each
# launch in step 2 of
# python -m xfdtd_gb300.run --config heterogeneous --steps 6 --precision fp32 --no-graph --no-autotune
#     --kernel-variant 22,19 --shell-variant 6,3
# E: 2900.65 + 1209.39 MB (wide) + 771.83 + 213.49 MB (z edges);
# H: 2521.39 + 1068.52 MB (interior) + 891.77 + 356.84 MB (shell).
NCU_TRAFFIC = {
    ("update_e", "fp32", (280, 280, 280), True): 535.400704e6 + 192.98304e6 + 219.822848e6 + 40.7488e6,
    ("update_h", "fp32", (280, 280, 280), True): 504.384e6 + 190.464e6 + 187.740672e6 + 34.299904e6,
    ("update_e", "fp32", (532, 532, 404), True): 2900.651264e6 + 1209.392128e6 + 771.828736e6 + 213.485312e6,
    ("update_h", "fp32", (532, 532, 404), False): 2521.388032e6 + 1068.519424e6 + 891.773952e6 + 356.841984e6,
}


def dominant(prof) -> str:
    """The main-stream entry with the largest device time."""
    return max((k for k in prof if k not in SIDE_STREAM_KERNELS), key=lambda k: prof[k][0])


def algorithmic_bytes(n, slab_layers, precision: str, kernel: str, split=None, ib: int = 1) -> float:
    """Bytes one E (or H) volume update must move at least: per cell read
    the 3 own components and the 3 curl components, write the 3 own
    components, read the material index (ib bytes); inside CPML slabs read and
    write one psi per (component, slab axis) pair (2 per slab axis).  The
    update runs as two concurrent launches, an interior and a shell launch
    (cells split["e_interior"] / ["e_shell"], likewise for H); in the narrow
    decomposition the shell launch carries all psi traffic, in the wide one
    (split["e_wide"]) the interior launch carries the x- and y-slab psi and
    the shell launch the z-slab psi.  "update_e" / "update_h" is the pair.
    Fused sweep (E and H of one step): read and write all 6 components once
    and the index once; psi traffic of both halves."""
    nx, ny, nz = n
    cells = nx * ny * nz
    w = 8 if precision == "fp64" else 4
    psi_xy = (slab_layers[0] * ny * nz + slab_layers[1] * nx * nz) * 2 * 2 * w
    psi_z = slab_layers[2] * nx * ny * 2 * 2 * w
    psi = psi_xy + psi_z
    if kernel == "sweep_eh":
        return cells * (12 * w + ib) + psi * 2
    if split is not None:
        side = kernel[7]
        wide = split.get(side + "_wide", False)
        if kernel.endswith("_interior"):
            return split[side + "_interior"] * (9 * w + ib) + (psi_xy if wide else 0)
        if kernel.endswith("_shell"):
            return split[side + "_shell"] * (9 * w + ib) + (psi_z if wide else psi)
        return (split[side + "_interior"] + split[side + "_shell"]) * (9 * w + ib) + psi
    return cells * (9 * w + ib) + psi


def _slab_layers(sc):
    lay = [0, 0, 0]
    for b in sc.boundaries:
        lay[b.orientation // 2] += b.thickness
    return lay


# -------------------------------------------------------------------- arms ---
def headline_config(world: int) -> dict:
    """The workload both arms report on (the same dict on both lines)."""
    return {"workload": WORKLOAD, "cells": 532 * 532 * 404, "grid": [532, 532, 404], "steps_per_job": 1000,
            "l2": "no flush: inputs larger than L2 (each field component 456 MB in FP32, 912 MB in FP64, "
                  "against the 129 MB L2)",
            "parallelism": f"replicas x{world}"}


def run_cpu_oracle(threads: int, sample_steps: int, scale: int = 2):
    """FP64 CPU oracle on the headline workload at 1/`scale` per axis (the
    same scene family and per-cell arithmetic): init untimed,
    `sample_steps` steps timed.  Returns (Mcell-updates/s, cores, sample
    description)."""
    import oracle
    oracle.build()
    cores = oracle.set_threads(threads)
    sc, _ = configs.heterogeneous(scale=scale)
    o = oracle.OracleSim(sc, sample_steps + 1)
    o.step(1)   # first touch
    t0 = time.perf_counter()
    o.step(sample_steps)
    dt = time.perf_counter() - t0
    cells = o.n[0] * o.n[1] * o.n[2]
    grid = "x".join(str(v) for v in o.n)
    del o
    return cells * sample_steps / dt / 1e6, cores, (f"{sample_steps} steps of the {grid} grid (the heterogeneous "
                                                    f"medium at 1/{scale} per axis), {cores} thread(s), {dt:.1f} s")


def reference_arm(args, world, rank):
    """The reference's algorithm (its FP64 CPU step loop, restated in
    oracle/: the reference itself does not build here) on all host threads,
    on the headline workload.  Each bench step is one oracle time step of
    the heterogeneous-medium scene on a grid sized so that the whole
    --warmup W --steps K run stays within about --ref-budget seconds."""
    base = {"metric": METRIC, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": headline_config(world)}
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle
    oracle.build()
    cores = oracle.set_threads(threads)
    cal, _ = configs.heterogeneous(scale=8)   # calibration: seconds per cell-update
    oc = oracle.OracleSim(cal, 6)
    oc.step(1)
    t0 = time.perf_counter()
    oc.step(4)
    per_cell = (time.perf_counter() - t0) / 4 / (oc.n[0] * oc.n[1] * oc.n[2])
    del oc
    budget_step = args.ref_budget / (args.warmup + args.steps)
    scale = 1
    for s in (1, 2, 4, 8):
        scale = s
        nx, ny, nz = 512 // s + 20, 512 // s + 20, 384 // s + 20
        if nx * ny * nz * per_cell <= budget_step:
            break
    sc, _ = configs.heterogeneous(scale=scale)
    o = oracle.OracleSim(sc, args.warmup + args.steps + 1)
    cells = o.n[0] * o.n[1] * o.n[2]
    o.step(1)
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    tot = time.perf_counter() - t0
    v = cells * args.steps / tot / 1e6
    grid = "x".join(map(str, o.n))
    line = dict(base)
    line.update({"value": v, "ms_per_step": 1e3 * tot / args.steps,
                 "cpu_baseline": dict({"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                       "sample": f"{args.steps} oracle steps (after {args.warmup} warm-up steps) of "
                                                 f"the {grid} grid: the headline workload at 1/{scale} per axis, "
                                                 f"{cores} threads"}, **_cpu_info()),
                 "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                 "note": "the reference does not build here (xtensor, xtensor-blas, xtensor-fftw, FFTW3, BLAS and "
                         "LAPACK are absent); its FP64 step loop is restated in oracle/"})
    print(json.dumps(line), flush=True)


def run_batched_form(args, local):
    """The batched form: many uneven scatterer problems (interior 32 .. 160
    cells per axis, 8-cell CPML, 500 .. 1500 steps each) advanced as one
    batch (TMA-staged volume launches for the members whose grids allow
    them), against the same problems run one after another with the plain
    single-simulation kernels on the same GPU.  Both timed with CUDA events
    over the step loops (set-up excluded), FP32."""
    import xfdtd_gb300 as X
    probs = configs.batched_scatterers(n=args.batch_problems)
    members = [X.Simulation(sc, st, precision="fp32", fused=False, autotune=False, device=local) for sc, st in probs]
    cells = [m.n[0] * m.n[1] * m.n[2] for m in members]
    work = sum(c * st for c, (_, st) in zip(cells, probs))
    b = X.Batch(members, graph=True)
    n_tma = b.tma_members()
    ms_b = b.step_timed(max(st for _, st in probs))
    b.synchronize()
    launches = b.status()["launches"]
    for m in members:
        m.check_finite()
    del b, members
    ms_s = 0.0
    alone = []   # (cells, cell-updates, ms) of each problem run alone
    for sc, st in probs:   # sequential: each problem alone, plain split kernels, graph replay
        s = X.Simulation(sc, st, precision="fp32", fused=False, autotune=False, device=local)
        ms = s.step_timed(st)
        alone.append((s.n[0] * s.n[1] * s.n[2], s.n[0] * s.n[1] * s.n[2] * st, ms))
        ms_s += ms
        del s
    # throughput of the problems alone, by size: the batch's gain is in packing the small ones
    bins = {}
    for lo, hi, name in ((0, 5e5, "<0.5M cells"), (5e5, 2e6, "0.5-2M cells"), (2e6, 1e12, ">=2M cells")):
        sel = [a for a in alone if lo <= a[0] < hi]
        if sel:
            bins[name] = {"problems": len(sel), "alone_value": sum(a[1] for a in sel) / (sum(a[2] for a in sel) / 1e3) / 1e6}
    return {"problems": len(probs), "cells_total": sum(cells), "cell_updates": work,
            "value": work / (ms_b / 1e3) / 1e6, "unit": UNIT, "ms": ms_b, "launches": launches,
            "sequential_value": work / (ms_s / 1e3) / 1e6, "sequential_ms": ms_s,
            "speedup_vs_sequential": ms_s / ms_b, "tma_members": n_tma, "sequential_by_size": bins,
            "workload": "64 dielectric-sphere problems, interior U{32..160}^3 + 8-cell CPML, "
                        "steps U{500..1500}, seeds 4000+i"}


def run_adjoint_form(args, local):
    """The adjoint form: dL/d eps_r over a 64 x 64 x 32 design region of the
    160 x 160 x 96 (+ 10-cell CPML) dipole problem, L = sum of Ez^2 over a
    64 x 64 plane over the last 400 of 2000 steps, FP32 forward and reverse
    passes.  `adjoint_checkpoint` K: 0 records the design box at every step
    (no recomputation; about 6 GB here, small beside the GPU's HBM), K > 0
    keeps a full checkpoint every K steps and recomputes each segment in the
    backward pass.  Times: the plain FP32 forward run (CUDA events), the
    recording forward and the backward pass (wall clock around the
    synchronous calls).  Check: central differences of the FP64 forward loss
    (eps_r +- 1e-4, set in double) at `adjoint_fd` seeded design voxels."""
    import xfdtd_gb300 as X
    sc, st, spec = configs.adjoint_dipole()
    keys = ("design_lo", "design_hi", "plane_axis", "plane_index", "plane_lo", "plane_hi", "t_begin", "t_end",
            "loss_comp", "checkpoint_every")
    sa = {q: spec[q] for q in keys}
    sa["checkpoint_every"] = args.adjoint_checkpoint
    plain = X.Simulation(sc, st, precision="fp32", fused=False, autotune=False, device=local)
    fwd_ms = plain.step_timed(st)
    cells = plain.n[0] * plain.n[1] * plain.n[2]
    del plain
    g = X.Simulation(sc, st, precision="fp32", fused=False, autotune=False, device=local)
    t0 = time.perf_counter()
    loss = g.adjoint_forward(**sa)
    t1 = time.perf_counter()
    dev_bytes = g.device_bytes()
    ge, _ = g.adjoint_backward()
    t2 = time.perf_counter()
    del g
    out = {"grid": cells, "steps": st, "design_cells": int(ge.size), "loss": loss,
           "forward_ms": fwd_ms, "adjoint_forward_ms": (t1 - t0) * 1e3, "backward_ms": (t2 - t1) * 1e3,
           "backward_over_forward": (t2 - t1) * 1e3 / fwd_ms,
           "gradient_over_forward": (t2 - t0) * 1e3 / fwd_ms,
           "value": cells * st / ((t2 - t1)) / 1e6, "unit": "Mcell-updates/s (reverse pass)",
           "checkpoint_every": args.adjoint_checkpoint, "device_bytes": dev_bytes}
    if args.adjoint_checkpoint > 0:
        # the same gradient with the design box recorded at every step (no
        # re-run of the segments; the records fit GB300's HBM many times over)
        g0 = X.Simulation(sc, st, precision="fp32", fused=False, autotune=False, device=local)
        t0 = time.perf_counter()
        g0.adjoint_forward(**dict(sa, checkpoint_every=0))
        t1 = time.perf_counter()
        ge0, _ = g0.adjoint_backward()
        t2 = time.perf_counter()
        out["record_every_step"] = {"adjoint_forward_ms": (t1 - t0) * 1e3, "backward_ms": (t2 - t1) * 1e3,
                                    "gradient_over_forward": (t2 - t0) * 1e3 / fwd_ms,
                                    "device_bytes": g0.device_bytes(),
                                    "same_gradient": bool(np.array_equal(ge0, ge))}
        del g0
    if args.adjoint_fd > 0:
        import copy
        rng = np.random.default_rng(5002)
        dsz = ge.shape
        picks = [tuple(int(rng.integers(0, n)) for n in dsz) for _ in range(args.adjoint_fd)]
        sb = dict(sa, checkpoint_every=st)   # one checkpoint: the FD runs only need the loss

        def loss_with(cell, eps):
            # eps_r set in double (the float Material ctor would round the
            # 1e-4 step)
            sc2 = copy.copy(sc)
            sc2.voxel_materials = list(sc.voxel_materials)
            q = 1 + int(np.ravel_multi_index(cell, dsz))
            sc2.voxel_materials[q] = S.Material("d", eps, 1.0, 0.0, 0.0, exact_eps=True)
            s64 = X.Simulation(sc2, st, precision="fp64", fused=False, autotune=False, device=local)
            return s64.adjoint_forward(**sb)

        rel = []
        for cell in picks:
            e0 = float(spec["eps"][cell])
            lp = loss_with(cell, e0 + 1e-4)
            lm = loss_with(cell, e0 - 1e-4)
            fd = (lp - lm) / 2e-4
            rel.append(abs(ge[cell] - fd) / abs(fd))
        out["fd_check"] = {"voxels": len(picks), "h": 1e-4, "forward": "fp64", "eps_r": "double",
                           "max_rel_err": float(max(rel)), "median_rel_err": float(np.median(rel))}
    return out


def _timed(sc, precision, steps, warmup, local, grp=None, fused=False, variants=None):
    """The production path over `steps` timed steps: after `warmup` steps
    the run is brought to a graph boundary (untimed steps, one graph
    captured and replayed), then exactly `steps` steps are timed with CUDA
    events on the engine's stream (graph replays of GRAPH_STEPS steps,
    single launches for the rest).  Returns the run's facts."""
    import xfdtd_gb300 as X
    setup = GRAPH_STEPS - warmup % GRAPH_STEPS + GRAPH_STEPS
    sim = X.Simulation(sc, warmup + setup + steps, precision=precision, graph=True, device=local, fused=fused)
    if variants:
        sim.set_kernel_variant(*variants[0])
        sim.set_shell_variant(*variants[1])
    n = sim.n
    sim.step(warmup)
    sim.step(setup)
    sim.synchronize()
    l0 = sim.launch_count()
    if grp is not None:
        grp.barrier()
    ms = sim.step_timed(steps)
    sim.synchronize()
    if grp is not None:
        grp.barrier()
    out = {"n": tuple(n), "cells": n[0] * n[1] * n[2], "ms": ms, "launches": sim.launch_count() - l0,
           "variants": sim.kernel_variants(), "shell_variants": sim.shell_variants(), "split": sim.volume_split(),
           "tfsf_folded": sim.tfsf_fusion(), "nffft_schedule": sim.nffft_split(), "index_bytes": sim.index_bytes(),
           "setup_steps": setup,
           "timed_path": f"{steps // GRAPH_STEPS} CUDA graph replays of {GRAPH_STEPS} steps + "
                         f"{steps % GRAPH_STEPS} single steps, after {warmup} warm-up steps and {setup} untimed "
                         f"steps to reach a graph boundary and capture the graph"}
    sim.check_finite()
    del sim
    return out


def _profiled(sc, precision, steps, warmup, local, run, fused=False):
    """Per-kernel device times of `steps` steps with CUDA events around every
    launch (no graph), with the timed run's variants, and the roofline of
    the dominant main-stream entry (algorithmic bytes / its mean time)."""
    import xfdtd_gb300 as X
    psim = X.Simulation(sc, warmup + steps, precision=precision, graph=False, profile=True, device=local,
                        fused=fused)
    psim.set_kernel_variant(run["variants"]["e"], run["variants"]["h"])
    psim.set_shell_variant(run["shell_variants"]["e"], run["shell_variants"]["h"])
    psim.set_tfsf_fusion(*run["tfsf_folded"])
    psim.set_nffft_split(run["nffft_schedule"]["split"])
    assert psim.volume_split() == run["split"]
    assert psim.tfsf_fusion() == run["tfsf_folded"]
    psim.step(warmup)
    psim.synchronize()
    psim.profile_reset()
    total_ms = psim.step_timed(steps)
    prof = psim.profile()
    del psim
    side = {k: prof.pop(k) for k in SIDE_STREAM_KERNELS if k in prof}
    dom = dominant(prof)
    dom_ms, dom_n = prof[dom]
    slabs = _slab_layers(sc)
    n, split, ib = run["n"], run["split"], run["index_bytes"]
    alg = algorithmic_bytes(n, slabs, precision, dom, split, ib)
    peak, peak_kind = _peaks()
    achieved = alg / (dom_ms / dom_n / 1e3) / 1e9
    total_prof = sum(v[0] for v in prof.values())
    shares = {k: round(v[0] / total_prof, 4) for k, v in prof.items()}
    shares.update({f"{k} (concurrent)": round(v[0] / total_prof, 4) for k, v in side.items()})
    concurrent = {k: {"ms_per_launch": v[0] / max(v[1], 1),
                      "algorithmic_GBs": algorithmic_bytes(n, slabs, precision, k, split, ib) / (v[0] / max(v[1], 1) / 1e3) / 1e9}
                  for k, v in side.items() if k.startswith("update_")}
    # both volume updates over the whole profiled step: 2 x the pair's bytes
    # per step over the step time (the small surface launches included)
    pair = (algorithmic_bytes(n, slabs, precision, "update_e", split, ib)
            + algorithmic_bytes(n, slabs, precision, "update_h", split, ib))
    step_frac = pair / (total_ms / steps / 1e3) / 1e9 / peak
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind,
            "traffic": NCU_TRAFFIC.get((dom, precision, tuple(n), split.get(dom[7] + "_wide"))),
            "algorithmic_bytes_per_launch": alg, "index_bytes": ib, "launch_ms": dom_ms / dom_n,
            "step_frac": step_frac,
            "timing": f"CUDA events around each launch in a profiled pass of {steps} steps "
                      f"({total_ms / steps:.4f} ms/step, no graph)"}
    return roof, shares, concurrent


def _e2e(sc, precision, steps, local, fused=False, readout="rcs"):
    """One whole job through the public API (the reference's
    Simulation(...); run(steps); outputs): host scene -> plan (lowering on
    the host) -> engine create (device allocation, upload, autotuning) ->
    `steps` steps -> far field / monitors copied back to the host.  Wall
    clock per phase."""
    import xfdtd_gb300 as X
    t0 = time.perf_counter()
    job = X.Simulation(sc, steps, precision=precision, graph=True, device=local, fused=fused)
    t1 = time.perf_counter()
    ct = job.create_times()
    job.step(steps)
    job.synchronize()
    t2 = time.perf_counter()
    if readout == "rcs":
        result = job.rcs_db()
    else:
        result = np.stack([job.read_monitor(m) for m in range(len(sc.monitors))])
    t3 = time.perf_counter()
    h2d, d2h = job.transfer_bytes()
    n = job.n
    del job
    assert np.isfinite(result).all()
    cells = n[0] * n[1] * n[2]
    wall = t3 - t0
    create_s = t1 - t0
    phases = {"lowering_s": create_s - (ct["alloc_upload_ms"] + ct["autotune_ms"]) / 1e3,
              "alloc_upload_s": ct["alloc_upload_ms"] / 1e3, "autotune_s": ct["autotune_ms"] / 1e3,
              "steps_s": t2 - t1, "readout_s": t3 - t2}
    e2e = {"value": cells * steps / wall / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d / steps,
           "d2h_bytes_per_step": d2h / steps, "wall_s": wall, "steps": steps, "phases": phases,
           "scope": "host scene -> plan lowering -> device allocation and upload -> autotuning -> "
                    f"{steps} steps (CUDA graph replay) -> "
                    + ("far field and RCS copied to the host" if readout == "rcs" else "probe series copied to the host")}
    return e2e, result


def _rcs_err(a, b):
    d = np.abs(a - b)
    return {"rcs_db_max": float(d.max()), "rcs_db_median": float(np.median(d))}


def _probe_err(a, b):
    rel = np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)
    return {"probe_l2_max": float(rel.max()), "probe_l2_median": float(np.median(rel))}


def run_fp64_form(args, local, sc, timed_steps, job_steps, fp32_out, readout, fused):
    """The FP64 form (the reference's arithmetic) of a workload: timed steps
    through graph replay, the dominant kernel's roofline at 146 B per
    cell-update, the whole job end to end, and the FP32 form's error
    against it (probe series or RCS of the same job)."""
    run = _timed(sc, "fp64", timed_steps, args.warmup, local, fused=fused)
    roof, shares, _ = _profiled(sc, "fp64", min(timed_steps, PROFILE_STEPS), args.warmup, local, run, fused=fused)
    e2e, out64 = _e2e(sc, "fp64", job_steps, local, fused=fused, readout=readout)
    err = None
    if fp32_out is not None:
        err = dict(_rcs_err(fp32_out, out64) if readout == "rcs" else _probe_err(fp32_out, out64),
                   against="this FP64 form, same job", steps=job_steps)
    return {"value": run["cells"] * timed_steps / (run["ms"] / 1e3) / 1e6, "unit": UNIT,
            "steps": timed_steps, "ms_per_step": run["ms"] / timed_steps, "dtype": "f64",
            "timed_path": run["timed_path"], "roofline": roof, "kernel_shares": shares, "e2e": e2e,
            "fp32_form_error": err,
            "note": "GB300 runs FP64 at 1/64 of the FP32 rate: the FP64 volume kernels are bound by "
                    "the FP64 pipe, not by HBM (frac is of the copy bandwidth)"}


def run_dielectric_form(args, local):
    """The dielectric-sphere scattering configuration: 256^3 interior +
    12-cell CPML (280^3 cells), eps_r 4 sphere of radius 60 cells, TFSF
    x-polarised +z Gaussian plane wave (tau = 40 dt), NF-FF DFT at 1, 2 and
    3 GHz, bistatic RCS at 181 angles in two planes, 2000 steps.  FP32 form
    (its update's target: 70 % of the copy bandwidth): timed steps, roofline, the whole job end
    to end; FP64 form likewise, with the FP32 RCS error against it."""
    sc, job_steps = configs.dielectric_sphere()
    fused = False   # the split E and H kernels (the fused sweep is slower on this grid)
    run = _timed(sc, "fp32", args.dielectric_steps, args.warmup, local, fused=fused)
    roof, shares, conc = _profiled(sc, "fp32", min(args.dielectric_steps, PROFILE_STEPS), args.warmup, local, run,
                                   fused=fused)
    e2e, rcs32 = _e2e(sc, "fp32", job_steps, local, fused=fused, readout="rcs")
    v, sv = run["variants"], run["shell_variants"]
    out = {"workload": "dielectric sphere scattering: 256^3 interior + 12-cell CPML (280^3 cells), dx 2 mm, "
                       "eps_r 4 sphere r=60 cells, TFSF x-pol +z Gaussian, NF-FF 1/2/3 GHz",
           "grid": list(run["n"]), "cells": run["cells"], "steps": args.dielectric_steps,
           "value": run["cells"] * args.dielectric_steps / (run["ms"] / 1e3) / 1e6, "unit": UNIT,
           "ms_per_step": run["ms"] / args.dielectric_steps, "dtype": "f32", "timed_path": run["timed_path"],
           "launches": run["launches"], "roofline": roof, "kernel_shares": shares,
           "volume_split_cells": run["split"], "volume_kernels_concurrent": conc,
           "autotuned_variants": {"update_e": v["e"], "update_h": v["h"], "shell_e": sv["e"], "shell_h": sv["h"],
                                  "tfsf_folded": {"e": run["tfsf_folded"][0], "h": run["tfsf_folded"][1]},
                                  "nffft_schedule": run["nffft_schedule"],
                                  "trial_ms_e": [round(q, 4) for q in v["trials_e"]],
                                  "trial_ms_h": [round(q, 4) for q in v["trials_h"]]},
           "e2e": e2e, "l2": "no flush: fields 6 x %.0f MB > 129 MB L2" % (run["cells"] * 4 / 1e6)}
    if args.dielectric_fp64_steps > 0:
        out["fp64_form"] = run_fp64_form(args, local, sc, args.dielectric_fp64_steps, job_steps, rcs32, "rcs", fused)
        out["fp32_form_error"] = out["fp64_form"]["fp32_form_error"]
    return out


def _cpu_info():
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k = line.split(":")[0].strip().lower()
                if k in ("model name", "cpu model", "hardware") and ":" in line:
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if not model:
        try:
            r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
            for line in r.stdout.splitlines():
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    import platform
    return {"cpu_model": model or platform.processor() or platform.machine(), "nproc": os.cpu_count(),
            "machine": platform.machine()}


def ours_arm(args, world, rank, local, grp):
    import xfdtd_gb300 as X
    X.build()
    clock = ClockSampler(local)
    clock.start()
    sc, job_steps = configs.heterogeneous()
    fused = {"auto": None, "fused": True, "split": False}[args.volume]
    fixed = None
    if args.kernel_variant or args.shell_variant:
        fixed = (tuple(int(v) for v in (args.kernel_variant or "0,0").split(",")),
                 tuple(int(v) for v in (args.shell_variant or "0,0").split(",")))
    # the headline: the FP32 form of the heterogeneous medium, timed steps
    # through the production path
    run = _timed(sc, "fp32", args.steps, args.warmup, local, grp=grp, fused=fused, variants=fixed)
    n, cells, split = run["n"], run["cells"], run["split"]
    max_ms = grp.max(run["ms"])
    value = aggregate_value(cells, args.steps, world, max_ms)
    roof, shares, concurrent = _profiled(sc, "fp32", min(args.steps, PROFILE_STEPS), args.warmup, local, run,
                                         fused=fused)

    # e2e: the config's whole job through the public API, host scene to host probe series
    grp.barrier()
    e2e, p32 = _e2e(sc, "fp32", args.e2e_steps or job_steps, local, fused=fused, readout="probes")
    e2e_wall = grp.max(e2e["wall_s"])
    e2e["value"] = cells * e2e["steps"] * world / e2e_wall / 1e6
    e2e["wall_s"] = e2e_wall

    fp64 = None
    if args.fp64_steps > 0 and rank == 0:
        fp64 = run_fp64_form(args, local, sc, args.fp64_steps, args.e2e_steps or job_steps, p32, "probes", fused)
    dielectric = run_dielectric_form(args, local) if (args.dielectric_steps > 0 and rank == 0) else None
    batched = run_batched_form(args, local) if (args.batch_problems > 0 and rank == 0) else None
    adjoint = run_adjoint_form(args, local) if (args.adjoint and rank == 0) else None

    cpu = None
    if rank == 0 and world == 1 and args.cpu_sample > 0:
        v, cores, sample = run_cpu_oracle(1, args.cpu_sample)
        cpu = dict({"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}, **_cpu_info())
    clocks = clock.stop()

    if rank != 0:
        return
    v = run["variants"]
    sv = run["shell_variants"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(world),
        "timed_path": run["timed_path"],
        "roofline": roof,
        "kernel_shares": shares,
        "volume_split_cells": split,
        "volume_kernels_concurrent": concurrent,
        "autotuned_variants": {"update_e": v["e"], "update_h": v["h"], "shell_e": sv["e"], "shell_h": sv["h"],
                               "tfsf_folded": {"e": run["tfsf_folded"][0], "h": run["tfsf_folded"][1]},
                               "trial_ms_e": [round(q, 4) for q in v["trials_e"]],
                               "trial_ms_h": [round(q, 4) for q in v["trials_h"]]},
        "e2e": e2e,
        "gpu_launches": run["launches"],
        "clocks": clocks,
        "cpu_baseline": cpu,
        "accuracy": {
            "fp32_vs_fp64_engine": (fp64 or {}).get("fp32_form_error"),
            "against_oracle": "tests/test_gpu_fullsize.py compares the FP64 form with the CPU oracle at every "
                              "config's full grid (1e-10) and bounds the FP32 form's errors against it",
        },
        "fp64_form": fp64,
        "dielectric_form": dielectric,
        "batched_form": batched,
        "adjoint_form": adjoint,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=100, help="timed steps of the headline's FP64 form (0: skip)")
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="steps of the headline's whole job end to end (0: the config's 1000)")
    ap.add_argument("--cpu-sample", type=int, default=10, help="oracle steps timed for cpu_baseline (0: skip)")
    ap.add_argument("--ref-budget", type=float, default=120.0, help="seconds of oracle work for --impl reference")
    ap.add_argument("--volume", default="auto", choices=["split", "fused", "auto"],
                    help="volume kernels of the headline: the split E and H kernels, the fused E/H sweep, or the "
                         "autotuner's choice")
    ap.add_argument("--dielectric-steps", type=int, default=2000,
                    help="timed steps of the dielectric-sphere form (0: skip)")
    ap.add_argument("--dielectric-fp64-steps", type=int, default=200,
                    help="timed steps of the dielectric-sphere FP64 form (0: skip)")
    ap.add_argument("--batch-problems", type=int, default=64, help="problems of the batched form (0: skip)")
    ap.add_argument("--adjoint", type=int, default=1, help="run the adjoint form (0: skip)")
    ap.add_argument("--adjoint-fd", type=int, default=16, help="design voxels of the adjoint FD check (0: skip)")
    ap.add_argument("--adjoint-checkpoint", type=int, default=100,
                    help="adjoint form: checkpoint every K steps (0: record the design box at every step)")
    ap.add_argument("--kernel-variant", default=None, metavar="E,H",
                    help="fix the interior variants of the headline run (after autotuning; for a launch list "
                         "under a profiler, whose timings would mislead the autotuner)")
    ap.add_argument("--shell-variant", default=None, metavar="E,H", help="fix the shell variants likewise")
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, world, rank)
        return
    grp = _Group(world, local)
    try:
        ours_arm(args, world, rank, local, grp)
    finally:
        grp.close()


if __name__ == "__main__":
    main()
