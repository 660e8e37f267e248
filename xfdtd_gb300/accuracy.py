"""Accuracy of the FP32 form against the FP64 form on the benchmark
configurations (the FP64 engine matches the CPU restatement of the
reference within 1e-10 on the test scenes).

    python -m xfdtd_gb300.accuracy --config dielectric_sphere [--steps N]

prints one JSON line: relative L2 error of every field component at the
last step, the RCS error in dB (median, max, and max over the angles within
30 dB of the peak) where the scene has an NF-FF box, and the relative L2
error of the monitor time series where it has monitors.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import Simulation, configs


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def compare(sc, steps):
    out = {"steps": steps}
    t0 = time.perf_counter()
    ref = Simulation(sc, steps, precision="fp64")
    ref.step(steps)
    f32 = Simulation(sc, steps, precision="fp32")
    f32.step(steps)
    out["run_s"] = time.perf_counter() - t0
    out["grid"] = list(ref.n)
    out["field_l2"] = [_rel_l2(f32.read_field(c), ref.read_field(c)) for c in range(6)]
    if sc.nffft is not None:
        d64, d32 = ref.rcs_db(), f32.rcs_db()
        err = np.abs(d32 - d64)
        near = d64 >= d64.max(axis=(1, 2), keepdims=True) - 30
        out["rcs_db"] = {"median": float(np.median(err)), "max": float(err.max()),
                         "max_within_30dB_of_peak": float(err[near].max())}
    if sc.monitors:
        out["monitor_l2"] = max(_rel_l2(f32.read_monitor(m), ref.read_monitor(m)) for m in range(len(sc.monitors)))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--config", default="dielectric_sphere", choices=sorted(configs.CONFIGS))
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--scale", type=int, default=1)
    a = ap.parse_args(argv)
    sc, steps = configs.CONFIGS[a.config](scale=a.scale)
    if a.steps:
        steps = a.steps
    out = {"config": a.config, "scale": a.scale}
    out.update(compare(sc, steps))
    print(json.dumps(out))


if __name__ == "__main__":
    main()
