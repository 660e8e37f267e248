"""Writes the golden vectors in tests/golden/ from the CPU oracle.

For each small test scene (tests/scenes.py) it runs the oracle and stores
per-component x-plane sums and the middle x-slice of every field, every
monitor time series and (with NF-FF) three far-field arrays; for the
output-format scenes, every frame of their field and movie monitors and
their broadband far field.  The files pin
the oracle between machines and commits; regenerate only after a deliberate
change of the restatement:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import oracle as O  # noqa: E402
import scenes  # noqa: E402


def main():
    O.set_threads(8)
    for name, fn in sorted(scenes.SCENES.items()):
        sc, steps = fn()
        o = O.OracleSim(sc, steps)
        o.step(steps)
        out = {"steps": np.array(steps)}
        for c in range(6):
            f = o.read_field(c)
            out[f"f{c}_xsum"] = f.sum(axis=(1, 2))
            out[f"f{c}_slice"] = f[f.shape[0] // 2].astype(np.float64)
        for m in range(len(sc.monitors)):
            out[f"m{m}"] = o.read_monitor(m)
        if sc.nffft is not None:
            for w in (0, 1, 8):
                out[f"ff{w}"] = o.far_field(w)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, os.path.getsize(os.path.join(HERE, f"{name}.npz")))
    # the output formats: every frame of the field and movie monitors, the
    # broadband far field (e_theta, e_phi, power_theta and the bin frequencies)
    for name, fn in sorted(scenes.OUTPUT_SCENES.items()):
        sc, steps = fn()
        o = O.OracleSim(sc, steps)
        o.step(steps)
        out = {"steps": np.array(steps)}
        for m, mon in enumerate(sc.monitors):
            if mon.kind != 2:   # field and movie monitors only
                continue
            _, _, frames = o.field_monitor_frames(m)
            out[f"steps{m}"] = np.array(frames)
            for f in range(len(frames)):
                out[f"mon{m}_{f}"] = o.read_field_monitor(m, f)
        if sc.nffft is not None:
            for w in (0, 1, 8, 10):
                out[f"ff{w}"] = o.far_field(w)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, os.path.getsize(os.path.join(HERE, f"{name}.npz")))


if __name__ == "__main__":
    main()
