"""Writes the golden vectors in tests/golden/ from the CPU oracle.

For each small test scene (tests/scenes.py) it runs the oracle and stores
per-component x-plane sums and the middle x-slice of every field, every
monitor time series and (with NF-FF) three far-field arrays.  The files pin
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


if __name__ == "__main__":
    main()
