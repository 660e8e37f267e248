"""Command-line runner for the built-in configurations.

    python -m xfdtd_gb300.run --config dielectric_sphere --steps 20 --precision fp32
    python -m xfdtd_gb300.run --config pec_sphere_rcs --steps 800 --out out_dir

Builds the scene, runs it on the GPU engine and prints one JSON line with
the grid, the device time per step and Mcell-updates/s; with --out it also
writes the reference's .npy outputs (far field, monitors).  It is also the
small driver that profilers wrap.
"""
import argparse
import json
import os
import time

from . import Simulation, build, configs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="dielectric_sphere", choices=sorted(configs.CONFIGS))
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--scale", type=int, default=1)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--volume", default="auto", choices=["auto", "fused", "split"],
                    help="volume kernels: autotuned choice, the fused E/H sweep, or the split E and H kernels")
    ap.add_argument("--kernel-variant", default=None, metavar="E,H",
                    help="interior-kernel variants of the E and H updates (after autotuning; for profiling a "
                         "fixed variant)")
    ap.add_argument("--shell-variant", default=None, metavar="E,H",
                    help="shell-kernel variants of the E and H updates (after the interior variants)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the autotuner's trials (with --kernel-variant, for profiling one launch per step)")
    ap.add_argument("--tfsf-fusion", default="auto", choices=["auto", "on", "off"],
                    help="TFSF corrections inside the wide TMA launches: the autotuner's choice, or fixed")
    ap.add_argument("--nffft-split", default="auto", choices=["auto", "on", "off"],
                    help="NF-FF sampling schedule: the autotuner's choice, split halves beside the volume "
                         "updates (on) or one launch after the H update (off)")
    ap.add_argument("--out", default=None)
    ap.add_argument("--adjoint", action="store_true",
                    help="run the adjoint-gradient problem (forward with checkpoints, then backward) instead")
    args = ap.parse_args()
    build()
    if args.adjoint:
        run_adjoint(args)
        return
    sc, steps = configs.CONFIGS[args.config](scale=args.scale)
    if args.steps is not None:
        steps = args.steps
    if args.out and sc.nffft is not None:
        sc.nffft.output_dir_path = args.out
    t0 = time.perf_counter()
    fused = {"auto": None, "fused": True, "split": False}[args.volume]
    sim = Simulation(sc, steps, precision=args.precision, graph=not args.no_graph, fused=fused,
                     autotune=not args.no_autotune)
    if args.kernel_variant:
        sim.set_kernel_variant(*(int(v) for v in args.kernel_variant.split(",")))
    if args.shell_variant:
        sim.set_shell_variant(*(int(v) for v in args.shell_variant.split(",")))
    if args.tfsf_fusion != "auto":
        sim.set_tfsf_fusion(args.tfsf_fusion == "on", args.tfsf_fusion == "on")
    if args.nffft_split != "auto":
        sim.set_nffft_split(args.nffft_split == "on")
    t1 = time.perf_counter()
    ms = sim.step_timed(steps)
    sim.synchronize()
    cells = sim.n[0] * sim.n[1] * sim.n[2]
    res = {"config": args.config, "grid": sim.n, "steps": steps, "precision": args.precision,
           "setup_s": t1 - t0, "ms_per_step": ms / steps, "Mcell_updates_per_s": cells * steps / ms / 1e3,
           "device_bytes": sim.device_bytes(), "volume_kernels": sim.kernel_variants(),
           "shell_variants": sim.shell_variants(), "tfsf_folded": sim.tfsf_fusion(), "nffft_schedule": sim.nffft_split()}
    if args.out:
        os.makedirs(args.out, exist_ok=True)
        sim.output()
    print(json.dumps(res))


def run_adjoint(args):
    sc, steps, spec = configs.adjoint_dipole(scale=args.scale)
    if args.steps is not None:
        steps = args.steps
        spec["t_begin"], spec["t_end"] = steps - steps // 5, steps
    keys = ("design_lo", "design_hi", "plane_axis", "plane_index", "plane_lo", "plane_hi", "t_begin", "t_end",
            "loss_comp", "checkpoint_every")
    sim = Simulation(sc, steps, precision=args.precision, fused=False, autotune=False)
    t0 = time.perf_counter()
    loss = sim.adjoint_forward(**{k: spec[k] for k in keys})
    t1 = time.perf_counter()
    ge, _ = sim.adjoint_backward()
    t2 = time.perf_counter()
    print(json.dumps({"config": "adjoint_dipole", "scale": args.scale, "grid": sim.n, "steps": steps,
                      "loss": loss, "forward_s": t1 - t0, "backward_s": t2 - t1,
                      "grad_eps_absmax": float(abs(ge).max())}))


if __name__ == "__main__":
    main()
