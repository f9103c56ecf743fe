"""Small profiling case: the 1M impact's geometry at a chosen particle count.

Uploads the two-layer impact (90% target, 10% impactor, synthetic iron /
dunite tables), runs the prologue and a few steps, and prints the per-segment
device times.  Meant to run under a profiler on a case that keeps a capture
small (e.g. 400,000 particles hold about 1.5 GB on the device):

    python -m fdps_sph_gb300.profile_case --n 400000 --steps 2
"""
import argparse
import time

from . import eos, ic, lib


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=400_000, help="total particles")
    ap.add_argument("--steps", type=int, default=2, help="steps after the prologue")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--tpi", type=int, default=4, choices=[1, 2, 4],
                    help="threads per particle of the mixed derivative / hydro kernels")
    a = ap.parse_args(argv)
    n_t = int(a.n * 0.9)
    F, ids, mats, _ = ic.config_1m_impact(seed=2024, n_target=n_t, n_impactor=a.n - n_t)
    ctx = lib.Context(precision=a.precision)
    for k, name in enumerate(("iron", "dunite")):
        ctx.set_material(k, eos.synthetic_table(name))
    ctx.upload(F, ids, mats)
    if a.precision == "mixed":
        ctx.set_tune(a.tpi, a.tpi)
    t = time.time()
    ctx.prologue()
    print(f"prologue {1e3 * (time.time() - t):.1f} ms (host clock)", flush=True)
    if a.steps > 0:
        ctx.enable_timing(True)
        ctx.step(a.steps)
        print({k: round(v / a.steps, 3) for k, v in ctx.timings().items()})
    print(ctx.counters())


if __name__ == "__main__":
    main()
