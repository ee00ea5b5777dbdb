"""Timed CPU baseline: the oracle's propagator on the host cores.

TEST INFRASTRUCTURE ONLY: run by bench.py's CPU legs (the reference arm and
the cpu_baseline field), one process per library build and thread count,
so that each build is loaded alone.

    python -m oracle.cpu_time --workload cfg2 --variant fast --threads 16 --steps 20 --warmup 1

Prints one JSON line: the median over `--repeats` samples of the time per
step (each sample runs `--steps` steps, or fewer once `--budget` seconds of
that sample have passed), the steps and the threads used.
"""
import argparse
import json
import os
import statistics
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cfg2")
    ap.add_argument("--variant", default="fast", choices=["", "o3", "fast"])
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--budget", type=float, default=None, help="seconds per sample (cap on --steps)")
    args = ap.parse_args()

    from oracle import oracle as O
    O.use_variant(args.variant)
    threads = O.threads(args.threads if args.threads > 0 else (os.cpu_count() or 1))
    import bench
    hp, psi, run, _ = bench.workload("fp64", args.workload)
    P = O.Propagator(O.System(hp), run["name"], run["params"], dt=run["dt"])
    x = psi.copy()
    step = 0
    for _ in range(args.warmup):
        P.apply(x, step)
        step += 1
    samples, total = [], 0
    for _ in range(args.repeats):
        t0 = time.perf_counter()
        n = 0
        while n < args.steps:
            P.apply(x, step)
            step += 1
            n += 1
            if args.budget is not None and time.perf_counter() - t0 > args.budget:
                break
        samples.append((time.perf_counter() - t0) / n)
        total += n
    med = statistics.median(samples)
    print(json.dumps({"variant": args.variant, "threads": threads, "steps": total, "repeats": args.repeats,
                      "s_per_step_median": med, "s_per_step_samples": samples,
                      "value": hp.size / med, "unit": "grid-pt*steps/s", "workload": args.workload}))


if __name__ == "__main__":
    main()
