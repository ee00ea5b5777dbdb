"""FFT schedule autotuner: picks the radix order (and, for the persistent
step kernel, the lines per batch) of every line length the benchmark
workloads use, by timing the candidates on the GPU, and writes the table
that libqdg.so reads at plan and ensemble creation (fft_schedules.txt next
to the library).  This is the engine's counterpart of FFTW's planning and
wisdom, which the reference relies on (src/fft/FFTGlobal.cpp:26-84,
src/fft/fft.cpp:98-122).

    python -m qdng_gb300.autotune [--quick] [--out PATH]

Every candidate runs whole Chebyshev steps of a workload of that line
length (a two-state 2-D grid, a 1-D Morse line, a 3-D grid, or an ensemble
of members of that size), timed with CUDA events after warm-up; a candidate
whose wave function differs from the greedy schedule's by more than 1e-11
(relative; 1e-2 for the FP32 form) is rejected.  A winner enters the table
only if it beats the greedy order by more than 2 %.
"""
import argparse
import ctypes as C
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

RADICES = (16, 8, 4, 2, 3, 5)
PREC_NAMES = {0: "fp64", 1: "mixed", 2: "df64"}
CTX_NAMES = {0: "plan", 1: "ensemble"}


def orders(n, extra_stages=1, cap=12):
    """Ordered factorisations of n into the supported radices with the fewest
    stages (and up to `extra_stages` more), fewest stages first."""
    found = set()

    def rec(m, seq):
        if m == 1:
            found.add(tuple(seq))
            return
        if len(seq) >= 8:
            return
        for r in RADICES:
            if m % r == 0:
                rec(m // r, seq + [r])

    rec(n, [])
    if not found:
        return []
    least = min(len(s) for s in found)
    keep = sorted((s for s in found if len(s) <= least + extra_stages), key=lambda s: (len(s), [-r for r in s]))
    return [list(s) for s in keep[:cap]]


def greedy(n):
    """The library's default order (largest radices first)."""
    seq, m = [], n
    while m % 16 == 0:
        seq.append(16)
        m //= 16
    for r in (8, 4, 2):
        if m % r == 0:
            seq.append(r)
            m //= r
    for r in (3, 5):
        while m % r == 0:
            seq.append(r)
            m //= r
    return seq


class Tuner:
    def __init__(self):
        from qdng_gb300 import _lib, build, engine
        build.build()
        self.L = _lib.load()
        self.engine = engine
        self.rows = []

    def set(self, ctx, n, prec, radices, lines):
        arr = (C.c_int32 * len(radices))(*radices)
        if self.L.qdg_fft_schedule_set(ctx, n, prec, arr, len(radices), lines) != 0:
            raise ValueError(f"schedule rejected: {ctx} {n} {prec} {radices} {lines}")

    def time_plan(self, hp, psi, run, prec, steps):
        import torch
        eng = self.engine
        plan = eng.Plan(hp, PREC_NAMES[prec])
        stream = torch.cuda.Stream()
        plan.set_stream(stream.cuda_stream)
        P = eng.Propagator(plan, run["name"], run["params"], dt=run["dt"])
        w = plan.wavefunction(psi)
        P.run(w, 0, 2)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        P.run(w, 2, steps)
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps, w.download()

    def time_ensemble(self, members, prec, steps):
        E = self.engine.Ensemble(members, dt=10.0, precision=PREC_NAMES[prec])
        E.upload([m["psi"] for m in members])
        E.run(0, 1)
        t0 = time.perf_counter()
        E.run(1, steps)
        dt = (time.perf_counter() - t0) * 1e3 / steps
        return dt, np.concatenate(E.download())

    def tune(self, ctx, n, prec, runner, line_caps=(0,)):
        base_r = greedy(n)
        cands = [(base_r, 0)] + [(r, l) for r in orders(n) for l in line_caps if (r, l) != (base_r, 0)]
        results, ref = [], None
        for r, l in cands:
            self.L.qdg_fft_schedule_reset(0)
            self.set(ctx, n, prec, r, l)
            try:
                ms, psi = runner()
            except Exception as e:  # a schedule the kernels cannot take (shared memory) is skipped
                print(f"  {r} lines {l}: skipped ({e})", flush=True)
                continue
            if ref is None:
                ref, ok = psi, True
            else:
                ok = float(np.abs(psi - ref).max() / np.abs(ref).max()) < (1e-11 if prec != 1 else 1e-2)
            results.append((ms, r, l, ok))
            print(f"  {CTX_NAMES[ctx]} n={n} {PREC_NAMES[prec]} {r} lines {l}: {ms:.4f} ms/step"
                  f"{'' if ok else ' REJECTED'}", flush=True)
        self.L.qdg_fft_schedule_reset(0)
        if not results:
            return
        base = results[0][0]
        best = min((x for x in results if x[3]), key=lambda x: x[0])
        if best[0] < 0.98 * base:
            self.rows.append((ctx, n, prec, best[1], best[2], best[0], base))

    def write(self, path):
        lines = ["# FFT schedules of the GB300 engine's line transforms, written by",
                 "# `python -m qdng_gb300.autotune` from CUDA-event timings of the candidates.",
                 "# context n precision radices lines_per_batch   # winner / greedy ms per step"]
        for ctx, n, prec, r, l, ms, base in sorted(self.rows):
            lines.append(f"{CTX_NAMES[ctx]} {n} {PREC_NAMES[prec]} {','.join(map(str, r))} {l}"
                         f"   # {ms:.4f} / {base:.4f} ms")
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="fewer sizes and steps")
    ap.add_argument("--out", default=os.path.join(HERE, "fft_schedules.txt"))
    args = ap.parse_args()
    from tests import cases
    T = Tuner()
    steps = 3 if args.quick else 5
    # plans: the benchmark grids (2-D two-state 256^2, 2-D 128^2, 1-D 1024, 3-D)
    plan_cases = [
        (256, lambda: cases.cfg2_two_state(256), (0, 4, 8)),
        (128, lambda: cases.cfg5_double_well(128), (0, 4, 8)),
        (1024, lambda: cases.cfg1_morse(1024), (0,)),
    ]
    if not args.quick:
        plan_cases.append((64, lambda: cases.cfg3_anharmonic(64), (0, 8, 16)))
    for n, mk, caps in plan_cases:
        hp, psi, run = mk()
        for prec in (0, 1):
            T.tune(0, n, prec, lambda: T.time_plan(hp, psi, run, prec, steps), caps)
    # ensembles: members of one size class each
    rng = np.random.default_rng(3)
    ens_1d = [256, 512, 1024, 2048, 4096] if not args.quick else [1024, 4096]
    ens_2d = [64, 128, 256] if not args.quick else [128]
    for n in ens_1d:
        mem = [cases.cfg4_member(rng, 1, n, nt=16) for _ in range(32)]
        for prec in (0, 1):
            T.tune(1, n, prec, lambda: T.time_ensemble(mem, prec, 2))
    for n in ens_2d:
        mem = [cases.cfg4_member(rng, 2, n, nt=16) for _ in range(8)]
        for prec in (0, 1):
            T.tune(1, n, prec, lambda: T.time_ensemble(mem, prec, 2))
    T.write(args.out)
    print(open(args.out).read())


if __name__ == "__main__":
    main()
