"""Benchmark: QDng Chebyshev propagation of the 256x256 two-state grid.

Workload (the reference's two-state 2-D benchmark, Chebyshev part): 2-D two-state
diabatic model, 256 x 256 grid on [-4,4]^2, masses (1836, 3672), harmonic
surfaces with k = 0.02, Gaussian coupling V12 = 0.01 exp(-(x-0.5)^2 - y^2),
displaced Gaussian start on state 1, dt = 5 a.u.  One "step" is one
Chebyshev time step U(dt) psi (the series is cut by the reference's norm
criterion).  Metric: grid-pt*steps/s = (states * grid points) * steps / s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
    python bench.py --impl reference ...   # the reference algorithm on the host cores

Timing: per step, L2 is flushed by writing a 512 MB buffer (outside the
timed interval); each step is bracketed by CUDA events on the engine's
stream.  `e2e` repeats the steps through the drop-in call with the wave
function in pinned host memory (upload, step, download inside the timed
region).  N > 1: independent replicas (the single-wavepacket path does not
shard), timing = max over ranks, value = sum of the ranks' work / that time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic bytes per Chebyshev term (one launch of the fused term kernel):
# N_pts * [S*5*c + (S + C + D)*r]; c/r = bytes per complex/real.
def term_bytes(npts, S, C, D, precision):
    if precision in ("fp64", "df64"):
        return npts * (S * 5 * 16 + (S + C + D) * 8)
    return npts * (S * 56 + (S + C + D) * 4)  # phi FP32 (3 x 8 B) + psi FP64 (2 x 16 B)


def read_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


WORKLOADS = {
    # name: (builder, description, coupling grids C, dipole grids D)
    "cfg2": ("cfg2_two_state", "cfg2 two-state 2-D Chebyshev, 256x256 grid x 2 states, dt=5 a.u.", 1, 0),
    "cfg2gspo": ("cfg2_two_state", "cfg2 two-state 2-D GSPO, 256x256 grid x 2 states, dt=5 a.u.", 1, 0),
    "cfg1": ("cfg1_morse", "cfg1 1-D Morse Chebyshev, 1024 points, dt=10 a.u.", 0, 0),
    "cfg3": ("cfg3_anharmonic", "cfg3 3-D anharmonic Chebyshev, 128^3 grid, dt=10 a.u.", 0, 0),
    "cfg5sil": ("cfg5_double_well", "cfg5 2-D double well, 128x128, real-time SIL (Krylov 16), dt=20 a.u., "
                "from the superposition of the 8 lowest relaxed states", 0, 0),
    "cfg5arnoldi": ("cfg5_double_well", "cfg5 2-D double well, 128x128, real-time Arnoldi (Krylov 16), dt=20 a.u., "
                    "from the superposition of the 8 lowest relaxed states", 0, 0),
}


def cfg5_start(hp, psi, on_gpu):
    """Start of the double-well Krylov workloads: the normalised equal-weight
    superposition of its 8 lowest states, relaxed by imaginary-time Chebyshev
    steps with projection and basis diagonalisation (up to 300 steps per
    state).  The relaxation uses dt = 2 a.u.: at dt = 20 the imaginary-time
    series' e^{-scaling dt} prefactor (e^{-42}) lies below the rounding of its
    terms in binary64.  The engine arm relaxes on the GPU, the CPU arms with
    the oracle."""
    from tests import cases
    nef, steps, conv, dt = 8, 300, 1e-8, 2.0
    if on_gpu:
        from qdng_gb300 import engine
        plan = engine.Plan(hp, "fp64")
        P = engine.Propagator(plan, "Cheby", "", dt=dt, imaginary_time=True, backward=True)
        efs = P.eigen_imag(psi, nef, steps, conv, diag=True)[0]
    else:
        from oracle import oracle as O
        P = O.Propagator(O.System(hp), "Cheby", "", dt=dt, imaginary_time=True, backward=True)
        efs = P.eigen_imag(psi, nef, steps, conv, diag=True)[0]
    return cases.superposition(hp, efs)


def workload(precision, name="cfg2", on_gpu=False):
    from tests import cases
    builder, desc, C, D = WORKLOADS[name]
    hp, psi, run = getattr(cases, builder)(gspo=True) if name == "cfg2gspo" else getattr(cases, builder)()
    if name.startswith("cfg5"):
        psi = cfg5_start(hp, psi, on_gpu)
    # a mixed plan runs Krylov propagators on its FP64 copy unless the FP32
    # basis is asked for; the mixed bench line measures the FP32 basis
    fp32 = " krylov_fp32=1" if precision == "mixed" else ""
    if name == "cfg5sil":
        run = dict(run, name="SIL", params="order=16" + fp32)
    elif name == "cfg5arnoldi":
        run = dict(run, name="Arnoldi", params="order=16" + fp32)
    cfg = {"workload": desc, "grid": list(hp.grid.n), "states": hp.nstates, "dt": run["dt"],
           "propagator": run["name"], "precision": precision,
           "l2": "flushed between timed steps (512 MB write)", "C": C, "D": D}
    return hp, psi, run, cfg


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # one process per GPU; the engine uses the device made visible here
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def reduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_time(workload, variant, threads, steps, warmup=1, repeats=3, budget=None):
    """The oracle (a restatement of QDng's propagator) timed on the host
    cores in a process of its own (oracle/cpu_time.py): median over
    `repeats` samples of `steps` steps (or `budget` seconds) each."""
    cmd = [sys.executable, "-m", "oracle.cpu_time", "--workload", workload, "--variant", variant,
           "--threads", str(threads), "--steps", str(steps), "--warmup", str(warmup), "--repeats", str(repeats)]
    if budget is not None:
        cmd += ["--budget", str(budget)]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CPU baseline failed: {r.stderr[-2000:]}")
    return json.loads(r.stdout.strip().splitlines()[-1])


VARIANT_TEXT = {"fast": "g++ -O3 -funroll-loops -ffast-math (QDng's configure default)",
                "o3": "g++ -O3 -funroll-loops", "": "g++ -O2"}


def cpu_baseline(workload_name, steps, budget):
    """CPU baselines of the workload: the oracle built with QDng's optimised
    flags and with -O3 alone, on all host cores, and the -O3 build on one
    core (QDng runs one thread unless given -p).  Returns the fastest
    all-core figure with every variant listed."""
    cores = os.cpu_count() or 1
    runs = [cpu_time(workload_name, "fast", cores, steps, budget=budget),
            cpu_time(workload_name, "o3", cores, steps, budget=budget),
            cpu_time(workload_name, "o3", 1, max(1, steps // 4), budget=budget)]
    best = max(runs[:2], key=lambda r: r["value"])
    variants = [{"build": VARIANT_TEXT[r["variant"]], "threads": r["threads"], "value": round(r["value"], 1),
                 "ms_per_step_median": round(r["s_per_step_median"] * 1e3, 3), "steps": r["steps"]}
                for r in runs]
    return best, variants


def mixed_error(hp, psi, run, nsteps):
    """Observables of the mixed-precision path against the FP64 path over
    nsteps from the same start (the FP64 path equals the oracle to 1e-12):
    largest error over the steps of the norm, each state population, <H>
    and the autocorrelation <psi0|psi(t)> (populations and autocorrelation
    relative to the norm, which bounds them; norm and <H> relative to their
    values)."""
    import numpy as np

    from qdng_gb300 import engine
    rows = {}
    for prec in ("fp64", "mixed"):
        plan = engine.Plan(hp, prec)
        prop = engine.Propagator(plan, run["name"], run["params"], dt=run["dt"])
        w, w0 = plan.wavefunction(psi), plan.wavefunction(psi)
        rows[prec], _ = prop.propagate(w, w0, nsteps)
    a, b = rows["mixed"], rows["fp64"]
    S = hp.nstates
    ac_a, ac_b = a[:, S + 2] + 1j * a[:, S + 3], b[:, S + 2] + 1j * b[:, S + 3]
    return {"steps": nsteps,
            "norm_rel": float(np.max(np.abs(a[:, 0] - b[:, 0]) / np.abs(b[:, 0]))),
            "populations": float(np.max(np.abs(a[:, 1:S + 1] - b[:, 1:S + 1]) / b[:, :1])),
            "energy_rel": float(np.max(np.abs(a[:, S + 1] - b[:, S + 1]) / np.abs(b[:, S + 1]))),
            "autocorrelation": float(np.max(np.abs(ac_a - ac_b) / b[:, 0]))}


def engine_arm(args, world, rank, local):
    import numpy as np
    import torch

    from qdng_gb300 import build, engine

    build.build()
    torch.cuda.set_device(0)
    hp, psi, run, cfg = workload(args.precision, args.workload, on_gpu=True)
    stream = torch.cuda.Stream()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    plan = engine.Plan(hp, args.precision)
    plan.set_stream(stream.cuda_stream)
    prop = engine.Propagator(plan, run["name"], run["params"], dt=run["dt"])
    w = plan.wavefunction(psi)
    info = prop.info()

    step = 0
    for _ in range(args.warmup):
        prop.run(w, step, 1)
        step += 1

    def timed_steps(k, profile=False):
        nonlocal step
        evs = []
        terms = 0
        if profile:
            plan.profile(True)
        for _ in range(k):
            with torch.cuda.stream(stream):
                flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            terms += prop.run(w, step, 1)
            b.record(stream)
            evs.append((a, b))
            step += 1
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs)
        prof = plan.profile_read() if profile else None
        if profile:
            plan.profile(False)
            phases.update({k: round(v / 1e3 / max(terms - 2 * k_steps, 1), 3)
                           for k, v in prop.phase_times().items()})
        return ms, terms, prof

    phases = {}
    k_steps = args.steps

    barrier(world)
    torch.cuda.synchronize()
    l0 = engine.kernel_launches()
    with ClockSampler(local) as clk:
        ms, terms, _ = timed_steps(args.steps)
    launches = engine.kernel_launches() - l0
    torch.cuda.synchronize()
    barrier(world)
    clocks = clk.summary()
    ms_max = reduce_max(ms, world)
    value = hp.size * args.steps * world / (ms_max / 1e3)

    # dominant kernel: device time of every launch of the engine's step /
    # pass kernels over the same number of steps (events around each launch)
    pms, pterms, (prof_ms, prof_n) = timed_steps(args.steps, profile=True)
    modes = engine.PASS_MODES
    top = int(np.argmax(prof_ms[:len(modes)]))
    npts, S = hp.npts, hp.nstates
    C, D = cfg.pop("C"), cfg.pop("D")  # distinct off-diagonal coupling and dipole grids
    peak, peak_src = read_peak()
    roof = None
    if prof_n[top] > 0:
        avg_s = prof_ms[top] / prof_n[top] / 1e3
        if modes[top] == "cheby_step":
            # one launch = one time step = terms_per_step Chebyshev terms
            tps = pterms / prof_n[top]
            per_launch = term_bytes(npts, S, C, D, args.precision) * tps
            what = (f"one time step = {tps:.1f} Chebyshev terms x [read phi_(n-1), phi_(n-2), psi, "
                    "potentials; write phi_n, psi]")
            kname = "cheby_step_kernel (persistent, whole step)"
        elif modes[top] == "cheby_term":
            per_launch = term_bytes(npts, S, C, D, args.precision)
            what = "one Chebyshev term: read phi_(n-1), phi_(n-2), psi, potentials; write phi_n, psi"
            kname = "combine_kernel (cheby_term)"
        elif modes[top] == "gspo_kin":
            per_launch = npts * S * 2 * 16
            what = "GSPO kinetic pass along one dimension: read psi, write exp(c T_d) psi (complex128)"
            kname = "linepass_kernel (gspo_kin)"
        else:
            per_launch = npts * S * 2 * (8 if args.precision == "mixed" else 16)
            what = "kinetic line pass: read phi, write T_d phi"
            kname = f"kin_all_kernel ({modes[top]})"
        ach = per_launch / avg_s / 1e9
        # DRAM bytes (read + write) of one launch of the dominant kernel, from
        # an ncu capture of the same command (dram__bytes_read.sum +
        # dram__bytes_write.sum, profiles/); the 256^2 x 2 working set stays
        # in L2, the 128^3 step streams the kinetic parts of three dimensions;
        # workloads not captured report null
        traffic = None
        if args.workload == "cfg2" and modes[top] == "cheby_step":
            traffic = {"fp64": 6.13e6, "mixed": 3.75e6}.get(args.precision)
        elif args.workload == "cfg3" and modes[top] == "cheby_step" and args.precision == "fp64":
            traffic = 9.52e9
        elif args.workload == "cfg1" and modes[top] == "cheby_step" and args.precision == "fp64":
            traffic = 7.35e4
        elif args.workload == "cfg2gspo" and modes[top] == "gspo_kin":
            traffic = 2.21e6
        if args.workload == "cfg1" and modes[top] == "cheby_step":
            kname = "cheby_line64_kernel (one line on a cluster of 16 blocks, whole step)"
        # what binds these kernels instead: binary64 arithmetic on GB300's FP64
        # pipe (the mixed and double-float forms: latency of the term chain)
        limiter = ("FP64 pipe (binary64 FFTs; cfg2: 60% busy in ncu, working set L2-resident)"
                   if args.precision == "fp64" and modes[top] == "cheby_step" else None)
        # the bound that does apply to the binary64 step kernels: how busy the
        # FP64 pipe is, from the ncu capture of the same kernel
        # (sm__inst_executed_pipe_fp64.avg.pct_of_peak_sustained_active, profiles/)
        fp64_busy = None
        if args.precision == "fp64" and modes[top] == "cheby_step":
            fp64_busy = {"cfg2": 59.5, "cfg1": 36.1}.get(args.workload)
        roof = {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "traffic": traffic, "kernel": kname, "limiter": limiter,
                "fp64_pipe_busy_pct_ncu": fp64_busy,
                "algorithmic_bytes_per_launch": int(per_launch), "bytes_note": what,
                "avg_launch_us": round(avg_s * 1e6, 2), "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)"}
    per_mode = {modes[i]: {"ms": round(float(prof_ms[i]), 3), "launches": int(prof_n[i])}
                for i in range(len(modes)) if prof_n[i] > 0}
    term_rate = None
    if terms > 0:
        term_s = (ms / 1e3) / terms
        tb = term_bytes(npts, S, C, D, args.precision)
        term_rate = {"terms_per_step": terms / args.steps, "us_per_term": round(term_s * 1e6, 2),
                     "algorithmic_GBps_per_term": round(tb / term_s / 1e9, 1)}

    # e2e through the drop-in call with host (pinned) buffers
    host = torch.empty(hp.size * 2, dtype=torch.float64, pin_memory=True).numpy().view(np.complex128)
    host[:] = psi
    scratch = plan.wavefunction()
    e2e_s = 0.0
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prop.apply_host(scratch, host, i)
        e2e_s += time.perf_counter() - t0
    e2e_s = reduce_max(e2e_s, world)
    e2e_val = hp.size * args.steps * world / e2e_s

    err = None
    if args.precision == "mixed" and rank == 0 and args.err_steps > 0:
        err = mixed_error(hp, psi, run, args.err_steps)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        best, variants = cpu_baseline(args.workload, steps=50, budget=args.cpu_budget / 3)
        cpu = {"value": round(best["value"], 1), "unit": "grid-pt*steps/s", "cores": best["threads"], "kind": "port",
               "sample": f"median of 3 samples ({best['steps']} steps in all) of the same workload, oracle "
                         f"restatement of the QDng propagator built with {VARIANT_TEXT[best['variant']]}, "
                         "OpenMP over FFT lines; QDng itself does not build here",
               "variants": variants}

    line = {
        "metric": "grid-pt*steps/s" + (" (Chebyshev, 256^2 x 2 states)" if args.workload == "cfg2" else ""),
        "value": round(value, 1),
        "unit": "grid-pt*steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_max / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        # fp64: binary64 throughout; df64: phi, H phi and the FFTs of the
        # multi-dimensional step in double-float (2 x f32), psi and the
        # reductions binary64; mixed: FP32 bulk, binary64 psi and reductions
        "dtype": {"fp64": "f64", "df64": "f64+df32" if hp.grid.ndims > 1 else "f64",
                  "mixed": "f32+f64"}[args.precision],
        "data": "synthetic (seeded analytic potentials and Gaussian start)",
        "config": dict(cfg, parallelism="replicas" if world > 1 else "single",
                       cheby_order=info["order"]),
        "e2e": {"value": round(e2e_val, 1), "unit": "grid-pt*steps/s",
                "h2d_bytes_per_step": hp.size * 16, "d2h_bytes_per_step": hp.size * 16},
        "gpu_launches": int(launches),
        "roofline": roof,
        "per_term": term_rate,
        "pass_profile": per_mode,
        "step_phases_us_per_term": phases or None,
        "error_vs_fp64": err,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line))


def ensemble_timeline_report(ens, se, blk):
    """Per member class (dimensions, points) of the timed run: members, time
    on their block (min, max) and the latest end, in ms from the launch's
    first start; then the makespan and the busy time per block (stderr)."""
    import collections

    import numpy as np
    t0 = se[:, 0].min()
    dur = (se[:, 1] - se[:, 0]) / 1e6
    end = (se[:, 1] - t0) / 1e6
    cls = collections.defaultdict(list)
    for i, m in enumerate(ens):
        cls[(m["grid"].ndims, m["grid"].npts)].append(i)
    for k in sorted(cls):
        ix = cls[k]
        print("timeline class %dD %7d pts: %3d members, on-block %.1f-%.1f ms, last end %.1f ms"
              % (k[0], k[1], len(ix), dur[ix].min(), dur[ix].max(), end[ix].max()), file=sys.stderr)
    busy = collections.defaultdict(float)
    for i in range(len(ens)):
        busy[int(blk[i])] += dur[i]
    b = np.array(sorted(busy.values()))
    print("timeline makespan %.1f ms; busy per block min %.1f median %.1f max %.1f ms over %d blocks"
          % (end.max(), b.min(), np.median(b), b.max(), len(b)), file=sys.stderr)


def ensemble_arm(args, world, rank, local):
    """Ensemble of 512 laser-driven members, one persistent launch per
    call; wavepackets/s = members x (steps / 5000) / time."""
    import numpy as np
    import torch

    from qdng_gb300 import build, engine
    from tests import cases

    build.build()
    torch.cuda.set_device(0)
    ens = cases.cfg4_ensemble(n=args.members, seed=4)
    if world > 1:  # shard members across ranks by LPT (no collective on the data path)
        costs = [m["grid"].npts * np.log2(m["grid"].npts) for m in ens]
        parts, _ = cases.lpt_partition(costs, world)
        ens = [ens[i] for i in parts[rank]]
    E = engine.Ensemble(ens, dt=10.0, precision=args.precision)
    psi0 = [m["psi"] for m in ens]
    E.upload(psi0)
    E.run(0, args.warmup)
    barrier(world)
    torch.cuda.synchronize()
    l0 = engine.kernel_launches()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        terms = E.run(args.warmup, args.steps)
        dt_s = time.perf_counter() - t0
    launches = engine.kernel_launches() - l0
    if args.timeline and rank == 0:
        ensemble_timeline_report(ens, *E.timeline())
    clocks = clk.summary()
    dt_max = reduce_max(dt_s, world)
    total_members = args.members
    value = total_members * (args.steps / 5000.0) / dt_max
    # e2e: host psi (pinned) up, steps, down
    host = [torch.from_numpy(np.ascontiguousarray(p).view(np.float64)).pin_memory() for p in psi0]
    t0 = time.perf_counter()
    E.upload([h.numpy().view(np.complex128) for h in host])
    E.run(0, args.steps)
    out = E.download()
    e2e_s = reduce_max(time.perf_counter() - t0, world)
    err = None
    if args.precision == "mixed" and rank == 0:
        R = engine.Ensemble(ens, dt=10.0, precision="fp64")
        E.upload(psi0)
        R.upload(psi0)
        E.run(0, args.steps)
        R.run(0, args.steps)
        errs, acs, nrms = [], [], []
        for p0, a, b in zip(psi0, E.download(), R.download()):
            errs.append(float(np.abs(a - b).max() / np.abs(b).max()))
            ac, ac_ref = np.vdot(p0, a), np.vdot(p0, b)
            acs.append(float(abs(ac - ac_ref) / abs(ac_ref)))
            n, n_ref = np.vdot(a, a).real, np.vdot(b, b).real
            nrms.append(float(abs(n - n_ref) / n_ref))
        err = {"max_rel_psi_error_vs_fp64": max(errs), "median": float(np.median(errs)),
               "max_rel_autocorrelation_error": max(acs), "max_rel_norm_error": max(nrms), "steps": args.steps}
    plain = None
    if args.plain_baseline and rank == 0:
        plain = plain_fp64_members(ens, E, psi0, args.steps, dt_max / args.steps)
    bytes_io = int(sum(p.size for p in psi0) * 16)
    line = {
        "metric": "wavepackets/s (512 laser-driven members, 5000 steps each)",
        "value": round(value, 4),
        "unit": "wavepackets/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(dt_max / args.steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "strong",
        "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded Morse members)",
        "config": {"workload": "cfg4 ensemble: 512 members, 1-D 256-4096 / 2-D 64^2-256^2, dt=10, mass 1728",
                   "precision": args.precision, "l2": "members larger than L2 in total (not flushed)",
                   "terms_per_step_total": terms / args.steps},
        "e2e": {"value": round(total_members * (args.steps / 5000.0) / e2e_s, 4), "unit": "wavepackets/s",
                "h2d_bytes_per_step": bytes_io // args.steps, "d2h_bytes_per_step": bytes_io // args.steps},
        "gpu_launches": int(launches),
        "error_vs_fp64": err,
        "plain_fp64_path": plain,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line))


def plain_fp64_members(ens, E, psi0, steps, batched_s_per_step):
    """The batched form against the plain binary64 GPU path: the same members
    one at a time, each through its own plan and Chebyshev propagator (the
    qdg_prop_run call), device time of the steps only (plan set-up excluded),
    and the largest difference between the two results per member."""
    import numpy as np
    import torch

    from qdng_gb300 import engine
    from tests import cases

    total = 0.0
    outs = []
    for m in ens:
        plan = engine.Plan(cases.member_hplan(m), "fp64")
        P = engine.Propagator(plan, "Cheby", "", dt=10.0)
        w = plan.wavefunction(m["psi"])
        plan.synchronize()
        t0 = time.perf_counter()
        P.run(w, 0, steps)
        plan.synchronize()
        total += time.perf_counter() - t0
        outs.append(w.download())
        P.close()
        w.close()
        plan.close()
    torch.cuda.synchronize()
    R = engine.Ensemble(ens, dt=10.0, precision="fp64")
    R.upload(psi0)
    R.run(0, steps)
    diff = max(float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(R.download(), outs))
    plain_s = total / steps
    return {"ms_per_step": round(plain_s * 1e3, 3), "batched_speedup": round(plain_s / batched_s_per_step, 2),
            "max_rel_diff_batched_fp64_vs_plain": diff, "steps": steps,
            "what": "every member one at a time: its own plan, Cheby propagator and qdg_prop_run (binary64)"}


def reference_arm(args, world, rank):
    """The reference algorithm on the host cores: the oracle (QDng's
    propagator restated; QDng itself needs FFTW, LAPACK, SLATEC and protobuf,
    none of which exist here) built with QDng's optimised flags and with
    -O3 alone, on all cores; the faster build is the arm's value."""
    if rank != 0:
        return
    name = args.workload if args.workload not in ("ensemble",) else "cfg2"
    hp, psi, run, cfg = workload("fp64", name)
    cfg.pop("C"), cfg.pop("D")
    cores = os.cpu_count() or 1
    runs = [cpu_time(name, v, cores, args.steps, warmup=args.warmup, repeats=3) for v in ("fast", "o3")]
    best = max(runs, key=lambda r: r["value"])
    v = best["value"]
    line = {
        "metric": "grid-pt*steps/s" + (" (Chebyshev, 256^2 x 2 states)" if name == "cfg2" else ""),
        "value": round(v, 1),
        "unit": "grid-pt*steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(best["s_per_step_median"] * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded analytic potentials and Gaussian start)",
        "config": dict(cfg, l2="n/a (host)"),
        "impl": "reference",
        "cpu_baseline": {"value": round(v, 1), "unit": "grid-pt*steps/s", "cores": best["threads"], "kind": "port",
                         "sample": f"median of 3 samples of {args.steps} steps of the workload on {best['threads']} "
                                   f"host threads, oracle built with {VARIANT_TEXT[best['variant']]} "
                                   "(QDng is not buildable here: FFTW/LAPACK/SLATEC/protobuf missing; "
                                   "the oracle restatement of the propagator stands in)",
                         "variants": [{"build": VARIANT_TEXT[r["variant"]], "threads": r["threads"],
                                       "value": round(r["value"], 1)} for r in runs]},
        "e2e": {"value": round(v, 1), "unit": "grid-pt*steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--precision", default=None, choices=["fp64", "df64", "mixed"],
                    help="default: fp64 (the drop-in path); mixed for the ensemble workload")
    ap.add_argument("--err-steps", type=int, default=400,
                    help="steps of the mixed-vs-FP64 observable comparison (0: skip)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="cfg2", choices=list(WORKLOADS) + ["ensemble"])
    ap.add_argument("--members", type=int, default=512)
    ap.add_argument("--timeline", action="store_true",
                    help="ensemble: per member class times of the timed run, on stderr")
    ap.add_argument("--plain-baseline", action="store_true",
                    help="ensemble: also run the members one at a time through the plain binary64 plan API")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.precision is None:
        args.precision = "mixed" if args.workload == "ensemble" else "fp64"
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        reference_arm(args, world, rank)
    elif args.workload == "ensemble":
        ensemble_arm(args, world, rank, local)
    else:
        engine_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
