"""Benchmark of the intracule hot path on GB300 (one JSON line on stdout, rank 0).

Workload ("ch4_radial_scan_590"): the CH4 system of the benchmark configurations -- C + 4 H,
27 primitives, DM2 from a seeded closed-shell 1-RDM with 5 orbitals, all 142 884 quartets --
evaluated as radial_plot with s = 0..10 bohr step 0.05 (201 shells) at nang = 590
(62 390 grid points), thresh 1e-12, plus the same system's radial integral (nrad 50, nang 110)
for the FP64-vs-mixed comparison. Inputs are synthetic (seeded); see
inca_parallel_gb300/workloads.py.

A step is one pass of the hot path with the quartet records and the grid resident in HBM:
screening/set-up of every quartet (inca_prepare), the evaluation of all surviving quartets at
every grid point (inca_eval, mixed FP32/FP64 form at tolerance 1e-8 relative per I(s)) and
the I(s) reduction. value = (survivors x grid points) / step time. The records and grid fit
in L2, so L2 is flushed (256 MiB write) before every timed step, outside the event bracket.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "quartet-point evals/s"
THRESH = 1e-12
SCAN = dict(start=[0.0], end=[10.0], step=[0.05], nang=[590])
TOL_SCAN = 1e-8
TOL_INTEGRAL = 1e-10
TOL_CUBE = 1e-8
CUBE = ([0.0, 0.0, 0.0], [0.15, 0.15, 0.15], [48, 48, 48])


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU baseline sample")
    p.add_argument("--no-ring", dest="ring", action="store_false",
                   help="leave out the 12-atom ring's radial-integral leg (about 45 s)")
    p.add_argument("--no-batch", dest="batch", action="store_false",
                   help="leave out the batched-molecules leg")
    p.add_argument("--shard", default="replicas", choices=["replicas", "points"],
                   help="N > 1: each rank evaluates its own copy of the workload (replicas, weak scaling) or "
                        "its share of the scan's shells (points, strong scaling: one scan split over the ranks)")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def workload():
    from inca_parallel_gb300 import workloads as W
    b = W.ch4_basis()
    D, S = W.closed_shell_density(b, 5, W.SEED0 + 0)
    ijkl, v = W.folded_records(D)
    return b, D, ijkl, v


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline (oracle port)
def cpu_rate(b, ijkl, v, seconds):
    """The oracle (C++ FP64 restatement of the reference loop, OpenMP on all host cores) on a
    bounded sample of the scan grid; returns quartet-point evals/s and the sample used."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    sys_ = {"alpha": b["alpha"], "tmn": b["tmn"], "xyz": b["xyz"], "ijkl": ijkl, "v": v}
    g = O.gridpoints2(SCAN["start"], SCAN["end"], SCAN["step"], SCAN["nang"])
    pts = g["r"]
    n = 64
    while True:
        idx = np.linspace(0, len(pts) - 1, n).astype(int)
        t0 = time.perf_counter()
        _, cnt = O.intracule(sys_, THRESH, pts[idx])
        dt = time.perf_counter() - t0
        if dt > seconds / 4 or n >= len(pts):
            break
        n = min(len(pts), int(n * max(2.0, (seconds / 4) / max(dt, 1e-3))))
    reps = max(1, int(seconds / max(dt, 1e-3)))
    t0 = time.perf_counter()
    for _ in range(reps):
        O.intracule(sys_, THRESH, pts[idx])
    dt = (time.perf_counter() - t0) / reps
    qp = cnt[2] * len(idx)
    return qp / dt, {"points": int(len(idx)), "of_points": int(len(pts)), "survivors": int(cnt[2]),
                     "repeats": reps, "seconds_per_sample": dt}


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    b, D, ijkl, v = workload()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    per_step = max(2.0, min(args.cpu_seconds, 60.0) / max(1, args.steps))
    rates = []
    sample = None
    for i in range(args.warmup + args.steps):
        r, sample = cpu_rate(b, ijkl, v, per_step)
        if i >= args.warmup:
            rates.append(r)
    val = statistics.median(rates)
    # one step of the whole workload (every surviving quartet at all 62 390 points) at that rate
    ms_full = sample["survivors"] * sample["of_points"] / val * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "quartet-points/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_full, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded CH4 closed-shell DM2)",
            "config": {"workload": "ch4_radial_scan_590", "points": 62390, "quartets": int(len(v)),
                       "cpu_sample": sample, "step_rates": rates,
                       "step_rate_rel_std": (statistics.pstdev(rates) / val) if len(rates) > 1 else 0.0,
                       "ms_per_step_basis": "the full scan (all surviving quartets at all points) at the "
                                            "sampled rate"},
            "cpu_baseline": {"value": val, "unit": "quartet-points/s", "cores": cores, "kind": "port",
                             "sample": f"oracle (C++ FP64 restatement of the reference OpenMP loop) on "
                                       f"{sample['points']} of {sample['of_points']} scan points, all quartets"},
            "e2e": {"value": val, "unit": "quartet-points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def scan_for_rank(shard, rank, world):
    """grid_scan arguments of this rank: the whole scan, or its share of the shells."""
    if not shard or world == 1:
        return SCAN["start"], SCAN["end"], SCAN["step"], SCAN["nang"]
    from inca_parallel_gb300 import sharding as SH
    part = SH.scan_shard(SCAN["start"][0], SCAN["end"][0], SCAN["step"][0], rank, world)
    if part is None:
        raise SystemExit("more ranks than shells")
    return [part[0]], [part[1]], SCAN["step"], SCAN["nang"]


# ------------------------------------------------------------------ 12-atom ring leg
def ring_leg(ctx, stream, flush):
    """Radial integral of the 12-atom ring (198 primitives, l <= 2, exponents 0.1-5000, 21
    occupied orbitals, symmetry-unique DM2 of 194 074 551 records generated on the device),
    nrad 75, nang 302 on the automatic centres (nosym), thresh 1e-12: the mixed form at 1e-10
    on the whole grid, and the plain FP64 form on every 97th grid point, whose rate gives the
    FP64 time of the whole grid. Error: the mixed form's values at those points against the FP64
    form's, relative to the largest |I| there."""
    import torch
    from inca_parallel_gb300 import INCA_FP64, INCA_MIXED, centercalc, workloads as W
    b, D = W.ring_workload()
    ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
    nrec = ctx.gen_closed_shell_dm2(D, unique=True)
    counts = ctx.prepare(THRESH)
    cent, Ps, alf = centercalc(b["an"], b["cartes"])
    ctx.grid_radial([75] * len(Ps), [302] * len(Ps), alf, cent, Ps, nosym=True)
    ng = ctx.ngrid
    pts = ctx.grid_copy(weights=False)["r"]

    def run(fn):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), out

    def mixed():
        I = ctx.eval(mode=INCA_MIXED, tol=TOL_INTEGRAL)
        return I, ctx.radial_integral()[0]

    run(mixed)  # sorts the grid and sizes the buffers
    t_mix, (Imix, R) = run(mixed)
    stats = ctx.stats()
    sub = np.arange(0, ng, 97)
    ctx.grid_points(pts[sub])
    t_sub, I64 = run(lambda: ctx.eval(mode=INCA_FP64))
    rate64 = counts[2] * len(sub) / (t_sub * 1e-3)
    qp = counts[2] * ng
    err = float(np.abs(Imix[sub] - I64).max() / np.abs(I64).max())
    return {"records": int(nrec), "survivors": int(counts[2]), "grid_points": int(ng), "centres": int(len(Ps)),
            "tolerance": TOL_INTEGRAL, "radial_integral": R, "mixed_ms": t_mix,
            "mixed_value": qp / (t_mix * 1e-3), "fp64_value_sampled": rate64,
            "fp64_ms_whole_grid_at_sampled_rate": qp / rate64 * 1e3, "fp64_sample_points": int(len(sub)),
            "speedup_vs_fp64_form": qp / rate64 * 1e3 / t_mix, "max_err_rel_max_at_sample": err,
            "tiers": stats}


# ------------------------------------------------------------------ batched molecules leg
def batch_leg(ctx, device):
    """Molecules of the 64-molecule batch workload (3-20 atoms, 20-300 primitives, exponents up
    to 200, symmetry-unique closed-shell DM2s) with at most 60 primitives -- a subset that fits
    one batch -- each as radial_plot s = 0..10 step 0.1 at nang 302 (nosym), thresh 1e-12, with
    records and grids resident: one batched preparation plus one replay of the captured
    evaluation graph (mixed, 1e-8 per I(s), and again at 1e-10) and the I(s) reduction, against
    the molecules run one after the other (preparation, plain FP64 evaluation, I(s)), each in its
    own context. Host wall time around the (synchronous) calls."""
    from inca_parallel_gb300 import INCA_FP64, INCA_MIXED, Context, workloads as W
    scan = ([0.0], [10.0], [0.1], [302])
    mols = W.batch_workload(max_prims=60)
    ctxs = []
    for _, b, D in mols:
        c = Context(device)
        c.set_primitives(b["alpha"], b["tmn"], b["xyz"])
        c.gen_closed_shell_dm2(D, unique=True)
        c.grid_scan(*scan, nosym=True)
        ctxs.append(c)
    ctx.batch_clear()
    for _, b, D in mols:
        ctx.batch_add_closed_shell(b["alpha"], b["tmn"], b["xyz"], D, *scan, unique=True, nosym=True)
    cnt = ctx.batch_prepare(THRESH)

    def batched(tol=TOL_SCAN):
        ctx.prepare(THRESH)
        ctx.eval_graph(mode=INCA_MIXED, tol=tol, copy=False)
        return ctx.radial_plot()[1]

    def sequential(mode):
        res, qp = [], 0
        for c in ctxs:
            n = c.prepare(THRESH)
            c.eval(mode=mode, tol=TOL_SCAN, copy=False)
            res.append(c.radial_plot()[1])
            qp += n[2] * c.ngrid
        return np.concatenate(res), qp

    def wall(fn, reps):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            out = fn()
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts) * 1e3, out

    t_b, Ib = wall(batched, 5)  # the first call captures the graph; the timed ones replay it
    t_b10, Ib10 = wall(lambda: batched(TOL_INTEGRAL), 5)  # the same at the radial integral's 1e-10
    t_64, (I64, qp) = wall(lambda: sequential(INCA_FP64), 2)
    t_mx, _ = wall(lambda: sequential(INCA_MIXED), 3)
    for c in ctxs:
        c.close()
    err = float(np.max(np.abs(Ib - I64) / np.abs(I64)))
    err10 = float(np.max(np.abs(Ib10 - I64) / np.abs(I64)))
    return {"molecules": len(mols), "of_workload": 64, "primitives": [len(b["alpha"]) for _, b, _ in mols],
            "records": int(cnt[0]), "survivors": int(cnt[2]), "grid_points": int(ctx.ngrid),
            "quartet_points": int(qp), "batched_graph_ms": t_b, "batched_value": qp / (t_b * 1e-3),
            "sequential_fp64_ms": t_64, "sequential_mixed_ms": t_mx,
            "speedup_vs_sequential_fp64": t_64 / t_b, "speedup_vs_sequential_mixed": t_mx / t_b,
            "max_rel_err_I_s_vs_fp64": err, "tolerance_I_s": TOL_SCAN,
            "at_tolerance_1e-10": {"batched_graph_ms": t_b10, "speedup_vs_sequential_fp64": t_64 / t_b10,
                                   "max_rel_err_I_s_vs_fp64": err10},
            "note": "batched: one preparation of the whole batch and one graph replay of its mixed "
                    "evaluation; sequential: one context per molecule; preparation and I(s) on both sides"}


# ------------------------------------------------------------------ GPU arm
def gpu_arm(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from inca_parallel_gb300 import INCA_FP64, INCA_FP64_SCREENED, INCA_MIXED, Context
    b, D, ijkl, v = workload()
    ctx = Context(local)
    ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
    ctx.set_quartets(ijkl, v)
    counts = ctx.prepare(THRESH)
    shard = args.shard == "points"
    scan_args = scan_for_rank(shard, rank, world)
    nradi, ngrid = ctx.grid_scan(*scan_args)
    rec = ctx.records()
    Lbar = float(rec["L"].sum(axis=1).mean())
    qp = counts[2] * ngrid
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def step(mode, tol):
        ctx.prepare(THRESH)
        ctx.eval(mode=mode, tol=tol, copy=False)
        return ctx.radial_plot()[1]

    def timed(mode, tol, k, w):
        for _ in range(w):
            step(mode, tol)
        times, kern = [], []
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        n0 = ctx.kernel_launches()
        t_wall = time.perf_counter()
        for _ in range(k):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = step(mode, tol)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            kern.append(ctx.phases())
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
        launched = ctx.kernel_launches() - n0
        if world > 1:
            torch.distributed.barrier()
        return times, kern, t_wall, out, launched

    fp32_tflops = ctx.fp32_peak_tflops()
    # FP64 reference form (plain GPU form), fewer steps (it is ~2 orders slower)
    t64, k64, _, I64, _ = timed(INCA_FP64, 0.0, max(2, args.steps // 3), 1)
    # mixed form: the headline, on the schedule the library's autotuner picks for this grid and
    # these records (outside the timed region; every candidate schedule meets the tolerance)
    t_tune = time.perf_counter()
    sched = ctx.autotune(tol=TOL_SCAN, reps=2)
    t_tune = time.perf_counter() - t_tune
    with ClockSampler(local) as clk:
        tm, km, wall, Imix, launches = timed(INCA_MIXED, TOL_SCAN, args.steps, args.warmup)
    stats = ctx.stats()
    # the FP64 form with the same leaving-out of negligible (quartet, tile) pairs, on the same
    # schedule: the mixed form against it differs only in the arithmetic of the terms
    t64s, _, _, I64s, _ = timed(INCA_FP64_SCREENED, TOL_SCAN, max(2, args.steps // 3), 1)
    stats64s = ctx.stats()
    ctx.set_tuning()  # the other legs start from the default schedule
    ms = statistics.mean(tm)
    ms64 = statistics.mean(t64)
    ms64s = statistics.mean(t64s)
    rel_scan = float(np.max(np.abs(Imix - I64) / np.abs(I64)))
    rel_scan64s = float(np.max(np.abs(I64s - I64) / np.abs(I64)))
    # radial integral (nrad 50, nang 110, multicentre centres of CH4): time and error, both forms
    from inca_parallel_gb300 import centercalc
    cent, Ps, alf = centercalc(b["an"], b["cartes"])
    ctx.grid_radial([50] * len(Ps), [110] * len(Ps), alf, cent, Ps)
    # the library's autotuner on this grid (outside the timed region; every schedule meets the
    # tolerance); the FP64 form has no schedule
    ri_sched = ctx.autotune(tol=TOL_INTEGRAL, reps=2)
    ri = {}
    for name, mode in (("fp64", INCA_FP64), ("mixed", INCA_MIXED)):
        ts = []
        for i in range(4):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.prepare(THRESH)
            ctx.eval(mode=mode, tol=TOL_INTEGRAL, copy=False)
            val = ctx.radial_integral()[0]
            e1.record(stream)
            e1.synchronize()
            if i:
                ts.append(e0.elapsed_time(e1))
        ri[name] = {"ms": statistics.mean(ts), "value": val}
    ri_rel = abs(ri["mixed"]["value"] - ri["fp64"]["value"]) / abs(ri["fp64"]["value"])
    ctx.set_tuning()  # the cube and ring legs run the default schedule

    # vector cube (cubeintra lattice, 48^3 at 0.15 bohr): the FP64 form against INCA_MIXED, which
    # takes the separable double-float form on a lattice
    ctx.grid_cube(*CUBE)
    cube = {}
    for name, mode in (("fp64", INCA_FP64), ("mixed", INCA_MIXED)):
        ts = []
        for i in range(3 if mode == INCA_MIXED else 2):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.eval(mode=mode, tol=TOL_CUBE, copy=False)
            e1.record(stream)
            e1.synchronize()
            if i:
                ts.append(e0.elapsed_time(e1))
        cube[name] = {"ms": statistics.mean(ts), "I": ctx.eval(mode=mode, tol=TOL_CUBE)}
    cube_err = float(np.abs(cube["mixed"]["I"] - cube["fp64"]["I"]).max() / np.abs(cube["fp64"]["I"]).max())
    cube_qp = counts[2] * int(np.prod(CUBE[2]))

    ring = ring_leg(ctx, stream, flush) if args.ring else None
    batch = batch_leg(ctx, local) if args.batch else None

    # end to end through the C ABI with host buffers (the call sequence of the Fortran program's
    # bind(C) shim), tuned schedule;
    # the quartet input and the I(r) output live in pinned host memory
    ctx.set_tuning(sched["items_per_cta"], sched["sample_stride"], sched["estimate_safety"], sched["drop_fraction"],
                   sched["ctas_per_sm"], sched["cheap_slack"], sched["points_per_lane"])
    ctx.grid_scan(*scan_args)
    pin_ijkl = torch.empty(ijkl.size, dtype=torch.int32, pin_memory=True).numpy()
    pin_v = torch.empty(v.size, dtype=torch.float64, pin_memory=True).numpy()
    pin_out = torch.empty(ngrid, dtype=torch.float64, pin_memory=True).numpy()
    pin_ijkl[:] = ijkl.reshape(-1)
    pin_v[:] = v
    h2d = int(ijkl.nbytes + v.nbytes + b["alpha"].nbytes * 4 + b["tmn"].nbytes)
    d2h = int(8 * ngrid + 8 * nradi)
    e2e_t = []
    for i in range(2 + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
        ctx.set_quartets(pin_ijkl, pin_v)
        ctx.prepare(THRESH)
        ctx.grid_scan(*scan_args)
        ctx.eval(mode=INCA_MIXED, tol=TOL_SCAN, out=pin_out)
        ctx.radial_plot()
        torch.cuda.synchronize()
        if i >= 2:
            e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.mean(e2e_t)

    # roofline of the dominant kernel (k_pass1, the one-pass evaluation): algorithmic FP32 pipe
    # operations of one launch -- every surviving quartet at every grid point, 12 + L each
    # (3 FMA for r', 3 for |r'|^2, 1 exponent scale, L Horner FMA, 4 products, 1 add; the
    # reference loop's count) -- over its CUDA-event duration, against the FP32 FMA rate
    # measured on this GPU by the library's own microkernel (one FMA = one op)
    kms = statistics.mean(k["pass1_ms"] for k in km)
    pass2_ms = statistics.mean(k["pass2_ms"] for k in km)
    ops_per_qp = 12.0 + Lbar
    achieved = qp * ops_per_qp / (kms * 1e-3) / 1e12
    csum = clk.summary()
    peak = fp32_tflops / 2.0
    cpu_val, cpu_sample, cores = None, None, os.cpu_count() or 1
    if rank == 0 and world == 1:
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        cpu_val, cpu_sample = cpu_rate(b, ijkl, v, args.cpu_seconds)

    # whole-job aggregate: max time over ranks (each rank evaluates its own copy: weak scaling)
    t_step = ms
    qp_all, e2e_all = world * qp, world * qp / e2e_s
    if world > 1 and shard:  # strong scaling: the ranks' shares add up to one scan
        tq = torch.tensor([float(qp)], dtype=torch.float64, device=f"cuda:{local}")
        torch.distributed.all_reduce(tq)
        qp_all = float(tq.item())
        te = torch.tensor([e2e_s], dtype=torch.float64, device=f"cuda:{local}")
        torch.distributed.all_reduce(te, op=torch.distributed.ReduceOp.MAX)
        e2e_all = qp_all / float(te.item())
    if world > 1:
        tt = torch.tensor([t_step], device=f"cuda:{local}")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_step = float(tt.item())
    value = qp_all / (t_step * 1e-3)
    if rank == 0:
        prof = os.path.join(ROOT, "profiles", "k_pass1_ch4_radial_scan_590.md")
        traffic = None
        if os.path.exists(prof):
            for ln in open(prof):
                if ln.startswith("traffic_bytes_per_launch:"):
                    traffic = float(ln.split(":")[1])
        # the two bounds of the contract, for comparison: HBM (traffic of one launch from the ncu
        # summary over the launch time, against the measured copy bandwidth) and tensor (0: no
        # contraction on this path)
        hbm_peak, hbm_src = 6800.0, "fallback 6.8 TB/s (no MEASURED_PEAKS.json)"
        mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(mp):
            try:
                hbm_peak, hbm_src = float(json.load(open(mp))["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs"
            except (ValueError, KeyError):
                pass
        hbm_gbs = traffic / (kms * 1e-3) / 1e9 if traffic else None
        line = {
            "metric": METRIC, "value": value, "unit": "quartet-points/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True,
            "scaling": "strong" if (shard and world > 1) else "weak",
            "vs_baseline": None, "dtype": "f32 (double-float correction tier, f64 accumulation)",
            "data": "synthetic (seeded CH4 closed-shell DM2, 5 orbitals)",
            "config": {"workload": "ch4_radial_scan_590", "system": "CH4 27 primitives", "quartets": int(counts[0]),
                       "parallelism": (f"points split over {world} ranks (whole shells)" if (shard and world > 1)
                                       else f"{world} replica(s), one per GPU"),
                       "survivors": int(counts[2]), "grid_points": int(ngrid), "shells": int(nradi), "nang": 590,
                       "thresh": THRESH, "tolerance_I_s": TOL_SCAN, "l2": "flushed before each step (256 MiB write)",
                       "mean_L": Lbar,
                       "fp64_form": {"ms_per_step": ms64, "value": qp / (ms64 * 1e-3)},
                       "speedup_vs_fp64_form": ms64 / ms, "max_rel_err_I_s_vs_fp64": rel_scan,
                       "tiers": stats,
                       "schedule": {"source": "inca_autotune on this grid and records, before the timed steps",
                                    "items_per_cta": sched["items_per_cta"], "sample_stride": sched["sample_stride"],
                                    "estimate_safety": sched["estimate_safety"],
                                    "drop_fraction": sched["drop_fraction"], "ctas_per_sm": sched["ctas_per_sm"],
                                    "cheap_slack": sched["cheap_slack"],
                                    "points_per_lane": sched["points_per_lane"],
                                    "default_ms": sched["default_ms"],
                                    "tuned_ms": sched["best_ms"], "tuning_s": t_tune},
                       "radial_integral_nrad50_nang110": {"fp64_ms": ri["fp64"]["ms"], "mixed_ms": ri["mixed"]["ms"],
                                                          "rel_err": ri_rel, "value": ri["fp64"]["value"],
                                                          "tolerance": TOL_INTEGRAL,
                                                          "schedule": {k: ri_sched[k] for k in (
                                                              "items_per_cta", "sample_stride", "estimate_safety",
                                                              "drop_fraction", "ctas_per_sm", "cheap_slack",
                                                              "points_per_lane")}},
                       "fp64_screened_form": {"ms_per_step": ms64s, "value": qp / (ms64s * 1e-3),
                                              "max_rel_err_I_s_vs_fp64": rel_scan64s,
                                              "pairs_evaluated": stats64s["precise_pairs"],
                                              "pairs_left_out": stats64s["skipped_pairs"],
                                              "note": "every term in FP64, leaving out the same negligible "
                                                      "(quartet, tile) pairs as the mixed form, same schedule"},
                       "speedup_vs_fp64_screened_form": ms64s / ms,
                       "ring_radial_integral": ring,
                       "batched_graph": batch,
                       "vector_cube_48": {"fp64_ms": cube["fp64"]["ms"], "mixed_ms": cube["mixed"]["ms"],
                                          "mixed_value": cube_qp / (cube["mixed"]["ms"] * 1e-3),
                                          "max_err_rel_max": cube_err, "tolerance": TOL_CUBE,
                                          "form": "separable double-float lattice factors (k_cube_sep)"}},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "T FP32-ops/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_pass1 (one-pass evaluation)", "kernel_ms_per_launch": kms,
                         "correction_pass_ms": pass2_ms, "ops_per_quartet_point": ops_per_qp,
                         "peak_source": "measured: FP32 FMA microkernel (inca_fp32_fma_peak) on this GPU, "
                                        "%.1f TFLOP/s = %.1f T FMA/s" % (fp32_tflops, fp32_tflops / 2.0),
                         "note": "FP32-pipe bound (no contraction, ~0 bytes per quartet-point); "
                                 "MEASURED_PEAKS.json has no FP32 figure",
                         "hbm_view": {"achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s",
                                      "frac": (hbm_gbs / hbm_peak) if hbm_gbs else None, "peak_source": hbm_src},
                         "tensor_view": {"achieved": 0.0, "unit": "TFLOP/s",
                                         "note": "sm__pipe_tensor_cycles_active 0 % (ncu)"}},
            "clocks": csum,
            "e2e": {"value": e2e_all, "unit": "quartet-points/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3},
            "gpu_launches": int(launches),
        }
        if cpu_val is not None:
            line["cpu_baseline"] = {"value": cpu_val, "unit": "quartet-points/s", "cores": cores, "kind": "port",
                                    "sample": f"oracle (C++ FP64, OpenMP) on {cpu_sample['points']} of "
                                              f"{cpu_sample['of_points']} scan points, all {cpu_sample['survivors']} "
                                              f"surviving quartets"}
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
