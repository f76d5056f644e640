"""Full-size runs of the two largest synthetic workloads, one JSON object on stdout.

    python -m inca_parallel_gb300.fullsize [batch|cube|both]

batch: the 64-molecule workload (3-20 atoms, 20-300 primitives, exponents up to 200,
    symmetry-unique closed-shell DM2s, 1.38e10 generated records in all), radial_plot
    s = 0..10 step 0.1 at nang 302 (nosym), tolerance 1e-8 per I(s), evaluated in waves of at
    most 1.5e9 generated records (one batch each: the whole list does not fit on the device at
    once). The plain FP64 form is timed on the smallest and the largest molecule, and its rate
    stands for the whole workload.
cube: cubeintra on the 128^3 lattice at 0.1 bohr for the 20-atom molecule (300 primitives,
    1.02e9 symmetry-unique records), separable mixed form at 1e-8 of max|I|; the FP64 form is
    timed on the central 16^3 sub-lattice and its rate stands for the lattice.
Every time is host wall time around the library's (synchronous) calls.
"""
import json
import sys
import time

import numpy as np

THRESH = 1e-12


def run_batch(ctx):
    from . import INCA_FP64, batch_waves as BW, workloads as W
    scan = ([0.0], [10.0], [0.1], [302])
    t0 = time.perf_counter()
    mols = [(b, D) for _, b, D in W.batch_workload()]
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    Is, info = BW.run_waves(ctx, mols, scan, THRESH, 1, 1e-8, max_records=1.5e9, unique=True, nosym=True)
    t_mixed = time.perf_counter() - t0
    surv = sum(w["survivors"] for w in info)
    # every molecule has the same scan grid, so its quartet-points are its survivors times that
    g = info[0]["grid_points"] // len(info[0]["molecules"])
    qp = surv * g
    # the plain FP64 form on the smallest and the largest molecule
    sizes = [len(b["alpha"]) for b, _ in mols]
    rates = {}
    for k in (int(np.argmin(sizes)), int(np.argmax(sizes))):
        b, D = mols[k]
        ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
        ctx.gen_closed_shell_dm2(D, unique=True)
        n = ctx.prepare(THRESH)
        ctx.grid_scan(*scan, nosym=True)
        t0 = time.perf_counter()
        ctx.eval(mode=INCA_FP64, copy=False)
        I64 = ctx.radial_plot()[1]
        dt = time.perf_counter() - t0
        rates[sizes[k]] = n[2] * ctx.ngrid / dt
        err = float(np.max(np.abs(Is[k] - I64) / np.abs(I64)))
        rates[f"{sizes[k]}_err"] = err
    r64 = min(v for k, v in rates.items() if not str(k).endswith("_err"))
    return {"workload": "64 molecules, radial_plot 101 shells, nang 302", "molecules": len(mols),
            "waves": len(info), "records": int(sum(w["records"] for w in info)), "survivors": int(surv),
            "quartet_points": int(qp), "host_generation_s": t_gen, "mixed_s": t_mixed,
            "mixed_value": qp / t_mixed, "fp64_rates_by_primitives": rates,
            "fp64_s_at_lower_rate": qp / r64, "speedup_vs_fp64_form": qp / r64 / t_mixed}


def run_cube(ctx):
    from . import INCA_FP64, INCA_MIXED, workloads as W
    b, D = W.cube_workload()
    ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
    nrec = ctx.gen_closed_shell_dm2(D, unique=True)
    t0 = time.perf_counter()
    n = ctx.prepare(THRESH)
    t_prep = time.perf_counter() - t0
    ng = ctx.grid_cube([0.0, 0.0, 0.0], [0.1, 0.1, 0.1], [128, 128, 128])
    t0 = time.perf_counter()
    Imx = ctx.eval(mode=INCA_MIXED, tol=1e-8, copy=True)
    t_mixed = time.perf_counter() - t0
    stats = ctx.stats()
    ctx.grid_cube([0.0, 0.0, 0.0], [0.1, 0.1, 0.1], [16, 16, 16])
    t0 = time.perf_counter()
    I64 = ctx.eval(mode=INCA_FP64)
    t64 = time.perf_counter() - t0
    Is = ctx.eval(mode=INCA_MIXED, tol=1e-8)
    rate64 = n[2] * 16 ** 3 / t64
    qp = n[2] * ng
    return {"workload": "cubeintra 128^3 at 0.1 bohr, 20-atom molecule", "records": int(nrec),
            "survivors": int(n[2]), "prepare_s": t_prep, "lattice_points": int(ng), "mixed_s": t_mixed,
            "mixed_value": qp / t_mixed, "max_abs_I": float(np.abs(Imx).max()), "tiers": stats,
            "fp64_value_16cube": rate64, "fp64_s_at_that_rate": qp / rate64,
            "speedup_vs_fp64_form": qp / rate64 / t_mixed,
            "err_16cube_vs_fp64_rel_max": float(np.abs(Is - I64).max() / np.abs(I64).max())}


def main(argv=None):
    from . import Context
    what = (argv if argv is not None else sys.argv[1:]) or ["both"]
    out = {}
    with Context(0) as ctx:
        if what[0] in ("batch", "both"):
            out["batch"] = run_batch(ctx)
        if what[0] in ("cube", "both"):
            out["cube"] = run_cube(ctx)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
