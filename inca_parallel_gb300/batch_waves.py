"""Batches larger than the device: molecules evaluated in waves.

The batch ABI (inca_batch_*, csrc/batch.cu) holds every molecule of a batch on the device at
once: its generated DM2 records (24 B each), the screening and sort buffers of inca_batch_prepare
(about 25 B per record), and the survivor records. A list of molecules whose generated records
exceed a budget is therefore split into waves of consecutive molecules (a molecule above the
budget forms a wave of its own), and each wave is one batch: one preparation and one evaluation
launch sequence for all of its molecules. Results come back per molecule, in input order.

Closed-shell records of a molecule with n primitives: with P = n (n + 1) / 2 primitive pairs,
P^2 records (the .dm2p convention, i <= k and j <= l) or P (P + 1) / 2 symmetry-unique ones.
"""


def records(nprim, unique=True):
    """Generated closed-shell DM2 records of a molecule with nprim primitives."""
    P = nprim * (nprim + 1) // 2
    return P * (P + 1) // 2 if unique else P * P


def plan_waves(nprims, max_records, unique=True):
    """Consecutive molecules grouped so that each group's records stay within max_records."""
    waves, cur, tot = [], [], 0
    for i, n in enumerate(nprims):
        r = records(int(n), unique)
        if cur and tot + r > max_records:
            waves.append(cur)
            cur, tot = [], 0
        cur.append(i)
        tot += r
    if cur:
        waves.append(cur)
    return waves


def run_waves(ctx, molecules, scan, thresh, mode, tol, max_records=1.5e9, unique=True, nosym=False):
    """I(s) of every molecule (basis dict, closed-shell 1-RDM D) on its radial-scan grid
    (scan = (start, end, step, nang) lists as for inca_grid_scan), evaluated in waves of at most
    max_records generated records. Returns the list of I(s) arrays and one dict per wave."""
    nprims = [len(b["alpha"]) for b, _ in molecules]
    out = [None] * len(molecules)
    info = []
    for w in plan_waves(nprims, max_records, unique):
        ctx.batch_clear()
        for i in w:
            b, D = molecules[i]
            ctx.batch_add_closed_shell(b["alpha"], b["tmn"], b["xyz"], D, *scan, unique=unique, nosym=nosym)
        counts = ctx.batch_prepare(thresh)
        parts = ctx.batch_eval(mode=mode, tol=tol)
        for i, p in zip(w, parts):
            out[i] = p
        info.append({"molecules": list(w), "records": int(counts[0]), "survivors": int(counts[2]),
                     "grid_points": int(ctx.ngrid)})
    return out, info
