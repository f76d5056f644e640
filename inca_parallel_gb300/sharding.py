"""Point sharding of the intracule evaluation over ranks (one process per GPU).

The point loop of calculate_intracule (src/mod_intracule.f90:345-358) is independent per grid
point, so the work partitions by points with no exchange on the data path: every rank holds
all surviving quartet records and evaluates them on its own contiguous slice of the grid. The
only communication is at the end: a gather of the disjoint Ivec slices (cube / points jobs),
or one FP64 sum of per-rank partial sums (radial integral, Vee), or a gather of whole shells
(radial plot; a shell never straddles two ranks, so each I(s) is summed on one rank). The
reference's own reduction over OpenMP threads (mod_intracule.f90:376-381) is replaced by
these; partial sums are combined in rank order, so results do not depend on arrival order.

The evaluator is a callable ``evaluate(points) -> I`` (points (n, 3) bohr, I (n,) FP64). On
a GPU rank it wraps a Context (see ``context_evaluator``); any other callable with the same
contract can be sharded the same way.
"""
import numpy as np


def shard_bounds(n, rank, world):
    """Contiguous, balanced slice [lo, hi) of n points for `rank` of `world`."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("bad shard arguments")
    return (n * rank) // world, (n * (rank + 1)) // world


def shard_shells(smn, rank, world):
    """Whole shells for `rank`: a contiguous run of shells whose point counts (smn) are split
    as evenly as shell boundaries allow. Returns (first shell, end shell, first point, end point)."""
    smn = np.asarray(smn, dtype=np.int64)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad shard arguments")
    off = np.concatenate([[0], np.cumsum(smn)])
    total = int(off[-1])
    # shell k goes to the rank whose equal share contains the shell's first point
    owner = np.minimum((off[:-1] * world) // max(total, 1), world - 1)
    mine = np.nonzero(owner == rank)[0]
    if len(mine) == 0:
        # an empty rank still gets an empty range at a consistent place
        k = int(np.searchsorted(owner, rank))
        return k, k, int(off[k]), int(off[k])
    s0, s1 = int(mine[0]), int(mine[-1]) + 1
    return s0, s1, int(off[s0]), int(off[s1])


def _dist():
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        raise RuntimeError("torch.distributed is not initialised")
    return dist


def gather_slices(local, n, group=None):
    """All-gather the disjoint slices (rank order) into the full length-n FP64 array."""
    import torch
    dist = _dist()
    world = dist.get_world_size(group)
    local = np.ascontiguousarray(local, dtype=np.float64)
    sizes = [shard_bounds(n, r, world) for r in range(world)]
    width = max(hi - lo for lo, hi in sizes) if sizes else 0
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    buf = torch.zeros(width, dtype=torch.float64, device=dev)
    buf[:len(local)] = torch.from_numpy(local).to(dev)
    parts = [torch.zeros(width, dtype=torch.float64, device=dev) for _ in range(world)]
    dist.all_gather(parts, buf, group=group)
    out = np.empty(n, dtype=np.float64)
    for (lo, hi), p in zip(sizes, parts):
        out[lo:hi] = p[:hi - lo].cpu().numpy()
    return out


def sum_in_rank_order(values, group=None):
    """Sum a small FP64 vector over ranks, adding the ranks' contributions in rank order."""
    import torch
    dist = _dist()
    world = dist.get_world_size(group)
    v = np.atleast_1d(np.asarray(values, dtype=np.float64))
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.from_numpy(v.copy()).to(dev)
    parts = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    acc = np.zeros_like(v)
    for p in parts:
        acc = acc + p.cpu().numpy()
    return acc


def sharded_ivec(evaluate, points, group=None):
    """Ivec at every point (cube / explicit points jobs): each rank evaluates its slice."""
    dist = _dist()
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    points = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    lo, hi = shard_bounds(len(points), rank, world)
    local = evaluate(points[lo:hi]) if hi > lo else np.zeros(0)
    return gather_slices(local, len(points), group)


def sharded_radial_integral(evaluate, points, w, wvee=None, group=None):
    """sum_g w_g I_g (and sum_g wvee_g I_g) over a radial grid, points sharded over ranks."""
    dist = _dist()
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    points = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    lo, hi = shard_bounds(len(points), rank, world)
    I = evaluate(points[lo:hi]) if hi > lo else np.zeros(0)
    part = [float(np.dot(w[lo:hi], I))]
    if wvee is not None:
        part.append(float(np.dot(wvee[lo:hi], I)))
    tot = sum_in_rank_order(part, group)
    return (tot[0], tot[1]) if wvee is not None else tot[0]


def sharded_radial_plot(evaluate, points, w_ang, smn, group=None):
    """I(s) per shell of a scan grid: each rank evaluates whole shells; gathered in order."""
    dist = _dist()
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    points = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    smn = np.asarray(smn, dtype=np.int64)
    s0, s1, p0, p1 = shard_shells(smn, rank, world)
    I = evaluate(points[p0:p1]) if p1 > p0 else np.zeros(0)
    local = np.zeros(len(smn))
    k = 0
    for s in range(s0, s1):
        local[s] = float(np.dot(w_ang[p0 + k:p0 + k + smn[s]], I[k:k + smn[s]]))
        k += smn[s]
    # each shell has exactly one non-zero contributor, so the rank-order sum is exact
    return sum_in_rank_order(local, group)


def scan_shard(start, end, step, rank, world):
    """The rank's share of one radial-scan block (shells s_k = start + k step, k < npb, as
    gridpoints2 counts them: npb = int((end - start) / step) + 1): a contiguous run of whole
    shells, itself a scan block (start', end', step) -- so each rank builds its part of the grid
    on its own device and every I(s) is summed on one rank. Returns (start', end', k0, k1), or
    None for a rank with no shell."""
    if world < 1 or not 0 <= rank < world or not step > 0:
        raise ValueError("bad shard arguments")
    npb = int((end - start) / step) + 1
    k0, k1 = (npb * rank) // world, (npb * (rank + 1)) // world
    if k1 <= k0:
        return None
    s0 = start + k0 * step
    # half a step past the last shell, so the shell count comes out exact despite rounding
    return s0, s0 + (k1 - k0 - 1 + 0.5) * step, k0, k1


def sharded_scan_plot(ctx, start, end, step, nang, mode, tol=1e-8, nosym=False, group=None):
    """I(s) of one radial-scan block with its shells split over ranks: each rank builds and
    evaluates its own shells (mixed form: the one-pass scan evaluation with its per-shell
    tolerance), then the shells are gathered in order. ctx: a prepared Context on this rank's
    GPU. Returns the full I(s) array (every rank)."""
    dist = _dist()
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    npb = int((end - start) / step) + 1
    local = np.zeros(npb)
    part = scan_shard(start, end, step, rank, world)
    if part is not None:
        s0, s1, k0, k1 = part
        nr, _ = ctx.grid_scan([s0], [s1], [step], [nang], nosym=nosym)
        if nr != k1 - k0:
            raise RuntimeError("scan shard: shell count mismatch")
        ctx.eval(mode=mode, tol=tol, copy=False)
        local[k0:k1] = ctx.radial_plot()[1]
    # each shell has exactly one non-zero contributor, so the rank-order sum is exact
    return sum_in_rank_order(local, group)


def context_evaluator(ctx, mode, tol=1e-10):
    """evaluate(points) on a prepared Context (explicit-point grid, per-point tolerance)."""
    def evaluate(points):
        ctx.grid_points(points)
        return ctx.eval(mode=mode, tol=tol)
    return evaluate
