"""Learned per-centre radial grids for the automatic multicentre grids.

mod_autogrid (src/mod_autogrid.f90:12-185) puts integration centres at the origin and at the
interatomic vectors R_j - R_k and gives each a radial map r = a (1 + x) / (1 - x) whose scale a
comes from Bragg-Slater radii; every centre then gets the same nrad (mod_build_grid.f90:13-277).
Near a centre the intracule is a sum of Gaussians whose exponents come from the primitives of
the atoms behind the centre (e = 2 a_i a_j / (a_i + a_j) for primitives i on atom A and j on
atom B: the product Gaussians of the quartet terms with (i, k) on A and (j, l) on B peak exactly
at R_B - R_A). Bragg-Slater radii do not see those exponents.

This module trains a small network -- the library's own GPU kernels, inca_mlp_* -- to predict
for each centre (1) a multiplier of autogrid's scale and (2) the number of radial nodes, from
geometry and exponent features. The training targets come from the one-dimensional problem each
centre solves: for the centre's Gaussian components, the scale that minimises the relative
Gauss-Legendre error of their radial integrals (int r^2 exp(-e r^2) dr over the mapped rule) at a
given nrad, and the smallest nrad whose best error is below the target. Autogrid's centres and
Ps stay; its scale and the caller's nrad stay the fallback where the features leave the training
range or a prediction leaves its bounds. A grid is measured by its radial integral against a
dense reference grid (nrad 150, nang 974) computed by the engine itself.
"""
import math

import numpy as np

NFEAT = 9
NRAD_SET = (20, 30, 50, 75)
NRAD_MIN, NRAD_MAX = 10, 150
SCALE_BOUNDS = (0.25, 4.0)
TARGET_ERR = 1e-10
_GL = {}


def gauss_legendre(n):
    if n not in _GL:
        x, w = np.polynomial.legendre.leggauss(n)
        _GL[n] = (x, w)
    return _GL[n]


def radial_errors(scales, expo, nrad):
    """Relative error of the mapped Gauss-Legendre rule for int_0^inf r^2 exp(-e r^2) dr, for
    every scale (rows) and exponent (columns)."""
    x, w = gauss_legendre(nrad)
    a = np.asarray(scales, dtype=np.float64)[:, None]
    r = a * (1.0 + x[None, :]) / (1.0 - x[None, :])                # (S, n)
    wr = w[None, :] * 2.0 * a / (1.0 - x[None, :]) ** 2 * r * r     # (S, n)
    e = np.asarray(expo, dtype=np.float64)
    q = np.einsum("sn,sne->se", wr, np.exp(-np.minimum(e[None, None, :] * (r * r)[:, :, None], 700.0)))
    exact = math.sqrt(math.pi) / 4.0 * e ** -1.5
    return np.abs(q - exact[None, :]) / exact[None, :]


def best_scale(expo, nrad, a_ref, span=8.0, nscan=60):
    """The scale (within a_ref / span .. a_ref * span) minimising the mean relative error over
    the exponents, and that error."""
    scales = a_ref * np.exp(np.linspace(-math.log(span), math.log(span), nscan))
    err = radial_errors(scales, expo, nrad).mean(axis=1)
    k = int(np.argmin(err))
    return float(scales[k]), float(err[k])


def centre_pairs(an, cartes, cent, tol=0.3):
    """For each centre, the atom pairs (A, B) with R_B - R_A at the centre (the origin: A == B)."""
    R = np.asarray(cartes, dtype=np.float64)
    out = []
    for c in np.asarray(cent, dtype=np.float64):
        if np.linalg.norm(c) < 1e-8:
            out.append([(a, a) for a in range(len(R))])
            continue
        d = R[None, :, :] - R[:, None, :] - c[None, None, :]
        A, B = np.nonzero(np.linalg.norm(d, axis=2) < tol)
        out.append([(int(a), int(b)) for a, b in zip(A, B) if a != b])
    return out


def centre_exponents(basis, pairs, cap=16):
    """Quantiles (at most `cap`) of the product exponents 2 a_i a_j / (a_i + a_j) behind a centre."""
    al, X, R = basis["alpha"], basis["xyz"], basis["cartes"]
    atom_of = np.argmin(np.linalg.norm(X[:, None, :] - R[None, :, :], axis=2), axis=1)
    by_atom = [al[atom_of == a] for a in range(len(R))]
    es = []
    for a, b in pairs:
        ea, eb = by_atom[a], by_atom[b]
        if len(ea) and len(eb):
            es.append((2.0 * ea[:, None] * eb[None, :] / (ea[:, None] + eb[None, :])).ravel())
    if not es:
        return np.array([1.0])
    e = np.sort(np.concatenate(es))
    if len(e) > cap:
        e = e[np.round(np.linspace(0, len(e) - 1, cap)).astype(int)]
    return e


def features(basis, cent, Ps, alf, nrad):
    """Per-centre features: log scale, log Ps, log(1 + |c|), log(1 + nearest other centre),
    10/50/90 % quantiles of log exponent, log(number of atom pairs + 1), log nrad."""
    cent = np.asarray(cent, dtype=np.float64).reshape(-1, 3)
    pairs = centre_pairs(basis["an"], basis["cartes"], cent)
    F, E = [], []
    for k, c in enumerate(cent):
        e = centre_exponents(basis, pairs[k])
        le = np.log(e)
        dn = np.linalg.norm(cent - c, axis=1)
        dn = dn[dn > 1e-9]
        F.append([math.log(alf[k]), math.log(max(Ps[k], 1e-3)), math.log1p(np.linalg.norm(c)),
                  math.log1p(dn.min() if len(dn) else 10.0), np.quantile(le, 0.1), np.quantile(le, 0.5),
                  np.quantile(le, 0.9), math.log1p(len(pairs[k])), math.log(nrad)])
        E.append(e)
    return np.asarray(F, dtype=np.float64), E


def targets(E, alf, nrad):
    """Per centre: log(best scale / autogrid scale) at nrad, and log of the smallest nrad whose
    best error is below TARGET_ERR (NRAD_MAX if none is)."""
    T = []
    for e, a in zip(E, alf):
        s, _ = best_scale(e, nrad, a)
        need = NRAD_MAX
        for n in (10, 15, 20, 25, 30, 40, 50, 60, 75, 90, 110, 130, 150):
            if best_scale(e, n, a)[1] <= TARGET_ERR:
                need = n
                break
        T.append([math.log(s / a), math.log(need)])
    return np.asarray(T, dtype=np.float64)


def training_set(nmol=500, seed=20261207, nrad_set=NRAD_SET):
    """Features and targets from autogrid's centres for nmol seeded geometries of 2-20 atoms."""
    from . import centercalc
    from . import workloads as W
    rng = np.random.default_rng(seed)
    X, Y = [], []
    for _ in range(nmol):
        natoms = int(rng.integers(2, 21))
        b = W.random_molecule(rng, natoms, int(rng.integers(2 * natoms, 8 * natoms + 1)))
        cent, Ps, alf = centercalc(b["an"], b["cartes"])
        for nrad in nrad_set:
            F, E = features(b, cent, Ps, alf, nrad)
            X.append(F)
            Y.append(targets(E, alf, nrad))
    return np.vstack(X), np.vstack(Y)


class LearnedGrid:
    """Per-centre radial scales and node counts predicted by a network trained on GPU."""

    def __init__(self, nhidden=32, seed=1):
        from ._lib import MLP
        self.net = MLP(NFEAT, nhidden, 2, seed=seed)
        self.mu = self.sd = self.lo = self.hi = None
        self.tmu = self.tsd = None

    def fit(self, X, Y, epochs=300, batch=256, lr=3e-3, seed=7):
        X = np.asarray(X, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        self.mu, self.sd = X.mean(0), X.std(0) + 1e-9
        self.lo, self.hi = X.min(0), X.max(0)
        self.tmu, self.tsd = Y.mean(0), Y.std(0) + 1e-9
        Xn = ((X - self.mu) / self.sd).astype(np.float32)
        Yn = ((Y - self.tmu) / self.tsd).astype(np.float32)
        return self.net.train(Xn, Yn, epochs=epochs, batch=batch, lr=lr, seed=seed)

    def predict_raw(self, X):
        Xn = ((np.asarray(X, dtype=np.float64) - self.mu) / self.sd).astype(np.float32)
        return self.net.forward(Xn).astype(np.float64) * self.tsd + self.tmu

    def grid(self, basis, nrad, nohydro=True):
        """Centres, Ps and per-centre (scale, nrad) for inca_grid_radial: autogrid's values where
        the features leave the training range or a prediction leaves its bounds."""
        from . import centercalc
        cent, Ps, alf = centercalc(basis["an"], basis["cartes"], nohydro=nohydro)
        F, _ = features(basis, cent, Ps, alf, nrad)
        pred = self.predict_raw(F)
        inside = np.all((F >= self.lo) & (F <= self.hi), axis=1)
        mult = np.exp(pred[:, 0])
        ok = inside & (mult >= SCALE_BOUNDS[0]) & (mult <= SCALE_BOUNDS[1])
        scale = np.where(ok, alf * mult, alf)
        nr = np.clip(np.round(np.exp(pred[:, 1])), NRAD_MIN, NRAD_MAX).astype(np.int32)
        nr = np.where(inside, nr, nrad).astype(np.int32)
        return cent, Ps, scale, nr, ok


def mlp_reference(params, nin, nh, nout, X, T=None):
    """The same network in numpy (float64): outputs, and with targets the loss and its gradient
    in the parameter layout of inca_mlp_* (used to check the GPU kernels)."""
    p = np.asarray(params, dtype=np.float64)
    o = 0

    def take(k):
        nonlocal o
        v = p[o:o + k]
        o += k
        return v
    W1 = take(nh * nin).reshape(nh, nin); b1 = take(nh)
    W2 = take(nh * nh).reshape(nh, nh); b2 = take(nh)
    W3 = take(nout * nh).reshape(nout, nh); b3 = take(nout)
    X = np.asarray(X, dtype=np.float64)
    a1 = np.tanh(X @ W1.T + b1)
    a2 = np.tanh(a1 @ W2.T + b2)
    y = a2 @ W3.T + b3
    if T is None:
        return y
    n = len(X)
    d = y - np.asarray(T, dtype=np.float64)
    loss = float((d * d).sum() / n)
    dy = 2.0 * d / n
    gW3, gb3 = dy.T @ a2, dy.sum(0)
    d2 = (dy @ W3) * (1.0 - a2 * a2)
    gW2, gb2 = d2.T @ a1, d2.sum(0)
    d1 = (d2 @ W2) * (1.0 - a1 * a1)
    gW1, gb1 = d1.T @ X, d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return y, loss, g


def compare_with_dense(lg, cases, nrad=50, nang=302, dense=(150, 974), nohydro=True, ctx=None):
    """Radial integrals of each case (basis, ijkl, v) on autogrid's grid and on the learned grid
    (learned scales and node counts), both against a dense autogrid grid; returns one dict per
    case with the relative errors and the point counts."""
    from . import Context, centercalc
    own = ctx is None
    ctx = ctx or Context(0)
    out = []
    try:
        for b, ijkl, v in cases:
            ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
            ctx.set_quartets(ijkl, v)
            ctx.prepare(1e-12)
            cent, Ps, alf = centercalc(b["an"], b["cartes"], nohydro=nohydro)
            nq = len(Ps)

            def integral(c, P, a, nr, na):
                _, _, ng = ctx.grid_radial(np.broadcast_to(nr, (nq,)).astype(np.int32),
                                           np.broadcast_to(na, (nq,)).astype(np.int32), a, c, P)
                ctx.eval(mode=0)
                return ctx.radial_integral()[0], ng
            ref, nref = integral(cent, Ps, alf, dense[0], dense[1])
            auto, nauto = integral(cent, Ps, alf, nrad, nang)
            c2, P2, a2, nr2, ok = lg.grid(b, nrad, nohydro=nohydro)
            mine, nmine = integral(c2, P2, a2, nr2, nang)
            out.append({"centres": nq, "predicted": int(ok.sum()), "dense": ref, "dense_points": nref,
                        "auto_err": abs(auto - ref) / abs(ref), "auto_points": nauto,
                        "learned_err": abs(mine - ref) / abs(ref), "learned_points": nmine})
    finally:
        if own:
            ctx.close()
    return out


MULTS = (0.5, 0.7, 1.0, 1.4, 2.0)


def centre_components(ctx, cent, Ps, scale, nrad, nang, tol=1e-12):
    """Each centre's TFVC component of the radial integral (inca_radial_integral's per-centre
    values) on the multicentre grid with the given per-centre scales and node counts."""
    nq = len(Ps)
    ctx.grid_radial(np.broadcast_to(nrad, (nq,)).astype(np.int32), np.broadcast_to(nang, (nq,)).astype(np.int32),
                    np.asarray(scale, dtype=np.float64), cent, Ps)
    ctx.eval(mode=1, tol=tol)
    tot, _, pc, _ = ctx.radial_integral()
    return tot, pc, ctx.ngrid


def targets_3d(ctx, cent, Ps, alf, nrad, nang=302, dense=(150, 974), mults=MULTS, ref=None):
    """Per centre: log of the multiplier of autogrid's scale (from mults) whose grid gives the
    centre's TFVC component of the radial integral closest to the dense grid's. The partition
    weight of a point depends on the centres and Ps, not on the scales, so a centre's component
    changes only with its own scale and one grid per multiplier serves every centre."""
    if ref is None:
        ref = centre_components(ctx, cent, Ps, alf, dense[0], dense[1])[1]
    errs = np.array([np.abs(centre_components(ctx, cent, Ps, alf * m, nrad, nang)[1] - ref) for m in mults])
    return np.log(np.asarray(mults)[np.argmin(errs, axis=0)]), errs


def _dense_case_molecule(rng, natoms_range=(2, 7), nprim_range=(10, 36)):
    """A seeded molecule with s and p primitives of exponents up to 50 (where the reference's
    polynomial fit is exact) and its closed-shell 1-RDM."""
    from . import workloads as W
    b = W.random_molecule(rng, int(rng.integers(*natoms_range)), int(rng.integers(*nprim_range)))
    keep = (b["tmn"].sum(1) <= 1) & (b["alpha"] <= 50.0)
    b = {**b, "alpha": b["alpha"][keep], "tmn": b["tmn"][keep], "xyz": b["xyz"][keep]}
    nocc = max(1, min(W.electrons(b) // 2, len(b["alpha"]) // 3))
    D, _ = W.closed_shell_density(b, nocc, int(rng.integers(1 << 30)))
    return b, D


def training_set_3d(ctx, nmol=60, seed=20261208, nrad_set=(30, 50), nang=302):
    """Features and targets from per-centre dense-grid errors: the scale column from
    targets_3d, the node-count column from the 1D rule (targets). Molecules with real DM2s
    (generated on the device), evaluated by the engine."""
    from . import centercalc
    rng = np.random.default_rng(seed)
    X, Y = [], []
    for _ in range(nmol):
        b, D = _dense_case_molecule(rng)
        ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
        ctx.gen_closed_shell_dm2(D, unique=True)
        ctx.prepare(1e-12)
        cent, Ps, alf = centercalc(b["an"], b["cartes"])
        ref = centre_components(ctx, cent, Ps, alf, 150, 974)[1]
        for nrad in nrad_set:
            F, E = features(b, cent, Ps, alf, nrad)
            t3, _ = targets_3d(ctx, cent, Ps, alf, nrad, nang, ref=ref)
            X.append(F)
            Y.append(np.stack([t3, targets(E, alf, nrad)[:, 1]], axis=1))
    return np.vstack(X), np.vstack(Y)


def compare_at_equal_points(lg, cases, nrads=(30, 50), nang=302, dense=(150, 974), ctx=None):
    """Per case and nrad: the radial-integral error against the dense grid with autogrid's scales
    and with the learned scales, both with nrad nodes on every centre (equal points)."""
    from . import Context, centercalc
    own = ctx is None
    ctx = ctx or Context(0)
    out = []
    try:
        for b, D in cases:
            ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
            ctx.gen_closed_shell_dm2(D, unique=True)
            ctx.prepare(1e-12)
            cent, Ps, alf = centercalc(b["an"], b["cartes"])
            ref = centre_components(ctx, cent, Ps, alf, dense[0], dense[1])[0]
            row = {"centres": len(Ps)}
            for nrad in nrads:
                _, _, scale, _, ok = lg.grid(b, nrad)
                auto, _, na = centre_components(ctx, cent, Ps, alf, nrad, nang)
                mine, _, nm = centre_components(ctx, cent, Ps, scale, nrad, nang)
                row[nrad] = {"auto_err": abs(auto - ref) / abs(ref), "learned_err": abs(mine - ref) / abs(ref),
                             "points": [na, nm], "predicted": int(ok.sum())}
            out.append(row)
    finally:
        if own:
            ctx.close()
    return out


LEVELS = ((10, 26), (15, 50), (20, 86), (30, 146), (40, 194), (50, 302), (75, 434), (100, 590))


def level_study(ctx, nmol=20, seed=4242, levels=LEVELS, auto=(50, 302), dense=(150, 974)):
    """What any per-centre choice of (nrad, nang) could gain over autogrid's uniform grid.

    For each seeded molecule (2-8 atoms, s and p primitives, real closed-shell DM2) every centre's
    TFVC component of the radial integral is computed on the dense grid and at every level
    (one grid per level serves all centres: a component depends only on its own centre's grid).
    The best possible allocation with a per-centre error budget of autogrid's error / centres is
    then read off the table -- an upper bound of what a predictor of per-centre levels can do.
    Returns one dict per molecule: autogrid's relative error, the allocation's relative error
    and its points relative to autogrid's."""
    from . import centercalc
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nmol):
        b, D = _dense_case_molecule(rng, natoms_range=(2, 9), nprim_range=(10, 60))
        ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
        ctx.gen_closed_shell_dm2(D, unique=True)
        ctx.prepare(1e-12)
        cent, Ps, alf = centercalc(b["an"], b["cartes"])
        nc = len(Ps)
        tot_ref, ref, _ = centre_components(ctx, cent, Ps, alf, *dense)
        comps, pts = [], []
        for nr, na in levels:
            _, pc, ng = centre_components(ctx, cent, Ps, alf, nr, na)
            comps.append(pc)
            pts.append(ng / nc)
        comps = np.asarray(comps)
        err = np.abs(comps - ref[None, :])
        ia = list(levels).index(tuple(auto))
        auto_err = abs(comps[ia].sum() - tot_ref)
        budget = max(auto_err, 1e-300) / nc
        k = [next((i for i in range(len(levels)) if err[i, c] <= budget), len(levels) - 1) for c in range(nc)]
        alloc = abs(sum(comps[k[c], c] for c in range(nc)) - tot_ref)
        out.append({"centres": nc, "auto_rel_err": auto_err / abs(tot_ref), "alloc_rel_err": alloc / abs(tot_ref),
                    "alloc_points_rel": sum(pts[i] for i in k) / (pts[ia] * nc),
                    "levels": np.bincount(k, minlength=len(levels)).tolist()})
    return out


def main(argv=None):
    """Train on autogrid's centres for 500 seeded geometries of 2-20 atoms and compare the learned
    grids against dense grids (nrad 150, nang 974) on held-out molecules with real DM2s:
        python -m inca_parallel_gb300.learned_grid [nmol] [out.npz]"""
    import json
    import sys
    import time
    from . import workloads as W
    args = list(sys.argv[1:] if argv is None else argv)
    nmol = int(args[0]) if args else 500
    t0 = time.time()
    X, Y = training_set(nmol=nmol)
    t1 = time.time()
    lg = LearnedGrid(nhidden=32, seed=1)
    loss = lg.fit(X, Y, epochs=300)
    t2 = time.time()
    if len(args) > 1:
        np.savez(args[1], params=lg.net.params(), mu=lg.mu, sd=lg.sd, lo=lg.lo, hi=lg.hi, tmu=lg.tmu, tsd=lg.tsd)
    rng = np.random.default_rng(909)
    cases = []
    for _ in range(8):
        b = W.random_molecule(rng, int(rng.integers(2, 7)), int(rng.integers(10, 36)))
        keep = (b["tmn"].sum(1) <= 1) & (b["alpha"] <= 50.0)  # where the reference's fit is exact
        b = {**b, "alpha": b["alpha"][keep], "tmn": b["tmn"][keep], "xyz": b["xyz"][keep]}
        nocc = max(1, min(W.electrons(b) // 2, len(b["alpha"]) // 3))
        D, _ = W.closed_shell_density(b, nocc, int(rng.integers(1 << 30)))
        ijkl, v = W.folded_records(D)
        cases.append((b, ijkl, v))
    res = compare_with_dense(lg, cases)
    print(json.dumps({"molecules": nmol, "samples": len(X), "targets_s": t1 - t0, "train_s": t2 - t1,
                      "train_loss": loss, "held_out": res}, indent=1))


if __name__ == "__main__":
    main()
