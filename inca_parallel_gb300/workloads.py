"""Seeded synthetic workloads for the benchmark and the GPU tests.

No quantum-chemistry package is available, so the DM2s are built from seeded closed-shell
1-RDMs in a primitive Cartesian Gaussian basis: random orbitals, orthonormal in the overlap
metric of the normalised primitives, D = 2 C C^T, Gamma_{ik,jl} = D_ik D_jl - 1/2 D_il D_jk
(the library folds it into the .dm2p record convention). With that convention the records
satisfy sum v S_ik S_jl = N(N-1), like the reference's CH4 fixture.

Workloads (seed = 20261203 + index):
  0  CH4: C at the origin, 4 H tetrahedral at (+-1.1968)^3 bohr; C 6 s (71.6, 13.0, 3.53,
     2.94, 0.684, 0.222) + 3x3 p (2.94, 0.684, 0.222); H 3 s (3.425, 0.6239, 0.1689);
     5 occupied orbitals.
  2  12-atom planar ring (6 heavy atoms on a 2.64-bohr circle + 6 H), ~200 primitives l<=2,
     exponents log-uniform in [0.1, 5000], 21 occupied orbitals.
  3  molecules of 3..20 atoms at random non-overlapping positions (>= 1.8 bohr apart),
     20..300 primitives l<=2.
  4  a 20-atom molecule of that kind with about 300 primitives (exponents up to 200) and 60
     occupied orbitals, for the vector cube.
"""
import math

import numpy as np

SEED0 = 20261203

CH4_C_S = [71.6, 13.0, 3.53, 2.94, 0.684, 0.222]
CH4_C_P = [2.94, 0.684, 0.222]
CH4_H_S = [3.425, 0.6239, 0.1689]
CH4_H = 1.1968


def _dfact(a):
    r = 1
    while a > 1:
        r *= a
        a -= 2
    return r


def primitive_norm(alpha, t):
    """Normalisation of x^t y^m z^n exp(-alpha r^2) (the reference's normprim)."""
    L = sum(t)
    df = _dfact(2 * t[0] - 1) * _dfact(2 * t[1] - 1) * _dfact(2 * t[2] - 1)
    return (2 * alpha / math.pi) ** 0.75 * math.sqrt((4 * alpha) ** L / df)


def _overlap_1d(a, b, A, B, ta, tb):
    p = a + b
    P = (a * A + b * B) / p
    K = math.exp(-a * b / p * (A - B) ** 2)
    s = 0.0
    for i in range(ta + 1):
        for j in range(tb + 1):
            n = i + j
            if n % 2:
                continue
            mom = _dfact(n - 1) / (2 * p) ** (n // 2) * math.sqrt(math.pi / p)
            s += math.comb(ta, i) * math.comb(tb, j) * (P - A) ** (ta - i) * (P - B) ** (tb - j) * mom
    return K * s


def overlap(basis):
    """Overlap matrix of the normalised primitives."""
    a, t, x = basis["alpha"], basis["tmn"], basis["xyz"]
    n = len(a)
    N = np.array([primitive_norm(a[i], t[i]) for i in range(n)])
    S = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            v = N[i] * N[j]
            for d in range(3):
                v *= _overlap_1d(a[i], a[j], x[i, d], x[j, d], int(t[i, d]), int(t[j, d]))
            S[i, j] = S[j, i] = v
    return S


def closed_shell_density(basis, nocc, seed):
    """D = 2 C C^T from nocc random orbitals, orthonormal in the overlap metric."""
    rng = np.random.default_rng(seed)
    S = overlap(basis)
    n = len(S)
    C = rng.normal(size=(n, nocc))
    # Loewdin-style: C <- C (C^T S C)^(-1/2)
    M = C.T @ S @ C
    w, U = np.linalg.eigh(M)
    C = C @ (U @ np.diag(w ** -0.5) @ U.T)
    return 2.0 * C @ C.T, S


def _shells(alpha_list, l):
    comps = {0: [(0, 0, 0)], 1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
             2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]}[l]
    return [(a, c) for a in alpha_list for c in comps]


def ch4_basis():
    atoms = [(6, (0.0, 0.0, 0.0))]
    for sx, sy, sz in [(1, 1, 1), (-1, -1, 1), (-1, 1, -1), (1, -1, -1)]:
        atoms.append((1, (sx * CH4_H, sy * CH4_H, sz * CH4_H)))
    prims = []
    for z, pos in atoms:
        if z == 6:
            pr = _shells(CH4_C_S, 0)
            # p components grouped like the fixture: x block, y block, z block
            for c in [(1, 0, 0), (0, 1, 0), (0, 0, 1)]:
                pr += [(a, c) for a in CH4_C_P]
        else:
            pr = _shells(CH4_H_S, 0)
        prims += [(a, c, pos) for a, c in pr]
    return _basis(atoms, prims)


def _basis(atoms, prims):
    return {"alpha": np.array([p[0] for p in prims]),
            "tmn": np.array([p[1] for p in prims], dtype=np.int32),
            "xyz": np.array([p[2] for p in prims], dtype=np.float64),
            "an": np.array([a[0] for a in atoms], dtype=np.int32),
            "cartes": np.array([a[1] for a in atoms], dtype=np.float64)}


def random_atom_basis(rng, nprim_target, lmax=2, lo=0.1, hi=5000.0):
    """A random contracted-free basis for one atom: s, p, d shells with log-uniform exponents."""
    prims = []
    ncomp = {0: 1, 1: 3, 2: 6}
    while len(prims) < nprim_target:
        l = int(rng.integers(0, lmax + 1))
        a = float(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        if len(prims) + ncomp[l] > nprim_target and l > 0:
            continue
        prims += _shells([a], l)
    return prims


def ring_molecule(seed=SEED0 + 2, nprim_target=200):
    """12-atom planar ring: 6 heavy atoms on a circle of radius 2.64 bohr plus 6 H outside."""
    rng = np.random.default_rng(seed)
    atoms = []
    heavy = [6, 6, 7, 6, 8, 6]
    for k in range(6):
        ang = 2 * math.pi * k / 6
        atoms.append((heavy[k], (2.64 * math.cos(ang), 2.64 * math.sin(ang), 0.0)))
    for k in range(6):
        ang = 2 * math.pi * k / 6
        atoms.append((1, (4.70 * math.cos(ang), 4.70 * math.sin(ang), 0.0)))
    per_heavy = int(nprim_target * 0.8 / 6)
    prims = []
    for z, pos in atoms:
        n = per_heavy if z > 1 else max(3, (nprim_target - 6 * per_heavy) // 6)
        prims += [(a, c, pos) for a, c in random_atom_basis(rng, n, lmax=2 if z > 1 else 1)]
    return _basis(atoms, prims)


def random_molecule(rng, natoms, nprim_target, mind=1.8, hi=5000.0):
    pos = []
    while len(pos) < natoms:
        p = rng.uniform(-0.9, 0.9, size=3) * (2.0 + natoms ** (1 / 3) * 1.6)
        if all(np.linalg.norm(p - q) >= mind for q in pos):
            pos.append(p)
    zs = [int(rng.choice([1, 6, 7, 8])) for _ in range(natoms)]
    per = max(1, nprim_target // natoms)
    atoms, prims = [], []
    for z, p in zip(zs, pos):
        atoms.append((z, tuple(p)))
        prims += [(a, c, tuple(p)) for a, c in random_atom_basis(rng, per, lmax=2 if z > 1 else 1, hi=hi)]
    return _basis(atoms, prims)


def ring_workload(nprim_target=200, nocc=21):
    """Workload 2: the 12-atom ring and its closed-shell 1-RDM (D, overlap)."""
    b = ring_molecule(nprim_target=nprim_target)
    D, S = closed_shell_density(b, nocc, SEED0 + 2)
    return b, D


def cube_molecule(seed=SEED0 + 4, natoms=20, nprim_target=300, hi=200.0):
    """Workload 4 (cubeintra): a 20-atom molecule with about 300 primitives, l <= 2, exponents
    log-uniform in [0.1, 200] (beyond a few hundred the reference's polynomial fit breaks down for
    d shells on different atoms, so larger exponents would only test that breakdown)."""
    rng = np.random.default_rng(seed)
    return random_molecule(rng, natoms, nprim_target, hi=hi)


def cube_workload(nocc=60):
    """Workload 4: the 20-atom molecule and its closed-shell 1-RDM with 60 occupied orbitals."""
    b = cube_molecule()
    D, S = closed_shell_density(b, nocc, SEED0 + 4)
    return b, D


def electrons(basis):
    return int(basis["an"].sum())


def folded_records(D):
    """Host-side folding of Gamma into .dm2p records (i<=k, j<=l), 1-based, for checks."""
    n = len(D)
    pairs = [(i, k) for i in range(n) for k in range(i, n)]
    ijkl, v = [], []
    for (i, k) in pairs:
        for (j, l) in pairs:
            s = 0.0
            for a, b in ({(i, k), (k, i)}):
                for c, d in ({(j, l), (l, j)}):
                    s += D[a, b] * D[c, d] - 0.5 * D[a, d] * D[c, b]
            ijkl.append((i + 1, j + 1, k + 1, l + 1))
            v.append(s)
    return np.array(ijkl, dtype=np.int32), np.array(v)


def batch_workload(n=64, seed=SEED0 + 3, hi=200.0, max_prims=None):
    """Workload 3: n molecules of 3..20 atoms (random non-overlapping positions, >= 1.8 bohr apart)
    with 20..300 primitives (l <= 2, exponents up to 200) and uneven closed-shell 1-RDMs
    (min(electrons / 2, primitives / 3) occupied orbitals). Returns [(index, basis, D)];
    max_prims keeps only the molecules with at most that many primitives (the others are drawn
    all the same, so every molecule is the same whatever the subset)."""
    rng = np.random.default_rng(seed)
    mols = []
    for i in range(n):
        natoms = int(rng.integers(3, 21))
        nprim = int(rng.integers(20, 301))
        b = random_molecule(rng, natoms, nprim, hi=hi)
        nocc = max(1, min(electrons(b) // 2, len(b["alpha"]) // 3))
        dseed = int(rng.integers(1 << 30))
        if max_prims is not None and len(b["alpha"]) > max_prims:
            continue
        D, _ = closed_shell_density(b, nocc, dseed)
        mols.append((i, b, D))
    return mols
