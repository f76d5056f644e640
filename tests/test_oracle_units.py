"""Unit checks of the oracle's building blocks against independent implementations (CPU)."""
import math
import os
import re

import numpy as np
import pytest

import oracle_lib as O

RULES = [6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194, 230, 266, 302, 350, 434, 590, 770,
         974, 1202, 1454, 1730, 2030, 2354, 2702, 3074, 3470, 3890, 4334, 4802, 5294, 5810]
ORDERS = [3, 5, 7, 9, 11, 13, 15, 17, 19, 21, 23, 25, 27, 29, 31, 35, 41, 47, 53, 59, 65, 71, 77,
          83, 89, 95, 101, 107, 113, 119, 125, 131]


@pytest.mark.parametrize("nang,order", list(zip(RULES, ORDERS)))
def test_lebedev_rules_match_scipy(nang, order):
    integ = pytest.importorskip("scipy.integrate")
    if not hasattr(integ, "lebedev_rule"):
        pytest.skip("scipy without lebedev_rule")
    x, y, z, w = O.lebedev(nang)
    assert abs(w.sum() - 1.0) < 1e-13
    np.testing.assert_allclose(x * x + y * y + z * z, 1.0, atol=1e-15)
    pts, ws = integ.lebedev_rule(order)
    ws = ws / (4 * math.pi)
    mine = np.round(np.stack([x, y, z, w], 1), 12)
    theirs = np.round(np.stack([pts[0], pts[1], pts[2], ws], 1), 12)
    mine = mine[np.lexsort(mine.T[::-1])]
    theirs = theirs[np.lexsort(theirs.T[::-1])]
    np.testing.assert_allclose(mine, theirs, atol=2e-12)


def _sphere_moment(a, b, c):
    """Mean of x^a y^b z^c over the unit sphere: 2 G((a+1)/2) G((b+1)/2) G((c+1)/2) /
    G((a+b+c+3)/2) / (4 pi) when a, b, c are all even, else 0."""
    if a % 2 or b % 2 or c % 2:
        return 0.0
    g = math.lgamma((a + 1) / 2) + math.lgamma((b + 1) / 2) + math.lgamma((c + 1) / 2)
    return 2.0 * math.exp(g - math.lgamma((a + b + c + 3) / 2)) / (4.0 * math.pi)


@pytest.mark.parametrize("nang,order", list(zip(RULES, ORDERS)))
def test_lebedev_rules_exact(nang, order):
    # independent of any library: a rule of algebraic order p averages every monomial of degree
    # <= p over the sphere exactly (checked up to degree 24, where the moments stay well scaled)
    x, y, z, w = O.lebedev(nang)
    assert len(w) == nang
    deg = min(order, 24)
    for a in range(deg + 1):
        xa = x ** a
        for b in range(deg + 1 - a):
            xyab = xa * y ** b
            for c in range(deg + 1 - a - b):
                got = float(np.dot(w, xyab * z ** c))
                assert abs(got - _sphere_moment(a, b, c)) < 1e-13, (nang, a, b, c, got)
    # and one degree beyond the order is not integrated exactly by the smallest rules
    if order <= 7:
        errs = [abs(float(np.dot(w, x ** a * y ** b * z ** (order + 1 - a - b))) - _sphere_moment(a, b, order + 1 - a - b))
                for a in range(order + 2) for b in range(order + 2 - a)]
        assert max(errs) > 1e-6


@pytest.mark.parametrize("n", [1, 2, 5, 50, 75, 150])
def test_gauss_legendre(n):
    t, w = O.gauleg(n)
    tn, wn = np.polynomial.legendre.leggauss(n)
    np.testing.assert_allclose(t, tn, atol=1e-14)
    # the reference stops Newton at |dz| <= 1e-14 and uses the previous iterate for the weight
    np.testing.assert_allclose(w, wn, rtol=1e-10, atol=1e-15)


def _c_table(src, name):
    """The rows of `static const double name[R][C] = {{...}, ...};` in a generated header."""
    body = src[src.index(name + "["):]
    body = body[body.index("{") + 1:body.index("};")]
    return [[float(x) for x in row.split(",") if x.strip()] for row in re.findall(r"\{([^{}]*)\}", body)]


def test_hermite_table():
    # the generated table's n-node rule integrates x^(2k) exp(-x^2) exactly for 2k < 2n
    # (moments Gamma(k + 1/2)), its nodes are symmetric and ascending, and it agrees with
    # numpy's Gauss-Hermite rule
    src = open(os.path.join(O.ROOT, "inca_parallel_gb300", "csrc", "hermite_table.h")).read()
    nodes, weights = _c_table(src, "kNode"), _c_table(src, "kWeight")
    assert len(nodes) == len(weights) == 12
    for n in range(1, 12):
        x, w = np.array(nodes[n][:n]), np.array(weights[n][:n])
        assert np.all(np.diff(x) > 0) and np.allclose(x, -x[::-1], rtol=0, atol=1e-15)
        assert np.all(w > 0) and np.all(np.array(weights[n][n:]) == 0.0)
        for k in range(n):
            mom = math.gamma(k + 0.5)
            assert abs((w * x ** (2 * k)).sum() - mom) < 1e-12 * max(1.0, mom), (n, k)
        xn, wn = np.polynomial.hermite.hermgauss(n)
        np.testing.assert_allclose(x, xn, rtol=1e-13, atol=1e-14)
        np.testing.assert_allclose(w, wn, rtol=1e-12)


@pytest.mark.parametrize("seed", range(5))
def test_lu_solve_matches_dgesv(seed):
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(seed)
    for n in range(1, 14):
        # Vandermonde systems like polycoef's (mod_intrastuff.f90:151-169)
        base = rng.uniform(0.2, 3.0) * (np.arange(1, n + 1) - 0.5 + rng.uniform(-2, 2))
        M = np.array([[b ** (n - 1 - j) for j in range(n)] for b in base])
        b = rng.normal(size=n)
        lu, piv, x_ref, info = lapack.dgesv(M.copy(), b.copy())
        Mr = np.ascontiguousarray(M.copy())
        x = b.copy()
        inf = O.lib().orc_lu_solve(n, O._d(Mr), O._d(x))
        assert inf == info == 0
        np.testing.assert_allclose(x, x_ref, rtol=1e-9 * np.linalg.cond(M) * 1e-3 + 1e-10, atol=1e-12 * np.abs(x_ref).max())


def test_lu_singular_reports_info():
    M = np.ascontiguousarray(np.array([[1.0, 2.0], [2.0, 4.0]]))
    b = np.array([1.0, 1.0])
    assert O.lib().orc_lu_solve(2, O._d(M), O._d(b)) == 2


@pytest.mark.parametrize("t,m,n", [(0, 0, 0), (1, 0, 0), (0, 1, 1), (2, 0, 0), (1, 1, 1), (3, 0, 0)])
def test_normprim(t, m, n):
    def df(a):
        return 1 if a <= 0 else a * df(a - 2)
    alpha = 0.73
    L = t + m + n
    ref = (2 * alpha / math.pi) ** 0.75 * math.sqrt((4 * alpha) ** L / (df(2 * t - 1) * df(2 * m - 1) * df(2 * n - 1)))
    assert abs(O.lib().orc_normprim(alpha, t, m, n) - ref) < 1e-14 * ref


def test_gridpoints3_even_odd_rule():
    r = O.gridpoints3([0.0, 1.0, -2.0], [0.1, 0.2, 0.5], [4, 3, 2])
    # even np: first point at c - s/2 - (np-2)/2 s; odd: c - (np-1)/2 s (mod_build_grid.f90:422-428)
    assert np.allclose(r[0], [-0.15, 0.8, -2.25])
    assert np.allclose(r[-1], [0.15, 1.2, -1.75])
    # x outer, z inner
    assert np.allclose(r[1], [-0.15, 0.8, -1.75])


def test_gridpoints2_symmetry_halving():
    g = O.gridpoints2([0.0, 1.0], [0.5, 2.0], [0.5, 1.0], [6, 14])
    # s=0 shell keeps all points with unit weight; other shells keep z>=0, doubling z>0
    assert g["smn"][0] == 6 and abs(g["w_ang"][:6].sum() - 1.0) < 1e-15
    k = 6
    for n in g["smn"][1:]:
        assert abs(g["w_ang"][k:k + n].sum() - 1.0) < 1e-14
        k += n
    assert len(g["radi"]) == 4 and np.allclose(g["radi"], [0.0, 0.5, 1.0, 2.0])


def test_multicentre_grid_weights_partition():
    # three-centre TFVC partition: the weights integrate a smooth Gaussian to half its norm.
    # The radial weight carries 2*pi rather than 4*pi (mod_build_grid.f90:132), which turns
    # the integral of I(r) (= N(N-1) for the DM2 normalisation) into the number of pairs.
    cent = np.array([[0.0, 0.0, 0.0], [1.4, 0.0, 0.8], [-1.4, 0.0, -0.8]])
    Ps = np.array([3.0, 1.0, 1.0])
    g = O.gridpoints([60, 60, 60], [302, 302, 302], [1.2, 1.0, 1.0], cent, Ps, nosym=True)
    f = np.exp(-((g["r"] - [0.7, 0, 0.4]) ** 2).sum(1))
    assert abs((g["w"] * f).sum() - math.pi ** 1.5 / 2) < 1e-7
    gs = O.gridpoints([60, 60, 60], [302, 302, 302], [1.2, 1.0, 1.0], cent, Ps, nosym=False)
    fs = np.exp(-((gs["r"] - [0.7, 0, 0.4]) ** 2).sum(1)) + np.exp(-((gs["r"] + [0.7, 0, 0.4]) ** 2).sum(1))
    assert abs((gs["w"] * fs).sum() - math.pi ** 1.5) < 1e-7


def test_centercalc_merges_and_snaps():
    an = np.array([6, 6, 1])
    cart = np.array([[0.0, 0.0, 0.0], [2.5, 0.0, 0.3], [0.0, 2.0, 0.0]])
    cent, Ps, alf = O.centercalc(an, cart, nohydro=True)
    # origin + the +-(R1-R2) pair with z snapped to 0 (|z| < 0.5)
    assert len(Ps) == 3 and np.allclose(cent[1], [-2.5, 0.0, 0.0]) and np.allclose(cent[2], [2.5, 0, 0])
    assert Ps[0] == 30.0 and Ps[1] == 18.0
    cent2, Ps2, _ = O.centercalc(an, cart, nohydro=False)
    assert len(Ps2) == 7


def test_dm2p_formats_and_truncation(ch4):
    raw = ch4["raw"]
    ijkl, v = O.parse_dm2p_bytes(raw, 27)
    assert len(v) == 142884
    # sequential unformatted with 4-byte markers (format 1)
    rec = np.frombuffer(raw, dtype=O.DM2P_DTYPE)[:100]
    seq = b"".join(np.int32(24).tobytes() + r.tobytes() + np.int32(24).tobytes() for r in rec)
    a, b = O.parse_dm2p_bytes(seq, 27)
    assert len(b) == 100 and np.array_equal(a, ijkl[:100]) and np.array_equal(b, v[:100])
    # a partial trailing record is ignored (EOF inside a record)
    a, b = O.parse_dm2p_bytes(raw[:24 * 10 + 7], 27)
    assert len(b) == 10
    # an out-of-range index ends the data
    bad = bytearray(raw[:24 * 10])
    bad[24 * 4:24 * 4 + 4] = np.int32(99).tobytes()
    a, b = O.parse_dm2p_bytes(bytes(bad), 27)
    assert len(b) == 4
    with pytest.raises(ValueError):
        O.parse_dm2p_bytes(np.int32(24).tobytes() + np.int32(0).tobytes() + b"\0" * 40, 27)


def test_radial_smearing_normalisation(ch4):
    # P(u) of a sum of point masses integrates to sum of masses (inside the axis)
    r = np.array([[1.0, 0, 0], [0, 2.0, 0], [0, 0, 3.0]])
    w = np.array([1.0, 2.0, 3.0])
    u, P, I = O.radial_smearing(r, w, np.ones(3), u_max=8.0, n_bins=801, sigma=0.15)
    # the kernel is cut at +-4 sigma (mod_intracule.f90:618-619): mass erf(4/sqrt 2) each
    assert abs(np.trapezoid(P, u) - 6.0 * math.erf(4 / math.sqrt(2))) < 1e-4
