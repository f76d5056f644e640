"""GPU parity of libinca_gpu.so against the CPU oracle and the reference's goldens.

Tolerances (written here, per the precision contract of the hot path):
  * screening values, flags and survivor records: bit-identical to the oracle;
  * grids: bit-identical (same operation sequence, no FMA contraction on either side);
  * FP64 form: 1e-12 relative to the oracle (summation order only);
  * mixed form: 1e-10 relative on the radial integral, 1e-8 relative on each I(s),
    1e-8 of max|I| on the vector cube, 1e-8 relative at explicit points.
"""
import numpy as np
import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu

THRESH = 1e-12


@pytest.fixture(scope="module")
def ctx():
    from inca_parallel_gb300 import build
    build.build()
    from inca_parallel_gb300 import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def ch4_ctx(ctx, ch4):
    ctx.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
    ctx.set_quartets(ch4["ijkl"], ch4["v"])
    counts = ctx.prepare(THRESH)
    return ctx, counts


def test_screening_bit_identical(ch4_ctx, ch4):
    ctx, counts = ch4_ctx
    assert counts == (142884, 111248, 111080)
    ref = O.prepare(ch4, THRESH)
    flags, s1, s2 = ctx.screening()
    np.testing.assert_array_equal(flags, ref["flags"])
    np.testing.assert_array_equal(s1, ref["s1"])
    np.testing.assert_array_equal(s2, ref["s2"])


def test_records_bit_identical(ch4_ctx, ch4):
    ctx, _ = ch4_ctx
    ref = O.prepare(ch4, THRESH, records=True)
    rec = ctx.records()
    for k in ("A", "sqe", "d", "L", "C"):
        np.testing.assert_array_equal(rec[k], ref[k], err_msg=k)


def test_radial_grid_matches_oracle(ch4_ctx, ch4):
    ctx, _ = ch4_ctx
    cent, Ps, alf = O.centercalc(ch4["an"], ch4["cartes"])
    mg, rg, ng = ctx.grid_radial([50], [110], alf, cent, Ps)
    g = O.gridpoints([50], [110], alf, cent, Ps)
    assert (mg, rg, ng) == (g["maxgrid"], g["rgrid"], len(g["w"]))
    mine = ctx.grid_copy(weights=True, vee=True, cmap=True)
    np.testing.assert_array_equal(mine["r"], g["r"])
    np.testing.assert_array_equal(mine["w"], g["w"])
    np.testing.assert_array_equal(mine["wvee"], g["wvee"])
    np.testing.assert_array_equal(mine["cmap"], g["cmap"] + 1)


def test_multicentre_grid_matches_oracle(ctx):
    cent = np.array([[0.0, 0.0, 0.0], [1.4, 0.3, 0.8], [-1.4, -0.3, -0.8], [0.0, 2.1, 0.0], [0.0, -2.1, 0.0]])
    Ps = np.array([3.0, 1.0, 1.0, 2.0, 2.0])
    alf = np.array([1.2, 1.0, 1.0, 0.8, 0.8])
    for nosym in (False, True):
        mg, rg, ng = ctx.grid_radial([40] * 5, [110, 110, 146, 110, 146], alf, cent, Ps, nosym=nosym)
        g = O.gridpoints([40] * 5, [110, 110, 146, 110, 146], alf, cent, Ps, nosym=nosym)
        assert (mg, rg, ng) == (g["maxgrid"], g["rgrid"], len(g["w"]))
        mine = ctx.grid_copy(weights=True, vee=True, cmap=True)
        np.testing.assert_array_equal(mine["r"], g["r"])
        np.testing.assert_array_equal(mine["w"], g["w"])
        np.testing.assert_array_equal(mine["cmap"], g["cmap"] + 1)


def test_scan_and_cube_grids_match_oracle(ctx):
    nr, ng = ctx.grid_scan([0.0, 1.0], [0.95, 3.0], [0.05, 0.1], [110, 302])
    g = O.gridpoints2([0.0, 1.0], [0.95, 3.0], [0.05, 0.1], [110, 302])
    assert nr == len(g["smn"]) and ng == len(g["w_ang"])
    mine = ctx.grid_copy(weights=True)
    np.testing.assert_array_equal(mine["r"], g["r"])
    np.testing.assert_array_equal(mine["w"], g["w_ang"])
    ctx.grid_cube([0.1, -0.2, 0.3], [0.1, 0.2, 0.15], [7, 6, 5])
    np.testing.assert_array_equal(ctx.grid_copy(weights=False)["r"],
                                  O.gridpoints3([0.1, -0.2, 0.3], [0.1, 0.2, 0.15], [7, 6, 5]))


@pytest.fixture(scope="module")
def ch4_integral_ref(ch4):
    cent, Ps, alf = O.centercalc(ch4["an"], ch4["cartes"])
    g = O.gridpoints([50], [110], alf, cent, Ps)
    Iv, _ = O.intracule(ch4, THRESH, g["r"])
    return cent, Ps, alf, g, Iv


@pytest.mark.parametrize("mode,rtol", [(0, 1e-12), (1, 1e-10)])
def test_radial_integral(ch4_ctx, ch4, ch4_integral_ref, mode, rtol):
    ctx, _ = ch4_ctx
    cent, Ps, alf, g, Iv_ref = ch4_integral_ref
    ctx.grid_radial([50], [110], alf, cent, Ps)
    ctx.eval(mode=mode, tol=1e-10)
    total, vee, pc, vc = ctx.radial_integral()
    R_ref = float((g["w"] * Iv_ref).sum())
    assert abs(total - R_ref) <= rtol * abs(R_ref), (total, R_ref)
    assert abs(total - ch4["gold"]["radial_integral"]) <= max(rtol, 1e-13) * 45.0
    assert abs(vee - float((g["wvee"] * Iv_ref).sum())) <= max(rtol, 1e-12) * abs(vee)


@pytest.mark.parametrize("mode,rtol", [(0, 1e-12), (1, 1e-8)])
def test_radial_plot(ch4_ctx, ch4, mode, rtol):
    ctx, _ = ch4_ctx
    ctx.grid_scan([0.0], [5.0], [0.05], [110])
    ctx.eval(mode=mode, tol=1e-8)
    radi, rintra = ctx.radial_plot()
    g = O.gridpoints2([0.0], [5.0], [0.05], [110])
    Iv, _ = O.intracule(ch4, THRESH, g["r"])
    ref, k = [], 0
    for n in g["smn"]:
        ref.append((g["w_ang"][k:k + n] * Iv[k:k + n]).sum())
        k += n
    np.testing.assert_allclose(rintra, ref, rtol=rtol, atol=0)
    np.testing.assert_allclose(rintra, O.ref_rad()[:, 1], rtol=1e-8)


@pytest.mark.parametrize("mode", [0, 1])
def test_vector_cube(ch4_ctx, mode):
    ctx, _ = ch4_ctx
    ctx.grid_cube([0, 0, 0], [0.1, 0.1, 0.1], [20, 20, 20])
    Iv = ctx.eval(mode=mode, tol=1e-8)
    ref, _ = O.ref_cube()
    scale = np.abs(ref).max()
    tol = 1e-12 if mode == 0 else 1e-8
    assert np.abs(Iv - ref).max() <= tol * scale


@pytest.mark.parametrize("mode", [0, 1])
def test_zero_and_two_points(ch4_ctx, ch4, mode):
    ctx, _ = ch4_ctx
    gold = ch4["gold"]
    ctx.grid_points(np.zeros((1, 3)))
    I0 = ctx.eval(mode=mode, tol=1e-10)
    assert abs(I0[0] / 2 - gold["intracule_at_zero"]) <= 1e-10 * gold["intracule_at_zero"]
    ctx.grid_points(np.array([[0.0, 0, 0], [1.0, 0, 0]]))
    I2 = ctx.eval(mode=mode, tol=1e-10)
    np.testing.assert_allclose(I2, gold["two_points"], rtol=1e-10)


def test_deterministic_repeat(ch4_ctx):
    ctx, _ = ch4_ctx
    ctx.grid_cube([0.3, 0, 0], [0.2, 0.2, 0.2], [9, 9, 9])
    for mode in (0, 1):
        a = ctx.eval(mode=mode)
        b = ctx.eval(mode=mode)
        np.testing.assert_array_equal(a, b)


def test_smearing_matches_oracle(ch4_ctx, ch4_integral_ref):
    ctx, _ = ch4_ctx
    cent, Ps, alf, g, Iv_ref = ch4_integral_ref
    ctx.grid_radial([50], [110], alf, cent, Ps)
    ctx.eval(mode=0)
    u, P, I = ctx.radial_smearing(5.0, 1000, 0.15)
    ur, Pr, Ir = O.radial_smearing(g["r"], g["w"], Iv_ref, 5.0, 1000, 0.15)
    np.testing.assert_allclose(u, ur, rtol=0, atol=0)
    np.testing.assert_allclose(P, Pr, rtol=1e-11, atol=1e-14 * np.abs(Pr).max())


def test_closed_shell_generator_matches_host_folding(ctx):
    from inca_parallel_gb300 import workloads as W
    b = W.ch4_basis()
    D, S = W.closed_shell_density(b, 5, W.SEED0)
    ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
    n = ctx.gen_closed_shell_dm2(D, unique=False)
    ijkl, v = W.folded_records(D)
    assert n == len(v)
    ctx.prepare(1e-12)
    ref = O.prepare({"alpha": b["alpha"], "tmn": b["tmn"], "xyz": b["xyz"], "ijkl": ijkl, "v": v}, 1e-12)
    flags, s1, s2 = ctx.screening()
    np.testing.assert_array_equal(flags, ref["flags"])
    np.testing.assert_allclose(s1, ref["s1"], rtol=1e-13, atol=0)
    # unique list: same integral with nosym
    cent, Ps, alf = O.centercalc(b["an"], b["cartes"])
    ctx.grid_radial([40], [110], alf, cent, Ps, nosym=True)
    ctx.eval(mode=0)
    full = ctx.radial_integral()[0]
    nu = ctx.gen_closed_shell_dm2(D, unique=True)
    assert nu == 378 * 379 // 2
    ctx.prepare(1e-12)
    ctx.eval(mode=0)
    uniq = ctx.radial_integral()[0]
    assert abs(full - uniq) <= 1e-9 * abs(full)


def test_errors_are_reported(ctx):
    from inca_parallel_gb300 import IncaError
    with pytest.raises(IncaError, match="INCA_E_IO"):
        ctx.load_dm2p("/nonexistent/file.dm2p")
    with pytest.raises(IncaError, match="INCA_E_ARG"):
        ctx.grid_scan([0.0], [1.0], [0.1], [111])
    with pytest.raises(IncaError, match="INCA_E_ARG"):
        ctx.set_quartets(np.array([[1, 1, 1, 99]]), np.array([1.0]))
        ctx.prepare(1e-12)
