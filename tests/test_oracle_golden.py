"""Pin the CPU oracle against the reference's own golden vectors (CPU only).

The reference's tests (tests/run_tests.py:96-255) compare the CH4 outputs of the Fortran
program with an absolute tolerance of 1e-5. The oracle restates the algorithm in FP64, so it
is held to much tighter bounds here: the goldens carry ~16 digits except the .rad file (ES20.8,
9 digits).
"""
import numpy as np

import oracle_lib as O

THRESH = 1e-12  # tests/inputs/test_*.inp


def test_counts_match_reference_screening(ch4):
    # 142 884 records; 111 248 after screen 1; 111 080 after screen 2 (CH4, thresh 1e-12)
    pr = O.prepare(ch4, THRESH)
    assert list(pr["counts"]) == [142884, 111248, 111080]


def test_radial_integral_golden(ch4):
    cent, Ps, alf = O.centercalc(ch4["an"], ch4["cartes"])  # multicenter=.true., nohydro
    assert len(Ps) == 1 and abs(alf[0] - 0.70 * 1.8897) < 1e-15 and Ps[0] == 15.0
    g = O.gridpoints([50], [110], alf, cent, Ps)
    assert g["r"].shape == (3050, 3) and g["maxgrid"] == 5500
    Iv, cnt = O.intracule(ch4, THRESH, g["r"])
    R = float((g["w"] * Iv).sum())
    gold = ch4["gold"]
    assert abs(R - gold["radial_integral"]) <= 1e-13 * gold["radial_integral"]
    npairs = ch4["nelec"] * (ch4["nelec"] - 1) // 2
    assert abs((R - npairs) - gold["radial_integral_error"]) < 1e-8


def test_intracule_at_zero_and_two_points_golden(ch4):
    gold = ch4["gold"]
    I0, _ = O.intracule(ch4, THRESH, np.zeros((1, 3)))
    assert abs(I0[0] / 2 - gold["intracule_at_zero"]) <= 1e-13 * gold["intracule_at_zero"]
    I2, _ = O.intracule(ch4, THRESH, np.array([[0.0, 0, 0], [1.0, 0, 0]]))
    for got, exp in zip(I2, gold["two_points"]):
        assert abs(got - exp) <= 1e-13 * abs(exp)


def test_radial_plot_golden(ch4):
    g = O.gridpoints2([0.0], [5.0], [0.05], [110])
    assert len(g["smn"]) == 101 and g["smn"][0] == 110
    Iv, _ = O.intracule(ch4, THRESH, g["r"])
    rad, k = [], 0
    for n in g["smn"]:
        rad.append((g["w_ang"][k:k + n] * Iv[k:k + n]).sum())
        k += n
    ref = O.ref_rad()
    np.testing.assert_allclose(g["radi"], ref[:, 0], atol=5e-7)
    # ES20.8 carries 9 significant digits
    np.testing.assert_allclose(rad, ref[:, 1], rtol=1e-8, atol=0)


def test_vector_cube_golden(ch4):
    r = O.gridpoints3([0, 0, 0], [0.1, 0.1, 0.1], [20, 20, 20])
    Iv, _ = O.intracule(ch4, THRESH, r)
    ref, _ = O.ref_cube()
    np.testing.assert_allclose(Iv, ref, rtol=1e-12, atol=1e-14)


def test_result_independent_of_thread_count(ch4):
    r = O.gridpoints3([0, 0, 0], [0.3, 0.3, 0.3], [4, 4, 4])
    a, _ = O.intracule(ch4, THRESH, r, nthreads=1)
    b, _ = O.intracule(ch4, THRESH, r, nthreads=4)
    np.testing.assert_allclose(a, b, rtol=1e-13)


def test_eval_records_equals_full_path(ch4):
    pr = O.prepare(ch4, THRESH, records=True)
    r = O.gridpoints3([0.2, -0.1, 0.05], [0.4, 0.4, 0.4], [3, 3, 3])
    a = O.eval_records(pr, r)
    b, _ = O.intracule(ch4, THRESH, r)
    np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-15)
