"""Edge cases of the oracle itself (CPU): the checker must behave on empty and degenerate inputs
before it is trusted on the GPU's. Everything screened out, no points, linearity in the DM2
values, independence of the record order, and the screening decisions under a change of
normalisation scale."""
import numpy as np

import oracle_lib as O

PTS = np.array([[0.0, 0.0, 0.0], [0.7, -0.2, 0.4], [1.5, 1.0, -0.5], [3.0, 0.0, 0.0]])


def _sys(ch4, v=None, ijkl=None):
    return {"alpha": ch4["alpha"], "tmn": ch4["tmn"], "xyz": ch4["xyz"],
            "ijkl": ch4["ijkl"] if ijkl is None else ijkl, "v": ch4["v"] if v is None else v}


def test_everything_screened_out(ch4):
    I, counts = O.intracule(_sys(ch4), 1e30, PTS)
    assert tuple(counts) == (len(ch4["v"]), 0, 0)
    assert np.all(I == 0.0)


def test_no_points(ch4):
    I, counts = O.intracule(_sys(ch4), 1e-12, np.zeros((0, 3)))
    assert I.shape == (0,)
    assert tuple(counts) == (142884, 111248, 111080)


def test_linear_in_the_dm2_values(ch4):
    # without screening (thresh 0 keeps every non-zero record) the sum is linear in v
    rng = np.random.default_rng(11)
    v1 = ch4["v"] * rng.uniform(0.5, 1.5, len(ch4["v"]))
    v2 = ch4["v"] - v1
    Ia, _ = O.intracule(_sys(ch4, v1), 0.0, PTS)
    Ib, _ = O.intracule(_sys(ch4, v2), 0.0, PTS)
    Iab, _ = O.intracule(_sys(ch4, v1 + v2), 0.0, PTS)
    scale = np.abs(Iab).max()
    assert np.abs(Ia + Ib - Iab).max() <= 1e-12 * scale


def test_record_order_does_not_matter(ch4):
    rng = np.random.default_rng(12)
    perm = rng.permutation(len(ch4["v"]))
    I, c = O.intracule(_sys(ch4), 1e-12, PTS)
    Ip, cp = O.intracule(_sys(ch4, ch4["v"][perm], ch4["ijkl"][perm]), 1e-12, PTS)
    assert tuple(c) == tuple(cp)
    np.testing.assert_allclose(Ip, I, rtol=1e-13, atol=0)


def test_screening_scales_with_the_values(ch4):
    # both screens compare |v| times a bound with thresh / npairs: scaling v and thresh by the
    # same power of two scales every screened value exactly and keeps every decision
    a = O.prepare(_sys(ch4), 1e-12)
    b = O.prepare(_sys(ch4, ch4["v"] * 1024.0), 1e-12 * 1024.0)
    np.testing.assert_array_equal(a["flags"], b["flags"])
    np.testing.assert_array_equal(a["s1"] * 1024.0, b["s1"])
