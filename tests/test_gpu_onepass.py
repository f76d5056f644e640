"""One-pass mixed evaluation (grids of at least 2 048 points) against the FP64 GPU form.

The FP64 GPU form is checked against the oracle at 1e-12 in test_gpu_parity.py and serves as
the full-size oracle here. Tolerances: 1e-8 relative on each I(s), 1e-10 relative on the radial
integral, 1e-8 of max|I| on the vector cube. The threshold estimates are also forced to both
extremes (INCA_EST_SAFETY): 0 corrects every term in the one pass; 1e6 leaves the corrections
to the correction pass, which must then run and still meet the tolerance. The estimate pass's
work split (INCA_SAMPLE_ITEMS_PER_CTA) is driven to 1, 4 and 48 items per CTA.
"""
import numpy as np
import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu

THRESH = 1e-12
SCAN = ([0.0], [10.0], [0.05], [590])


@pytest.fixture(scope="module")
def ctx(ch4):
    from inca_parallel_gb300 import build
    build.build()
    from inca_parallel_gb300 import Context
    c = Context(0)
    c.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
    c.set_quartets(ch4["ijkl"], ch4["v"])
    c.prepare(THRESH)
    yield c
    c.close()


@pytest.fixture(scope="module")
def scan_fp64(ctx):
    nr, ng = ctx.grid_scan(*SCAN)
    assert ng == 62390
    ctx.eval(mode=0)
    return ctx.radial_plot()[1]


def _scan_mixed(ctx):
    ctx.grid_scan(*SCAN)
    ctx.eval(mode=1, tol=1e-8)
    return ctx.radial_plot()[1]


def test_radial_plot_one_pass(ctx, scan_fp64):
    I = _scan_mixed(ctx)
    rel = np.abs(I - scan_fp64) / np.abs(scan_fp64)
    assert rel.max() <= 1e-8, rel.max()
    assert ctx.stats()["corrected_terms"] > 0


@pytest.mark.parametrize("safety", ["0", "1e6"])
def test_estimate_extremes(ctx, scan_fp64, monkeypatch, safety):
    monkeypatch.setenv("INCA_EST_SAFETY", safety)
    I = _scan_mixed(ctx)
    rel = np.abs(I - scan_fp64) / np.abs(scan_fp64)
    assert rel.max() <= 1e-8, rel.max()
    if safety == "1e6":
        assert ctx.phases()["pass2_ms"] > 0.0
        assert ctx.stats()["precise_pairs"] > 0


@pytest.mark.parametrize("items", ["1", "4", "48"])
def test_estimate_pass_items(ctx, scan_fp64, monkeypatch, items):
    # the estimate pass's work split (INCA_SAMPLE_ITEMS_PER_CTA) changes its partial sums, hence
    # the estimated thresholds and the set of inline corrections, never the tolerance met; a
    # captured graph follows the knob
    monkeypatch.setenv("INCA_SAMPLE_ITEMS_PER_CTA", items)
    I = _scan_mixed(ctx)
    rel = np.abs(I - scan_fp64) / np.abs(scan_fp64)
    assert rel.max() <= 1e-8, rel.max()
    eager = ctx.eval(mode=1, tol=1e-8)
    np.testing.assert_array_equal(ctx.eval_graph(mode=1, tol=1e-8), eager)
    np.testing.assert_array_equal(ctx.eval_graph(mode=1, tol=1e-8), eager)


@pytest.mark.parametrize("cheap,drop,slack", [("1", "0.4", "0"), ("1", "0.05", "0"), ("0", "0.05", "0"),
                                              ("1", "0.2", "6"), ("1", "0.2", "30")])
def test_cheap_tier(ctx, scan_fp64, monkeypatch, cheap, drop, slack):
    # pairs whose rigorous FP32 error bound fits under the drop threshold (times 2^slack) take
    # the cheap tier (plain FP32, hardware ex2); the tolerance holds with and without it, with a
    # large share of the tolerance given to left-out and cheap pairs, and with a slack so large
    # that the left-out mass exceeds its check and the pass is repeated without leaving out
    monkeypatch.setenv("INCA_CHEAP_TIER", cheap)
    monkeypatch.setenv("INCA_DROP_FRACTION", drop)
    monkeypatch.setenv("INCA_CHEAP_SLACK", slack)
    I = _scan_mixed(ctx)
    rel = np.abs(I - scan_fp64) / np.abs(scan_fp64)
    assert rel.max() <= 1e-8, rel.max()
    st = ctx.stats()
    if cheap == "1" and slack != "30":
        assert st["cheap_pairs"] > 0
    else:  # off, or repeated without leaving anything out
        assert st["cheap_pairs"] == 0
    eager = ctx.eval(mode=1, tol=1e-8)
    np.testing.assert_array_equal(ctx.eval_graph(mode=1, tol=1e-8), eager)


def test_fp64_screened_form(ctx, scan_fp64):
    # every term in FP64 with the mixed form's leaving-out of negligible (quartet, tile) pairs:
    # the left-out bound mass is checked after the pass to stay within half the tolerance (else
    # the pass is repeated without leaving out), so the result is within 0.5e-8 of the plain form
    from inca_parallel_gb300 import INCA_FP64_SCREENED
    ctx.grid_scan(*SCAN)
    ctx.eval(mode=INCA_FP64_SCREENED, tol=1e-8)
    I = ctx.radial_plot()[1]
    rel = np.abs(I - scan_fp64) / np.abs(scan_fp64)
    assert rel.max() <= 0.5e-8, rel.max()
    st = ctx.stats()
    assert st["skipped_pairs"] > 0 and st["precise_pairs"] > 0 and st["corrected_terms"] == 0
    np.testing.assert_array_equal(ctx.eval(mode=INCA_FP64_SCREENED, tol=1e-8), ctx.eval(mode=INCA_FP64_SCREENED,
                                                                                      tol=1e-8))


def test_one_pass_deterministic(ctx):
    a = _scan_mixed(ctx)
    b = _scan_mixed(ctx)
    np.testing.assert_array_equal(a, b)


def test_radial_integral_one_pass(ctx, ch4):
    cent, Ps, alf = O.centercalc(ch4["an"], ch4["cartes"], nohydro=False)
    nq = len(Ps)
    _, _, ng = ctx.grid_radial([50] * nq, [110] * nq, alf, cent, Ps)
    assert ng >= 16384
    ctx.eval(mode=0)
    ref, vref, _, _ = ctx.radial_integral()
    ctx.eval(mode=1, tol=1e-10)
    tot, vee, _, _ = ctx.radial_integral()
    assert abs(tot - ref) <= 1e-10 * abs(ref), (tot, ref)
    assert abs(vee - vref) <= 1e-10 * abs(vref), (vee, vref)
    # sum rule N(N-1)/2 = 45 up to the grid's own quadrature error
    assert abs(tot - 45.0) < 0.1


def test_cube_one_pass(ctx, monkeypatch):
    # the general one-pass form on a cube (INCA_MIXED otherwise takes the separable form there)
    monkeypatch.setenv("INCA_CUBE_SEPARABLE", "0")
    ctx.grid_cube([0.0, 0.0, 0.0], [0.15, 0.15, 0.15], [32, 32, 32])
    ref = ctx.eval(mode=0)
    I = ctx.eval(mode=1, tol=1e-8)
    assert np.abs(I - ref).max() <= 1e-8 * np.abs(ref).max()


@pytest.mark.parametrize("grid", ["scan", "cube", "small"])
def test_graph_replay_matches_eager(ctx, grid, monkeypatch):
    monkeypatch.setenv("INCA_CUBE_SEPARABLE", "0")  # the cube case captures the general form
    if grid == "scan":
        ctx.grid_scan(*SCAN)
    elif grid == "cube":
        ctx.grid_cube([0.0, 0.0, 0.0], [0.15, 0.15, 0.15], [32, 32, 32])
    else:
        ctx.grid_scan([0.0], [2.0], [0.1], [110])  # below the one-pass size: two passes
    eager = ctx.eval(mode=1, tol=1e-8)
    first = ctx.eval_graph(mode=1, tol=1e-8)   # captures (this result comes from an eager run)
    n0 = ctx.kernel_launches()
    again = ctx.eval_graph(mode=1, tol=1e-8)   # replays
    third = ctx.eval_graph(mode=1, tol=1e-8)
    np.testing.assert_array_equal(first, eager)
    np.testing.assert_array_equal(again, eager)
    np.testing.assert_array_equal(third, eager)
    assert ctx.kernel_launches() > n0


def test_autotune_keeps_tolerance(ctx, scan_fp64):
    ctx.grid_scan(*SCAN)
    t = ctx.autotune(tol=1e-8, reps=2)
    assert t["items_per_cta"] in (4, 8, 12, 24, 48)
    assert t["sample_stride"] in (8, 16, 32, 64)
    assert t["estimate_safety"] in (0.3, 0.5, 0.7, 1.0, 1.25)
    assert t["drop_fraction"] in (0.02, 0.05, 0.1, 0.2, 0.3)
    assert (t["points_per_lane"], t["ctas_per_sm"]) in ((4, 12), (4, 16), (4, 20), (3, 16), (3, 20), (5, 12),
                                                        (5, 16))
    assert t["cheap_slack"] in (0, 2, 4, 6, 8)
    assert 0 < t["best_ms"] <= t["default_ms"]
    try:
        # the tuned schedule stays in the context; every schedule meets the tolerance
        I = _scan_mixed(ctx)
        rel = np.abs(I - scan_fp64) / np.abs(scan_fp64)
        assert rel.max() <= 1e-8, rel.max()
        for ipc, stride, safety, drop, ctas, slack, ppt in ((4, 32, 0.3, 0.2, 12, 8, 4), (48, 8, 0.7, 0.02, 20, 0, 3),
                                                           (12, 16, 0.5, 0.05, 16, 30, 5), (24, 16, 0.7, 0.1, 16, 4, 3),
                                                           (24, 32, 0.7, 0.1, 12, 4, 5)):
            ctx.set_tuning(ipc, stride, safety, drop, ctas, slack, ppt)
            I = _scan_mixed(ctx)
            rel = np.abs(I - scan_fp64) / np.abs(scan_fp64)
            assert rel.max() <= 1e-8, (ipc, stride, safety, rel.max())
        # a tile shape that is not compiled (five points per lane need the larger register budgets)
        from inca_parallel_gb300 import IncaError
        for ctas, ppt in ((20, 5), (12, 3), (16, 6)):
            with pytest.raises(IncaError, match="INCA_E_ARG"):
                ctx.set_tuning(24, 16, 0.7, 0.1, ctas, 4, ppt)
    finally:
        ctx.set_tuning()


def test_graph_follows_schedule_knobs_and_reprepare(ctx, monkeypatch):
    # a captured graph holds the plan's sizes by value: a new schedule or knob must be captured
    # anew (results equal to the eager run with that schedule), and a new inca_prepare of the
    # same input gives tables of the same shape, which the graph keeps serving
    ctx.grid_scan(*SCAN)
    ref = ctx.eval(mode=1, tol=1e-8)
    ctx.eval_graph(mode=1, tol=1e-8)
    np.testing.assert_array_equal(ctx.eval_graph(mode=1, tol=1e-8), ref)
    try:
        # a new schedule, then a new tile shape (the sorted grid is rebuilt with 160-point tiles)
        for tune in ((4, 32, 0.7, 0.1), (24, 16, 0.7, 0.1, 16, 4, 5)):
            ctx.set_tuning(*tune)
            eager = ctx.eval(mode=1, tol=1e-8)
            for _ in range(2):
                np.testing.assert_array_equal(ctx.eval_graph(mode=1, tol=1e-8), eager)
    finally:
        ctx.set_tuning()
    monkeypatch.setenv("INCA_DROP_FRACTION", "0")
    eager = ctx.eval(mode=1, tol=1e-8)
    for _ in range(2):
        np.testing.assert_array_equal(ctx.eval_graph(mode=1, tol=1e-8), eager)
    monkeypatch.delenv("INCA_DROP_FRACTION")
    np.testing.assert_array_equal(ctx.eval_graph(mode=1, tol=1e-8), ref)
    ctx.prepare(THRESH)
    for _ in range(2):
        np.testing.assert_array_equal(ctx.eval_graph(mode=1, tol=1e-8), ref)
