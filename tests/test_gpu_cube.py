"""Separable evaluation of cube lattices (INCA_MIXED on a cube grid, csrc/cube_eval.cu) against
the FP64 GPU form and the oracle.

The separable form evaluates every term in double-float (~2^-44 relative). Without dropping
(INCA_DROP_FRACTION=0) it is held to 1e-12 of max|I| against the FP64 form (itself 1e-12 from
the oracle in test_gpu_parity.py). With the default dropping it leaves out records whose bound
over a tile is below 0.05 tol max|I| / N (max|I| from a coarse pre-pass on lattices of 16 points
per axis or more), so it is held to tol max|I|. The general mixed form on the same cube
(INCA_CUBE_SEPARABLE=0) meets its own 1e-8. Cases: the reference's CH4 cube (20^3, 0.1 bohr,
tests/refs/ch4_ref.cube), lattices whose sizes are not multiples of the 8 x 8 x 16 tile, a single
point, negative steps, and d shells (L_d up to 8, A' beyond the FP32 range: the exact power-of-two
scale is split over the three factors).
"""
import numpy as np
import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu

THRESH = 1e-12


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


@pytest.fixture
def exact(monkeypatch):
    monkeypatch.setenv("INCA_DROP_FRACTION", "0")


def _both(ctx, tol=1e-8):
    I64 = ctx.eval(mode=0)
    Is = ctx.eval(mode=1, tol=tol)
    return I64, Is


def test_reference_cube(ctx, exact):
    ctx.grid_cube([0, 0, 0], [0.1, 0.1, 0.1], [20, 20, 20])
    I64, Is = _both(ctx)
    ref, _ = O.ref_cube()
    scale = np.abs(ref).max()
    assert np.abs(Is - ref).max() <= 1e-12 * scale
    assert np.abs(Is - I64).max() <= 1e-12 * scale
    st = ctx.stats()
    assert st["precise_pairs"] > 0 and st["fp32_pairs"] == 0 and st["corrected_terms"] == 0


@pytest.mark.parametrize("center,step,npts", [
    ([0.1, -0.2, 0.3], [0.1, 0.2, 0.15], [7, 6, 5]),
    ([0.0, 0.0, 0.0], [0.15, 0.15, 0.15], [33, 17, 40]),
    ([0.5, 0.0, -0.5], [-0.2, 0.25, -0.1], [9, 10, 11]),
    ([0.3, 0.2, 0.1], [0.1, 0.1, 0.1], [1, 1, 1]),
])
def test_ragged_lattices(ctx, exact, center, step, npts):
    ctx.grid_cube(center, step, npts)
    I64, Is = _both(ctx)
    assert Is.shape == I64.shape == (int(np.prod(npts)),)
    scale = np.abs(I64).max()
    assert np.abs(Is - I64).max() <= 1e-12 * scale


@pytest.mark.parametrize("tol", [1e-6, 1e-8, 1e-10])
def test_budgeted_dropping(ctx, monkeypatch, tol):
    # 40^3 at 0.25 bohr reaches 5 bohr: the outer tiles leave out most records at loose tolerances
    ctx.grid_cube([0, 0, 0], [0.25, 0.25, 0.25], [40, 40, 40])
    I64 = ctx.eval(mode=0)
    Is = ctx.eval(mode=1, tol=tol)
    skipped = ctx.stats()["skipped_pairs"]
    scale = np.abs(I64).max()
    assert np.abs(Is - I64).max() <= tol * scale
    monkeypatch.setenv("INCA_DROP_FRACTION", "0")
    ctx.eval(mode=1, tol=tol)
    assert ctx.stats()["skipped_pairs"] < skipped


def test_matches_general_mixed_form(ctx, monkeypatch):
    ctx.grid_cube([0, 0, 0], [0.15, 0.15, 0.15], [32, 32, 32])
    I64, Is = _both(ctx)
    monkeypatch.setenv("INCA_CUBE_SEPARABLE", "0")
    Ig = ctx.eval(mode=1, tol=1e-8)
    assert ctx.stats()["fp32_pairs"] > 0  # the general form ran
    scale = np.abs(I64).max()
    assert np.abs(Ig - I64).max() <= 1e-8 * scale
    assert np.abs(Is - I64).max() <= 1e-8 * scale


def test_reproducible_and_graph_entry(ctx):
    ctx.grid_cube([0.2, 0.1, 0.0], [0.12, 0.12, 0.12], [24, 24, 24])
    a = ctx.eval(mode=1, tol=1e-8)
    b = ctx.eval(mode=1, tol=1e-8)
    c = ctx.eval_graph(mode=1, tol=1e-8)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)


def test_d_shells(exact):
    from inca_parallel_gb300 import Context, workloads as W
    b = W.ring_molecule(nprim_target=60)
    D, _ = W.closed_shell_density(b, 6, 7)
    with Context(0) as ctx:
        ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
        ctx.gen_closed_shell_dm2(D, unique=True)
        ctx.prepare(THRESH)
        assert int(ctx.records()["L"].max()) >= 6
        ctx.grid_cube([0.0, 0.0, 0.0], [0.3, 0.3, 0.3], [20, 18, 16])
        I64, Is = _both(ctx)
        assert not np.isnan(Is).any()
        scale = np.abs(I64).max()
        assert np.abs(Is - I64).max() <= 1e-12 * scale


def test_fp64_screened_on_a_lattice_is_the_fp64_form(ch4):
    # cube lattices have no drop thresholds of the one-pass form: the screened mode runs as FP64
    from inca_parallel_gb300 import INCA_FP64_SCREENED, Context
    with Context(0) as ctx:
        ctx.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
        ctx.set_quartets(ch4["ijkl"], ch4["v"])
        ctx.prepare(1e-12)
        ctx.grid_cube([0, 0, 0], [0.2, 0.2, 0.2], [10, 10, 10])
        np.testing.assert_array_equal(ctx.eval(mode=INCA_FP64_SCREENED, tol=1e-8), ctx.eval(mode=0))
