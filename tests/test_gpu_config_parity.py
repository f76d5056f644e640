"""Parity at the full sizes of the synthetic workloads, against the CPU oracle on sampled points.

The oracle generates the same closed-shell DM2 records as the device generator (same enumeration
and arithmetic, so the same screening) in batches and never stores the list
(oracle_lib.intracule_closed_shell), so lists of 1e9 records can be checked.

(a) The 12-atom ring (198 primitives, l <= 2, exponents log-uniform in [0.1, 5000], 21 occupied
    orbitals, symmetry-unique DM2: 194 074 551 records), thresh 1e-12:
    * quartet counts identical to the oracle's;
    * the FP64 form at 200 points of the full multicentre grid (19 centres x 75 x 302, nosym)
      within 1e-11 relative (+ 1e-12 of max|I|) of the oracle: summation order only;
    * the mixed form at the same 200 points (explicit points: tolerance 1e-10 per point) within
      1e-10 relative (+ 1e-12 of max|I| for the oracle's own rounding);
    * the mixed radial integral at 1e-10 against the FP64 form on a reduced grid of the same
      records (every centre, nrad 12, nang 14): the FP64 form over the full grid would take
      about 20 minutes.
(b) The 20-atom molecule of the vector cube (300 primitives, exponents up to 200, 60 occupied
    orbitals, symmetry-unique DM2: 1 019 283 825 records): the separable mixed form on the
    central 16^3 sub-lattice (0.1 bohr) within 1e-8 of max|I| (its max-norm tolerance, + 1e-12
    for FP64 rounding) of the oracle at 32 lattice points, and the FP64 form at those points
    within 1e-11 relative.
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


def test_ring_full_size(ctx):
    from inca_parallel_gb300 import centercalc, workloads as W
    b, D = W.ring_workload()
    assert len(b["alpha"]) == 198 and int(b["tmn"].sum(1).max()) == 2
    ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
    assert ctx.gen_closed_shell_dm2(D, unique=True) == 194074551
    counts = ctx.prepare(THRESH)
    cent, Ps, alf = centercalc(b["an"], b["cartes"])
    assert len(Ps) == 19
    ctx.grid_radial([75] * len(Ps), [302] * len(Ps), alf, cent, Ps, nosym=True)
    g = ctx.grid_copy()
    pts = g["r"][np.linspace(0, len(g["r"]) - 1, 200).astype(np.int64)]
    Io, oc = O.intracule_closed_shell(b, D, THRESH, pts, unique=True)
    assert list(counts) == oc.tolist()
    scale = np.abs(Io).max()
    ctx.grid_points(pts)
    I64 = ctx.eval(mode=0)
    np.testing.assert_allclose(I64, Io, rtol=1e-11, atol=1e-12 * scale)
    Imx = ctx.eval(mode=1, tol=1e-10)
    np.testing.assert_allclose(Imx, Io, rtol=1e-10, atol=1e-12 * scale)
    # radial integral at 1e-10 against the FP64 form on a reduced grid of the same records
    ctx.grid_radial([12] * len(Ps), [14] * len(Ps), alf, cent, Ps, nosym=True)
    assert ctx.ngrid >= 2048  # the one-pass mixed form
    ctx.eval(mode=0, copy=False)
    r64 = ctx.radial_integral()[0]
    ctx.eval(mode=1, tol=1e-10, copy=False)
    rmx = ctx.radial_integral()[0]
    assert abs(rmx - r64) <= 1e-10 * abs(r64), (rmx, r64)


def test_cube_molecule_central_lattice(ctx):
    from inca_parallel_gb300 import workloads as W
    b, D = W.cube_workload()
    ctx.set_primitives(b["alpha"], b["tmn"], b["xyz"])
    assert ctx.gen_closed_shell_dm2(D, unique=True) == 1019283825
    counts = ctx.prepare(THRESH)
    ng = ctx.grid_cube([0.0, 0.0, 0.0], [0.1, 0.1, 0.1], [16, 16, 16])
    assert ng == 16 ** 3
    lattice = ctx.grid_copy(weights=False)["r"]
    Imx = ctx.eval(mode=1, tol=1e-8)
    idx = np.random.default_rng(20261207).choice(ng, 32, replace=False)
    pts = lattice[idx]
    Io, oc = O.intracule_closed_shell(b, D, THRESH, pts, unique=True)
    assert list(counts) == oc.tolist()
    scale = np.abs(Imx).max()
    assert np.abs(Imx[idx] - Io).max() <= (1e-8 + 1e-12) * scale
    ctx.grid_points(pts)
    I64 = ctx.eval(mode=0)
    np.testing.assert_allclose(I64, Io, rtol=1e-11, atol=1e-12 * scale)
