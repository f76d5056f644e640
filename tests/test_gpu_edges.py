"""Edge cases of the evaluation forms on the GPU: nothing survives the screening (every form
returns exact zeros, no kernel of the mixed forms runs on an empty record list), no quartets at
all (inca_prepare reports the state error, as the reference stops on an empty .dm2p), and grids of
a single shell at s = 0 (the scan's unit-weight shell)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(ch4):
    from inca_parallel_gb300 import build
    build.build()
    from inca_parallel_gb300 import Context
    c = Context(0)
    c.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
    c.set_quartets(ch4["ijkl"], ch4["v"])
    yield c
    c.close()


def test_nothing_survives(ctx, ch4):
    import oracle_lib as O
    counts = ctx.prepare(1e12)  # a screening limit no quartet reaches
    assert counts[0] == len(ch4["v"]) and counts[2] == 0
    cent, Ps, alf = O.centercalc(ch4["an"], ch4["cartes"])
    grids = [lambda: ctx.grid_radial([30] * len(Ps), [110] * len(Ps), alf, cent, Ps),
             lambda: ctx.grid_scan([0.0], [3.0], [0.1], [302]),
             lambda: ctx.grid_cube([0, 0, 0], [0.2, 0.2, 0.2], [20, 20, 20]),
             lambda: ctx.grid_points(np.zeros((1, 3)))]
    for make in grids:
        make()
        for mode in (0, 1):
            I = ctx.eval(mode=mode, tol=1e-8)
            assert I.shape == (ctx.ngrid,) and not np.any(I)


def test_no_quartets(ctx, ch4):
    from inca_parallel_gb300 import IncaError
    ctx.set_quartets(np.zeros((0, 4), dtype=np.int32), np.zeros(0))
    with pytest.raises(IncaError, match="no quartets"):
        ctx.prepare(1e-12)
    ctx.set_quartets(ch4["ijkl"], ch4["v"])  # restore for the next test


def test_single_shell_at_zero(ctx, ch4):
    ctx.prepare(1e-12)
    nr, ng = ctx.grid_scan([0.0], [0.0], [0.1], [110])
    assert nr == 1 and ng == 110  # s = 0 keeps every Lebedev point, unit weight
    I64 = ctx.eval(mode=0)
    Im = ctx.eval(mode=1, tol=1e-10)
    np.testing.assert_allclose(Im, I64, rtol=1e-10, atol=0)
    np.testing.assert_allclose(I64, I64[0], rtol=1e-14)  # every point is the origin
    assert abs(I64[0] / 2 - ch4["gold"]["intracule_at_zero"]) <= 1e-10 * ch4["gold"]["intracule_at_zero"]
