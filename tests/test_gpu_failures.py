"""Failure paths of the product through the C ABI, each followed by a good call on the same
context (the context stays usable).

* .dm2p through inca_load_dm2p (src/mod_intracule.f90:164-195, 229-262): the sequential file
  with 4-byte markers gives the same counts and results as the flat one; 8-byte and zero
  markers fail with INCA_E_FORMAT; an index above nprim fails with INCA_E_FORMAT; an i out of
  range ends the data.
* Primitives: a NaN, zero or negative exponent and a negative Cartesian power fail with
  INCA_E_ARG; a power above 4 (g) fails in inca_prepare with INCA_E_LIMIT.
* Bounded waits: with INCA_TEST_STAGE_TIMEOUT the pass-1 kernels start no staging copy and give
  up each wait after that many tries (no fault, no hang: nothing is in flight, every wait is
  bounded); inca_eval returns INCA_E_TIMEOUT, on the one-pass and the two-pass form, and the next
  evaluation without the knob matches the FP64 form (1e-10 relative on the radial integral).
"""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THRESH = 1e-12


@pytest.fixture(scope="module")
def ctx(ch4):
    from inca_parallel_gb300 import build
    build.build()
    from inca_parallel_gb300 import Context
    c = Context(0)
    c.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
    yield c
    c.close()


def _sequential(raw, marker=24, fmt="<i"):
    m = struct.pack(fmt, marker)
    return b"".join(m + raw[k:k + 24] + m for k in range(0, len(raw) - len(raw) % 24, 24))


def test_load_dm2p_formats(ctx, ch4, tmp_path):
    from inca_parallel_gb300 import IncaError
    flat = tmp_path / "flat.dm2p"
    flat.write_bytes(ch4["raw"])
    seq = tmp_path / "seq.dm2p"
    seq.write_bytes(_sequential(ch4["raw"]))
    pts = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.4, -0.3, 0.9]])
    ctx.grid_points(pts)
    res = []
    for path in (flat, seq):
        assert ctx.load_dm2p(str(path)) == 142884
        assert tuple(ctx.prepare(THRESH)) == (142884, 111248, 111080)
        res.append(ctx.eval(mode=0))
    np.testing.assert_array_equal(res[0], res[1])
    for marker, fmt in ((24, "<q"), (0, "<i")):
        bad = tmp_path / "bad.dm2p"
        bad.write_bytes(_sequential(ch4["raw"][:24 * 100], marker, fmt))
        with pytest.raises(IncaError, match="INCA_E_FORMAT"):
            ctx.load_dm2p(str(bad))
    raw = bytearray(ch4["raw"][:24 * 100])
    raw[24 * 40 + 8:24 * 40 + 12] = struct.pack("<i", 28)  # k above nprim in record 41
    bad = tmp_path / "above.dm2p"
    bad.write_bytes(bytes(raw))
    with pytest.raises(IncaError, match="INCA_E_FORMAT"):
        ctx.load_dm2p(str(bad))
    raw[24 * 40 + 8:24 * 40 + 12] = struct.pack("<i", 1)
    raw[24 * 60:24 * 60 + 4] = struct.pack("<i", 0)  # i out of range in record 61: end of data
    short = tmp_path / "short.dm2p"
    short.write_bytes(bytes(raw))
    assert ctx.load_dm2p(str(short)) == 60
    # the context is still usable
    assert ctx.load_dm2p(str(flat)) == 142884
    ctx.prepare(THRESH)
    np.testing.assert_array_equal(ctx.eval(mode=0), res[0])


def test_bad_primitives(ctx, ch4):
    from inca_parallel_gb300 import IncaError
    for bad in (np.nan, 0.0, -1.0):
        alpha = ch4["alpha"].copy()
        alpha[5] = bad
        with pytest.raises(IncaError, match="INCA_E_ARG"):
            ctx.set_primitives(alpha, ch4["tmn"], ch4["xyz"])
    tmn = ch4["tmn"].copy()
    tmn[3, 1] = -1
    with pytest.raises(IncaError, match="INCA_E_ARG"):
        ctx.set_primitives(ch4["alpha"], tmn, ch4["xyz"])
    tmn[3, 1] = 5  # an h-type power: beyond INCA_MAX_DEGREE for a quartet
    ctx.set_primitives(ch4["alpha"], tmn, ch4["xyz"])
    ctx.set_quartets(ch4["ijkl"], ch4["v"])
    with pytest.raises(IncaError, match="INCA_E_LIMIT"):
        ctx.prepare(THRESH)
    ctx.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
    ctx.set_quartets(ch4["ijkl"], ch4["v"])
    assert tuple(ctx.prepare(THRESH)) == (142884, 111248, 111080)


@pytest.mark.parametrize("grid", ["radial", "points"])
def test_bounded_wait_gives_up(ctx, ch4, monkeypatch, grid):
    from inca_parallel_gb300 import IncaError
    ctx.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
    ctx.set_quartets(ch4["ijkl"], ch4["v"])
    ctx.prepare(THRESH)
    from inca_parallel_gb300 import centercalc
    if grid == "radial":  # 3 050 points: the one-pass form (estimate pass and main pass)
        cent, Ps, alf = centercalc(ch4["an"], ch4["cartes"])
        ctx.grid_radial([50] * len(Ps), [110] * len(Ps), alf, cent, Ps)
        assert ctx.ngrid >= 2048
    else:  # a few points: the two-pass form
        ctx.grid_points(np.array([[0.0, 0.0, 0.0], [0.5, 0.2, -0.1], [1.5, 0.0, 0.0]]))
    ref = ctx.eval(mode=0)
    r64 = ctx.radial_integral()[0] if grid == "radial" else None
    monkeypatch.setenv("INCA_TEST_STAGE_TIMEOUT", "8")
    with pytest.raises(IncaError, match="INCA_E_TIMEOUT"):
        ctx.eval(mode=1, tol=1e-10)
    monkeypatch.delenv("INCA_TEST_STAGE_TIMEOUT")
    got = ctx.eval(mode=1, tol=1e-10)
    if grid == "radial":
        rmx = ctx.radial_integral()[0]
        assert abs(rmx - r64) <= 1e-10 * abs(r64)
    else:
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=0)
