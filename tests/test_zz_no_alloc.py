"""inca_eval_records_noalloc: FP64 evaluation from caller-owned device buffers, no allocation.

Called through the C ABI (ctypes) twice in a row and compared with inca_eval(INCA_FP64) on
the same records and points. Tolerance: 1e-12 of max|I| (the FP64-form tolerance of the
vector-cube parity test; only the summation order differs); the two calls agree bit for bit.
This file sorts last so that it also runs after every other test in the same process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THRESH = 1e-12
INCA_OK, INCA_E_ARG, INCA_E_LIMIT = 0, 1, 7
MAX_POINTS = 1 << 21


@pytest.fixture(scope="module")
def env():
    from inca_parallel_gb300 import build
    build.build()
    import torch
    from inca_parallel_gb300 import Context, _lib
    torch.cuda.init()
    ctx = Context(0)
    yield ctx, _lib.load(), torch
    ctx.close()


def _noalloc(lib, torch, rec, pts, out):
    dev = {k: torch.from_numpy(np.ascontiguousarray(rec[k])).cuda() for k in ("A", "sqe", "d", "L", "C")}
    r = torch.from_numpy(np.ascontiguousarray(pts, dtype=np.float64)).cuda()
    stream = torch.cuda.current_stream()
    st = lib.inca_eval_records_noalloc(
        len(rec["A"]), dev["A"].data_ptr(), dev["sqe"].data_ptr(), dev["d"].data_ptr(),
        dev["L"].data_ptr(), dev["C"].data_ptr(), len(pts), r.data_ptr(), out.data_ptr(),
        ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return st


def _check_twice(ctx, lib, torch, rec, pts):
    ctx.grid_points(pts)
    ref = ctx.eval(mode=0)
    outs = []
    for _ in range(2):
        out = torch.full((len(pts),), float("nan"), dtype=torch.float64, device="cuda")
        assert _noalloc(lib, torch, rec, pts, out) == INCA_OK
        outs.append(out.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(outs[0] - ref).max() <= 1e-12 * scale


def test_noalloc_matches_inca_eval_cube(env, ch4):
    ctx, lib, torch = env
    ctx.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
    ctx.set_quartets(ch4["ijkl"], ch4["v"])
    assert ctx.prepare(THRESH)[2] == 111080
    rec = ctx.records()
    ax = np.arange(-10, 10) * 0.1
    pts = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    pts = np.vstack([np.zeros((1, 3)), pts])
    _check_twice(ctx, lib, torch, rec, pts)


def test_noalloc_at_maximum_size(env, ch4):
    ctx, lib, torch = env
    ctx.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
    ctx.set_quartets(ch4["ijkl"][:3000], ch4["v"][:3000])
    ctx.prepare(THRESH)
    rec = ctx.records()
    pts = np.random.default_rng(11).uniform(-3.0, 3.0, size=(MAX_POINTS, 3))
    _check_twice(ctx, lib, torch, rec, pts)


def test_noalloc_limits_and_empty(env):
    ctx, lib, torch = env
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    pts = torch.zeros(12, dtype=torch.float64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    null = ctypes.c_void_p(0)
    # beyond the maximum: rejected before anything is queued
    assert lib.inca_eval_records_noalloc(0, null, null, null, null, null, MAX_POINTS + 1,
                                         pts.data_ptr(), out.data_ptr(), s) == INCA_E_LIMIT
    assert lib.inca_eval_records_noalloc(-1, null, null, null, null, null, 4,
                                         pts.data_ptr(), out.data_ptr(), s) == INCA_E_ARG
    assert lib.inca_eval_records_noalloc(5, null, null, null, null, null, 4,
                                         pts.data_ptr(), out.data_ptr(), s) == INCA_E_ARG
    # no records: the output is all zeros
    assert lib.inca_eval_records_noalloc(0, null, null, null, null, null, 4,
                                         pts.data_ptr(), out.data_ptr(), s) == INCA_OK
    torch.cuda.synchronize()
    assert out.cpu().numpy().tolist() == [0.0] * 4


def test_noalloc_empty_records_on_side_stream(env):
    """nrec == 0 queues one memset of the output on the caller's (non-default) stream."""
    ctx, lib, torch = env
    side = torch.cuda.Stream()
    out = torch.full((1000,), float("nan"), dtype=torch.float64, device="cuda")
    pts = torch.zeros(3000, dtype=torch.float64, device="cuda")
    null = ctypes.c_void_p(0)
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        assert lib.inca_eval_records_noalloc(0, null, null, null, null, null, 1000, pts.data_ptr(),
                                             out.data_ptr(), ctypes.c_void_p(side.cuda_stream)) == INCA_OK
    side.synchronize()
    assert not np.isnan(out.cpu().numpy()).any()
    assert np.all(out.cpu().numpy() == 0.0)
