"""Point sharding through the product path: two gloo ranks, each with its own Context on the
one visible GPU (independent evaluations; nothing on the device waits on the other rank).

* sharded_scan_plot: each rank builds and evaluates its own whole shells of the scan (mixed
  form, 1e-8 per I(s); FP64 form) and the shells are gathered in order: I(s) within 1e-8
  (mixed) and 1e-13 (FP64, summation order only) of the single-process FP64 result.
* sharded_ivec with context_evaluator (explicit points, FP64): within 1e-13 of single-process.
"""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THRESH = 1e-12
SCAN = (0.0, 5.0, 0.05, 110)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle_lib as O
        from inca_parallel_gb300 import INCA_FP64, INCA_MIXED, Context, sharding as SH
        s = O.ch4()
        with Context(0) as ctx:
            ctx.set_primitives(s["alpha"], s["tmn"], s["xyz"])
            ctx.set_quartets(s["ijkl"], s["v"])
            ctx.prepare(THRESH)
            start, end, step, nang = SCAN
            mixed = SH.sharded_scan_plot(ctx, start, end, step, nang, INCA_MIXED, tol=1e-8)
            fp64 = SH.sharded_scan_plot(ctx, start, end, step, nang, INCA_FP64)
            pts = np.random.default_rng(5).uniform(-2.0, 2.0, size=(41, 3))
            iv = SH.sharded_ivec(SH.context_evaluator(ctx, INCA_FP64), pts)
        if rank == 0:
            np.savez(os.path.join(out_dir, "sharded.npz"), mixed=mixed, fp64=fp64, iv=iv, pts=pts)
    finally:
        dist.destroy_process_group()


def test_sharded_scan_and_points_on_gpu(tmp_path, ch4):
    from inca_parallel_gb300 import build
    build.build()
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, start_method="spawn")
    got = np.load(tmp_path / "sharded.npz")
    from inca_parallel_gb300 import INCA_FP64, Context
    with Context(0) as ctx:
        ctx.set_primitives(ch4["alpha"], ch4["tmn"], ch4["xyz"])
        ctx.set_quartets(ch4["ijkl"], ch4["v"])
        ctx.prepare(THRESH)
        start, end, step, nang = SCAN
        nr, _ = ctx.grid_scan([start], [end], [step], [nang])
        ctx.eval(mode=INCA_FP64, copy=False)
        ref = ctx.radial_plot()[1]
        ctx.grid_points(got["pts"])
        ref_iv = ctx.eval(mode=INCA_FP64)
    assert len(got["fp64"]) == nr
    np.testing.assert_allclose(got["fp64"], ref, rtol=1e-13, atol=0)
    assert np.max(np.abs(got["mixed"] - ref) / np.abs(ref)) <= 1e-8
    np.testing.assert_allclose(got["iv"], ref_iv, rtol=1e-13, atol=0)
