"""Point sharding over ranks (inca_parallel_gb300/sharding.py) on CPU: gloo, world size 2.

The evaluator here is the oracle (one thread, so every point's sum has a fixed order): the
sharded Ivec must equal the single-process one bit for bit; the sharded radial integral and
I(s) differ from the single-process sums only by summation order (1e-14 relative).
"""
import os
import socket

import numpy as np
import pytest

import oracle_lib as O
from inca_parallel_gb300 import sharding as SH

THRESH = 1e-12


def test_shard_bounds_cover_and_balance():
    for n in (0, 1, 7, 62390):
        for world in (1, 2, 3, 8):
            b = [SH.shard_bounds(n, r, world) for r in range(world)]
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[r][1] == b[r + 1][0] for r in range(world - 1))
            sizes = [hi - lo for lo, hi in b]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        SH.shard_bounds(10, 2, 2)


def test_shard_shells_whole_and_contiguous():
    smn = np.array([110] + [61] * 100)
    for world in (1, 2, 3, 5):
        parts = [SH.shard_shells(smn, r, world) for r in range(world)]
        assert parts[0][0] == 0 and parts[-1][1] == len(smn)
        for r in range(world - 1):
            assert parts[r][1] == parts[r + 1][0] and parts[r][3] == parts[r + 1][2]
        loads = [p[3] - p[2] for p in parts]
        assert max(loads) - min(loads) <= 2 * smn.max()
    # more ranks than shells: some ranks own nothing, the cover is still exact
    parts = [SH.shard_shells([5, 5], r, 4) for r in range(4)]
    assert sum(p[1] - p[0] for p in parts) == 2


def test_scan_shard_whole_shells():
    # each rank's share of a scan block is itself a scan block of whole shells; together they
    # cover every shell once, in order, and gridpoints2 counts the same shells in each share
    for start, end, step in ((0.0, 10.0, 0.05), (0.0, 5.0, 0.1), (0.5, 3.0, 0.25)):
        npb = int((end - start) / step) + 1
        for world in (1, 2, 3, 4, 8):
            parts = [SH.scan_shard(start, end, step, r, world) for r in range(world)]
            parts = [p for p in parts if p is not None]
            assert parts[0][2] == 0 and parts[-1][3] == npb
            for a, b in zip(parts, parts[1:]):
                assert a[3] == b[2]
            for s0, s1, k0, k1 in parts:
                g = O.gridpoints2([s0], [s1], [step], [26])
                assert len(g["smn"]) == k1 - k0
                np.testing.assert_allclose(g["radi"], start + step * np.arange(k0, k1), rtol=0, atol=1e-12)
    assert SH.scan_shard(0.0, 0.1, 0.1, 0, 4) is None  # more ranks than shells: rank 0 has none


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
        sys_ = O.ch4()

        def evaluate(points):
            return O.intracule(sys_, THRESH, points, nthreads=1)[0]

        rng = np.random.default_rng(3)
        pts = rng.uniform(-2.0, 2.0, size=(37, 3))
        iv = SH.sharded_ivec(evaluate, pts)
        cent, Ps, alf = O.centercalc(sys_["an"], sys_["cartes"])
        g = O.gridpoints([20], [50], alf, cent, Ps)
        tot, vee = SH.sharded_radial_integral(evaluate, g["r"], g["w"], g["wvee"])
        g2 = O.gridpoints2([0.0], [1.0], [0.25], [26])
        rad = SH.sharded_radial_plot(evaluate, g2["r"], g2["w_ang"], g2["smn"])
        if rank == 0:
            np.savez(os.path.join(out_dir, "sharded.npz"), iv=iv, tot=tot, vee=vee, rad=rad)
    finally:
        dist.destroy_process_group()


def test_sharded_evaluation_matches_single_process(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    got = np.load(tmp_path / "sharded.npz")
    sys_ = O.ch4()
    rng = np.random.default_rng(3)
    pts = rng.uniform(-2.0, 2.0, size=(37, 3))
    ref = O.intracule(sys_, THRESH, pts, nthreads=1)[0]
    np.testing.assert_array_equal(got["iv"], ref)
    cent, Ps, alf = O.centercalc(sys_["an"], sys_["cartes"])
    g = O.gridpoints([20], [50], alf, cent, Ps)
    I = O.intracule(sys_, THRESH, g["r"], nthreads=1)[0]
    assert abs(got["tot"] - np.dot(g["w"], I)) <= 1e-14 * abs(got["tot"])
    assert abs(got["vee"] - np.dot(g["wvee"], I)) <= 1e-14 * abs(got["vee"])
    g2 = O.gridpoints2([0.0], [1.0], [0.25], [26])
    I2 = O.intracule(sys_, THRESH, g2["r"], nthreads=1)[0]
    ref_rad, k = [], 0
    for n in g2["smn"]:
        ref_rad.append(np.dot(g2["w_ang"][k:k + n], I2[k:k + n]))
        k += n
    np.testing.assert_allclose(got["rad"], ref_rad, rtol=1e-14, atol=0)
