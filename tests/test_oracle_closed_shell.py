"""The oracle's closed-shell DM2 path (records generated from a 1-RDM in batches, never stored)
against the oracle's record path on the same records folded on the host.

The generated records follow the library's device generator (inca_gen_closed_shell_dm2): pairs
(i,k) with i <= k in row-major packed order, Gamma summed over the distinct orderings, and for
the symmetry-unique list pair(ik) <= pair(jl) with the off-diagonal pairs doubled. Counts must
be identical and I equal up to summation order (1e-13 of max|I|).
"""
import numpy as np
import pytest

import oracle_lib as O
from inca_parallel_gb300 import workloads as W

THRESH = 1e-12


def _host_records(D, unique):
    n = len(D)
    pairs = [(i, k) for i in range(n) for k in range(i, n)]
    ijkl, v = [], []
    for a, (i, k) in enumerate(pairs):
        for b, (j, l) in enumerate(pairs):
            if unique and b < a:
                continue
            s = 0.0
            for p, q in ([(i, k)] if i == k else [(i, k), (k, i)]):
                for r, t in ([(j, l)] if j == l else [(j, l), (l, j)]):
                    s += D[p, q] * D[r, t] - 0.5 * D[p, t] * D[r, q]
            if unique and a != b:
                s *= 2.0
            ijkl.append((i + 1, j + 1, k + 1, l + 1))
            v.append(s)
    return np.array(ijkl, dtype=np.int32), np.array(v)


@pytest.mark.parametrize("unique", [False, True])
def test_closed_shell_matches_record_path(unique):
    rng = np.random.default_rng(W.SEED0 + 41)
    b = W.random_molecule(rng, 3, 14)
    D, _ = W.closed_shell_density(b, 3, 5)
    ijkl, v = _host_records(D, unique)
    pts = rng.uniform(-2.5, 2.5, size=(40, 3))
    pts[0] = 0.0
    sys_ = {"alpha": b["alpha"], "tmn": b["tmn"], "xyz": b["xyz"], "ijkl": ijkl, "v": v}
    ref, rc = O.intracule(sys_, THRESH, pts)
    got, gc = O.intracule_closed_shell(b, D, THRESH, pts, unique=unique)
    assert gc.tolist() == rc.tolist()
    assert rc[2] > 0
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
