"""Wave planning of batches larger than the device (inca_parallel_gb300/batch_waves.py), CPU part:
record counts of the closed-shell generator's conventions and the grouping rules."""
from inca_parallel_gb300 import batch_waves as BW


def test_record_counts():
    # CH4's 27 primitives: 378 pairs, 378^2 = 142 884 .dm2p records (the reference fixture's count)
    assert BW.records(27, unique=False) == 142884
    assert BW.records(27, unique=True) == 378 * 379 // 2
    assert BW.records(300, unique=True) == 1019283825  # the 20-atom, 300-primitive molecule


def test_plan_respects_budget_and_order():
    nprims = [20, 300, 40, 60, 250, 25, 30]
    budget = 5e8
    waves = BW.plan_waves(nprims, budget)
    assert [i for w in waves for i in w] == list(range(len(nprims)))
    for w in waves:
        tot = sum(BW.records(nprims[i]) for i in w)
        assert tot <= budget or len(w) == 1  # only a molecule above the budget stands alone
    assert [1] in waves  # 300 primitives: 1.0e9 records, a wave of its own
    assert BW.plan_waves(nprims, 1e12) == [list(range(len(nprims)))]
    assert BW.plan_waves([], 1e9) == []
