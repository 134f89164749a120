"""The hand-derived TMEM upload plans of tests/tmem_plans.py against the oracle's own load planning
(CPU only): the same RDRAM, loaded once through RDP command words and once through the plans, must
leave identical TMEM after each group of loads."""
import numpy as np

from oracle import Oracle
from tmem_plans import GROUP_FIRST, GROUP_SECOND, TEXTURE_BYTES, commands, plan


def _rdram(size=8 << 20):
    rd = np.zeros(size, np.uint8)
    lo, hi = TEXTURE_BYTES
    rd[lo:hi] = np.random.default_rng(1234).integers(0, 256, hi - lo, dtype=np.uint8)
    return rd


def test_hand_plans_match_the_oracles_planning():
    rd = _rdram()
    by_cmd, by_plan = Oracle(8 << 20), Oracle(8 << 20)
    try:
        by_cmd.write_rdram(rd)
        by_plan.write_rdram(rd)
        for group in (GROUP_FIRST, GROUP_SECOND):
            by_cmd.enqueue(np.array(sum((commands(l) for l in group), []), np.uint32))
            plans = np.concatenate([plan(l) for l in group])
            by_plan.L.oracle_apply_upload_plans(by_plan.h, plans.ctypes.data, len(group))
            a, b = by_cmd.tmem(), by_plan.tmem()
            assert np.array_equal(a, b), "TMEM differs in %d words" % int((a != b).sum())
            assert np.count_nonzero(a) > 1000  # the loads wrote real data
        modes = {int(plan(l)["mode"][0]) for l in GROUP_FIRST + GROUP_SECOND}
        assert modes == {0, 1, 2}
    finally:
        by_cmd.close()
        by_plan.close()
