"""CPU test of the autotuner's search logic with a fake context (the timed
calls themselves run on the GPU in the batched benchmark)."""
import gasoline_gb300 as g
from gasoline_gb300 import autotune


class FakeCtx:
    def __init__(self):
        self.tuning = None
        self.last = None

    def set_tuning(self, taskSize=0, walkBlocksPerSM=0, walkGroup=0, walkLists=0):
        self.tuning = (taskSize, walkBlocksPerSM, walkGroup, walkLists)

    def grav_all(self, gp):
        self.last = gp.nBucket

    def timings(self):
        ts, wb, wg, wl = self.tuning
        # a made-up cost surface with its minimum at nBucket 16, 4 blocks,
        # task 65536, the two-pass walk without groups
        return {"total": abs(self.last - 16) + abs(wb - 4) + (0 if ts == 65536 else 1)
                + (0 if wg == -1 else 0.5) + (0 if wl == 1 else 0.25) + 1.0}


def test_tune_gravity_picks_the_minimum_and_leaves_it_set():
    c = FakeCtx()
    best, table = autotune.tune_gravity(c, g.grav_params(nBucket=8), reps=1)
    assert len(table) == 3 * 2 * 2 * 3
    assert (best["nBucket"], best["walkBlocksPerSM"], best["taskSize"], best["walkGroup"],
            best["walkLists"]) == (16, 4, 65536, -1, 1)
    assert c.tuning == (65536, 4, -1, 1)
