"""The block-size search of pct_gb300.batch on the host, against a scripted
stand-in for a Reconstruction: the chosen size is the one with the shortest
time to the residual target, not the fastest iteration."""
import math
import types

from pct_gb300 import batch


class FakeScan:
    """Per block size: seconds per iteration and the residual after each iteration."""

    def __init__(self, curves, block_size, iterations):
        self.curves = curves
        self.cfg = types.SimpleNamespace(block_size=block_size, iterations=iterations)
        self.calls = []

    def set_block_size(self, b):
        self.cfg.block_size = b
        self.calls.append(("size", b))

    def reset_iterate(self):
        self.calls.append(("reset",))

    def drop(self, iterations):
        per_it, res = self.curves[self.cfg.block_size]
        res = list(res[:iterations])
        self.calls.append(("drop", self.cfg.block_size, iterations))
        return types.SimpleNamespace(residual=res, iterations_run=len(res), seconds=per_it * len(res))


CURVES = {
    # block size: (seconds per iteration, residual after iterations 1..6)
    200000: (2.6, [0.9, 0.7, 0.55, 0.45, 0.40, 0.36]),   # the current size: the target is 0.36
    20000: (4.3, [0.6, 0.40, 0.33, 0.30, 0.28, 0.27]),   # reaches 0.36 after 3 iterations: 12.9 s
    50000: (3.2, [0.7, 0.45, 0.35, 0.31, 0.29, 0.28]),   # after 3: 9.6 s (the best)
    400000: (2.5, [0.95, 0.8, 0.7, 0.6, 0.55, 0.5]),     # never reaches it
}


def test_picks_the_shortest_time_to_the_target():
    r = FakeScan(CURVES, 200000, 6)
    best, table = batch.autotune_block_size(r, candidates=(20000, 50000, 400000))
    assert best == 50000
    by_size = {t[0]: t for t in table}
    assert [t[0] for t in table] == [200000, 20000, 50000, 400000]   # the current size first
    assert math.isclose(by_size[50000][3], 3 * 3.2)
    assert math.isclose(by_size[20000][3], 3 * 4.3)
    assert math.isclose(by_size[200000][3], 6 * 2.6)
    assert by_size[400000][3] == math.inf
    # the scan is left with the chosen size and a fresh iterate
    assert r.cfg.block_size == 50000
    assert r.calls[-2:] == [("size", 50000), ("reset",)]
    # every candidate ran the same number of iterations from a fresh iterate
    drops = [c for c in r.calls if c[0] == "drop"]
    assert [c[2] for c in drops] == [6, 6, 6, 6]


def test_explicit_target_and_ties_prefer_the_smaller_block():
    curves = {100: (1.0, [0.5, 0.2]), 300: (1.0, [0.5, 0.2]), 200: (2.0, [0.1, 0.05])}
    r = FakeScan(curves, 300, 2)
    best, table = batch.autotune_block_size(r, candidates=(100, 200), target=0.2)
    # 100 and 300 both reach 0.2 in 2 s, 200 in 2 s too (one iteration of 2 s): a three-way tie
    assert {t[0]: t[3] for t in table} == {300: 2.0, 100: 2.0, 200: 2.0}
    assert best == 100


def test_no_candidate_reaches_the_target():
    curves = {10: (1.0, [0.9, 0.8]), 20: (0.5, [0.95, 0.85])}
    r = FakeScan(curves, 10, 2)
    best, table = batch.autotune_block_size(r, candidates=(20,), target=0.1)
    assert all(t[3] == math.inf for t in table)
    assert best == 10   # all infinite: the smallest block size
