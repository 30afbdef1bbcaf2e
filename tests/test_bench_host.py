"""Host-side logic of bench.py that needs no GPU: how an autotuned V-cycle
schedule is applied to a solver (the point smoother's sweep tile, the line
smoother's coarse-level schedule)."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


class _Solver:
    """Records the calls a schedule makes on a projection handle."""

    def __init__(self):
        self.calls = []

    def set_schedule(self, *a):
        self.calls.append(("schedule", a))

    def set_tile(self, t):
        self.calls.append(("tile", t))

    def set_coarse_sweeps(self, *a):
        self.calls.append(("coarse", a))


def _apply(schedule):
    import bench
    s = _Solver()
    bench.apply_schedule(s, schedule)
    return s.calls


def test_point_smoother_schedule_sets_the_tile():
    from simcoflow_gb300 import batch as Bt
    for name, code in Bt.TILES.items():
        assert _apply((2, 2, 1.9, name)) == [("schedule", (2, 2, 1.9)), ("tile", code),
                                             ("coarse", (0, 0))]
        assert _apply((2, 2, 1.9, name, (1, 4))) == [("schedule", (2, 2, 1.9)), ("tile", code),
                                                     ("coarse", (1, 4))]
        assert _apply([2, 2, 1.9, name, None])[-1] == ("coarse", (0, 0))


def test_line_smoother_schedule_sets_the_coarse_levels():
    assert _apply((2, 2, 1.97, (2, 4))) == [("schedule", (2, 2, 1.97)), ("coarse", (2, 4))]
    # as it comes back from JSON
    assert _apply([2, 2, 1.97, [1, 6]]) == [("schedule", (2, 2, 1.97)), ("coarse", (1, 6))]


def test_schedule_without_extra_clears_the_coarse_schedule():
    for sch in ((2, 2, 1.9), (2, 2, 1.95, None)):
        assert _apply(sch) == [("schedule", (2, 2, sch[2])), ("coarse", (0, 0))]


def test_every_candidate_is_a_valid_coarse_schedule():
    import bench
    for co in bench.LINE_COARSE + bench.POINT_COARSE:
        assert co is None or (0 <= co[0] <= 64 and 1 <= co[1] <= 8)
