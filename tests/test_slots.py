"""Slot bookkeeping of the Python front end (no GPU): allocation of
contiguous runs, reuse of released slots, growth of the engine."""
from s_spi_spring_gb300.phase_retrieval import _Slots


class FakeEngine:
    def __init__(self):
        self.reserved = []

    def reserve(self, cap):
        self.reserved.append(cap)


def test_runs_reuse_and_growth():
    e = FakeEngine()
    s = _Slots(e)
    a = s.alloc(4)
    assert a == 0 and s.cap >= 4 and e.reserved[-1] == s.cap
    b = s.alloc(3)
    assert b == 4 and s.cap >= 7
    for k in (1, 2):
        s.release(k)
    assert s.alloc(2) == 1  # the freed run is reused
    s.release(5)
    s.release(6)
    c = s.alloc(3)  # 5, 6 are free; the run continues into new slots at the end
    assert c == 5 and s.cap >= 8
    taken = set(range(0, 8)) - set(s.free)
    assert taken == set(range(0, 8))
    d = s.alloc(1)
    assert d not in taken and d < s.cap


def test_growth_is_geometric():
    e = FakeEngine()
    s = _Slots(e)
    for _ in range(50):
        s.alloc(1)
    assert len(e.reserved) < 15
    assert sorted(set(range(s.cap)) - set(s.free)) == list(range(50))
