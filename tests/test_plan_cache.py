"""The operator layer's plan cache (host logic only, no GPU): identity keying,
least-recently-used order, and the entry and byte limits."""
import torch

from pridediff_gb300.radontorch import _PlanCache


def _plan(nbytes):
    return torch.empty(nbytes, dtype=torch.uint8)


def test_same_tensor_hits_new_tensor_or_write_misses():
    c = _PlanCache(size=4, budget=1 << 20)
    a = torch.arange(8, dtype=torch.float32)
    builds = []
    get = lambda ang: c.get(("k",), ang, lambda: builds.append(1) or _plan(16))   # noqa: E731
    p1 = get(a)
    assert get(a) is p1 and len(builds) == 1
    b = torch.arange(8, dtype=torch.float32)      # equal values, another tensor: rebuilt
    assert get(b) is not p1 and len(builds) == 2
    a.add_(1.0)                                    # in-place write bumps the version: rebuilt
    get(a)
    assert len(builds) == 3


def test_entry_limit_and_lru_order():
    c = _PlanCache(size=2, budget=1 << 30)
    angs = [torch.zeros(3) for _ in range(3)]
    plans = [c.get((i,), angs[i], lambda: _plan(10)) for i in range(2)]
    c.get((0,), angs[0], lambda: _plan(10))        # touch 0: 1 is now least recently used
    c.get((2,), angs[2], lambda: _plan(10))
    keys = [e[0] for e in c.entries]
    assert keys == [(2,), (0,)]
    assert c.get((0,), angs[0], lambda: _plan(10)) is plans[0]


def test_byte_budget_evicts_oldest_but_keeps_newest():
    c = _PlanCache(size=8, budget=100)
    angs = [torch.zeros(2) for _ in range(3)]
    c.get((0,), angs[0], lambda: _plan(60))
    c.get((1,), angs[1], lambda: _plan(30))
    assert c.nbytes() == 90 and len(c.entries) == 2
    c.get((2,), angs[2], lambda: _plan(50))        # 140 > 100: the oldest goes
    assert [e[0] for e in c.entries] == [(2,), (1,)] and c.nbytes() == 80
    c.get((3,), angs[0], lambda: _plan(500))       # larger than the budget alone: kept, others go
    assert [e[0] for e in c.entries] == [(3,)]
    c.clear()
    assert c.nbytes() == 0


def test_tuple_entries_count_the_plan_bytes():
    c = _PlanCache(size=8, budget=1 << 20)
    a = torch.zeros(2)
    src = torch.zeros(4, 2)
    c.get(("3d",), a, lambda: (_plan(40), src))
    assert c.nbytes() == 40
