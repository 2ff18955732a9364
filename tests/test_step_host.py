"""Host logic of the one-node step loss (no GPU): the camera content key, the
plans kept per key (reuse, a busy plan skipped, the oldest pending forward taken
over at the limit) and a graph pass's first call at new addresses running its
body directly."""
import numpy as np
import torch

import __graft_entry__

__graft_entry__.load_package()

from ngt_gb300 import step  # noqa: E402


def mats():
    rng = np.random.default_rng(3)
    return [rng.standard_normal(s).astype(np.float32) for s in ((1, 16), (5, 16), (5, 16), (5, 6))]


def test_matrix_key_follows_content():
    M, V, P, F = mats()
    k = step._matrix_key(M, V, P, F)
    assert step._matrix_key(M.copy(), V.copy(), P.copy(), F.copy()) == k
    assert step._matrix_key(torch.as_tensor(M), V, P, F) == k
    assert step._matrix_key(M.tolist(), V, P, F) == k
    V[2, 3] += 1.0  # a camera moved in place: another key, so another step
    k2 = step._matrix_key(M, V, P, F)
    assert k2 != k
    assert step._matrix_key(M, V, P, F) == k2


class _FakeStep:
    made = 0

    def __init__(self):
        _FakeStep.made += 1
        self.n = _FakeStep.made


def test_take_plan_reuse_busy_and_takeover():
    key = ("test_take_plan", object())
    try:
        first = step._take_plan(key, _FakeStep)
        assert step._take_plan(key, _FakeStep) is first  # not busy: reused
        plans = [first]
        first.busy = True
        for g in range(1, step._MAX_PLANS):
            pl = step._take_plan(key, _FakeStep)
            assert pl not in plans
            pl.busy, pl.generation = True, g + 10
            plans.append(pl)
        first.generation = 5  # the oldest pending forward
        taken = step._take_plan(key, _FakeStep)
        assert taken is first and not taken.busy
        assert len(step._PLANS[key]) == step._MAX_PLANS
    finally:
        step._PLANS.pop(key, None)


def test_pass_runs_body_directly_at_new_addresses():
    calls = []
    p = step._Pass()
    p.run(("addresses", 1), lambda: calls.append(1))
    p.run(("addresses", 2), lambda: calls.append(2))
    assert calls == [1, 2] and not p.graphs
    assert list(p.seen) == [("addresses", 1), ("addresses", 2)]
