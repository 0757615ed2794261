"""CPU tests of the binomial checkpoint schedule used by the adjoint (host code only)."""
import math

import pytest

from phasefield_gb300 import build, capi


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.load()


def cost(lib, n, s):
    return lib.ppf_checkpoint_schedule_cost(n, s)


def test_storing_every_state_needs_no_recomputation(lib):
    for n in (1, 2, 7, 50):
        assert cost(lib, n, n) == n


def test_one_slot_recomputes_quadratically(lib):
    for n in (2, 5, 20):
        assert cost(lib, n, 1) == n + n * (n - 1) // 2


def test_more_slots_never_cost_more(lib):
    n = 200
    costs = [cost(lib, n, s) for s in range(1, 40)]
    assert all(a >= b for a, b in zip(costs, costs[1:]))


@pytest.mark.parametrize("n,s", [(500, 32), (1000, 16), (300, 4)])
def test_binomial_bound(lib, n, s):
    # with t the smallest repetition number such that C(s-1+t, t) >= n (s-1 free slots),
    # every step is computed at most t+1 times (once forward, t times in reversal)
    t = 0
    while math.comb(s - 1 + t, t) < n:
        t += 1
    assert cost(lib, n, s) <= (t + 1) * n
