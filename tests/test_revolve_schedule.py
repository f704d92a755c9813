"""The binomial (revolve) checkpoint schedule of the adjoint, on the host.

The schedule (mj_revolve_schedule, the plan mj_adj_create_revolve executes)
is simulated with integer states: it must visit x_{N-1}, ..., x_1 exactly
once each and in that order, restore only what a slot holds, never use more
than the snapshot budget, and take the fewest forward steps for that budget
(checked against a plain dynamic program written here, and against the known
closed forms: no snapshot besides x_1 costs L(L-1)/2, enough snapshots cost
L-1)."""
import ctypes

import numpy as np
import pytest

from montjoie_gb300 import _lib


def schedule(nsteps, snapshots):
    L = _lib.load()
    n, cost = ctypes.c_int(), ctypes.c_longlong()
    _lib.check(L.mj_revolve_schedule(nsteps, snapshots, 0, None, ctypes.byref(n), ctypes.byref(cost)))
    acts = np.zeros(3 * n.value, dtype=np.int32)
    _lib.check(L.mj_revolve_schedule(nsteps, snapshots, n.value, _lib.iptr(acts), ctypes.byref(n),
                                     ctypes.byref(cost)))
    return acts.reshape(-1, 3), cost.value


def simulate(acts, nsteps, snapshots):
    slots = {0: 1}  # slot -> k of the state it holds
    cur, steps, visits = 1, 0, []
    for kind, k, slot in acts:
        if kind == 0:
            assert slots.get(slot) == k
            cur = k
        elif kind == 1:
            assert k >= cur
            steps += k - cur
            cur = k
        elif kind == 2:
            assert cur == k and 0 <= slot < snapshots
            slots[slot] = k
        else:
            assert cur == k
            visits.append(k)
    return visits, steps


def min_cost(L, S):
    c = np.zeros((L + 1, S + 1), dtype=np.int64)
    c[:, 0] = [l * (l - 1) // 2 for l in range(L + 1)]
    for s in range(1, S + 1):
        for l in range(2, L + 1):
            c[l, s] = min(x + c[l - x, s - 1] + c[x, s] for x in range(1, l))
    return c[L, S]


@pytest.mark.parametrize("nsteps,snapshots", [(2, 1), (3, 1), (10, 1), (10, 3), (40, 4), (81, 9), (100, 100)])
def test_schedule_visits_every_state_once_in_reverse_order(nsteps, snapshots):
    acts, cost = schedule(nsteps, snapshots)
    visits, steps = simulate(acts, nsteps, snapshots)
    assert visits == list(range(nsteps - 1, 0, -1))
    assert steps == cost
    L = nsteps - 1
    assert cost == min_cost(L, min(snapshots, L) - 1)
    if snapshots == 1:
        assert cost == L * (L - 1) // 2
    if snapshots >= L:
        assert cost == L - 1


def test_cost_falls_with_the_budget():
    costs = [schedule(1000, s)[1] for s in (4, 8, 16, 32, 64)]
    assert all(a > b for a, b in zip(costs, costs[1:]))
    assert costs[-1] < 2 * 1000  # 64 snapshots: fewer than two recomputations per step
