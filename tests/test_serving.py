"""Serving loop host logic: admission under the HBM budget, slots, chunking (no GPU)."""

import pytest

from custom_madi_gb300.serving import Scheduler, poisson_arrivals


def test_fifo_admission_respects_budget_and_slots():
    s = Scheduler(budget_bytes=100, n_slots=2, chunk_walkers=10, launch_walkers=25)
    s.offer(0, 60, 30)
    s.offer(1, 50, 5)          # does not fit next to 0
    s.offer(2, 10, None)       # a fit request; FIFO keeps it behind 1
    assert s.admit() == [0]
    assert s.used == 60
    s.release(0)
    assert s.admit() == [1, 2]
    assert s.used == 60 and len(s.free_slots) == 1


def test_slots_bound_simulations_not_fits():
    s = Scheduler(budget_bytes=1000, n_slots=1, chunk_walkers=10, launch_walkers=10)
    s.offer(0, 1, 5)
    s.offer(1, 1, 5)
    assert s.admit() == [0]          # second simulation waits for the slot
    s.release(0)
    assert s.admit() == [1]


def test_oversized_request_is_rejected():
    s = Scheduler(budget_bytes=10, n_slots=1, chunk_walkers=1, launch_walkers=1)
    with pytest.raises(ValueError, match="budget"):
        s.offer(0, 11, 1)


def test_round_robin_chunks_cover_every_walker_once():
    s = Scheduler(budget_bytes=1000, n_slots=4, chunk_walkers=7, launch_walkers=16)
    for rid, n in enumerate((20, 3, 11)):
        s.offer(rid, 1, n)
    s.admit()
    covered = {0: [], 1: [], 2: []}
    finished = []
    launches = 0
    while s.has_work():
        ch = s.next_launch()
        assert ch and sum(c[3] for c in ch) <= 16
        assert all(c[3] <= 7 for c in ch)
        for rid, slot, base, n in ch:
            assert slot == s.slot_of[rid]
            covered[rid].extend(range(base, base + n))
        finished += s.complete(ch)
        launches += 1
    for rid, n in enumerate((20, 3, 11)):
        assert covered[rid] == list(range(n))
    assert sorted(finished) == [0, 1, 2]
    assert launches >= 3


def test_poisson_arrivals_are_seeded_and_increasing():
    a = poisson_arrivals(50, 50.0, seed=2)
    b = poisson_arrivals(50, 50.0, seed=2)
    assert (a == b).all() and (a[1:] > a[:-1]).all()
    assert 0.5 < a[-1] < 2.0


def test_chunks_stay_tile_aligned():
    s = Scheduler(budget_bytes=1000, n_slots=4, chunk_walkers=300, launch_walkers=700, align=128)
    s.offer(0, 1, 1000)
    s.offer(1, 1, 500)
    s.admit()
    while s.has_work():
        for rid, slot, base, n in s.next_launch():
            assert base % 128 == 0
            total = 1000 if rid == 0 else 500
            assert n % 128 == 0 or base + n == total
        # complete immediately
