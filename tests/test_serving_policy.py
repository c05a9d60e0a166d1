"""The serving loop's admission policy, without a GPU."""

from __future__ import annotations

import numpy as np
import pytest

from commkit_gb300.serving import Admission, Request


def _req(rid, frames):
    return Request(rid, "A", 4, np.zeros((frames, 8), np.complex64), 0.1, arrival=rid * 1e-3)


def test_admission_respects_budget_order_and_slots():
    adm = Admission(budget=1000, max_inflight=2, batch_overhead=100)
    for i, f in enumerate([3, 4, 3, 5]):
        adm.arrive(_req(i, f))
    cost = lambda r: 100 * r.frames  # noqa: E731
    b1 = adm.next_batch(cost)  # 100 + 300 + 400 = 800; the next (300) would exceed 1000
    assert [r.rid for r in b1] == [0, 1] and adm.in_use == 800 and adm.inflight == 1
    assert adm.next_batch(cost) == []  # 800 + 100 + 300 > 1000: waits for memory
    adm.release(800)
    b2 = adm.next_batch(cost)  # no overtaking: 2 (300) then 3 (500) -> 900
    assert [r.rid for r in b2] == [2, 3] and adm.in_use == 900


def test_admission_limits_batches_in_flight():
    adm = Admission(budget=10**9, max_inflight=1)
    adm.arrive(_req(0, 1))
    adm.arrive(_req(1, 1))
    assert len(adm.next_batch(lambda r: 1)) == 2
    adm.arrive(_req(2, 1))
    assert adm.next_batch(lambda r: 1) == []  # the slot is busy
    adm.release(2)
    assert [r.rid for r in adm.next_batch(lambda r: 1)] == [2]


def test_request_too_large_for_the_budget_raises():
    adm = Admission(budget=100, max_inflight=2, batch_overhead=10)
    adm.arrive(_req(0, 50))
    with pytest.raises(MemoryError, match="budget"):
        adm.next_batch(lambda r: 10 * r.frames)
