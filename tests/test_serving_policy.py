"""The serving loop's admission policy, without a GPU."""

from __future__ import annotations

import numpy as np
import pytest

from commkit_gb300.serving import Admission, Request


def _req(rid, frames, code="A"):
    return Request(rid, code, 4, np.zeros((frames, 8), np.complex64), 0.1, arrival=rid * 1e-3)


def _fits(cap):
    def fits(batch, r):
        return sum(q.frames for q in batch if q.code == r.code) + r.frames <= cap[r.code]

    return fits


def test_batches_take_fifo_requests_that_fit_a_slot():
    adm = Admission(slots=2)
    for i, (f, c) in enumerate([(3, "A"), (4, "A"), (2, "B"), (5, "A"), (1, "B")]):
        adm.arrive(_req(i, f, c))
    fits = _fits({"A": 8, "B": 8})
    b1 = adm.next_batch(fits)  # 3 + 4 A frames, 2 B frames, then 5 more A frames do not fit
    assert [r.rid for r in b1] == [0, 1, 2] and adm.free == 1
    b2 = adm.next_batch(fits)  # no overtaking: request 3 first
    assert [r.rid for r in b2] == [3, 4] and adm.free == 0
    adm.arrive(_req(5, 1))
    assert adm.next_batch(fits) == []  # no free slot
    adm.release()
    assert [r.rid for r in adm.next_batch(fits)] == [5]


def test_request_larger_than_a_slot_raises():
    adm = Admission(slots=1)
    adm.arrive(_req(0, 50))
    with pytest.raises(MemoryError, match="does not fit"):
        adm.next_batch(_fits({"A": 16}))
