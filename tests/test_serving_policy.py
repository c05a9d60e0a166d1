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


def test_server_fits_keeps_running_totals():
    """The server's slot test (frames per code, symbols per slot) keeps the
    batch's totals between calls; it must admit exactly what a pass over the
    whole batch admits."""
    from types import SimpleNamespace

    from commkit_gb300.serving import Server

    rng = np.random.default_rng(0)
    fake = SimpleNamespace(caps={"A": 40, "B": 30, "C": 12}, _sym_cap=900, _fit=None)

    def naive(batch, r):
        frames = sum(q.frames for q in batch if q.code == r.code) + r.frames
        syms = sum(q.frames * q.symbols.shape[1] for q in batch) + r.frames * r.symbols.shape[1]
        return frames <= fake.caps[r.code] and syms <= fake._sym_cap

    reqs = [Request(i, "ABC"[rng.integers(3)], 4, np.zeros((int(rng.integers(1, 9)), int(rng.integers(2, 12))),
                                                            np.complex64), 0.1, arrival=i * 1e-3)
            for i in range(400)]  # fmt: skip
    got, want = Admission(slots=1), Admission(slots=1)
    for r in reqs:
        got.arrive(r)
        want.arrive(r)
    while want.pending:
        a = got.next_batch(lambda b, r: Server._fits(fake, b, r))
        b = want.next_batch(naive)
        assert [r.rid for r in a] == [r.rid for r in b]
        got.release()
        want.release()
    assert not got.pending
