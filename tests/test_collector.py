"""Host-side rendezvous of island threads (no GPU): one fused evaluation per
epoch, a deadline when islands are missing, and failures that stay with the
epoch that raised them. The evaluation itself is replaced by a fake plan."""
import threading
import time

import numpy as np
import pytest

from pagmo2_gb300 import archipelago as A


class FakeEpoch:
    calls = []

    def __init__(self, shapes, fail=False):
        self.shapes = shapes
        self.fail = fail

    def run(self, batches):
        FakeEpoch.calls.append(len(batches))
        if self.fail:
            raise RuntimeError("device failure")
        return [(b.sum(axis=1), 2 * b) for b in batches]


def make(shapes, deadline=0.5, fail=False):
    c = A.Collector.__new__(A.Collector)
    c.shapes = shapes
    c.deadline_s = deadline
    c.ctx = None
    c._cv = threading.Condition()
    c._pending, c._results, c._errors = {}, {}, {}
    c._epoch, c._first, c.epochs_run = 0, None, 0
    c._plans = {}
    c._plan = lambda islands: FakeEpoch([shapes[i] for i in islands], fail)
    return c


def run_islands(c, islands, rows=4, nx=3, skip=(), raise_in=()):
    out, errs = {}, {}

    def body(i):
        try:
            if i in raise_in:
                raise ValueError("island algorithm failed before evaluating")
            x = np.full((rows, nx), float(i))
            out[i] = c.evaluate(i, x)
        except BaseException as e:
            errs[i] = e

    ts = [threading.Thread(target=body, args=(i,)) for i in islands if i not in skip]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=10)
    return out, errs


def test_all_islands_one_epoch():
    FakeEpoch.calls.clear()
    shapes = [(1, 3, 4, True)] * 8
    c = make(shapes, deadline=5.0)
    out, errs = run_islands(c, range(8))
    assert not errs and sorted(out) == list(range(8))
    assert FakeEpoch.calls == [8] and c.epochs_run == 1
    for i, (f, g) in out.items():
        assert np.all(f == 3.0 * i) and np.all(g == 2.0 * i)


def test_missing_island_flushes_at_deadline():
    FakeEpoch.calls.clear()
    c = make([(1, 3, 4, True)] * 4, deadline=0.3)
    t0 = time.monotonic()
    out, errs = run_islands(c, range(4), skip=(2,))
    assert time.monotonic() - t0 < 5.0
    assert not errs and sorted(out) == [0, 1, 3]
    assert FakeEpoch.calls == [3]


def test_island_that_raises_does_not_block_others():
    FakeEpoch.calls.clear()
    c = make([(1, 3, 4, True)] * 4, deadline=0.3)
    out, errs = run_islands(c, range(4), raise_in=(1,))
    assert sorted(out) == [0, 2, 3] and isinstance(errs[1], ValueError)


def test_device_failure_reaches_every_caller_of_the_epoch():
    c = make([(1, 3, 4, True)] * 3, deadline=5.0, fail=True)
    out, errs = run_islands(c, range(3))
    assert not out and len(errs) == 3 and all(isinstance(e, RuntimeError) for e in errs.values())
    # the next epoch works again
    c._plan = lambda islands: FakeEpoch([c.shapes[i] for i in islands])
    out, errs = run_islands(c, range(3))
    assert not errs and sorted(out) == [0, 1, 2]


def test_double_submission_is_rejected():
    c = make([(1, 3, 4, True)] * 2, deadline=0.2)
    c._pending[0] = np.zeros((4, 3))
    with pytest.raises(ValueError):
        c.evaluate(0, np.zeros((4, 3)))
