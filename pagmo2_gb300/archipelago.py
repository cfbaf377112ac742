"""Migration epochs of an archipelago on the GPU.

In pagmo every island's algorithm calls its bfe on its own schedule
(src/archipelago.cpp:325-330 -> src/island.cpp:428-655 -> src/bfe.cpp:91-110).
Here the batches all islands submit for one epoch are evaluated together:

    ep = Epoch([(kind, param, n_rows, grad), ...])   # plan once per shape list
    ep.run(batches)            # list of dvs arrays -> list of (fvs, grads)
    ep.submit(batches); ep.collect()   # two epochs in flight (double buffering)

`Collector` is the host-side rendezvous for island threads: each island calls
`collector.evaluate(island, dvs)` from its own thread; when every island of the
epoch has submitted (or the deadline passes, then with the islands that did),
one fused evaluation runs and every caller gets its own results back.
"""
from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np

from . import _native as N
from .workloads import nx_of


class Epoch:
    """A planned epoch over fixed request shapes (libpgx pgx_epoch_*)."""

    def __init__(self, shapes, ctx: N.Context | None = None):
        self.ctx = ctx or N.default_context()
        self.shapes = [(int(k), int(p), int(n), bool(g)) for k, p, n, g in shapes]
        reqs = (N.pgx_request * len(self.shapes))()
        self._dummy = np.zeros(1)
        for i, (k, p, n, g) in enumerate(self.shapes):
            reqs[i].kind, reqs[i].param, reqs[i].n_dvs = k, p, n
            reqs[i].dvs = self._dummy.ctypes.data
            reqs[i].fvs = self._dummy.ctypes.data
            reqs[i].grads = self._dummy.ctypes.data if g else None
        h = C.c_void_p()
        N.check(N.lib().pgx_epoch_create(self.ctx.handle, reqs, len(self.shapes), C.byref(h)))
        self.handle = h
        self._keep = [None, None]  # buffers of in-flight epochs
        self._slot = 0
        self._fifo = []

    def _requests(self, batches, outs):
        reqs = (N.pgx_request * len(self.shapes))()
        keep = []
        for i, ((k, p, n, g), x) in enumerate(zip(self.shapes, batches)):
            x = np.ascontiguousarray(x, dtype=np.float64).reshape(n, nx_of(k, p))
            f, gr = outs[i]
            keep += [x, f, gr]
            reqs[i].kind, reqs[i].param, reqs[i].n_dvs = k, p, n
            reqs[i].dvs = x.ctypes.data
            reqs[i].fvs = f.ctypes.data
            reqs[i].grads = gr.ctypes.data if gr is not None else None
        return reqs, keep

    def outputs(self):
        """Fresh output buffers [(fvs, grads or None), ...] for this plan."""
        return [(np.empty(n), np.empty((n, nx_of(k, p))) if g else None) for k, p, n, g in self.shapes]

    def run(self, batches, outs=None):
        """Evaluates one epoch; `outs` (from outputs()) is filled if given."""
        outs = outs if outs is not None else self.outputs()
        reqs, keep = self._requests(batches, outs)
        N.check(N.lib().pgx_epoch_run(self.handle, reqs))
        return outs

    def submit(self, batches, outs=None):
        outs = outs if outs is not None else self.outputs()
        reqs, keep = self._requests(batches, outs)
        N.check(N.lib().pgx_epoch_submit(self.handle, reqs))
        self._fifo.append((keep, outs))
        return outs

    def collect(self):
        N.check(N.lib().pgx_epoch_collect(self.handle))
        _, outs = self._fifo.pop(0)
        return outs

    def info(self, i):
        lanes = C.c_int()
        tiles = C.c_uint64()
        N.check(N.lib().pgx_epoch_info(self.handle, i, C.byref(lanes), C.byref(tiles)))
        return lanes.value, tiles.value

    def launch_device(self, stream=None):
        N.check(N.lib().pgx_epoch_launch_device(self.handle, stream))

    def close(self):
        if self.handle:
            N.lib().pgx_epoch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_plain(shapes, batches, ctx: N.Context | None = None, outs=None):
    """The island-by-island baseline: one host-buffer batch call per request."""
    ctx = ctx or N.default_context()
    reqs = (N.pgx_request * len(shapes))()
    if outs is None:
        outs = [(np.empty(n), np.empty((n, nx_of(k, p))) if g else None) for k, p, n, g in shapes]
    keep = []
    for i, ((k, p, n, g), x) in enumerate(zip(shapes, batches)):
        x = np.ascontiguousarray(x, dtype=np.float64)
        f, gr = outs[i]
        keep.append(x)
        reqs[i].kind, reqs[i].param, reqs[i].n_dvs = k, p, n
        reqs[i].dvs, reqs[i].fvs = x.ctypes.data, f.ctypes.data
        reqs[i].grads = gr.ctypes.data if gr is not None else None
    N.check(N.lib().pgx_requests_run_plain(ctx.handle, reqs, len(shapes)))
    return outs


class Collector:
    """Rendezvous of island threads for one fused evaluation per epoch.

    `evaluate(island, dvs)` blocks until the epoch that contains the island's
    request has been evaluated and returns (fvs, grads). An epoch is flushed
    when every expected island has submitted, or when `deadline_s` passes
    after the first submission (then only the islands that submitted are
    evaluated, through a plan of their shapes). An island that raises or never
    comes does not block the others beyond the deadline.
    """

    def __init__(self, shapes, deadline_s: float = 1.0, ctx: N.Context | None = None, grad: bool = True):
        self.shapes = list(shapes)
        self.deadline_s = deadline_s
        self.ctx = ctx or N.default_context()
        self._cv = threading.Condition()
        self._pending: dict[int, np.ndarray] = {}
        self._results: dict[int, tuple] = {}
        self._errors: dict[int, BaseException] = {}
        self._epoch = 0
        self._first = None
        self._plans: dict[tuple, Epoch] = {}
        self.epochs_run = 0

    def _plan(self, islands):
        key = tuple(islands)
        ep = self._plans.get(key)
        if ep is None:
            ep = Epoch([self.shapes[i] for i in islands], self.ctx)
            self._plans[key] = ep
        return ep

    def _flush_locked(self):
        islands = sorted(self._pending)
        batches = [self._pending[i] for i in islands]
        try:
            outs = self._plan(islands).run(batches)
            for i, o in zip(islands, outs):
                self._results[i] = o
        except BaseException as e:  # every caller of this epoch sees the failure
            for i in islands:
                self._errors[i] = e
        self._pending.clear()
        self._first = None
        self._epoch += 1
        self.epochs_run += 1
        self._cv.notify_all()

    def evaluate(self, island: int, dvs):
        with self._cv:
            if island in self._pending:
                raise ValueError(f"island {island} already submitted to this epoch")
            my_epoch = self._epoch
            self._pending[island] = np.ascontiguousarray(dvs, dtype=np.float64)
            if self._first is None:
                self._first = time.monotonic()
            if len(self._pending) == len(self.shapes):
                self._flush_locked()
            while self._epoch == my_epoch:
                remaining = self.deadline_s - (time.monotonic() - self._first)
                if remaining <= 0:
                    self._flush_locked()
                    break
                self._cv.wait(remaining)
            if island in self._errors:
                raise self._errors.pop(island)
            return self._results.pop(island)
