"""flow.OutputWriter's host logic against a fake context and job (no GPU):
outputs are consumed in submission order on the writer thread, at most
`slots` are outstanding, every ticket is released, and a failure in a wait
or in the consumer comes back from close()."""
import threading
import time

import numpy as np
import pytest

import flow
import fvc


class FakeCtx:
    def __init__(self, fail_ticket=None):
        self.lock = threading.Lock()
        self.held = set()
        self.max_held = 0
        self.released = []
        self.next = 0
        self.fail_ticket = fail_ticket

    def begin(self):
        with self.lock:
            t = self.next
            self.next += 1
            self.held.add(t)
            self.max_held = max(self.max_held, len(self.held))
            return t

    def output_wait(self, t):
        time.sleep(0.002)  # the copy in flight
        if t == self.fail_ticket:
            raise fvc.FvcError(fvc.FVC_ERR_WALK, "a queued advance failed")
        return np.full((3, 3), float(t))

    def output_release(self, t):
        with self.lock:
            self.held.discard(t)
            self.released.append(t)


class FakeJob:
    def __init__(self, ctx):
        self.ctx = ctx

    def output_begin(self, always=0):
        return self.ctx.begin()


def test_outputs_in_order_within_the_slots():
    ctx = FakeCtx()
    got = []
    w = flow.OutputWriter(ctx, lambda i, a: got.append((i, float(a[0, 0]))), slots=3)
    for k in range(20):
        w.submit(k, FakeJob(ctx))
    w.close()
    assert got == [(k, float(k)) for k in range(20)]
    assert ctx.max_held <= 3 and not ctx.held and sorted(ctx.released) == list(range(20))


def test_failures_come_back_from_close():
    ctx = FakeCtx(fail_ticket=4)
    got = []
    w = flow.OutputWriter(ctx, lambda i, a: got.append(i), slots=2)
    for k in range(8):
        w.submit(k, FakeJob(ctx))
    with pytest.raises(fvc.FvcError) as e:
        w.close()
    assert e.value.status == fvc.FVC_ERR_WALK
    assert got == [0, 1, 2, 3]  # nothing consumed after the failure
    assert not ctx.held  # every ticket released all the same

    ctx = FakeCtx()
    w = flow.OutputWriter(ctx, lambda i, a: 1 / 0, slots=2)
    for k in range(3):
        w.submit(k, FakeJob(ctx))
    with pytest.raises(ZeroDivisionError):
        w.close()
    assert not ctx.held
