"""The host-buffer discipline of the pipelined end-to-end loop (bench.py
``pipelined_steps``), on CPU against a stand-in for the pipelined C ABI.

The stand-in keeps the library's rules (include/jif3d_gb300.h, the
j3g_batched_*_async calls): a call reads its input host buffers and writes
its output host buffer at some time until it completes; it completes when it
is waited for or when the ring of four slots is reused four calls later.
Every call queued and every host access of the misfit is checked against the
calls still in flight: no host write to a buffer a call may still read or
write, no host read of a buffer a call may still write, no two calls in
flight writing one buffer or one reading what another writes.
"""
import numpy as np
import pytest

import bench

SLOTS = 4


class Hazard(AssertionError):
    pass


class FakePipeline:
    def __init__(self):
        self.next = 0
        self.live = {}  # ticket -> (reads, writes) of calls in flight
        self.calls = []

    def _check(self, reads, writes, what):
        for t, (r, w) in self.live.items():
            if writes & (r | w) or reads & w:
                raise Hazard(f"{what} overlaps call {t} in flight")

    def _queue(self, kind, reads, writes):
        # the call four tickets back has completed: its slot is reused
        self.live.pop(self.next - SLOTS, None)
        self._check(reads, writes, f"call {self.next} ({kind})")
        t = self.next
        self.next += 1
        self.live[t] = (reads, writes)
        self.calls.append(kind)
        return t

    def batched_forward_async(self, models, out):
        return self._queue("forward", {id(models)}, {id(out)})

    def batched_lqderivative_async(self, models, misfits, out):
        return self._queue("derivative", {id(models), id(misfits)}, {id(out)})

    def batched_wait(self, ticket):
        assert 0 <= ticket < self.next
        self.live.pop(ticket, None)

    def misfit(self, st):
        self._check({id(st["data"])}, set(), "host read of the data")
        self._check(set(), {id(st["mis"])}, "host write of the misfit")


def make_sets(n):
    return [{k: np.zeros(3) for k in ("models", "data", "mis", "grads")} for _ in range(n)]


@pytest.mark.parametrize("nsteps", [1, 2, 3, 4, 7, 20])
def test_bench_loop_keeps_buffers_apart(nsteps):
    """Three sets with the gradient of two steps back waited for (the loop the
    bench times): no hazard, every call waited for at the end, a forward and
    a derivative per step."""
    p = FakePipeline()
    bench.pipelined_steps(p, make_sets(3), nsteps, p.misfit)
    assert not p.live
    assert p.calls.count("forward") == nsteps and p.calls.count("derivative") == nsteps


@pytest.mark.parametrize("nsteps", [1, 3, 20])
def test_one_step_back_with_two_sets_is_safe(nsteps):
    """The earlier order (two sets, the gradient of one step back) is safe too."""
    p = FakePipeline()
    bench.pipelined_steps(p, make_sets(2), nsteps, p.misfit, nsets=2, back=1)
    assert not p.live


def test_two_steps_back_needs_three_sets():
    """With two sets, waiting two steps back lets the misfit of step i + 1
    overwrite what the derivative of step i - 1 may still read; the stand-in
    catches it (the check itself is live)."""
    p = FakePipeline()
    with pytest.raises(Hazard):
        bench.pipelined_steps(p, make_sets(2), 6, p.misfit, nsets=2, back=2)
