"""Host-side logic of the ctypes binding that needs no GPU: a pipelined
call's host arrays stay referenced until the call has surely completed --
PIPELINE_SLOTS tickets later, when the library's ring has reused its slot
(and so waited for it) -- or until it is waited for."""
import types

from jif3d_gb300 import capi


def test_pipelined_arrays_held_for_the_ring_depth():
    held = types.SimpleNamespace(_inflight={}, PIPELINE_SLOTS=capi.Context.PIPELINE_SLOTS)
    assert held.PIPELINE_SLOTS == 4  # the ring of j3g_batched_*_async (jif3d_gb300.h)
    for t in range(10):
        capi.Context._hold(held, t, ("arrays of", t))
        # every call of the last PIPELINE_SLOTS tickets may still be in flight
        live = sorted(held._inflight)
        assert live == list(range(max(0, t - held.PIPELINE_SLOTS + 1), t + 1)), (t, live)
