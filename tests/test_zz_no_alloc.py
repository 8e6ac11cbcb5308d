"""mks_replay_noalloc — the replay entry point that allocates no device memory.

Some callers of this library cannot call cudaMalloc during a run (for
example a host that has already given its device-memory budget to the
lattice, or one that must not grow a stream-ordered memory pool).  This entry
point stages the event trace in a fixed device array owned by the library
instead of allocating a buffer per call.  The tests drive it through the C
ABI and check that, on two calls in a row, it leaves exactly the lattice
that the allocating mks_replay leaves (the state is integer bytes, so the
tolerance is zero) while the device's memory counters stay put, that a trace
longer than the array is refused, and that after an event that does not
apply the shared array serves the next call correctly.
Kept in a file collected last so that a failure here cannot hide others."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MKS_ERR_INVARIANT = 3        # include/mulskips_gpu.h
# cudaMemPoolAttr values of the CUDA runtime (driver_types.h)
ATTR_RESERVED_HIGH, ATTR_USED_CURRENT, ATTR_USED_HIGH = 0x6, 0x7, 0x8


class DeviceMemory:
    """The default memory pool of device 0 and the device's free memory, read
    through the CUDA runtime (the pool is a driver object shared by every
    runtime in the process, the engine's included)."""

    def __init__(self):
        cand = ["libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"]
        self.rt = None
        for c in cand:
            try:
                self.rt = C.CDLL(c)
                break
            except OSError:
                continue
        if self.rt is None:
            pytest.skip("libcudart not found")
        self.pool = C.c_void_p()
        assert self.rt.cudaDeviceGetDefaultMemPool(C.byref(self.pool), 0) == 0

    def attr(self, a):
        v = C.c_uint64()
        assert self.rt.cudaMemPoolGetAttribute(self.pool, a, C.byref(v)) == 0
        return v.value

    def reset_high(self):
        zero = C.c_uint64(0)
        for a in (ATTR_RESERVED_HIGH, ATTR_USED_HIGH):
            assert self.rt.cudaMemPoolSetAttribute(self.pool, a, C.byref(zero)) == 0

    def free(self):
        f, t = C.c_size_t(), C.c_size_t()
        assert self.rt.cudaMemGetInfo(C.byref(f), C.byref(t)) == 0
        return f.value

    def snapshot(self):
        return (self.attr(ATTR_USED_CURRENT), self.attr(ATTR_USED_HIGH), self.attr(ATTR_RESERVED_HIGH), self.free())


def last_error(lib):
    buf = C.create_string_buffer(512)
    lib.mks_last_error(buf, 512)
    return buf.value


def test_noalloc_replay_matches_replay(oracle_lib, engine_lib):
    from mulskips_gb300 import Lattice
    from mulskips_gb300 import _native as N
    start = os.path.join(GOLDEN, "Si-SL", "start.dat")
    o = oracle_lib.Oracle(start, 480, 480, 480)
    o.init()
    pE, pD = o.rates()
    o.trace_enable()
    ref = Lattice(480, 480, 480, sf=0.4525)
    dut = Lattice(480, 480, 480, sf=0.4525)
    mem = DeviceMemory()
    try:
        for lat in (ref, dut):
            lat.set_rates(pE, pD)
            lat.init_flat("S", 360)
        for call in range(2):                      # two calls in a row on the shared array
            o.run(30000)
            tr = np.ascontiguousarray(o.trace(), dtype=N.EVENT_DTYPE)
            assert len(tr) == 30000
            # existing entry point: it allocates its trace buffer from the pool
            mem.reset_high()
            used0 = mem.attr(ATTR_USED_CURRENT)
            ref.replay(tr)
            assert mem.attr(ATTR_USED_HIGH) >= used0 + tr.nbytes, "mks_replay should allocate its trace buffer"
            # the new entry point: no pool growth, no allocation, same free memory
            mem.reset_high()
            before = mem.snapshot()
            N.check(engine_lib.mks_replay_noalloc(dut._h, N.ptr(tr), len(tr)))
            after = mem.snapshot()
            assert after[1] == before[0], f"call {call}: the memory pool saw an allocation"
            assert after == before, f"call {call}: device memory changed {before} -> {after}"
            a, b = ref.state(), dut.state()
            assert np.array_equal(a, b), f"call {call}: lattices differ"
            assert np.array_equal(ref.class_histogram(), dut.class_histogram())
        # the oracle agrees too
        st, off = oracle_lib.compact_state(o)
        assert off == 0 and np.array_equal(dut.state(), st)
        # longer than the fixed array: refused with a clear error, lattice untouched
        big = np.zeros(65537, dtype=N.EVENT_DTYPE)
        before = dut.state()
        rc = engine_lib.mks_replay_noalloc(dut._h, N.ptr(big), len(big))
        assert rc == 1
        assert b"per-call limit" in last_error(engine_lib)
        assert np.array_equal(dut.state(), before)
    finally:
        ref.close()
        dut.close()
        o.close()


def test_noalloc_replay_recovers_after_a_bad_event(oracle_lib, engine_lib):
    """A trace whose k-th event does not apply stops there with the invariant
    error naming event k; the progress counter and the status word that live
    in and beside the shared array are reset, so the next call on the same
    array replays a valid trace exactly as mks_replay does."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300 import _native as N
    start = os.path.join(GOLDEN, "Si-SL", "start.dat")
    o = oracle_lib.Oracle(start, 480, 480, 480)
    o.init()
    pE, pD = o.rates()
    o.trace_enable()
    o.run(4000)
    good = np.ascontiguousarray(o.trace(), dtype=N.EVENT_DTYPE)
    ref = Lattice(480, 480, 480, sf=0.4525)
    dut = Lattice(480, 480, 480, sf=0.4525)
    try:
        for lat in (ref, dut):
            lat.set_rates(pE, pD)
            lat.init_flat("S", 360)
        k = 1234
        bad = good[:2000].copy()
        # evaporation of a site deep in the bulk (coordination 4): not an event site
        bad[k]["x"], bad[k]["y"], bad[k]["z"], bad[k]["itrans"] = 0, 0, 120, 4
        rc = engine_lib.mks_replay_noalloc(dut._h, N.ptr(bad), len(bad))
        assert rc == MKS_ERR_INVARIANT
        assert f"event {k} ".encode() in last_error(engine_lib)
        assert dut.status()["error"] == 0
        # the first k events were applied: continue from there on both lattices
        ref.replay(good[:k])
        assert np.array_equal(ref.state(), dut.state())
        rest = np.ascontiguousarray(good[k:])
        ref.replay(rest)
        N.check(engine_lib.mks_replay_noalloc(dut._h, N.ptr(rest), len(rest)))
        assert np.array_equal(ref.state(), dut.state())
        assert np.array_equal(ref.class_histogram(), dut.class_histogram())
        # a negative coordinate is refused, not wrapped to a periodic image:
        # the oracle's next event applies to this state, its image at x - LenX
        # must not
        o.run(1)
        nxt = np.ascontiguousarray(o.trace(), dtype=N.EVENT_DTYPE)
        assert len(nxt) == 1
        neg = nxt.copy()
        neg[0]["x"] -= 480
        assert neg[0]["x"] < 0
        assert engine_lib.mks_replay_noalloc(dut._h, N.ptr(neg), 1) == MKS_ERR_INVARIANT
        assert np.array_equal(ref.state(), dut.state())
        N.check(engine_lib.mks_replay_noalloc(dut._h, N.ptr(nxt), 1))
        ref.replay(nxt)
        assert np.array_equal(ref.state(), dut.state())
    finally:
        ref.close()
        dut.close()
        o.close()
