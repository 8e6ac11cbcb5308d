"""mks_replay_noalloc — the replay entry point that allocates no device memory.

Some callers of this library cannot call cudaMalloc during a run (for
example a host that has already given its device-memory budget to the
lattice, or one that must not grow a stream-ordered memory pool).  This entry
point stages the event trace in a fixed device array owned by the library
instead of allocating a buffer per call.  The test drives it through the C
ABI and checks that, on two calls in a row, it leaves exactly the lattice
that the allocating mks_replay leaves (the state is integer bytes, so the
tolerance is zero), and that a trace longer than the array is refused.
Kept in a file collected last so that a failure here cannot hide others."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


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
    try:
        for lat in (ref, dut):
            lat.set_rates(pE, pD)
            lat.init_flat("S", 360)
        for call in range(2):                      # two calls in a row on the shared array
            o.run(30000)
            tr = np.ascontiguousarray(o.trace(), dtype=N.EVENT_DTYPE)
            assert len(tr) == 30000
            ref.replay(tr)                          # existing entry point (allocates)
            N.check(engine_lib.mks_replay_noalloc(dut._h, N.ptr(tr), len(tr)))
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
        buf = C.create_string_buffer(512)
        engine_lib.mks_last_error(buf, 512)
        assert b"per-call limit" in buf.value
        assert np.array_equal(dut.state(), before)
    finally:
        ref.close()
        dut.close()
        o.close()
