"""Checkpoint / resume and failure detection on the GPU, without a GPU fault.

* A run saved with mks_get_state + mks_get_clock and restored into a fresh
  handle with the same seed continues bit for bit.
* Failure injection on the host side of the contract: a tile that never
  publishes its progress (mks_debug_hold_tile) makes its neighbours' bounded
  waits run out; the run returns MKS_ERR_TIMEOUT and a new handle on the same
  device runs normally.  A lattice holding a species its NCrystal does not
  have is rejected when it is loaded.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lattice(seed=9):
    from mulskips_gb300 import Lattice, arrhenius_tables
    lat = Lattice(480, 480, 480, seed=seed)
    lat.set_rates(*arrhenius_tables(1100.0))
    return lat


def test_resume_is_bit_exact():
    a = _lattice()
    a.init_flat("S", 240)
    tau = a.suggest_tau(0.3)
    a.run(tau, 16)
    snap, clk = a.state().copy(), a.clock()
    a.run(tau, 16)
    s1, c1 = a.state().copy(), a.clock()
    a.close()
    b = _lattice()
    b.set_state(snap)
    b.set_clock(*clk)
    b.run(tau, 16)
    assert np.array_equal(b.state(), s1)
    assert b.clock() == c1
    b.close()


def test_stalled_neighbour_times_out_and_device_stays_usable():
    from mulskips_gb300 import _native as N
    a = _lattice()
    a.init_flat("S", 240)
    tau = a.suggest_tau(0.3)
    # about 10 ms of spinning instead of 2 s
    N.check(N.lib().mks_debug_hold_tile(a._h, 5, 20_000_000))
    with pytest.raises(N.MksError) as e:
        a.run(tau, 8)
    assert "timed out" in str(e.value)
    a.close()
    b = _lattice()
    b.init_flat("S", 240)
    ev, t = b.run(tau, 8)
    assert ev > 0 and b.status()["error"] == 0
    b.close()


def test_foreign_species_is_rejected_on_load():
    from mulskips_gb300 import _native as N
    a = _lattice()
    a.init_flat("S", 240)
    st = a.state().copy()
    z, bb, aa = np.argwhere((st & 3) == 1)[0]
    st[z, bb, aa] = (int(st[z, bb, aa]) & 0xFC) | 2     # species 2 in an NCrystal = 1 lattice
    with pytest.raises(N.MksError):
        a.set_state(st)
    a.close()
