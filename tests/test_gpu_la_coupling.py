"""In-process LA coupling: the arrays of the reference's FEM <-> KMC socket
messages (mulskips-source-LaserAnnealing/main.f:160-345) through the C ABI
(GPU).

On the reference's LA regression lattice (480x240x240, built by the oracle's
pinned InitSt LA initializer):
* a temperature field given as the SENDFIELD message (mks_batch_set_field,
  SetT's rule: 10 keeps a wall's temperature) drives the same LA run, bit
  for bit, as the LattCoo temperatures it encodes (mks_batch_load_temperature);
* mks_batch_get_phases returns the GETPHASES / GETXGE arrays of main.f:796-817
  (coordination / species of occupied sites, 10 on walls) of the lattice that
  mks_get_lattice returns, at every grid point.
"""
import numpy as np
import pytest

from test_gpu_la_regression import BOX, _inputs, _startdat

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def la_lattice(oracle_lib, tmp_path_factory):
    geo, tsub, txt = _inputs()
    p = tmp_path_factory.mktemp("cpl") / "start.dat"
    p.write_text(_startdat(txt, 77))
    o = oracle_lib.Oracle(str(p), *BOX, numbers=None)
    o.set_la_input(geo, tsub)
    o.init()
    lc = o.lattcoo()
    pE, pD = o.rates()
    o.close()
    return lc, pE, pD


def socket_field(lc):
    """SENDFIELD array b(LenZ, LenX*LenY) of a LattCoo: T bits, 10 on walls."""
    lz = lc.shape[0] - 1
    body = lc[:lz]                                   # [z, y, x]
    T = np.where((body & 255) == 113, 10, (body >> 9) & 8191)
    return T.reshape(lz, -1)                         # [z, x + LenX*y]


def reference_phases(lc):
    """GETPHASES / GETXGE of LaserAnnealing main.f:796-817 applied to LattCoo."""
    lz = lc.shape[0] - 1
    body = lc[:lz]
    wall = (body & 255) == 113
    occ = (body >> 23) & 1
    coo = np.where(wall, 10, np.where(occ == 1, (body >> 24) & 7, 0))
    sp = np.where(wall, 10, np.where(occ == 1, (body >> 27) & 7, 0))
    return coo.reshape(lz, -1), sp.reshape(lz, -1)


def _run(lc, pE, pD, via_field):
    from mulskips_gb300 import Batch, la
    b = Batch([BOX], seeds=[19], sf=5.43 / 12)
    b.set_rates(pE[None], pD[None])
    b.load_lattice(0, lc)
    if via_field:
        b.set_field(0, socket_field(lc))
    else:
        b.load_temperature(0, lc)
    mat = la.Material(P0=(1.33e17,), Tm=(1688.0,), Tflex=(1080.0,), A=(280.0,))
    prm = la.la_params(mat, la.Pulse(), zsurf=1e30, score=False)
    prm.liquid_weighting = 0
    b.set_la(prm)
    b.run(2e-12, 64)
    out = b.get_phases(0), b.lattcoo(), b.observables()[0]
    b.close()
    return out


def test_field_message_drives_the_same_run(la_lattice):
    lc, pE, pD = la_lattice
    (c1, s1), lc1, o1 = _run(lc, pE, pD, via_field=False)
    (c2, s2), lc2, o2 = _run(lc, pE, pD, via_field=True)
    assert o1["events"] > 1000 and o1["events"] == o2["events"]
    assert np.array_equal(lc1, lc2)
    assert np.array_equal(c1, c2) and np.array_equal(s1, s2)


def test_phase_messages_match_the_reference_rule(la_lattice):
    lc, pE, pD = la_lattice
    (coo, sp), lc1, _ = _run(lc, pE, pD, via_field=True)
    rc, rs = reference_phases(lc1)
    assert coo.shape == rc.shape == (BOX[2], BOX[0] * BOX[1])
    assert np.array_equal(coo, rc)
    assert np.array_equal(sp, rs)
    # the solid sites pymulskips maps to the FEM mesh (values 1..4)
    n_solid = int(np.isin(coo, [1, 2, 3, 4]).sum())
    assert n_solid > 0.5 * int(((lc1 >> 23) & 1).sum() - ((lc1 & 255) == 113).sum())
