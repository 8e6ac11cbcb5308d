"""The window-factor tuner (mulskips_gb300/autotune.py choose_f) on two
models whose validated factors differ: it must keep the long window of the
plain Si(001) etch (f = 0.3) and shorten the window of the 3C-SiC(001)
`surface` rates, where f = 0.3 grows about 10 % too slowly (fast carbon
desorption across tile borders)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

NPILOT = 16


def test_choose_f_keeps_the_plain_si_window():
    from mulskips_gb300 import Batch, arrhenius_tables
    from mulskips_gb300.autotune import ACCURATE_F, choose_f
    pE, pD = arrhenius_tables(1100.0)

    def make(f):
        b = Batch([(480, 480, 480)] * NPILOT, seeds=[300 + s for s in range(NPILOT)], sf=0.4525)
        b.set_rates(np.stack([pE] * NPILOT), np.stack([pD] * NPILOT))
        b.init_flat("S", [120] * NPILOT)
        return b

    f, record = choose_f(make, 4e-7)
    print(record)
    assert f == ACCURATE_F


def test_choose_f_shortens_the_sic_window():
    from mulskips_gb300 import Batch
    from mulskips_gb300.autotune import choose_f
    from mulskips_gb300.startdat import parse_startdat
    d = parse_startdat(os.path.join(GOLDEN, "surface", "start.dat"))

    def make(f):
        b = Batch([(480, 480, 480)] * NPILOT, seeds=[400 + s for s in range(NPILOT)], ncrystal=2,
                  list_crystal=(14, 6), sf=d["sf"])
        b.set_rates(np.stack([d["ptransE"]] * NPILOT), np.stack([d["ptransD"]] * NPILOT))
        b.init_flat("C", [d["len"][0]] * NPILOT)
        return b

    f, record = choose_f(make, 2e5)
    print(record)
    first = next(r for r in record if r["f"] == 0.3)
    assert not first["accepted"], "f = 0.3 should fail the equivalence test on the SiC rates"
    assert f < 0.3
