"""Replay parity: the reference's event sequence (from the pinned oracle),
applied by the GPU engine through the C ABI, gives bit-identical lattice
occupancy, coordination, neighbour-list head, dummy flags and coverage, and
the same rate-class histogram as the oracle's own lists."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def oracle_hist(ora, o):
    cls, _ = ora.mc_classes(o)
    return np.bincount(cls, minlength=64)[:64]


def replay_case(ora, startdat, len1, kind, total, chunk, lenxyz=480):
    from mulskips_gb300 import Lattice
    o = ora.Oracle(startdat, lenxyz, lenxyz, lenxyz)
    o.init()
    d = __import__("mulskips_gb300.startdat", fromlist=["x"]).parse_startdat(startdat)
    pE, pD = o.rates()
    lat = Lattice(lenxyz, lenxyz, lenxyz, ncrystal=d["ncrystal"], list_crystal=d["list_crystal"], sf=d["sf"],
                  list_cov=d["list_cov"])
    try:
        lat.set_rates(pE, pD)
        if d["list_cov"]:
            lat.set_coverage_rates(*o.cov_rates())
        if kind:
            lat.init_flat(kind, len1)
        else:                               # the oracle's own initializer, through LattCoo
            lat.load_lattcoo(o.lattcoo())
        st0, off = ora.compact_state(o)
        assert off == 0
        assert np.array_equal(lat.state(), st0), "initial lattice differs"
        o.trace_enable()
        done = 0
        while done < total:
            r = o.run(chunk)
            tr = o.trace()
            lat.replay(tr)
            done += len(tr)
            st, off = ora.compact_state(o)
            assert off == 0
            g = lat.state()
            bad = np.argwhere(g != st)
            assert bad.size == 0, f"after {done} events: {len(bad)} sites differ, first {bad[:3]}"
            h = lat.class_histogram()
            ho = oracle_hist(ora, o)
            assert np.array_equal(h[1:], ho[1:]), f"class histogram differs after {done} events"
            if r:
                break
        return done
    finally:
        lat.close()
        o.close()


def test_replay_si001(oracle_lib):
    n = replay_case(oracle_lib, os.path.join(GOLDEN, "Si-SL", "start.dat"), 360, "S", 400000, 100000)
    assert n == 400000


def test_replay_sic001(oracle_lib):
    n = replay_case(oracle_lib, os.path.join(GOLDEN, "surface", "start.dat"), 120, "C", 200000, 100000)
    assert n == 200000


def test_replay_cvd_si001_hydrogen(oracle_lib):
    """CVD of Si(001) under one coverage species (H), the reference's
    CVD-Si-SiH2 case: absorption (itrans 6) and desorption (5) events among
    the depositions and evaporations replay exactly, covered sites included."""
    n = replay_case(oracle_lib, os.path.join(GOLDEN, "CVD-Si-SiH2", "start.dat"), 48, "S", 400000, 100000)
    assert n == 400000


def test_replay_cvd_two_coverage_species(oracle_lib, tmp_path):
    """CVD of Si(001) under two coverage species (H and Cl, the input of
    tests/cvd2.py): depositions, evaporations, desorptions and absorptions of
    either species (itrans 6 and 7, IndexEvent_Abs of Get_Prob.f:22-52)
    replay exactly, covered sites of each species and the 19 atom classes
    keyed by their covered neighbours (PE(1, n1, 0, 0, c1, c2, 0)) included."""
    from cvd2 import two_coverage_startdat
    p = two_coverage_startdat(str(tmp_path / "start.dat"))
    n = replay_case(oracle_lib, p, 48, "S", 400000, 100000)
    assert n == 400000


def test_replay_sic_cube(oracle_lib):
    """The free-standing 3C-SiC parallelepiped of the reference's `cube` case
    (SetNC, no walls), loaded from the oracle's LattCoo through
    mks_load_lattice: the growth of its six faces replays exactly."""
    n = replay_case(oracle_lib, os.path.join(GOLDEN, "cube", "start.dat"), 0, None, 300000, 100000)
    assert n == 300000


def test_replay_etch_to_walls(oracle_lib, tmp_path):
    """T=1100 K plain Si(001) (the benchmark model): etches through to the
    walls and stops on the few-MC-particles rule; replay stays exact."""
    from mulskips_gb300.startdat import write_plain_si_startdat
    p = tmp_path / "start.dat"
    write_plain_si_startdat(str(p), T=1100.0, len1=120, max_iter=1000000, seed=1)
    n = replay_case(oracle_lib, str(p), 120, "S", 1000000, 40000)
    assert 100000 < n < 1000000


def test_replay_rejects_inapplicable_event(oracle_lib):
    from mulskips_gb300 import Lattice, arrhenius_tables
    from mulskips_gb300._native import EVENT_DTYPE, MksError
    pE, pD = arrhenius_tables(1100.0)
    with Lattice(480, 480, 480) as lat:
        lat.set_rates(pE, pD)
        lat.init_flat("S", 120)
        ev = np.zeros(1, dtype=EVENT_DTYPE)
        ev[0] = (0, 0, 300, 1, 0, 0)      # empty, untracked site far above the surface
        with pytest.raises(MksError):
            lat.replay(ev)


def site_rates_case(ora, startdat, len1, kind, events):
    """The engine's rate of every MC particle of the oracle against the
    oracle's tree leaf (ProbTrans), at the start and after `events` replayed
    events; returns the number of sites compared at each point."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    d = parse_startdat(startdat)
    o = ora.Oracle(startdat, 480, 480, 480)
    o.init()
    pE, pD = o.rates()
    lat = Lattice(480, 480, 480, ncrystal=d["ncrystal"], list_crystal=d["list_crystal"], sf=d["sf"],
                  list_cov=d["list_cov"])
    counts = []
    try:
        lat.set_rates(pE, pD)
        if d["list_cov"]:
            lat.set_coverage_rates(*o.cov_rates())
        if kind:
            lat.init_flat(kind, len1)
        else:
            lat.load_lattcoo(o.lattcoo())
        o.trace_enable()
        for step in range(2):
            if step:
                o.run(events)
                lat.replay(o.trace())
            xyz = ora.mc_sites(o)
            cls_o, rate_o = ora.mc_classes(o)
            cls_g, rate_g = lat.site_rates(xyz)
            assert np.array_equal(cls_g, cls_o), f"step {step}: classes differ at {np.argwhere(cls_g != cls_o)[:3]}"
            keep = cls_o != 5                      # isolated atoms: 1e5 x Tree(1), dynamic
            # FP32 class rates of the engine against the FP64 leaves of the reference
            assert np.array_equal(rate_g[keep], rate_o[keep].astype(np.float32)), f"step {step}: rates differ"
            counts.append((int(keep.sum()), int(np.count_nonzero(cls_o == 63)), int(np.count_nonzero(cls_o == 2))))
        return counts
    finally:
        lat.close()
        o.close()


@pytest.mark.parametrize("case,len1,kind", [("Si-SL", 360, "S"), ("CVD-Si-SiH2", 48, "S"), ("cube", 0, None)])
def test_site_rates_match_oracle_leaves(oracle_lib, case, len1, kind):
    """Per-site rates, not only classes: every MC particle's tree leaf in the
    oracle (Get_Prob / Get_Prob_Ini's ProbTrans) equals the engine's rate of
    that site, right after initialization and after 20000 replayed events.
    The cube's initializer (SetNC) rates its unsupported coor-1 sites with
    Get_Prob_Ini's 1e-6, which they keep until they change; later dummies
    take Get_Prob's 1e-8."""
    counts = site_rates_case(oracle_lib, os.path.join(GOLDEN, case, "start.dat"), len1, kind, 20000)
    print(case, counts)
    assert counts[0][0] > 1000
    if case == "cube":
        assert counts[0][1] > 0                    # initial dummies at 1e-6
