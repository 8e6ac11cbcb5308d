"""Arm-chair (hexagonal) stacking on the GPU: the explicit-neighbour engine
of handles with PtransZig < 1 (mulskips_gb300/csrc/stacking.cu).

Replay parity: the reference's `cube-zigzag` case (a free-standing 3C-SiC
parallelepiped, SetNC, PtransZig = 0.8: ties of IF_Arm_Choice.f:44-51 go
arm-chair one time in five), loaded from the pinned oracle with its lists,
and the oracle's own event trace applied by the engine, must give the
oracle's LattCoo word at every grid point and its list entries (grid point,
NextN in order, list, event and FP32 rate) after every chunk -- atoms off the
diamond sub-grid (FIND_SN.f:67, FIND_NN.f:25-77) included."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CUBE_ZZ = os.path.join(GOLDEN, "cube-zigzag", "start.dat")


def oracle_lists(ora, o):
    e = ora.list_entries(o)
    lx, ly, _ = o.dims
    key = e["xyz"][:, 0].astype(np.int64) + lx * (e["xyz"][:, 1] + ly * e["xyz"][:, 2].astype(np.int64))
    order = np.argsort(key)
    return key[order], {k: v[order] for k, v in e.items()}


def gpu_lists(lat):
    e = lat.lists()
    lx, ly, _ = lat.dims
    key = e["xyz"][:, 0].astype(np.int64) + lx * (e["xyz"][:, 1] + ly * e["xyz"][:, 2].astype(np.int64))
    order = np.argsort(key)
    return key[order], {k: v[order] for k, v in e.items()}


def ini_flags(e):
    """Unsupported coor-1 sites still at Get_Prob_Ini's dummy rate 1e-6."""
    return ((e["kind"] == 1) & (e["prob"] == float(np.float32(1e-6)))).astype(np.uint8)


def compare_state(ora, o, lat, where):
    lo = o.lattcoo()
    lg = lat.lattcoo()
    bad = np.argwhere(lo != lg)
    assert bad.size == 0, f"{where}: {len(bad)} LattCoo words differ, first [z, y, x] {bad[:3].tolist()}"
    ko, eo = oracle_lists(ora, o)
    kg, eg = gpu_lists(lat)
    assert np.array_equal(ko, kg), f"{where}: listed sites differ ({len(ko)} oracle, {len(kg)} GPU)"
    assert np.array_equal(eo["nn"], eg["nn"]), f"{where}: NextN lists differ"
    assert np.array_equal(eo["kind"], eg["kind"]), f"{where}: list membership differs"
    mc = eo["kind"] == 1
    dep = mc & (eo["ind_event"] <= 3)
    dummy = dep & ((eo["prob"] == float(np.float32(1e-8))) | (eo["prob"] == float(np.float32(1e-6))))
    assert np.array_equal(eg["event"][dep & ~dummy], np.full(np.count_nonzero(dep & ~dummy), 1))
    assert np.array_equal(eg["event"][dummy], np.full(np.count_nonzero(dummy), 2))
    evap = mc & (eo["ind_event"] == 4)
    assert np.all((eg["event"][evap] == 4) | (eg["event"][evap] == 5))
    rated = (dep | evap) & (eg["event"] != 5)
    assert np.array_equal(eg["rate"][rated], eo["prob"][rated].astype(np.float32)), f"{where}: rates differ"
    return int(np.count_nonzero(mc)), lg


def load_from_oracle(ora, o, lat):
    e = ora.list_entries(o)
    lat.load_lists(o.lattcoo(), e["xyz"], e["nn"], ini_flags(e))


def stacking_replay(ora, startdat, warm, total, chunk, box=480):
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    d = parse_startdat(startdat)
    o = ora.Oracle(startdat, box, box, box)
    o.init()
    if warm:
        o.run(warm)
    pE, pD = o.rates()
    lat = Lattice(box, box, box, ncrystal=d["ncrystal"], list_crystal=d["list_crystal"], sf=d["sf"],
                  ptrans_zig=d["ptrans_zig"])
    try:
        lat.set_rates(pE, pD)
        load_from_oracle(ora, o, lat)
        compare_state(ora, o, lat, f"after loading at event {warm}")
        o.trace_enable()
        done, arm = 0, 0
        while done < total:
            r = o.run(chunk)
            tr = o.trace()
            arm += int(np.count_nonzero(tr["arm"]))
            lat.replay(tr)
            done += len(tr)
            _, lg = compare_state(ora, o, lat, f"after {warm + done} events")
            if r:
                break
        x, y, z = np.nonzero(np.transpose(lg[:box], (2, 1, 0)))
        v = lg[:box][z, y, x]
        occ = ((v >> 23) & 1) == 1
        off = occ & ((x % 3 != 0) | (y % 3 != 0) | (z % 3 != 0))
        return done, arm, int(np.count_nonzero(off))
    finally:
        lat.close()
        o.close()


def test_stacking_replay_from_start(oracle_lib):
    """From SetNC's initial lattice: the first arm-chair depositions and the
    growth on hexagonal sites replay exactly."""
    done, arm, off = stacking_replay(oracle_lib, CUBE_ZZ, 0, 600000, 150000)
    assert done == 600000
    assert arm > 1000, "the trace should hold arm-chair depositions"
    assert off > 100, "atoms should sit off the diamond sub-grid"


def test_stacking_replay_twinned_lattice(oracle_lib):
    """From the oracle's state after 3e6 events (about 5 % of the atoms off
    the diamond sub-grid): evaporation and growth around twinned atoms,
    FIND_NN's rotations about non-<111> bonds and their rounding, replay
    exactly."""
    done, arm, off = stacking_replay(oracle_lib, CUBE_ZZ, 3000000, 500000, 250000)
    assert done == 500000
    assert off > 1000


def test_stacking_expands_initializer_lattice(oracle_lib):
    """The compact lattice of an initializer (SetNC, InitSt 'C') expanded to
    the explicit form equals the oracle's SetNC lattice: every LattCoo word,
    the listed sites with their list, event and rate, and the NextN lists as
    sets of sites (the order after the first entry is not kept by the
    compact form)."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    ora = oracle_lib
    d = parse_startdat(CUBE_ZZ)
    o = ora.Oracle(CUBE_ZZ, 480, 480, 480)
    o.init()
    pE, pD = o.rates()
    lens = d["len"]
    with Lattice(480, 480, 480, ncrystal=d["ncrystal"], list_crystal=d["list_crystal"], sf=d["sf"],
                 ptrans_zig=d["ptrans_zig"]) as lat:
        lat.set_rates(pE, pD)
        lat.init_shape("C", lens)
        assert np.array_equal(lat.lattcoo(), o.lattcoo())
        ko, eo = oracle_lists(ora, o)
        kg, eg = gpu_lists(lat)
        assert np.array_equal(ko, kg)
        assert np.array_equal(eo["kind"], eg["kind"])
        assert np.array_equal(eo["nn"][:, 0], eg["nn"][:, 0]), "first NextN entries differ"
        so = np.sort(eo["nn"].reshape(-1, 4, 3).view(np.dtype((np.void, 12))).reshape(-1, 4), axis=1)
        sg = np.sort(eg["nn"].reshape(-1, 4, 3).view(np.dtype((np.void, 12))).reshape(-1, 4), axis=1)
        assert np.array_equal(so, sg), "NextN sets differ"
        mc = eo["kind"] == 1
        assert np.array_equal(eg["rate"][mc & (eg["event"] != 5)], eo["prob"][mc & (eg["event"] != 5)].astype(np.float32))
    o.close()


def test_stacking_run_grows_hexagonal_sites(oracle_lib):
    """The synchronous-sublattice run with PtransZig = 0.8 on the cube
    case: events happen, the lattice stays consistent (the engine checks the
    census of every re-rated atom against its coordination, Get_Prob.f:
    293-298), and atoms grow off the diamond sub-grid."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    ora = oracle_lib
    d = parse_startdat(CUBE_ZZ)
    o = ora.Oracle(CUBE_ZZ, 480, 480, 480)
    o.init()
    pE, pD = o.rates()
    o.close()
    with Lattice(480, 480, 480, ncrystal=d["ncrystal"], list_crystal=d["list_crystal"], sf=d["sf"],
                 ptrans_zig=d["ptrans_zig"], seed=7) as lat:
        lat.set_rates(pE, pD)
        lat.init_shape("C", d["len"])
        tau = lat.suggest_tau(0.03)
        n, t = lat.run(tau, 200)
        assert n > 100000
        ob = lat.observables()
        lg = lat.lattcoo()
        z, y, x = np.nonzero(lg[:480])
        v = lg[:480][z, y, x]
        occ = ((v >> 23) & 1) == 1
        off = occ & ((x % 3 != 0) | (y % 3 != 0) | (z % 3 != 0))
        assert np.count_nonzero(off) > 50
        assert ob["atoms"] == int(np.count_nonzero(occ & ((v & 255) != 113)))
        # lists are consistent with the lattice: every atom and every
        # coordinated empty site is listed once
        e = lat.lists()
        assert len(np.unique(e["xyz"], axis=0)) == len(e["xyz"])
        assert np.all(e["kind"] > 0)
