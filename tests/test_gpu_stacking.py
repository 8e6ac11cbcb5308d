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


def oracle_events(e):
    """The engine's event codes and FP32 rates of the oracle's list entries:
    1 deposition, 2 the dummy of an unsupported coor-1 site (1e-8 or, still
    from the initializer, 1e-6), 4 evaporation, 0 bulk atoms and voids."""
    mc = e["kind"] == 1
    dummy = mc & (e["ind_event"] <= 3) & ((e["prob"] == float(np.float32(1e-8))) |
                                         (e["prob"] == float(np.float32(1e-6))))
    ev = np.where(mc, np.where(e["ind_event"] <= 3, 1, 4), 0)
    ev[dummy] = 2
    return ev.astype(np.int32), np.where(mc, e["prob"], 0.0).astype(np.float32)


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
    ev, rate = oracle_events(e)
    lat.load_lists(o.lattcoo(), e["xyz"], e["nn"], ev, rate)


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


def test_stacking_replay_twinned_lattice(oracle_lib):
    """From the oracle's state after 8e6 events (atoms off the diamond
    sub-grid in the thousands: 440 at 3e6 events, 2657 at 1e7), loaded with
    its list entries and their saved rates: evaporation and growth around
    twinned atoms, FIND_NN's rotations about non-<111> bonds and their
    rounding, replay exactly."""
    done, arm, off = stacking_replay(oracle_lib, CUBE_ZZ, 8000000, 500000, 250000)
    assert done == 500000
    assert off > 1000


def test_stacking_replay_sic_facets(oracle_lib, tmp_path):
    """Config 2's stacking preference (PtransZig = 0.5362, a 0.02 eV
    preference for cubic stacking at 1600 K) on {111} facets: a 3C-SiC
    square pyramid with {111} faces on a (001) slab (InitSt SH point list,
    240^3 box), the reference's SiC `surface` rates.  About one coor-1
    deposition in five takes the hexagonal position here; 300k events of
    the oracle's trace replay exactly."""
    from test_shape_points import pyramid_points, sh_startdat, write_points
    xyz, sym, _, _ = pyramid_points(240, 60, 54)
    write_points(tmp_path / "p.xyz", xyz, sym)
    lines = [("0.5362 ! PtransZig" if "PtransZig" in ln else ln)
             for ln in open(os.path.join(GOLDEN, "surface", "start.dat")).read().splitlines()]
    p = tmp_path / "start.dat"
    sh_startdat(lines, p, str(tmp_path / "p.xyz"))
    done, arm, off = stacking_replay(oracle_lib, str(p), 0, 300000, 100000, box=240)
    assert done == 300000 and arm > 1000


def test_stacking_run_is_reproducible(oracle_lib):
    """Two runs with the same seed give the same lattice: list order never
    depends on the scheduling of warps or lanes (inbox drained in grid-point
    order, a tile's own new sites appended in lane order, lists sorted after
    a rebuild)."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    d = parse_startdat(CUBE_ZZ)
    out = []
    for _ in range(2):
        with Lattice(480, 480, 480, ncrystal=d["ncrystal"], list_crystal=d["list_crystal"], sf=d["sf"],
                     ptrans_zig=d["ptrans_zig"], seed=23) as lat:
            lat.set_rates(d["ptransE"], d["ptransD"])
            lat.init_shape("C", d["len"])
            n = 0
            for _ in range(24):
                m, _t = lat.run(lat.suggest_tau(0.01), 64)
                n += m
            out.append((n, lat.lattcoo()))
    assert out[0][0] == out[1][0] > 1000
    assert np.array_equal(out[0][1], out[1][1])


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


def test_stacking_frames_match_oracle_writer(oracle_lib, tmp_path):
    """The frame files of an arm-chair stacking handle (WriteMolMolXYZFile.f:
    22-406) against the oracle's writer on the same twinned state (the
    oracle's cube-zigzag lattice after 3e6 events, loaded with its lists):
    _d.xyz -- the non-epitaxial bulk atoms off the diamond sites, the
    reference's own stacking-fault output -- and _w.xyz byte for byte; the
    atom lines of .xyz in order and its voids, and the labelled voids of
    _v.xyz, as sets (the reference lists voids in ListVoid order)."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    ora = oracle_lib
    d = parse_startdat(CUBE_ZZ)
    o = ora.Oracle(CUBE_ZZ, 480, 480, 480)
    o.init()
    o.run(8000000)
    pE, pD = o.rates()
    with Lattice(480, 480, 480, ncrystal=d["ncrystal"], list_crystal=d["list_crystal"], sf=d["sf"],
                 ptrans_zig=d["ptrans_zig"]) as lat:
        lat.set_rates(pE, pD)
        load_from_oracle(ora, o, lat)
        lat.write_frame(str(tmp_path / "g"), 1.5, 8000000)
    o.write_frame(str(tmp_path / "o"), 1.5, 8000000)
    o.close()

    def read(name):
        return (tmp_path / name).read_text().splitlines()

    assert read("g_d.xyz") == read("o_d.xyz")
    assert int(read("g_d.xyz")[0].split()[0]) > 200, "the twinned lattice holds non-epitaxial bulk atoms"
    assert read("g_w.xyz") == read("o_w.xyz")
    g, r = read("g.xyz"), read("o.xyz")
    assert g[:2] == r[:2]
    ga = [x for x in g[2:] if not x.startswith("O ")]
    ra = [x for x in r[2:] if not x.startswith("O ")]
    assert ga == ra
    assert sorted(x for x in g[2:] if x.startswith("O ")) == sorted(x for x in r[2:] if x.startswith("O "))
    gv, rv = read("g_v.xyz"), read("o_v.xyz")
    assert gv[:2] == rv[:2] and sorted(gv[2:]) == sorted(rv[2:])


# ---------------------------------------------------------------- statistics
NSEEDS = 32
T_OBS = 1.2e6          # s: about 3e6 events of the serial reference


def stacking_observables(lg):
    """From LattCoo [z, y, x] (z < LenZ): atoms, C atoms, atoms off the
    diamond sub-grid, and the non-epitaxial bulk atoms of _d.xyz
    (WriteMolMolXYZFile.f:120-160: coordination 4 on a grid point that is not
    a diamond site)."""
    z, y, x = np.nonzero(lg)
    v = lg[z, y, x]
    atom = (((v >> 23) & 1) == 1) & ((v & 255) != 113)
    dia = (x % 3 == 0) & (y % 3 == 0) & (z % 3 == 0)
    x1, y1, z1 = x // 3, y // 3, z // 3
    dia &= ((x1 & 1) == (y1 & 1)) & ((x1 & 1) == (z1 & 1)) & (((x1 + y1 + z1) & 3) % 3 == 0)
    co4 = ((v >> 24) & 7) == 4
    return {"atoms": int(atom.sum()), "C": int((atom & (((v >> 27) & 7) == 2)).sum()),
            "off-grid atoms": int((atom & ~dia).sum()), "non-epitaxial bulk": int((atom & co4 & ~dia).sum())}


def _oracle_seed(args):
    path, t_obs = args
    from oracle import ora
    o = ora.Oracle(path, 480, 480, 480)
    o.init()
    o.run_until(t_obs)
    out = stacking_observables(o.lattcoo()[:480])
    out["events"] = o.iter
    o.close()
    return out


def _gpu_seed(args):
    seed, d, t_obs, f = args
    from mulskips_gb300 import Lattice
    with Lattice(480, 480, 480, ncrystal=d["ncrystal"], list_crystal=d["list_crystal"], sf=d["sf"],
                 ptrans_zig=d["ptrans_zig"], seed=seed) as lat:
        lat.set_rates(d["ptransE"], d["ptransD"])
        lat.init_shape("C", d["len"])
        t, events, windows = 0.0, 0, 0
        while t < t_obs:
            tau = lat.suggest_tau(f)        # the window follows the state, as mulskips.e re-suggests it
            n, t1 = lat.run(tau, 64, 0, t_obs)
            assert t1 > t
            t = t1
            events += n
            windows += 64
        out = stacking_observables(lat.lattcoo()[:480])
        out["events"] = events
        return out


def test_stacking_statistics_match_serial_reference(tmp_path):
    """The sublattice KMC with arm-chair stacking against the serial
    reference: the cube-zigzag case (SiC rates of its start.dat, PtransZig =
    0.8), RunType R, 32 oracle seeds and 32 GPU replicas observed at t =
    1.2e6 s (about 3e6 events): atoms, C atoms, atoms off the diamond
    sub-grid and non-epitaxial bulk atoms -- the stacking-fault density --
    each inside its 95 % family band (Welch t, Bonferroni over the four)."""
    import multiprocessing as mp
    from concurrent.futures import ThreadPoolExecutor
    from mulskips_gb300.autotune import accurate_f
    from mulskips_gb300.startdat import parse_startdat
    from stat_bands import Family
    txt = open(CUBE_ZZ).read().replace("T   ! R = production run", "R   ! R = production run")
    paths = []
    for s in range(NSEEDS):
        p = tmp_path / f"zz{s}.dat"
        p.write_text(txt.replace("9117116 ! Random seed", f"{900 + s} ! Random seed"))
        paths.append(str(p))
    d = parse_startdat(paths[0])
    assert d["run_type"] == "R" and d["ptrans_zig"] == 0.8
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        ref = pool.map(_oracle_seed, [(p, T_OBS) for p in paths])
    f = accurate_f(2)
    with ThreadPoolExecutor(8) as ex:
        gpu = list(ex.map(_gpu_seed, [(31 + s, d, T_OBS, f) for s in range(NSEEDS)]))
    fam = Family(f"cube-zigzag, PtransZig = 0.8, t = {T_OBS:g} s, f = {f}", 4)
    for k in ("atoms", "C", "off-grid atoms", "non-epitaxial bulk"):
        fam.add(k, np.array([g[k] for g in gpu], float), np.array([r[k] for r in ref], float))
    assert np.mean([r["off-grid atoms"] for r in ref]) > 100
    fam.check()


# ---------------------------------------------------------------- config 2 as stated: an etching {111}-faceted slab
C2_SIDE, C2_T_OBS = 240, 2e-11      # s: about 8.4e3 events of the serial reference (a third of the atoms)


def slab_observables(lg):
    """From LattCoo [z, y, x]: atoms, C atoms, and the mean and RMS of the
    top atom's height over the (x, y) columns holding atoms."""
    z, y, x = np.nonzero(lg)
    v = lg[z, y, x]
    atom = (((v >> 23) & 1) == 1) & ((v & 255) != 113)
    top = np.full(lg.shape[1:], -1, np.int64)
    np.maximum.at(top, (y[atom], x[atom]), z[atom])
    h = top[top >= 0].astype(float)
    return {"atoms": int(atom.sum()), "C": int((atom & (((v >> 27) & 7) == 2)).sum()),
            "mean top height": float(h.mean()), "RMS roughness": float(h.std())}


def _config2_oracle(args):
    path, t_obs = args
    from oracle import ora
    o = ora.Oracle(path, C2_SIDE, C2_SIDE, C2_SIDE, numbers=None)
    o.init()
    o.run_until(t_obs)
    out = slab_observables(o.lattcoo()[:C2_SIDE])
    out["events"] = o.iter
    o.close()
    return out


def _config2_gpu(args):
    seed, E, D, sf, pzig, xyz, sp, t_obs, f = args
    from mulskips_gb300 import Lattice
    with Lattice(C2_SIDE, C2_SIDE, C2_SIDE, ncrystal=2, list_crystal=(14, 6), sf=sf, ptrans_zig=pzig,
                 seed=seed) as lat:
        lat.set_rates(E, D)
        lat.init_points(xyz, sp)
        t, events = 0.0, 0
        while t < t_obs:
            n, t1 = lat.run(lat.suggest_tau(f), 64, 0, t_obs)
            assert t1 > t
            t = t1
            events += n
        out = slab_observables(lat.lattcoo()[:C2_SIDE])
        out["events"] = events
        return out


def test_config2_faceted_etch_matches_serial_reference(tmp_path):
    """Config 2 as stated, on a small box: a 3C-SiC slab with {111} facets
    only (mulskips_gb300.shapes, square pyramids of period 60 in a 240^3
    box), per-species fluxes U(0.1, 1) ML/s and 18 evaporation barriers
    U(0.4, 0.9) eV with a 1e13 prefactor at 1600 K (table seed 2), PtransZig
    = 0.5362, on the explicit-neighbour engine.  The slab etches; 32 oracle
    seeds (RunType R) and 32 GPU runs observed at t = 2e-11 s: atoms, C
    atoms, mean top height and RMS roughness of the etched surface, each
    inside its 95 % family band (Welch t, Bonferroni over the four)."""
    import multiprocessing as mp
    from concurrent.futures import ThreadPoolExecutor
    from bench import PZIG_1600K, config2_tables
    from mulskips_gb300.autotune import accurate_f
    from mulskips_gb300.shapes import faceted_slab_points
    from mulskips_gb300.startdat import parse_startdat, write_startdat
    from stat_bands import Family
    E, D, _, _ = config2_tables()
    sf = parse_startdat(CUBE_ZZ)["sf"]
    xyz, sp = faceted_slab_points(C2_SIDE, 120, 60)
    pts = tmp_path / "slab.xyz"
    with open(pts, "w") as fh:
        fh.write(f"{len(xyz)}\nslab\n")
        fh.write("".join(f"{'Si' if s == 1 else 'C'} {x} {y} {z}\n" for (x, y, z), s in zip(xyz.tolist(), sp)))
    paths = []
    for s in range(NSEEDS):
        p = tmp_path / f"c2_{s}.dat"
        write_startdat(str(p), E, D, ncrystal=2, list_crystal=(14, 6), init_st="SH", points=str(pts), run_type="R",
                       seed=1300 + s, sf=sf, ptrans_zig=PZIG_1600K, max_iter=10 ** 9)
        paths.append(str(p))
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        ref = pool.map(_config2_oracle, [(p, C2_T_OBS) for p in paths])
    f = accurate_f(2)
    with ThreadPoolExecutor(8) as ex:
        gpu = list(ex.map(_config2_gpu, [(71 + s, E, D, sf, PZIG_1600K, xyz, sp, C2_T_OBS, f) for s in range(NSEEDS)]))
    fam = Family(f"config 2 faceted etch, PtransZig = {PZIG_1600K:.4f}, t = {C2_T_OBS:g} s, f = {f}", 4)
    for k in ("atoms", "C", "mean top height", "RMS roughness"):
        fam.add(k, np.array([g[k] for g in gpu], float), np.array([r[k] for r in ref], float))
    atoms0 = int(((xyz[:, 2] > 3) & (xyz[:, 2] < C2_SIDE - 4)).sum())
    assert 0.1 * atoms0 < atoms0 - np.mean([r["atoms"] for r in ref]) < 0.6 * atoms0
    fam.check()


# ---------------------------------------------------------------- InitSt E: SetSiCSF
@pytest.mark.parametrize("pzig", ["1.0", "0.5362"])
def test_sicsf_matches_oracle_and_replays(oracle_lib, tmp_path, pzig):
    """InitSt E (SetSiCSF.f: a 3C-SiC slab holding a triangular triple
    stacking fault, its atoms off the diamond sites) on the explicit-neighbour
    engine, at PtransZig = 1 (explicit_nn) and 0.5362: after the initializer
    the engine holds the oracle's LattCoo word for word and its list entries
    (NextN in order, event codes, FP32 rates); the oracle's event trace from
    there then replays exactly, chunk by chunk (a 120^3 box, vertex (24, 24,
    36), the cube-zigzag SiC rates, RunType T)."""
    from test_shape_points import sicsf_startdat
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    L = 120
    p = tmp_path / "start.dat"
    sicsf_startdat(p, 60, 24, 24, pzig)
    d = parse_startdat(str(p))
    o = oracle_lib.Oracle(str(p), L, L, L)
    o.init()
    pE, pD = o.rates()
    lat = Lattice(L, L, L, ncrystal=2, list_crystal=d["list_crystal"], sf=d["sf"], ptrans_zig=d["ptrans_zig"],
                  explicit_nn=True)
    try:
        lat.set_rates(pE, pD)
        lat.init_shape("E", [60, 24, 24])
        nmc, lg = compare_state(oracle_lib, o, lat, "after SetSiCSF")
        z, y, x = np.nonzero(((lg >> 23) & 1) == 1)
        assert nmc > 100 and ((x % 3 != 0) | (y % 3 != 0) | (z % 3 != 0)).sum() > 10
        o.trace_enable()
        done = 0
        while done < 40000:
            r = o.run(10000)
            tr = o.trace()
            lat.replay(tr)
            done += len(tr)
            compare_state(oracle_lib, o, lat, f"after {done} events")
            if r:
                break
        assert done >= 40000
    finally:
        lat.close()
        o.close()


def test_sicsf_needs_the_explicit_engine():
    from mulskips_gb300 import Lattice
    from mulskips_gb300._native import MksError
    with Lattice(120, 120, 120, ncrystal=2, list_crystal=(14, 6)) as lat:
        with pytest.raises(MksError, match="explicit-neighbour"):
            lat.init_shape("E", [60, 24, 24])
