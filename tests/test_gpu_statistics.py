"""Statistical parity of the sublattice KMC with the serial reference.

The plain Si(001) model at T = 1100 K (the benchmark's model, 480^3 box,
Len1 = 120 slab) etches.  Observable: atoms left at time T_obs (the etch
rate).  32 seeds of the serial oracle (RunType R, exact reference dynamics,
deterministic dt = 1/R_tot) against 32 GPU replicas (exponential waiting
times, synchronous sublattice windows of length tau).  The difference of the
means must lie inside the 3-sigma band of the difference (99.7 %; several
statistical checks run together, so a 95 % band would fail by chance too
often)."""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

T_OBS = 4e-7
NSEEDS = 32


def oracle_atoms(ora, tmp_path, seed):
    from mulskips_gb300.startdat import write_plain_si_startdat
    p = tmp_path / f"start{seed}.dat"
    write_plain_si_startdat(str(p), T=1100.0, len1=120, max_iter=10 ** 9, seed=seed)
    o = ora.Oracle(str(p), 480, 480, 480, numbers=None)
    o.init()
    o.run_until(T_OBS)
    n = o.atoms()
    o.close()
    return n


def gpu_atoms(tau, seeds):
    from mulskips_gb300 import Batch, arrhenius_tables
    pE, pD = arrhenius_tables(1100.0)
    n = len(seeds)
    b = Batch([(480, 480, 480)] * n, seeds=seeds)
    b.set_rates(np.stack([pE] * n), np.stack([pD] * n))
    b.init_flat("S", [120] * n)
    nwin = int(round(T_OBS / tau))
    b.run(tau, nwin)
    obs = b.observables()
    b.close()
    assert all(abs(o["time"] - nwin * tau) < 1e-12 for o in obs)
    return np.array([o["atoms"] for o in obs], dtype=float)


def band(x, y):
    d = x.mean() - y.mean()
    se = math.sqrt(x.var(ddof=1) / len(x) + y.var(ddof=1) / len(y))
    return d, 3.0 * se


@pytest.fixture(scope="module")
def oracle_sample(oracle_lib, tmp_path_factory):
    tmp = tmp_path_factory.mktemp("stat")
    return np.array([oracle_atoms(oracle_lib, tmp, 100 + s) for s in range(NSEEDS)], dtype=float)


# k2 = 1e13 exp(-1.2 eV / kT) at 1100 K is the coor-2 evaporation rate: 2e-9 s
# is k2 tau = 0.064; T_OBS / 43 is k2 tau = 0.296, the f = 0.3 window rule of
# the engine's tau suggestion
@pytest.mark.parametrize("tau", [2e-9, T_OBS / 43])
def test_etch_rate_matches_serial_reference(oracle_sample, tau):
    g = gpu_atoms(tau, [1 + s for s in range(NSEEDS)])
    d, hw = band(g, oracle_sample)
    start = 3200 * 36
    print(f"tau={tau}: gpu {g.mean():.1f}+-{g.std(ddof=1):.1f}  serial {oracle_sample.mean():.1f}"
          f"+-{oracle_sample.std(ddof=1):.1f}  diff {d:.1f}  3-sigma band +-{hw:.1f}")
    assert g.mean() < start and oracle_sample.mean() < start       # etching happened
    assert abs(d) <= hw, f"etch-rate difference {d:.1f} atoms outside the 3-sigma band {hw:.1f}"


def test_deposition_evaporation_regime_matches_serial_reference(oracle_lib, tmp_path):
    """The Si-SL regression rates with RunType R (deposition 9.3e-4 against
    coor-2 evaporation 2.0e-3, so both event kinds matter): atoms left at
    t = 1e4 s, 16 oracle seeds against 16 GPU replicas at the autotuned tau."""
    from mulskips_gb300 import Batch
    from mulskips_gb300.startdat import parse_startdat
    from conftest import GOLDEN
    txt = open(os.path.join(GOLDEN, "Si-SL", "start.dat")).read().replace("T   ! R = production run",
                                                                            "R   ! R = production run")
    ref = []
    for s in range(16):
        p = tmp_path / f"sl{s}.dat"
        p.write_text(txt.replace("9117116 ! Random seed", f"{200 + s} ! Random seed"))
        o = oracle_lib.Oracle(str(p), 480, 480, 480, numbers=None)
        o.init()
        o.run_until(1e4)
        ref.append(o.atoms())
        o.close()
    ref = np.array(ref, float)
    d = parse_startdat(str(tmp_path / "sl0.dat"))
    n = 16
    b = Batch([(480, 480, 480)] * n, seeds=[31 + s for s in range(n)], sf=d["sf"])
    b.set_rates(np.stack([d["ptransE"]] * n), np.stack([d["ptransD"]] * n))
    b.init_flat("S", [360] * n)
    tau = float(b.suggest_tau(0.3)[0])
    nwin = int(round(1e4 / tau))
    b.run(1e4 / nwin, nwin)
    g = np.array([o["atoms"] for o in b.observables()], float)
    b.close()
    diff, hw = band(g, ref)
    print(f"Si-SL rates: gpu {g.mean():.1f}+-{g.std(ddof=1):.1f} serial {ref.mean():.1f}+-{ref.std(ddof=1):.1f} "
          f"diff {diff:.1f} 3-sigma band +-{hw:.1f}")
    assert abs(diff) <= hw


def test_sic_surface_matches_serial_reference(oracle_lib, tmp_path):
    """3C-SiC(001), the rates of the reference's `surface` regression case
    (NCrystal 2, Si and C with 18 census-dependent evaporation rates), RunType
    R: atoms and C atoms at t = 2e5 s, 16 oracle seeds against 16 GPU
    replicas at the two-species window factor f = 0.03."""
    from mulskips_gb300 import Batch
    from mulskips_gb300.startdat import parse_startdat
    from conftest import GOLDEN
    t_obs = 2e5
    txt = open(os.path.join(GOLDEN, "surface", "start.dat")).read().replace(
        "T   ! R = production run", "R   ! R = production run")
    ref, ref_c = [], []
    for s in range(16):
        p = tmp_path / f"sic{s}.dat"
        p.write_text(txt.replace("9117116 ! Random seed", f"{400 + s} ! Random seed"))
        o = oracle_lib.Oracle(str(p), 480, 480, 480, numbers=None)
        o.init()
        o.run_until(t_obs)
        st, _ = oracle_lib.compact_state(o)
        ref.append(int(np.count_nonzero((st & 3) != 0)))
        ref_c.append(int(np.count_nonzero((st & 3) == 2)))
        o.close()
    ref, ref_c = np.array(ref, float), np.array(ref_c, float)
    d = parse_startdat(str(tmp_path / "sic0.dat"))
    n = 16
    b = Batch([(480, 480, 480)] * n, seeds=[51 + s for s in range(n)], ncrystal=2, list_crystal=(14, 6),
              sf=d["sf"])
    b.set_rates(np.stack([d["ptransE"]] * n), np.stack([d["ptransD"]] * n))
    b.init_flat("C", [d["len"][0]] * n)
    from mulskips_gb300.autotune import accurate_f
    tau = float(b.suggest_tau(accurate_f(2))[0])
    nwin = int(math.ceil(t_obs / tau))
    b.run(t_obs / nwin, nwin)
    obs = b.observables()
    b.close()
    g = np.array([o["atoms"] for o in obs], float)
    gc = np.array([o["species"][1] for o in obs], float)
    for name, x, y in (("atoms", g, ref), ("C atoms", gc, ref_c)):
        diff, hw = band(x, y)
        print(f"SiC {name}: gpu {x.mean():.1f}+-{x.std(ddof=1):.1f} serial {y.mean():.1f}+-{y.std(ddof=1):.1f} "
              f"diff {diff:.1f} 3-sigma band +-{hw:.1f} (tau {tau:.3e})")
        assert abs(diff) <= hw, name


def test_sic_facets_match_serial_reference(oracle_lib, tmp_path):
    """3C-SiC on {111} facets: a square pyramid with {111} faces on a (001)
    slab (InitSt SH point list, 240^3 box), the rates of the reference's
    `surface` case, RunType R: atoms and C atoms at t = 2e5 s (about 2.5e5
    events, the facets filling in), 16 oracle seeds against 16 GPU replicas
    at the two-species window factor."""
    from mulskips_gb300 import Batch
    from mulskips_gb300.autotune import accurate_f
    from mulskips_gb300.startdat import parse_startdat, read_shape_points
    from conftest import GOLDEN
    from test_shape_points import pyramid_points, sh_startdat, write_points
    t_obs, n, L = 2e5, 16, 240
    xyz, sym, _, _ = pyramid_points(L, 60, 54)
    write_points(tmp_path / "p.xyz", xyz, sym)
    txt = open(os.path.join(GOLDEN, "surface", "start.dat")).read().replace(
        "T   ! R = production run", "R   ! R = production run")
    ref, ref_c = [], []
    for s in range(n):
        p = tmp_path / f"fac{s}.dat"
        sh_startdat(txt.replace("9117116 ! Random seed", f"{600 + s} ! Random seed").splitlines(), p,
                    str(tmp_path / "p.xyz"))
        o = oracle_lib.Oracle(str(p), L, L, L, numbers=None)
        o.init()
        o.run_until(t_obs)
        st, _ = oracle_lib.compact_state(o)
        ref.append(int(np.count_nonzero((st & 3) != 0)))
        ref_c.append(int(np.count_nonzero((st & 3) == 2)))
        o.close()
    ref, ref_c = np.array(ref, float), np.array(ref_c, float)
    d = parse_startdat(str(tmp_path / "fac0.dat"))
    pts, sp = read_shape_points(str(tmp_path / "p.xyz"))
    b = Batch([(L, L, L)] * n, seeds=[81 + s for s in range(n)], ncrystal=2, list_crystal=(14, 6), sf=d["sf"])
    b.set_rates(np.stack([d["ptransE"]] * n), np.stack([d["ptransD"]] * n))
    for r in range(n):
        b.init_points(r, pts, sp)
    start = np.array([o["atoms"] for o in b.observables()], float)
    tau = float(b.suggest_tau(accurate_f(2))[0])
    nwin = int(math.ceil(t_obs / tau))
    b.run(t_obs / nwin, nwin)
    obs = b.observables()
    b.close()
    g = np.array([o["atoms"] for o in obs], float)
    gc = np.array([o["species"][1] for o in obs], float)
    assert g.mean() - start.mean() > 1000
    for name, x, y in (("atoms", g, ref), ("C atoms", gc, ref_c)):
        diff, hw = band(x, y)
        print(f"SiC facets {name}: gpu {x.mean():.1f}+-{x.std(ddof=1):.1f} serial {y.mean():.1f}+-{y.std(ddof=1):.1f} "
              f"diff {diff:.1f} 3-sigma band +-{hw:.1f} (tau {tau:.3e}, {nwin} windows)")
        assert abs(diff) <= hw, name


def _cvd_oracle(args):
    """One RunType R oracle run of the CVD case to t_obs: (atoms, covered)."""
    import sys
    path, t_obs, root = args
    sys.path.insert(0, root)
    from oracle import ora
    o = ora.Oracle(path, 480, 480, 480, numbers=None)
    o.init()
    o.run_until(t_obs)
    st, _ = ora.compact_state(o)
    out = (o.atoms(), int(np.count_nonzero((st & 3) == 3)))
    o.close()
    return out


@pytest.mark.parametrize("f", [0.3, 0.03])
def test_cvd_hydrogen_coverage_matches_serial_reference(oracle_lib, tmp_path, f):
    """CVD of Si(001) under one coverage species (H), the rates of the
    reference's CVD-Si-SiH2 case (deposition 85/s, absorption 287/s and
    desorption 40/s per site, evaporation keyed by covered neighbours),
    RunType R: atoms and covered sites at t = 3 s, 16 oracle seeds against 16
    GPU replicas at the window factors f = 0.3 (the one-crystal-species rule
    mulskips.e uses) and 0.03."""
    import multiprocessing as mp
    from mulskips_gb300 import Batch
    from mulskips_gb300.startdat import parse_startdat
    from conftest import GOLDEN, ROOT
    t_obs, n = 3.0, 16
    txt = open(os.path.join(GOLDEN, "CVD-Si-SiH2", "start.dat")).read().replace(
        "T ! RunType", "R ! RunType")
    paths = []
    for s in range(n):
        p = tmp_path / f"cvd{s}.dat"
        p.write_text(txt.replace("9117116 ! Random seed", f"{500 + s} ! Random seed"))
        paths.append(str(p))
    with mp.get_context("spawn").Pool(min(n, os.cpu_count() or 1)) as pool:
        ref = np.array(pool.map(_cvd_oracle, [(p, t_obs, ROOT) for p in paths]), float)
    d = parse_startdat(paths[0])
    assert d["run_type"] == "R" and d["list_cov"] == [1]
    b = Batch([(480, 480, 480)] * n, seeds=[71 + s for s in range(n)], sf=d["sf"], list_cov=d["list_cov"])
    b.set_rates(np.stack([d["ptransE"]] * n), np.stack([d["ptransD"]] * n))
    b.set_coverage_rates(np.stack([d["ptransAbs"][:, 1:]] * n), np.stack([d["ptransDes"][:, 1:]] * n))
    b.init_flat("S", [48] * n)
    tau = float(b.suggest_tau(f)[0])
    nwin = int(math.ceil(t_obs / tau))
    b.run(t_obs / nwin, nwin)
    obs = b.observables()
    b.close()
    g = np.array([(o["atoms"], o["covered"]) for o in obs], float)
    print(f"\nCVD tau {t_obs / nwin:.3e} ({nwin} windows)")
    for k, name in enumerate(("atoms", "covered")):
        diff, hw = band(g[:, k], ref[:, k])
        print(f"{name}: gpu {g[:, k].mean():.1f}+-{g[:, k].std(ddof=1):.1f} serial {ref[:, k].mean():.1f}"
              f"+-{ref[:, k].std(ddof=1):.1f} diff {diff:.1f} 3-sigma band +-{hw:.1f}")
        assert abs(diff) <= hw, name
    assert ref[:, 1].mean() > 1000 and g[:, 0].mean() > 0
