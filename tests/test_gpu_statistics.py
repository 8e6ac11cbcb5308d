"""Statistical parity of the sublattice KMC with the serial reference.

The sublattice engine and the serial reference are different samplers of the
same process: each test runs 32 GPU replicas (exponential waiting times,
synchronous sublattice windows of length tau, stated per test) and 32 seeds
of the serial oracle (RunType R: the reference's own dynamics with dt =
1/R_tot), each replica or seed with its own seed, and compares the means of
the trajectory observables the reference itself reports:

  atoms        atoms in the box at t_obs (the net grown or etched amount),
  growth rate  pymulskips' analyze_growth_rate ('finitediff', Nexclude = 2;
               pymulskips/analyze.py:209-416) of the surface heights
               (get_surface_height, :124-207) of nine frames at t = 0, t_obs/8,
               ..., t_obs, in micron/hour (mulskips_gb300.analyze restates
               both and is pinned to them by tests/test_analysis.py),
  RMS          RMS roughness of the column heights at t_obs,
  C atoms / covered sites where the model has them (3C-SiC / CVD coverage).

Band: Welch's two-sample t band of the difference of the means at level
1 - 0.05/k for each of the k observables of a test (Bonferroni), i.e. 95 %
confidence for the test as a whole (tests/stat_bands.py).  The window
length is stated per case as f = tau * r*, r* the rate of the class that
carries the largest share of the replica's rate (mks_suggest_tau)."""
import math
import multiprocessing as mp
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from stat_bands import Family

pytestmark = pytest.mark.gpu

NSEEDS = 32
NFRAMES = 8
KB = 0.00008617330350


def k2(T):
    """Coordination-2 evaporation rate of the plain Si(001) model."""
    return 1e13 * math.exp(-1.2 / (KB * T))


def _oracle_run(args):
    """One serial oracle run (RunType R): frames at `times`; returns (frame
    times, surface heights, observables of the last frame)."""
    import sys
    path, box, times, sf, cov, root = args
    sys.path.insert(0, root)
    from oracle import ora
    from mulskips_gb300 import analyze as an
    o = ora.Oracle(path, box[0], box[1], box[2], numbers=None)
    o.init()
    zl = box[2] * sf
    st, _ = ora.compact_state(o)
    ts, hs = [0.0], [an.surface_height(an.frame_z(st, sf, cov), zl)]
    for t in times:
        o.run_until(t)
        st, off = ora.compact_state(o)
        assert off == 0
        ts.append(o.time)
        hs.append(an.surface_height(an.frame_z(st, sf, cov), zl))
    obs = an.state_observables(st, cov)
    assert obs["atoms"] == o.atoms()
    o.close()
    return ts, hs, obs


def oracle_sample(paths, box, t_obs, sf, cov=False):
    """Serial runs of the start.dat files `paths` in parallel processes."""
    times = [t_obs * (k + 1) / NFRAMES for k in range(NFRAMES)]
    with mp.get_context("spawn").Pool(min(len(paths), os.cpu_count() or 1)) as pool:
        return pool.map(_oracle_run, [(p, box, times, sf, cov, ROOT) for p in paths])


def gpu_sample(b, tau, nwin, box, sf, cov=False):
    """Run batch b for nwin windows of length tau in NFRAMES chunks; returns
    per replica (frame times, surface heights, observables at the end)."""
    from mulskips_gb300 import analyze as an
    assert nwin % NFRAMES == 0
    zl = box[2] * sf
    hs = [[an.surface_height(an.frame_z(b.state(r), sf, cov), zl)] for r in range(b.n)]
    for k in range(NFRAMES):
        b.run(tau, nwin // NFRAMES)
        for r in range(b.n):
            hs[r].append(an.surface_height(an.frame_z(b.state(r), sf, cov), zl))
    obs = b.observables()
    ts = [tau * nwin * k / NFRAMES for k in range(NFRAMES + 1)]
    for r in range(b.n):
        assert abs(obs[r]["time"] - ts[-1]) <= 1e-9 * ts[-1], "a replica stopped early"
        # the device's column statistics are the host definition's
        so = an.state_observables(b.state(r), cov)
        m, rms = so["mean_height"], so["rms_roughness"]
        assert abs(obs[r]["mean_height"] - m) < 1e-9 * max(1.0, m) and abs(obs[r]["rms_roughness"] - rms) < 1e-9 * max(1.0, rms)
        assert obs[r]["covered"] == so["covered"]
        obs[r]["covered2"] = so["covered2"]        # the device's count holds both coverage species
    return [(ts, hs[r], obs[r]) for r in range(b.n)]


def growth(sample):
    from mulskips_gb300 import analyze as an
    return np.array([an.growth_rate(ts, hs)[1] for ts, hs, _ in sample])


def column(sample, key, idx=None):
    return np.array([o[key] if idx is None else o[key][idx] for _, _, o in sample], dtype=float)


def windows_for(t_obs, tau):
    """Window count: a multiple of the frame count, windows no longer than tau."""
    return NFRAMES * int(math.ceil(t_obs / tau / NFRAMES))


def startdats(tmp_path, case, runtype_line, seed0, n, name):
    txt = open(os.path.join(GOLDEN, case, "start.dat")).read()
    a, b_ = runtype_line
    assert a in txt
    txt = txt.replace(a, b_)
    paths = []
    for s in range(n):
        p = tmp_path / f"{name}{s}.dat"
        p.write_text(txt.replace("9117116 ! Random seed", f"{seed0 + s} ! Random seed"))
        paths.append(str(p))
    return paths


# ---------------------------------------------------------------- etch (the benchmark's model)
_ETCH_REF = {}


def etch_oracle(tmp_path_factory, T):
    """32 serial runs of the plain Si(001) model at T (480^3 box, Len1 = 120),
    to t_obs = 4e-7 s x k2(1100 K) / k2(T) (the same etched amount at each T)."""
    if T not in _ETCH_REF:
        from mulskips_gb300.startdat import write_plain_si_startdat
        tmp = tmp_path_factory.mktemp(f"etch{int(T)}")
        paths = []
        for s in range(NSEEDS):
            p = tmp / f"start{s}.dat"
            write_plain_si_startdat(str(p), T=T, len1=120, max_iter=10 ** 9, seed=100 + s)
            paths.append(str(p))
        t_obs = 4e-7 * k2(1100.0) / k2(T)
        _ETCH_REF[T] = (t_obs, oracle_sample(paths, (480, 480, 480), t_obs, 0.4525))
    return _ETCH_REF[T]


# (T, tile width, k2 tau, colours): the benchmark's window rule f = 0.3 at
# tile widths 6 and 8 (brick tiling, three colours) at its three
# temperatures, on the same model in a 480^3 box; width 6 on the four-colour
# grid; a shorter window at width 8
@pytest.mark.parametrize("T,width,f,colours", [(1000.0, 6, 0.3, 3), (1100.0, 6, 0.3, 3), (1200.0, 6, 0.3, 3),
                                               (1000.0, 8, 0.3, 3), (1100.0, 8, 0.3, 3), (1200.0, 8, 0.3, 3),
                                               (1100.0, 6, 0.3, 4), (1100.0, 8, 0.064, 3)])
def test_etch_matches_serial_reference(tmp_path_factory, T, width, f, colours):
    from mulskips_gb300 import Batch, arrhenius_tables
    t_obs, ref = etch_oracle(tmp_path_factory, T)
    pE, pD = arrhenius_tables(T)
    b = Batch([(480, 480, 480)] * NSEEDS, seeds=[1 + s for s in range(NSEEDS)], sf=0.4525)
    b.set_rates(np.stack([pE] * NSEEDS), np.stack([pD] * NSEEDS))
    b.init_flat("S", [120] * NSEEDS)
    b.set_tiling(width)
    b.set_colours(colours)
    assert b.colours() == colours
    nwin = windows_for(t_obs, f / k2(T))
    tau = t_obs / nwin
    g = gpu_sample(b, tau, nwin, (480, 480, 480), 0.4525)
    b.close()
    fam = Family(f"etch T={T:.0f} K width {width} colours {colours} k2*tau={k2(T) * tau:.3f} ({nwin} windows)", 3)
    fam.add("atoms", column(g, "atoms"), column(ref, "atoms"))
    fam.add("growth rate um/h", growth(g), growth(ref))
    fam.add("RMS roughness", column(g, "rms_roughness"), column(ref, "rms_roughness"))
    assert column(ref, "atoms").mean() < 3200 * 36 - 5000          # etching happened
    fam.check()


# ---------------------------------------------------------------- deposition + evaporation
def test_deposition_evaporation_regime_matches_serial_reference(tmp_path):
    """The Si-SL regression rates with RunType R (deposition 9.3e-4 against
    coor-2 evaporation 2.0e-3, so both event kinds matter): t_obs = 1e4 s at
    the single-species window f = 0.3."""
    from mulskips_gb300 import Batch
    from mulskips_gb300.startdat import parse_startdat
    paths = startdats(tmp_path, "Si-SL", ("T   ! R = production run", "R   ! R = production run"), 200, NSEEDS, "sl")
    d = parse_startdat(paths[0])
    ref = oracle_sample(paths, (480, 480, 480), 1e4, d["sf"])
    b = Batch([(480, 480, 480)] * NSEEDS, seeds=[31 + s for s in range(NSEEDS)], sf=d["sf"])
    b.set_rates(np.stack([d["ptransE"]] * NSEEDS), np.stack([d["ptransD"]] * NSEEDS))
    b.init_flat("S", [360] * NSEEDS)
    nwin = windows_for(1e4, float(b.suggest_tau(0.3)[0]))
    g = gpu_sample(b, 1e4 / nwin, nwin, (480, 480, 480), d["sf"])
    b.close()
    fam = Family(f"Si-SL rates, f = 0.3 ({nwin} windows)", 3)
    fam.add("atoms", column(g, "atoms"), column(ref, "atoms"))
    fam.add("growth rate um/h", growth(g), growth(ref))
    fam.add("RMS roughness", column(g, "rms_roughness"), column(ref, "rms_roughness"))
    fam.check()


# ---------------------------------------------------------------- 3C-SiC
_SURFACE_REF = {}


@pytest.mark.parametrize("window", ["fixed", "tuned"])
def test_sic_surface_matches_serial_reference(tmp_path_factory, window):
    """3C-SiC(001), the rates of the reference's `surface` regression case
    (NCrystal 2, Si and C with 18 census-dependent evaporation rates), RunType
    R, t_obs = 2e5 s, at the two-species window factor ("fixed",
    autotune.accurate_f) and at the factor the pilot tuner picks for these
    rates ("tuned", autotune.choose_f on 16 pilot replicas of its own seeds)."""
    from mulskips_gb300 import Batch
    from mulskips_gb300.autotune import accurate_f, choose_f
    from mulskips_gb300.startdat import parse_startdat
    if "ref" not in _SURFACE_REF:
        tmp = tmp_path_factory.mktemp("sic")
        paths = startdats(tmp, "surface", ("T   ! R = production run", "R   ! R = production run"), 400, NSEEDS,
                          "sic")
        d = parse_startdat(paths[0])
        _SURFACE_REF["ref"] = (d, oracle_sample(paths, (480, 480, 480), 2e5, d["sf"]))
    d, ref = _SURFACE_REF["ref"]

    def make(n, seed0):
        b = Batch([(480, 480, 480)] * n, seeds=[seed0 + s for s in range(n)], ncrystal=2, list_crystal=(14, 6),
                  sf=d["sf"])
        b.set_rates(np.stack([d["ptransE"]] * n), np.stack([d["ptransD"]] * n))
        b.init_flat("C", [d["len"][0]] * n)
        return b

    pilots = None
    if window == "fixed":
        f = accurate_f(2)
    else:
        f, pilots = choose_f(lambda f_: make(16, 900), 2e5)
    b = make(NSEEDS, 51)
    nwin = windows_for(2e5, float(b.suggest_tau(f)[0]))
    g = gpu_sample(b, 2e5 / nwin, nwin, (480, 480, 480), d["sf"])
    b.close()
    fam = Family(f"3C-SiC(001) surface rates, {window} f = {f} ({nwin} windows)", 4, extra={"pilots": pilots})
    fam.add("atoms", column(g, "atoms"), column(ref, "atoms"))
    fam.add("C atoms", column(g, "species", 1), column(ref, "species", 1))
    fam.add("growth rate um/h", growth(g), growth(ref))
    fam.add("RMS roughness", column(g, "rms_roughness"), column(ref, "rms_roughness"))
    fam.check()


def test_sic_facets_match_serial_reference(tmp_path):
    """3C-SiC on {111} facets: a square pyramid with {111} faces on a (001)
    slab (InitSt SH point list, 240^3 box), the rates of the reference's
    `surface` case, RunType R, t_obs = 2e5 s (about 2.5e5 events, the facets
    filling in), at the two-species window factor."""
    from mulskips_gb300 import Batch
    from mulskips_gb300.autotune import accurate_f
    from mulskips_gb300.startdat import parse_startdat, read_shape_points
    from test_shape_points import pyramid_points, sh_startdat, write_points
    L, t_obs = 240, 2e5
    xyz, sym, _, _ = pyramid_points(L, 60, 54)
    write_points(tmp_path / "p.xyz", xyz, sym)
    txt = open(os.path.join(GOLDEN, "surface", "start.dat")).read().replace(
        "T   ! R = production run", "R   ! R = production run")
    paths = []
    for s in range(NSEEDS):
        p = tmp_path / f"fac{s}.dat"
        sh_startdat(txt.replace("9117116 ! Random seed", f"{600 + s} ! Random seed").splitlines(), p,
                    str(tmp_path / "p.xyz"))
        paths.append(str(p))
    d = parse_startdat(paths[0])
    ref = oracle_sample(paths, (L, L, L), t_obs, d["sf"])
    pts, sp = read_shape_points(str(tmp_path / "p.xyz"))
    b = Batch([(L, L, L)] * NSEEDS, seeds=[81 + s for s in range(NSEEDS)], ncrystal=2, list_crystal=(14, 6),
              sf=d["sf"])
    b.set_rates(np.stack([d["ptransE"]] * NSEEDS), np.stack([d["ptransD"]] * NSEEDS))
    for r in range(NSEEDS):
        b.init_points(r, pts, sp)
    start = np.array([o["atoms"] for o in b.observables()], float)
    f = accurate_f(2)
    nwin = windows_for(t_obs, float(b.suggest_tau(f)[0]))
    g = gpu_sample(b, t_obs / nwin, nwin, (L, L, L), d["sf"])
    b.close()
    assert column(g, "atoms").mean() - start.mean() > 1000
    fam = Family(f"3C-SiC {{111}} facets, f = {f} ({nwin} windows)", 3)
    fam.add("atoms", column(g, "atoms"), column(ref, "atoms"))
    fam.add("C atoms", column(g, "species", 1), column(ref, "species", 1))
    fam.add("RMS roughness", column(g, "rms_roughness"), column(ref, "rms_roughness"))
    fam.check()


# ---------------------------------------------------------------- CVD with two coverage species
def test_cvd_two_coverage_species_match_serial_reference(tmp_path):
    """CVD of Si(001) under H and Cl (tests/cvd2.py: two coverage species,
    absorption split by IndexEvent_Abs, Get_Prob.f:22-52, atom rates keyed by
    covered neighbours of each species), RunType R, t_obs = 3 s, f = 0.3:
    atoms, H- and Cl-covered sites, growth rate and RMS roughness."""
    from cvd2 import two_coverage_startdat
    from mulskips_gb300 import Batch
    from mulskips_gb300.startdat import parse_startdat
    t_obs, f = 3.0, 0.3
    paths = [two_coverage_startdat(str(tmp_path / f"c2_{s}.dat"), "R", 700 + s, 100.0) for s in range(NSEEDS)]
    d = parse_startdat(paths[0])
    assert d["run_type"] == "R" and d["list_cov"] == [1, 17]
    ref = oracle_sample(paths, (480, 480, 480), t_obs, d["sf"], cov=True)
    b = Batch([(480, 480, 480)] * NSEEDS, seeds=[171 + s for s in range(NSEEDS)], sf=d["sf"], list_cov=d["list_cov"])
    b.set_rates(np.stack([d["ptransE"]] * NSEEDS), np.stack([d["ptransD"]] * NSEEDS))
    b.set_coverage_rates(np.stack([d["ptransAbs"][:, 1:]] * NSEEDS), np.stack([d["ptransDes"][:, 1:]] * NSEEDS))
    b.init_flat("S", [48] * NSEEDS)
    nwin = windows_for(t_obs, float(b.suggest_tau(f)[0]))
    g = gpu_sample(b, t_obs / nwin, nwin, (480, 480, 480), d["sf"], cov=True)
    b.close()
    fam = Family(f"CVD Si(001) + H + Cl, f = {f} ({nwin} windows)", 5)
    fam.add("atoms", column(g, "atoms"), column(ref, "atoms"))
    fam.add("H-covered sites", column(g, "covered") - column(g, "covered2"),
            column(ref, "covered") - column(ref, "covered2"))
    fam.add("Cl-covered sites", column(g, "covered2"), column(ref, "covered2"))
    fam.add("growth rate um/h", growth(g), growth(ref))
    fam.add("RMS roughness", column(g, "rms_roughness"), column(ref, "rms_roughness"))
    assert column(ref, "covered2").mean() > 100
    fam.check()


# ---------------------------------------------------------------- CVD with hydrogen coverage
_CVD_REF = {}


@pytest.mark.parametrize("f", [0.3, 0.03])
def test_cvd_hydrogen_coverage_matches_serial_reference(tmp_path_factory, f):
    """CVD of Si(001) under one coverage species (H), the rates of the
    reference's CVD-Si-SiH2 case (deposition 85/s, absorption 287/s and
    desorption 40/s per site, evaporation keyed by covered neighbours),
    RunType R, t_obs = 3 s, at the window factors f = 0.3 (the one-crystal-
    species rule mulskips.e uses) and 0.03."""
    from mulskips_gb300 import Batch
    from mulskips_gb300.startdat import parse_startdat
    t_obs = 3.0
    if "ref" not in _CVD_REF:
        tmp = tmp_path_factory.mktemp("cvd")
        paths = startdats(tmp, "CVD-Si-SiH2", ("T ! RunType", "R ! RunType"), 500, NSEEDS, "cvd")
        d = parse_startdat(paths[0])
        assert d["run_type"] == "R" and d["list_cov"] == [1]
        _CVD_REF["ref"] = (d, oracle_sample(paths, (480, 480, 480), t_obs, d["sf"], cov=True))
    d, ref = _CVD_REF["ref"]
    b = Batch([(480, 480, 480)] * NSEEDS, seeds=[71 + s for s in range(NSEEDS)], sf=d["sf"], list_cov=d["list_cov"])
    b.set_rates(np.stack([d["ptransE"]] * NSEEDS), np.stack([d["ptransD"]] * NSEEDS))
    b.set_coverage_rates(np.stack([d["ptransAbs"][:, 1:]] * NSEEDS), np.stack([d["ptransDes"][:, 1:]] * NSEEDS))
    b.init_flat("S", [48] * NSEEDS)
    nwin = windows_for(t_obs, float(b.suggest_tau(f)[0]))
    g = gpu_sample(b, t_obs / nwin, nwin, (480, 480, 480), d["sf"], cov=True)
    b.close()
    fam = Family(f"CVD Si(001) + H, f = {f} ({nwin} windows)", 4)
    fam.add("atoms", column(g, "atoms"), column(ref, "atoms"))
    fam.add("covered sites", column(g, "covered"), column(ref, "covered"))
    fam.add("growth rate um/h", growth(g), growth(ref))
    fam.add("RMS roughness", column(g, "rms_roughness"), column(ref, "rms_roughness"))
    assert column(ref, "covered").mean() > 1000 and column(g, "atoms").mean() > 0
    fam.check()
