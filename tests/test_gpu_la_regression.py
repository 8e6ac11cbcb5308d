"""The GPU's LA law on the reference's own LA regression input (GPU).

The 480x240x240 box of regression-tests' LA case (a Si slab with a molten
spherical pocket under a nearly uniform 1655-1661 K field; P0 = 1.33e17,
Tm = 1688 K, A = 280 K, Tflex = 1080 K, E = 0.96 eV per bond): the initial
lattice and per-site temperatures come from the oracle's InitSt LA
initializer (pinned byte for byte to the reference's frames), the rate law is
mulskips-source/mcevent/Get_Prob.f:127-149 (no liquid fraction).  Atoms at
t = 2e-10 s and 4e-10 s: 32 GPU replicas (sublattice windows, exponential
waiting times) against 32 oracle runs (RunType R, the reference's clock);
the difference of the means must lie inside the 95 % family band (Welch t,
Bonferroni over the two times, tests/stat_bands.py).
"""
import math
import multiprocessing as mp
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

BOX = (480, 240, 240)
N = 32
MARKS = (2e-10, 4e-10)


def _inputs():
    geo = np.load(os.path.join(GOLDEN, "LA", "geo_layers.npy")).astype(np.int8)
    shifted = geo.copy()
    shifted[4:] = geo[:-4]          # the layers the reference run used (see test_oracle_golden)
    tsub = np.load(os.path.join(GOLDEN, "LA", "temp_sub.npz"))["t"].astype(np.int16)
    txt = open(os.path.join(GOLDEN, "LA", "start.dat")).read()
    return shifted, tsub, txt


def _startdat(txt, seed):
    out = []
    for line in txt.splitlines():
        if "! RunType" in line:
            line = "R ! RunType"
        elif "! Random seed" in line:
            line = f"{seed} ! Random seed"
        out.append(line)
    return "\n".join(out) + "\n"


@pytest.fixture(scope="module")
def oracle_runs(oracle_lib):
    geo, tsub, txt = _inputs()
    jobs = [(_startdat(txt, 300 + i), BOX, geo, tsub, MARKS) for i in range(N)]
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        res = pool.map(oracle_lib.la_regression_replica, jobs)
    return np.array([[r[k][0] for k in range(len(MARKS))] for r in res], dtype=float)


@pytest.fixture(scope="module")
def initial(oracle_lib, tmp_path_factory):
    geo, tsub, txt = _inputs()
    d = tmp_path_factory.mktemp("la0")
    p = d / "start.dat"
    p.write_text(_startdat(txt, 299))
    o = oracle_lib.Oracle(str(p), *BOX, numbers=None)
    o.set_la_input(geo, tsub)
    o.init()
    lc = o.lattcoo()
    pE, pD = o.rates()
    atoms0 = o.atoms()
    o.close()
    return lc, pE, pD, atoms0


def test_la_law_matches_oracle_on_regression_input(initial, oracle_runs):
    from mulskips_gb300 import Batch, la
    lc, pE, pD, atoms0 = initial
    b = Batch([BOX] * N, seeds=[11 + i for i in range(N)], sf=5.43 / 12)
    b.set_rates(np.stack([pE] * N), np.stack([pD] * N))
    for i in range(N):
        b.load_lattice(i, lc)
        b.load_temperature(i, lc)
    mat = la.Material(P0=(1.33e17,), Tm=(1688.0,), Tflex=(1080.0,), A=(280.0,))
    prm = la.la_params(mat, la.Pulse(), zsurf=1e30, score=False)
    prm.liquid_weighting = 0
    b.set_la(prm)
    # window: f = 0.3 over the rate of the class with the largest share at the
    # hottest temperature of the field
    Tmax = float((lc >> 9 & 8191).max())
    r = la.share_rate(b.class_histogram(), la.class_rates_tables(pE, pD, mat, Tmax))
    k = math.ceil(MARKS[0] / 8.0 / (0.3 / float(r.max())))
    tau = MARKS[0] / (8.0 * k)
    got = []
    t = 0.0
    for m in MARKS:
        nw = int(round((m - t) / tau))
        b.run(tau, nw, 0, m - 0.5 * tau)
        t = m
        got.append([o["atoms"] for o in b.observables()])
    b.close()
    got = np.array(got, dtype=float).T
    from stat_bands import Family
    fam = Family(f"LA regression lattice, initial atoms {atoms0}, tau {tau:.3e}", len(MARKS))
    for j, m in enumerate(MARKS):
        assert oracle_runs[:, j].mean() > atoms0 + 100          # the pocket regrows
        fam.add(f"atoms at t={m:.1e}", got[:, j], oracle_runs[:, j])
    fam.check()
