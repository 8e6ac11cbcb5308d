"""InitSt ST on the GPU: per-site rates interpolated from a probability table
(mks_batch_set_tabulated) against the oracle's ST mode (GPU).

A Si trench (SetTrenchSi, 480^3 grid, Len = 60, Len2 = 60, Len3 = 120,
70 degrees) under a temperature gradient from 1000 K at the bottom to
1250 K at the top, rates tabulated at 950, 1100 and 1300 K (all rising with
T; coor-2 evaporation comparable to deposition), RunType R.  Atoms and RMS
roughness at t = 100 s: 32 oracle runs against 32 GPU replicas loaded from
the oracle's initial LattCoo (lattice and temperatures), window 0.3 / r*
with r* the rate of the class carrying the largest share at the hottest
temperature.  The differences of the means must lie inside the 95 % family
band (Welch t, Bonferroni over the two observables, tests/stat_bands.py)."""
import math
import multiprocessing as mp
import os

import numpy as np
import pytest

from test_oracle_st import write_st

pytestmark = pytest.mark.gpu

ROWS = [(950, (3.0e2, 0.15, 0.002), (0.5, 0.5, 0.5)),
        (1100, (5.0e2, 0.3, 0.004), (0.55, 0.55, 0.55)),
        (1300, (9.0e2, 0.6, 0.008), (0.6, 0.6, 0.6))]
TTOP, TBOTTOM = 1250.0, 1000.0
T_OBS = 100.0
N = 32


def _oracle_atoms(args):
    import sys
    path, root = args
    sys.path.insert(0, root)
    from oracle import ora
    o = ora.Oracle(path, 480, 480, 480, numbers=None)
    o.init()
    o.run_until(T_OBS)
    from mulskips_gb300 import analyze as an
    st, _ = ora.compact_state(o)
    n = (o.atoms(), an.height_stats(st)[1])
    o.close()
    return n


def _tables():
    E = np.zeros((len(ROWS), 3, 4, 4, 4, 4, 4, 4))
    D = np.zeros((len(ROWS), 3, 3))
    for k, (_, e, d) in enumerate(ROWS):
        for n in range(3):
            E[k, 0, n + 1, 0, 0, 0, 0, 0] = e[n]
            D[k, 0, n] = d[n]
    return np.array([r[0] for r in ROWS]), E, D


def test_tabulated_rates_match_oracle(oracle_lib, tmp_path):
    from conftest import ROOT
    from mulskips_gb300 import Batch
    paths = [write_st(str(tmp_path / f"s{i}"), TTOP, TBOTTOM, ROWS, run_type="R", iters=10 ** 9, seed=700 + i)
             for i in range(N)]
    with mp.get_context("spawn").Pool(min(N, os.cpu_count() or 1)) as pool:
        ref = np.array(pool.map(_oracle_atoms, [(p, ROOT) for p in paths]), float)
    o = oracle_lib.Oracle(paths[0], 480, 480, 480, numbers=None)
    o.init()
    lc, atoms0 = o.lattcoo(), o.atoms()
    o.close()
    T, E, D = _tables()
    b = Batch([(480, 480, 480)] * N, seeds=[41 + i for i in range(N)], sf=0.4525)
    b.set_rates(np.stack([E[-1]] * N), np.stack([D[-1]] * N))
    for i in range(N):
        b.load_lattice(i, lc)
        b.load_temperature(i, lc)
    b.set_tabulated(np.stack([T] * N), np.stack([E] * N), np.stack([D] * N))
    # class rates at the hottest temperature: C1, C2, C3 and atoms of coordination 1..3
    w = (TTOP - 1100.0) / 200.0
    hot = lambda lo, hi: (1 - w) * lo + w * hi
    rate = np.zeros(64)
    rate[1], rate[3], rate[4] = (hot(ROWS[1][2][n], ROWS[2][2][n]) for n in range(3))
    rate[6], rate[9], rate[15] = (hot(ROWS[1][1][n], ROWS[2][1][n]) for n in range(3))
    hist = b.class_histogram()[0]
    rstar = rate[int(np.argmax(hist[:64] * rate))]
    nwin = int(math.ceil(T_OBS / (0.3 / rstar)))
    b.run(T_OBS / nwin, nwin)
    g = np.array([(x["atoms"], x["rms_roughness"]) for x in b.observables()], float)
    b.close()
    from stat_bands import Family
    fam = Family(f"ST trench, atoms0 {atoms0} ({nwin} windows)", 2)
    fam.add("atoms", g[:, 0], ref[:, 0])
    fam.add("RMS roughness", g[:, 1], ref[:, 1])
    assert abs(ref[:, 0].mean() - atoms0) > 10 * ref[:, 0].std(ddof=1) / math.sqrt(N)   # the trench evolves
    fam.check()
