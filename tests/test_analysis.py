"""The trajectory observables of mulskips_gb300.analyze against the
reference's own post-processing (pymulskips/analyze.py), pinned by
tests/golden/analysis.json: get_surface_height of every golden frame, and
analyze_growth_rate of a synthetic frame series.  Also: the frame lines that
analyze.frame_z derives from a compact lattice are the lines of the
reference's initial frame, and the column statistics match a direct count."""
import gzip
import json
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

from mulskips_gb300 import analyze as an

FIX = json.load(open(os.path.join(GOLDEN, "analysis.json")))


def frame_lines(case, fr):
    with gzip.open(os.path.join(GOLDEN, case, fr + ".xyz.gz"), "rt") as f:
        lines = f.read().splitlines()
    return lines[0], lines[1], lines[2:]


def zl_of(box):
    return float(box.split()[3])


@pytest.mark.parametrize("key", sorted(FIX["surface_height"]))
def test_surface_height_matches_reference(key):
    case, fr = key.split("/")
    _, box, body = frame_lines(case, fr)
    z = np.array([float(l.split()[3]) for l in body])
    assert an.surface_height(z, zl_of(box)) == FIX["surface_height"][key]
    assert an.surface_height(z, zl_of(box), 3.0, 10.0) == FIX["surface_height_b3_r10"][key]


@pytest.mark.parametrize("method", ["finitediff", "polyfit"])
def test_growth_rate_matches_reference(method):
    sys.path.insert(0, GOLDEN)
    from make_fixtures import growth_series
    hdr, box, body = frame_lines("Si-SL", "I00000001")
    times, heights = [], []
    for k in range(9):
        t, fl = growth_series(body, k)
        times.append(float(repr(t)))
        heights.append(an.surface_height(np.array([float(l.split()[3]) for l in fl]), zl_of(box)))
    ref = FIX["growth"][method]
    assert np.allclose(heights, ref["heights"], rtol=0, atol=1e-9)
    _, rate = an.growth_rate(times, heights, method)
    assert rate == pytest.approx(ref["rate"], rel=1e-9)


@pytest.mark.parametrize("case", ["Si-SL", "surface", "CVD-Si-SiH2", "cube", "sphere"])
def test_frame_lines_of_initial_lattice(oracle_lib, case):
    """The oracle's initial lattice (pinned to the reference's I00000000.xyz)
    as a compact state gives, through frame_z, the z values of that frame's
    lines and so the same surface height."""
    from mulskips_gb300.startdat import parse_startdat
    start = os.path.join(GOLDEN, case, "start.dat")
    d = parse_startdat(start)
    o = oracle_lib.Oracle(start, 480, 480, 480)
    o.init()
    st, off = oracle_lib.compact_state(o)
    o.close()
    assert off == 0
    hdr, box, body = frame_lines(case, "I00000000")
    zf = np.sort(np.array([float(l.split()[3]) for l in body]))
    z = an.frame_z(st, d["sf"], cov=bool(d["list_cov"]))
    assert len(z) == int(hdr.split()[0]) == len(zf)
    assert np.allclose(np.sort(z), zf, rtol=0, atol=1e-5)
    assert an.surface_height(z, zl_of(box)) == pytest.approx(FIX["surface_height"][case + "/I00000000"], abs=1e-6)


def test_column_heights_by_direct_count():
    rng = np.random.default_rng(3)
    st = np.zeros((20, 8, 8), np.uint8)
    st[:3] = 0x80
    tops = rng.integers(3, 18, size=(8, 8))
    for b in range(8):
        for a in range(8):
            if (a + b) % 5 == 0:
                continue                                # an empty column
            for z in range(3, tops[b, a] + 1):
                st[z, b, a] = 0x11                      # species 1, coordination 4
    h = an.column_heights(st)
    exp = np.where((np.arange(8)[None, :] + np.arange(8)[:, None]) % 5 == 0, -1, 3 * tops)
    assert np.array_equal(h, exp)
    m, r = an.height_stats(st)
    v = exp[exp >= 0].astype(float)
    assert m == pytest.approx(v.mean()) and r == pytest.approx(v.std())
