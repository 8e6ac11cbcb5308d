"""The one-byte site rules of mulskips_gb300/csrc/lattice.cuh, compiled for
the host by a test helper, track the oracle exactly: every site byte, the
rate-class histogram (against the oracle's own list-based census) and every
MC site's rate, along the reference's event sequence."""
import os
import subprocess

import pytest

from conftest import GOLDEN, ROOT

HELPER_SRC = os.path.join(ROOT, "tests", "native", "compact_check.cpp")


@pytest.fixture(scope="module")
def helper(tmp_path_factory, oracle_lib):
    exe = str(tmp_path_factory.mktemp("native") / "compact_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", exe, HELPER_SRC,
                    os.path.join(ROOT, "oracle", "mks_oracle.c"), "-lm"], check=True)
    return exe


def run(helper, startdat, len1, kind, events, chunk):
    r = subprocess.run([helper, startdat, os.path.join(GOLDEN, "numberslist.txt"), str(len1), "480", kind,
                        str(events), str(chunk)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout[-3000:]
    return r.stdout


def test_si001_trace(helper):
    out = run(helper, os.path.join(GOLDEN, "Si-SL", "start.dat"), 360, "S", 3000000, 1000000)
    assert out.count("state_mismatch 0 hist_mismatch 0 rate_mismatch 0 offgrid 0") == 4


def test_sic001_trace(helper):
    out = run(helper, os.path.join(GOLDEN, "surface", "start.dat"), 120, "C", 2000000, 1000000)
    assert out.count("state_mismatch 0 hist_mismatch 0 rate_mismatch 0 offgrid 0") == 3


def test_etch_to_walls(helper, tmp_path):
    """Config-0 rates (T=1100 K): the slab etches away and the run ends on the
    reference's few-MC-particles rule; the walls are exercised."""
    from mulskips_gb300.startdat import write_plain_si_startdat
    p = tmp_path / "start.dat"
    write_plain_si_startdat(str(p), T=1100.0, len1=120, max_iter=1000000, seed=1)
    out = run(helper, str(p), 120, "S", 1000000, 50000)
    assert "oracle stopped (code 1)" in out
    assert "state_mismatch 0 hist_mismatch 0 rate_mismatch 0 offgrid 0" in out.splitlines()[-1]
