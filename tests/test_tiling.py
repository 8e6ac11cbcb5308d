"""The two tilings of the sublattice method (mulskips_gb300/csrc/tiling.cuh,
compiled for the host): every site in one tile, the band scan's mapping,
tiles of one colour four columns apart, near tiles listed as neighbours;
every even plane size from 16 to 96 sites and every width 4..8 (CPU)."""
import os
import subprocess

from conftest import ROOT


def test_tilings_keep_colours_apart(tmp_path):
    exe = str(tmp_path / "tiling_check")
    src = os.path.join(ROOT, "tests", "native", "tiling_check.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", src, "-o", exe], check=True)
    r = subprocess.run([exe, "96"], stdout=subprocess.PIPE, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout
