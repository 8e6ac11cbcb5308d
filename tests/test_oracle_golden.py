"""The oracle (serial C restatement of the reference) reproduces the
reference's own regression outputs byte for byte
(regression-tests/input-and-references-files: Si-SL and surface, 10^7 events
each, RunType T, IDUM 9117116, 480^3 box; cube and cube-zigzag, a free-standing
3C-SiC parallelepiped (SetNC) grown for 10^7 events, the latter with
PtransZig = 0.8, i.e. arm-chair stacking through IF_Arm_Choice / FIND_SN /
FIND_NN; sphere (SetNCSp); inverted-pyramid (SetInvPOff, 3C-SiC); finfet
(SetSiFINFET, Si between walls); CVD-Si-SiH2, Si(001) under one coverage
species to a KMC time of 105 s (4.3e7 events); LA, the laser-anneal rate law on a
480x240x240 box with a per-site temperature field, 10^6 events; CAD, SetCAD
on a per-site geometry grown by CVD with one coverage species)."""
import numpy as np
import gzip
import os
import re
import shutil
import subprocess

import pytest

from conftest import GOLDEN, ROOT

LA_BOX = ("480", "240", "240")

ORACLE_EXE = os.path.join(ROOT, "oracle", "_build", "mks_oracle")


def run_case(case, tmp_path):
    d = tmp_path / case
    d.mkdir()
    shutil.copy(os.path.join(GOLDEN, case, "start.dat"), d / "start.dat")
    r = subprocess.run([ORACLE_EXE, "480", "480", "480", os.path.join(GOLDEN, "numberslist.txt")], cwd=d,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    return d, r.stdout


def golden_log_numbers(case):
    txt = open(os.path.join(GOLDEN, case, "log.txt")).read()
    m = re.search(r"Iter, Time, Site\s+(\d+)\s+([0-9.Ee+-]+)\s+(\d+)\s+(\d+)\s+(\d+)", txt)
    n = re.search(r"NatNvoidNad\s+(\d+)\s+(\d+)\s+(\d+)", txt)
    return m.groups(), n.groups()


@pytest.mark.parametrize("case", ["Si-SL", "surface", "cube", "cube-zigzag", "sphere", "inverted-pyramid", "finfet",
                                  "CVD-Si-SiH2"])
def test_regression_frames_identical(case, oracle_lib, tmp_path):
    d, out = run_case(case, tmp_path)
    for fr in ("I00000000", "I00000001"):
        with gzip.open(os.path.join(GOLDEN, case, fr + ".xyz.gz"), "rb") as f:
            gold = f.read()
        mine = (d / (fr + ".xyz")).read_bytes()
        assert mine == gold, f"{case} {fr}.xyz differs from the reference"
    (it, t, x, y, z), (nat, nvoid, nad) = golden_log_numbers(case)
    m = re.search(r"Iter, Time, Site\s+(\d+)\s+([0-9.Ee+-]+)\s+(\d+)\s+(\d+)\s+(\d+)", out)
    assert m.group(1) == it and (m.group(3), m.group(4), m.group(5)) == (x, y, z)
    assert abs(float(m.group(2)) - float(t)) <= 1e-10 * abs(float(t))
    n = re.search(r"NatNvoidNad\s+(\d+)\s+(\d+)\s+(\d+)", out)
    assert n.groups() == (nat, nvoid, nad)


def test_la_regression_frames_identical(oracle_lib, tmp_path):
    """InitSt LA: SetT + SetCAD on the regression input (tests/golden/LA:
    LattGeo per layer, TempStat at the 3-grid points) and the LA law of
    Get_Prob.f:127-149 / Get_Prob_Ini.f:60-77 with RunType T.  The reference
    frames were written by a SetCAD that applied LattGeo line z-4 to layer z
    (it did not skip the file's four wall lines; the LaserAnnealing SetCAD
    notes this shift of the old geometry), so the layers are fed shifted."""
    d = tmp_path / "LA"
    d.mkdir()
    shutil.copy(os.path.join(GOLDEN, "LA", "start.dat"), d / "start.dat")
    geo = np.load(os.path.join(GOLDEN, "LA", "geo_layers.npy")).astype(np.int8)
    shifted = geo.copy()
    shifted[4:] = geo[:-4]
    shifted.tofile(d / "geo.bin")
    np.load(os.path.join(GOLDEN, "LA", "temp_sub.npz"))["t"].astype(np.int16).tofile(d / "temp.bin")
    r = subprocess.run([ORACLE_EXE, *LA_BOX, os.path.join(GOLDEN, "numberslist.txt"), "0", str(d / "geo.bin"),
                        str(d / "temp.bin")], cwd=d, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    for fr in ("I00000000", "I00000001"):
        with gzip.open(os.path.join(GOLDEN, "LA", fr + ".xyz.gz"), "rb") as f:
            gold = f.read()
        assert (d / (fr + ".xyz")).read_bytes() == gold, f"LA {fr}.xyz differs from the reference"
    (it, t, x, y, z), (nat, nvoid, nad) = golden_log_numbers("LA")
    m = re.search(r"Iter, Time, Site\s+(\d+)\s+([0-9.Ee+-]+)\s+(\d+)\s+(\d+)\s+(\d+)", r.stdout)
    assert m.group(1) == it and (m.group(3), m.group(4), m.group(5)) == (x, y, z)
    assert abs(float(m.group(2)) - float(t)) <= 1e-10 * abs(float(t))
    n = re.search(r"NatNvoidNad\s+(\d+)\s+(\d+)\s+(\d+)", r.stdout)
    assert n.groups() == (nat, nvoid, nad)
    assert "Atoms,Voids,AdAtoms 63828 0 2856" in " ".join(r.stdout.split())


def test_cad_regression_frames_identical(oracle_lib, tmp_path):
    """InitSt IN: SetCAD on the per-site regression geometry (tests/golden/CAD,
    480x240x240, Si below a patterned wall layer) grown by CVD with one
    coverage species (H: PtransAbs / PtransDes, SetProbability.f and
    Get_Prob.f's coverage branches), 3e6 events, RunType T.  As for the LA
    case the reference frames come from a SetCAD that applied LattGeo line
    z-4 to layer z, so the geometry is fed shifted by four layers."""
    d = tmp_path / "CAD"
    d.mkdir()
    shutil.copy(os.path.join(GOLDEN, "CAD", "start.dat"), d / "start.dat")
    geo = np.load(os.path.join(GOLDEN, "CAD", "geo.npz"))["g"].astype(np.int8)
    shifted = geo.copy()
    shifted[4:] = geo[:-4]
    shifted.tofile(d / "geo.bin")
    r = subprocess.run([ORACLE_EXE, *LA_BOX, os.path.join(GOLDEN, "numberslist.txt"), "0", str(d / "geo.bin")],
                       cwd=d, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    for fr in ("I00000000", "I00000001"):
        with gzip.open(os.path.join(GOLDEN, "CAD", fr + ".xyz.gz"), "rb") as f:
            gold = f.read()
        assert (d / (fr + ".xyz")).read_bytes() == gold, f"CAD {fr}.xyz differs from the reference"
    (it, t, x, y, z), (nat, nvoid, nad) = golden_log_numbers("CAD")
    m = re.search(r"Iter, Time, Site\s+(\d+)\s+([0-9.Ee+-]+)\s+(\d+)\s+(\d+)\s+(\d+)", r.stdout)
    assert m.group(1) == it and (m.group(3), m.group(4), m.group(5)) == (x, y, z)
    assert abs(float(m.group(2)) - float(t)) <= 1e-10 * abs(float(t))
    n = re.search(r"NatNvoidNad\s+(\d+)\s+(\d+)\s+(\d+)", r.stdout)
    assert n.groups() == (nat, nvoid, nad)
    assert "Atoms,Voids,AdAtoms 78400 0 3198" in " ".join(r.stdout.split())


def test_ran3_is_deterministic_and_in_range(oracle_lib):
    a = oracle_lib.ran3_sequence(9117116, 1000)
    b = oracle_lib.ran3_sequence(9117116, 1000)
    assert (a == b).all() and (a >= 0).all() and (a < 1).all()
    assert not (a == oracle_lib.ran3_sequence(1, 1000)).all()


def test_numbers_list_fixture():
    vals = [float(v) for v in open(os.path.join(GOLDEN, "numberslist.txt")).read().split()]
    assert len(vals) == 1000 and all(0 < v < 1 for v in vals)
