"""The drop-in mulskips.e (C++ host over the C ABI) on a GB300: reads the
reference's start.dat, writes the reference's frame files.  The initial
frame is deterministic and must equal the reference's I00000000.xyz byte for
byte; the run then follows the GPU engine's own dynamics."""
import gzip
import os
import shutil
import subprocess

import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu
EXE = os.path.join(ROOT, "mulskips_gb300", "_lib", "mulskips.e")


def run_exe(d, box="480 480 480"):
    env = dict(os.environ, MULSKIPS_BOX=box)
    r = subprocess.run([EXE], cwd=d, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    return r


def test_initial_frame_identical_and_run_completes(tmp_path):
    """Si-SL start.dat with the exit moved to 200000 events (the frame names
    follow Iter/OutMolMol as in the reference, so a run that stops early
    overwrites I00000000 with its final frame, like the reference)."""
    d = tmp_path / "si"
    d.mkdir()
    txt = open(os.path.join(GOLDEN, "Si-SL", "start.dat")).read()
    txt = txt.replace("10000000 ! IterMax", "200000 ! IterMax").replace("10000000  ! OutMolMol", "200000  ! OutMolMol")
    (d / "start.dat").write_text(txt)
    r = run_exe(d)
    assert r.returncode == 0, r.stdout[-3000:]
    with gzip.open(os.path.join(GOLDEN, "Si-SL", "I00000000.xyz.gz"), "rb") as f:
        gold = f.read()
    assert (d / "I00000000.xyz").read_bytes() == gold
    hdr = (d / "I00000001.xyz").read_text().splitlines()[0].split()
    assert hdr[1] == "angstroem" and int(hdr[-1]) >= 200000
    assert "NatNvoidNad" in r.stdout and "Atoms,Voids,AdAtoms" in r.stdout
    for name in ("I00000000_d.xyz", "I00000000_v.xyz", "I00000000.src", "movie.mos"):
        assert (d / name).exists()
    # movie.mos starts over in each run and lists every frame once;
    # DefAtEnergy.dat holds one blank record, Run_time.dat nothing
    assert (d / "movie.mos").read_text().count("zap") == 2
    assert (d / "DefAtEnergy.dat").read_text() == " \n"
    assert (d / "Run_time.dat").read_text() == ""
    r = run_exe(d)
    assert r.returncode == 0 and (d / "movie.mos").read_text().count("zap") == 2


def test_run_mulskips_wrapper_etch_stop(tmp_path):
    """pymulskips-style call; at 1100 K the slab etches away and the run ends
    on the few-MC-particles rule, which run_mulskips reports as False."""
    from mulskips_gb300.setuprun import PlainSi, run_mulskips
    os.environ["MULSKIPS_BOX"] = "240 240 240"
    try:
        ok = run_mulskips(runpath=str(tmp_path / "run"), Simulation="FS", mp=PlainSi(T=1100.0),
                          ExitStrategy="Iter", OutMolMol=4000, IterMax=10 ** 8, Seed_box=[72, 72, 72])
    finally:
        del os.environ["MULSKIPS_BOX"]
    assert ok is False
    log = open(tmp_path / "run" / "log.txt").read()
    assert "few MC particles: stop MC" in log
    assert (tmp_path / "run" / "I00000001.xyz").exists()


def test_cvd_start_dat_runs_with_coverage(tmp_path):
    """The reference's CVD-Si-SiH2 start.dat (one coverage species, H; Time
    exit) cut to 0.5 s: the initial frame equals the reference's byte for
    byte, and the final frame lists H lines for covered sites."""
    d = tmp_path / "cvd"
    d.mkdir()
    txt = open(os.path.join(GOLDEN, "CVD-Si-SiH2", "start.dat")).read()
    txt = txt.replace("105.144755160701223 ! TotTime", "0.5 ! TotTime").replace(
        "105.14475516070123 ! OutTime", "0.5 ! OutTime")
    (d / "start.dat").write_text(txt)
    r = run_exe(d)
    assert r.returncode == 0, r.stdout[-3000:]
    with gzip.open(os.path.join(GOLDEN, "CVD-Si-SiH2", "I00000000.xyz.gz"), "rb") as f:
        gold = f.read()
    assert (d / "I00000000.xyz").read_bytes() == gold
    assert "Coverage species (NCov= 1 )" in r.stdout
    lines = (d / "I00000001.xyz").read_text().splitlines()
    nh = sum(1 for ln in lines[2:] if ln.startswith("H "))
    assert int(lines[0].split()[0]) == len(lines) - 2 and nh > 500


def test_arm_chair_start_dat_runs(tmp_path):
    """The reference's cube-zigzag start.dat (3C-SiC parallelepiped, SetNC,
    PtransZig = 0.8: arm-chair stacking on ties, IF_Arm_Choice.f:44-51) cut
    to 1e6 events: mulskips.e runs it on the explicit-neighbour engine, its
    initial frame equals the reference's byte for byte, and every frame file
    (.xyz, the non-epitaxial bulk of _d.xyz, _v, and _w for SiC) is written
    with a header count that matches its lines."""
    d = tmp_path / "zz"
    d.mkdir()
    txt = open(os.path.join(GOLDEN, "cube-zigzag", "start.dat")).read()
    txt = txt.replace("10000000 ! IterMax", "1000000 ! IterMax").replace("10000000  ! OutMolMol",
                                                                          "1000000  ! OutMolMol")
    assert "1000000 ! IterMax" in txt
    (d / "start.dat").write_text(txt)
    r = run_exe(d)
    assert r.returncode == 0, r.stdout[-3000:]
    with gzip.open(os.path.join(GOLDEN, "cube-zigzag", "I00000000.xyz.gz"), "rb") as f:
        gold = f.read()
    assert (d / "I00000000.xyz").read_bytes() == gold
    for name in ("I00000001.xyz", "I00000001_d.xyz", "I00000001_v.xyz", "I00000001_w.xyz"):
        lines = (d / name).read_text().splitlines()
        assert int(lines[0].split()[0]) == len(lines) - 2, name
    hdr = (d / "I00000001.xyz").read_text().splitlines()[0].split()
    assert int(hdr[-1]) >= 1000000
    assert "NatNvoidNad" in r.stdout
