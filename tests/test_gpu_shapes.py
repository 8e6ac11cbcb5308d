"""The shaped initial lattices of the library (mks_init_shape: SetNC,
SetNCSp, SetInvPOff, SetSiFINFET, SetTrenchSi) against the oracle's, which
reproduce the reference's regression frames byte for byte (GPU): the
compact lattice after initialization is identical, and mulskips.e run on the
reference's own start.dat writes the reference's initial frame byte for
byte."""
import gzip
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from test_oracle_st import write_st

pytestmark = pytest.mark.gpu
EXE = os.path.join(ROOT, "mulskips_gb300", "_lib", "mulskips.e")
CASES = ["cube", "sphere", "inverted-pyramid", "finfet"]


def _lens(d):
    k, L = d["init_st"], d["len"]
    return [L[0]] if k == "S" else ([L[0], L[1]] if k == "I" else list(L))


@pytest.mark.parametrize("case", CASES)
def test_shape_matches_oracle(oracle_lib, case):
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    start = os.path.join(GOLDEN, case, "start.dat")
    d = parse_startdat(start)
    o = oracle_lib.Oracle(start, 480, 480, 480)
    o.init()
    ref, off = oracle_lib.compact_state(o)
    o.close()
    assert off == 0
    with Lattice(480, 480, 480, ncrystal=d["ncrystal"], list_crystal=d["list_crystal"], sf=d["sf"]) as lat:
        lat.set_rates(d["ptransE"], d["ptransD"])
        lat.init_shape(d["init_st"], _lens(d))
        st = lat.state()
    bad = np.argwhere(st != ref)
    assert bad.size == 0, f"{len(bad)} sites differ, first {bad[:3]}"


def test_trench_matches_oracle(oracle_lib, tmp_path):
    from mulskips_gb300 import Lattice
    rows = [(950, (3.0e2, 0.15, 0.002), (0.5, 0.5, 0.5)), (1300, (9.0e2, 0.6, 0.008), (0.6, 0.6, 0.6))]
    p = write_st(str(tmp_path / "st"), 1250.0, 1000.0, rows, lens=(60, 60, 120, 70.0))
    o = oracle_lib.Oracle(p, 480, 480, 480)
    o.init()
    ref, _ = oracle_lib.compact_state(o)
    o.close()
    with Lattice(480, 480, 480, sf=0.4525) as lat:
        lat.init_shape("ST", [60, 60, 120], [70.0, 1250.0, 1000.0])
        st = lat.state()
    assert np.array_equal(st, ref)


@pytest.mark.parametrize("case", CASES)
def test_mulskips_e_initial_frame(tmp_path, case):
    d = tmp_path / case
    d.mkdir()
    txt = open(os.path.join(GOLDEN, case, "start.dat")).read()
    out = []
    for line in txt.splitlines():
        if "! IterMax" in line:
            line = "4000 ! IterMax"
        elif "! OutMolMol" in line:
            line = "4000 ! OutMolMol"
        out.append(line)
    (d / "start.dat").write_text("\n".join(out) + "\n")
    r = subprocess.run([EXE], cwd=d, env=dict(os.environ, MULSKIPS_BOX="480 480 480"), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    with gzip.open(os.path.join(GOLDEN, case, "I00000000.xyz.gz"), "rb") as f:
        gold = f.read()
    assert (d / "I00000000.xyz").read_bytes() == gold
    assert (d / "I00000001.xyz").exists()


def test_mulskips_e_trench_with_tables(oracle_lib, tmp_path):
    """InitSt ST through mulskips.e: the table file, SetTrenchSi and the
    per-site interpolated rates; the initial frame equals the oracle's."""
    rows = [(950, (3.0e2, 0.15, 0.002), (0.5, 0.5, 0.5)), (1100, (5.0e2, 0.3, 0.004), (0.55, 0.55, 0.55)),
            (1300, (9.0e2, 0.6, 0.008), (0.6, 0.6, 0.6))]
    d = tmp_path / "st"
    p = write_st(str(d), 1250.0, 1000.0, rows, run_type="R", iters=200000)
    o = oracle_lib.Oracle(p, 480, 480, 480, numbers=None)
    o.init()
    o.write_frame(str(tmp_path / "ora"), 0.0, 0)
    o.close()
    r = subprocess.run([EXE], cwd=d, env=dict(os.environ, MULSKIPS_BOX="480 480 480"), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert (d / "I00000000.xyz").read_text() == (tmp_path / "ora.xyz").read_text()
    hdr = (d / "I00000001.xyz").read_text().splitlines()[0].split()
    assert hdr[1] == "angstroem" and int(hdr[-1]) >= 200000


def _cad_geometry():
    return np.load(os.path.join(GOLDEN, "CAD", "geo.npz"))["g"].astype(np.int8)


def test_cad_matches_oracle(oracle_lib, tmp_path):
    """SetCAD (InitSt IN) on the reference's CAD geometry, as the current
    SetCAD.f reads it (record z to layer z)."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    start = os.path.join(GOLDEN, "CAD", "start.dat")
    d = parse_startdat(start)
    geo = _cad_geometry()
    o = oracle_lib.Oracle(start, 480, 240, 240)
    o.set_geometry(geo)
    o.init()
    ref, _ = oracle_lib.compact_state(o)
    o.close()
    with Lattice(480, 240, 240, sf=d["sf"], list_cov=d["list_cov"]) as lat:
        lat.init_cad(geo)
        st = lat.state()
    bad = np.argwhere(st != ref)
    assert bad.size == 0, f"{len(bad)} sites differ, first {bad[:3]}"


def test_mulskips_e_cad(oracle_lib, tmp_path):
    """mulskips.e with the CAD start.dat (one coverage species) and its
    geometry file: the initial frame equals the oracle's."""
    geo = _cad_geometry()
    d = tmp_path / "cad"
    d.mkdir()
    with open(d / "LattGeo.dat", "w") as f:
        for z in range(geo.shape[0]):
            f.write(" ".join(map(str, geo[z].reshape(-1).tolist())) + "\n")
    out = []
    for line in open(os.path.join(GOLDEN, "CAD", "start.dat")).read().splitlines():
        if "LattGeo" in line:
            line = "LattGeo.dat"
        elif "! IterMax" in line:
            line = "4000 ! IterMax"
        elif "! OutMolMol" in line:
            line = "4000 ! OutMolMol"
        out.append(line)
    (d / "start.dat").write_text("\n".join(out) + "\n")
    o = oracle_lib.Oracle(str(d / "start.dat"), 480, 240, 240)
    o.set_geometry(geo)
    o.init()
    o.write_frame(str(tmp_path / "ora"), 0.0, 0)
    o.close()
    r = subprocess.run([EXE], cwd=d, env=dict(os.environ, MULSKIPS_BOX="480 240 240"), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert (d / "I00000000.xyz").read_text() == (tmp_path / "ora.xyz").read_text()


def test_mulskips_e_la(oracle_lib, tmp_path):
    """InitSt LA through mulskips.e (main.f:118-138, 287-291): TempStat and
    LattGeo files, SetT + SetCAD with a molten nucleus, the law of
    Get_Prob.f:127-149 on the static field.  A 120^3 box with the LA
    regression's rates and parameters (nucleus radius 20 A): the initial
    frame equals the oracle's, and the run writes the LA phases file.  The
    run is capped at 4000 events: the nucleus solidifies to the upper wall
    within about 13000, after which the reference stops on too few MC sites
    and its final frame (index 0) would overwrite I00000000.  Each layer of
    both files is wrapped over records of 997 values, as a Fortran runtime may
    write a list-directed record: SetT's and SetCAD's READ(*) read across
    them."""
    L = 120
    d = tmp_path / "la"
    d.mkdir()
    layers = np.where(np.arange(L) < 100, 1, 10).astype(np.int8)
    layers[:4] = 10
    T = np.where(layers == 10, 10, (1650 + 0.1 * np.arange(L)).astype(np.int64))
    def wrapped(vals, n=997):
        return "".join(" ".join(vals[i:i + n]) + "\n" for i in range(0, len(vals), n))

    with open(d / "LattGeo.dat", "w") as fg, open(d / "TempStat.dat", "w") as ft:
        for z in range(L):
            fg.write(wrapped([str(int(layers[z]))] * (L * L)))
            ft.write(wrapped([str(int(T[z]))] * (L * L)))
    out, skip = [], False
    for line in open(os.path.join(GOLDEN, "LA", "start.dat")).read().splitlines():
        if skip:
            skip = False
            continue
        if line.startswith("LattGeo"):
            line = "LattGeo.dat"
        elif line.startswith("TempStat"):
            line = "TempStat.dat"
        elif "! LenNuc" in line:
            line = "20.0 ! LenNuc"
        elif "! IterMax" in line:
            line = "4000 ! IterMax"
        elif "! OutMolMol" in line:
            line = "4000 ! OutMolMol"
        elif "! Save final state" in line:
            line, skip = "F ! Save final state", True
        out.append(line)
    (d / "start.dat").write_text("\n".join(out) + "\n")
    tsub = np.broadcast_to(T[::3, None, None], (L // 3, L // 3, L // 3)).astype(np.int16)
    o = oracle_lib.Oracle(str(d / "start.dat"), L, L, L)
    o.set_la_input(layers, np.ascontiguousarray(tsub))
    o.init()
    o.write_frame(str(tmp_path / "ora"), 0.0, 0)
    o.close()
    r = subprocess.run([EXE], cwd=d, env=dict(os.environ, MULSKIPS_BOX=f"{L} {L} {L}"), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert (d / "I00000000.xyz").read_text() == (tmp_path / "ora.xyz").read_text()
    hdr = (d / "I00000001.xyz").read_text().splitlines()[0].split()
    assert int(hdr[-1]) >= 4000
    assert len(open(d / "LattStat.dat").read().splitlines()) == L


def test_points_match_oracle(oracle_lib, tmp_path):
    """InitSt SH through the C ABI (mks_init_points): a 3C-SiC slab with a
    {111}-faceted pyramid, byte-identical to the oracle's SetShape."""
    from test_shape_points import pyramid_points, sic_startdat, write_points
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat, read_shape_points
    L = 240
    xyz, sym, _, _ = pyramid_points(L, 60, 54)
    write_points(tmp_path / "p.xyz", xyz, sym)
    sic_startdat(str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), L)
    o = oracle_lib.Oracle(str(tmp_path / "start.dat"), L, L, L)
    o.init()
    ref, _ = oracle_lib.compact_state(o)
    o.close()
    d = parse_startdat(str(tmp_path / "start.dat"))
    pts, sp = read_shape_points(str(tmp_path / "p.xyz"))
    with Lattice(L, L, L, ncrystal=2, list_crystal=[14, 6], sf=d["sf"]) as lat:
        lat.set_rates(d["ptransE"], d["ptransD"])
        lat.init_points(pts, sp)
        st = lat.state()
    bad = np.argwhere(st != ref)
    assert bad.size == 0, f"{len(bad)} sites differ, first {bad[:3]}"


def test_mulskips_e_shape_file(oracle_lib, tmp_path):
    """mulskips.e with InitSt SH and the point-list file: the initial frame
    equals the oracle's, and the run goes on from it."""
    from test_shape_points import pyramid_points, sic_startdat, write_points
    L = 240
    d = tmp_path / "sh"
    d.mkdir()
    xyz, sym, _, _ = pyramid_points(L, 60, 54)
    write_points(d / "shape.xyz", xyz, sym)
    sic_startdat(str(d / "start.dat"), "shape.xyz", L)
    txt = open(d / "start.dat").read().replace("1000000 ! IterMax", "4000 ! IterMax")
    txt = txt.replace("1000000 ! OutMolMol", "4000 ! OutMolMol")
    (d / "start.dat").write_text(txt)
    cwd = os.getcwd()
    try:
        os.chdir(d)
        o = oracle_lib.Oracle("start.dat", L, L, L)
        o.init()
        o.write_frame(str(tmp_path / "ora"), 0.0, 0)
        o.close()
    finally:
        os.chdir(cwd)
    r = subprocess.run([EXE], cwd=d, env=dict(os.environ, MULSKIPS_BOX=f"{L} {L} {L}"), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert (d / "I00000000.xyz").read_text() == (tmp_path / "ora.xyz").read_text()
    hdr = (d / "I00000001.xyz").read_text().splitlines()[0].split()
    assert int(hdr[-1]) >= 4000


def test_mulskips_e_sige(oracle_lib, tmp_path):
    """mulskips.e with InitSt SG (SetSiGex): the sites of SetSi's slab, Ge
    drawn on each atom with the alloy fraction (the reference draws it with
    the compiler's RAND, here a seeded generator)."""
    from mulskips_gb300.startdat import write_startdat
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    D = np.full((3, 3), 0.5)
    for s in range(2):
        for n1 in range(4):
            for n2 in range(4 - n1):
                if n1 + n2:
                    E[s, n1, n2] = 1e13 * np.exp(-0.6 * (n1 + n2) / (8.617e-5 * 1100.0))
    d = tmp_path / "sg"
    d.mkdir()
    write_startdat(str(d / "start.dat"), E, D, ncrystal=2, list_crystal=(14, 32), init_st="SG", len1=130,
                   max_iter=4000, alloy_fraction=0.3)
    write_startdat(str(tmp_path / "fs.dat"), E, D, ncrystal=1, list_crystal=(14,), init_st="FS", len1=120,
                   max_iter=4000, run_type="T")
    o = oracle_lib.Oracle(str(tmp_path / "fs.dat"), 480, 480, 480)
    o.init()
    o.write_frame(str(tmp_path / "ora"), 0.0, 0)
    o.close()
    r = subprocess.run([EXE], cwd=d, env=dict(os.environ, MULSKIPS_BOX="480 480 480"), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    mine = (d / "I00000000.xyz").read_text().splitlines()
    ref = (tmp_path / "ora.xyz").read_text().splitlines()
    assert len(mine) == len(ref) and mine[0] == ref[0]
    assert [l.split()[1:] for l in mine[2:]] == [l.split()[1:] for l in ref[2:]]
    sym = [l.split()[0] for l in mine[2:]]
    assert set(sym) <= {"Si", "Ge"} and 0.25 < sym.count("Ge") / len(sym) < 0.35


NEW_SHAPES = [("SS", (96, 0, 0)), ("D", (24, 90, 0)), ("Z", (24, 90, 0)), ("J", (24, 90, 0)), ("K", (24, 90, 0)),
              ("L", (24, 90, 0)), ("T", (30, 40, 90)), ("Fw", (130, 170, 0)), ("Fa", (130, 170, 75))]


@pytest.mark.parametrize("kind,lens", NEW_SHAPES, ids=[k for k, _ in NEW_SHAPES])
def test_mulskips_e_shape_variants(oracle_lib, tmp_path, kind, lens):
    """mulskips.e with the other shaped InitSt of main.f:224-278 (SetNCSpSi,
    the inverted-pyramid variants, SetTrench, SetSiC3Cww and its aperture
    form): the initial frame equals the oracle's, and the run goes on.  The
    run is short: with these rates the Si ball evaporates within a few
    thousand events, and the final frame of a run stopped on too few MC
    sites is numbered 0."""
    from mulskips_gb300.startdat import write_startdat
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    for s in range(2):
        for n1 in range(4):
            for n2 in range(4 - n1):
                if n1 + n2:
                    E[s, n1, n2] = 1e13 * np.exp(-0.6 * (n1 + n2) / (8.617e-5 * 1600.0))
    d = tmp_path / kind
    d.mkdir()
    write_startdat(str(d / "start.dat"), E, np.full((3, 3), 0.5), ncrystal=2, list_crystal=(14, 6), init_st=kind,
                   len1=lens[0], lens=lens[1:], max_iter=300, run_type="T")
    o = oracle_lib.Oracle(str(d / "start.dat"), 240, 240, 240)
    o.init()
    o.write_frame(str(tmp_path / "ora"), 0.0, 0)
    o.close()
    r = subprocess.run([EXE], cwd=d, env=dict(os.environ, MULSKIPS_BOX="240 240 240"), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert (d / "I00000000.xyz").read_text() == (tmp_path / "ora.xyz").read_text()
    assert int((d / "I00000001.xyz").read_text().splitlines()[0].split()[-1]) >= 300


def test_mulskips_e_continuation_run(tmp_path):
    """RunType C (main.f:178-182, SetCAD.f:54-80): a CAD run with one
    coverage species saves its final LattCoo (main.f:385-403), and a
    continuation run started from that checkpoint writes, as its initial
    frame, the final frame of the first run."""
    geo = _cad_geometry()
    d1, d2 = tmp_path / "first", tmp_path / "cont"
    d1.mkdir()
    d2.mkdir()
    with open(d1 / "LattGeo.dat", "w") as f:
        for z in range(geo.shape[0]):
            f.write(" ".join(map(str, geo[z].reshape(-1).tolist())) + "\n")

    def startdat(run_type, cadfile, save):
        out = []
        for line in open(os.path.join(GOLDEN, "CAD", "start.dat")).read().splitlines():
            if "LattGeo" in line:
                line = cadfile
            elif "! IterMax" in line:
                line = "4000 ! IterMax"
            elif "! OutMolMol" in line:
                line = "4000 ! OutMolMol"
            elif "! RunType" in line:
                line = f"{run_type} ! RunType"
            elif "! Save final state" in line and save:
                out.append("T ! Save final state")
                line = "final.dat  "
            out.append(line)
        return "\n".join(out) + "\n"

    (d1 / "start.dat").write_text(startdat("R", "LattGeo.dat", True))
    env = dict(os.environ, MULSKIPS_BOX="480 240 240")
    r = subprocess.run([EXE], cwd=d1, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert len((d1 / "final.dat").read_text().splitlines()) == 240
    (d2 / "start.dat").write_text(startdat("C", str(d1 / "final.dat"), False))
    r = subprocess.run([EXE], cwd=d2, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "continuation run" in r.stdout
    last = (d1 / "I00000001.xyz").read_text().splitlines()
    first = (d2 / "I00000000.xyz").read_text().splitlines()
    assert first[0].split()[0] == last[0].split()[0] and first[1:] == last[1:]
    assert int((d2 / "I00000001.xyz").read_text().splitlines()[0].split()[-1]) >= 4000
    # a checkpoint written by a Fortran runtime that wraps long list-directed
    # records across lines (here 37 values per line) reads as the same
    # LattCoo: each READ takes LenX*LenY values across line breaks and skips
    # the rest of its last record
    d3 = tmp_path / "wrapped"
    d3.mkdir()
    with open(d3 / "final.dat", "w") as f:
        for rec in (d1 / "final.dat").read_text().splitlines():
            vals = rec.split()
            for i in range(0, len(vals), 37):
                f.write(" " + " ".join(vals[i:i + 37]) + "\n")
    (d3 / "start.dat").write_text(startdat("C", str(d3 / "final.dat"), False))
    r = subprocess.run([EXE], cwd=d3, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert (d3 / "I00000000.xyz").read_text().splitlines()[1:] == first[1:]
    assert (d3 / "I00000001.xyz").read_text() == (d2 / "I00000001.xyz").read_text()


def test_mulskips_e_cad_sige(oracle_lib, tmp_path):
    """InitSt IN with a SiGe start.dat and alloy fraction 0.3 (SetCAD.f:215-222):
    the sites of the CAD geometry's Si, Ge drawn on each at the fraction (the
    reference draws with RAND(), here a seeded generator)."""
    from mulskips_gb300.startdat import write_startdat
    geo = _cad_geometry()
    d = tmp_path / "sige"
    d.mkdir()
    with open(d / "LattGeo.dat", "w") as f:
        for z in range(geo.shape[0]):
            f.write(" ".join(map(str, geo[z].reshape(-1).tolist())) + "\n")
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    for s in range(2):
        for n1 in range(4):
            for n2 in range(4 - n1):
                if n1 + n2:
                    E[s, n1, n2] = 1e13 * np.exp(-0.7 * (n1 + n2) / (8.617e-5 * 1000.0))

    def with_geometry(path, ncrystal, lc, alloy):
        write_startdat(str(path), E, np.full((3, 3), 0.5), ncrystal=ncrystal, list_crystal=lc, init_st="IN",
                       max_iter=300, run_type="T", alloy_fraction=alloy)
        lines = open(path).read().splitlines()
        lines[3] = "LattGeo.dat"
        open(path, "w").write("\n".join(lines) + "\n")

    with_geometry(d / "start.dat", 2, (14, 32), 0.3)
    with_geometry(tmp_path / "si.dat", 1, (14,), 0.0)
    o = oracle_lib.Oracle(str(tmp_path / "si.dat"), 480, 240, 240)
    o.set_geometry(geo)
    o.init()
    o.write_frame(str(tmp_path / "ora"), 0.0, 0)
    o.close()
    r = subprocess.run([EXE], cwd=d, env=dict(os.environ, MULSKIPS_BOX="480 240 240"), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    mine = (d / "I00000000.xyz").read_text().splitlines()
    ref = (tmp_path / "ora.xyz").read_text().splitlines()
    assert len(mine) == len(ref) and mine[0] == ref[0]
    assert [l.split()[1:] for l in mine[2:]] == [l.split()[1:] for l in ref[2:]]
    sym = [l.split()[0] for l in mine[2:]]
    assert set(sym) <= {"Si", "Ge"} and 0.25 < sym.count("Ge") / len(sym) < 0.35


def test_run_mulskips_la_call(tmp_path, monkeypatch):
    """The pymulskips-style LA call: mulskips_gb300.setuprun.run_mulskips
    writes the LA start.dat (energetics, files, LA block, the layout the
    reference writer gives) and runs mulskips.e on the geometry and
    temperature files, which writes the phases file."""
    import sys
    sys.path.insert(0, GOLDEN)
    import process_stubs
    from mulskips_gb300.setuprun import run_mulskips
    L = 120
    layers = np.where(np.arange(L) < 100, 1, 10).astype(np.int8)
    layers[:4] = 10
    T = np.where(layers == 10, 10, (1650 + 0.1 * np.arange(L)).astype(np.int64))
    work = tmp_path / "inputs"
    work.mkdir()
    with open(work / "LattGeo.dat", "w") as fg, open(work / "TempStat.dat", "w") as ft:
        for z in range(L):
            fg.write(" ".join([str(int(layers[z]))] * (L * L)) + "\n")
            ft.write(" ".join([str(int(T[z]))] * (L * L)) + "\n")
    monkeypatch.chdir(work)
    monkeypatch.setenv("PWD", str(work))
    monkeypatch.setenv("MULSKIPS_BOX", f"{L} {L} {L}")
    ok = run_mulskips(execpath=os.path.dirname(EXE), runpath=str(tmp_path / "run"), Simulation="LA",
                      mp=process_stubs.PhaseChange(), ExitStrategy="Time", TotTime=0.02, OutTime=0.01,
                      cadfilename="LattGeo.dat", tempfilename="TempStat.dat", LenVac=10.0, LenNuc=20.0,
                      initialState="inhomogeneous", LenSiGe=0.0, SaveCoo=True, coofilename="LattStat.dat",
                      restartfilename="restart.dat", RunType="R", IDUM=3)
    log = open(tmp_path / "run" / "log.txt").read()
    assert ok, log[-3000:]
    assert len(open(work / "LattStat.dat").read().splitlines()) == L
    assert (tmp_path / "run" / "I00000001.xyz").exists()


def test_batch_replicas_of_shapes_match_oracle(oracle_lib, tmp_path):
    """Replicas of one batch built by different shaped initializers (an
    antiphase-domain inverted pyramid and a SiC trench) and by SetShape, each
    byte-identical to the oracle's lattice."""
    from mulskips_gb300 import Batch
    from mulskips_gb300.startdat import parse_startdat, read_shape_points, write_startdat
    from test_shape_points import pyramid_points, sic_startdat, write_points
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    for s in range(2):
        for n1 in range(4):
            for n2 in range(4 - n1):
                if n1 + n2:
                    E[s, n1, n2] = 1e13 * np.exp(-0.6 * (n1 + n2) / (8.617e-5 * 1600.0))
    refs, paths = [], []
    for k, (kind, lens) in enumerate((("K", (24, 90, 0)), ("T", (30, 40, 90)))):
        p = tmp_path / f"{kind}.dat"
        write_startdat(str(p), E, np.full((3, 3), 0.5), ncrystal=2, list_crystal=(14, 6), init_st=kind,
                       len1=lens[0], lens=lens[1:], run_type="T")
        o = oracle_lib.Oracle(str(p), 240, 240, 240)
        o.init()
        refs.append(oracle_lib.compact_state(o)[0])
        o.close()
    xyz, sym, _, _ = pyramid_points(240, 60, 54)
    write_points(tmp_path / "p.xyz", xyz, sym)
    sic_startdat(str(tmp_path / "sh.dat"), str(tmp_path / "p.xyz"), 240)
    o = oracle_lib.Oracle(str(tmp_path / "sh.dat"), 240, 240, 240)
    o.init()
    refs.append(oracle_lib.compact_state(o)[0])
    o.close()
    d = parse_startdat(str(tmp_path / "K.dat"))
    b = Batch([(240, 240, 240)] * 3, seeds=[1, 2, 3], ncrystal=2, list_crystal=(14, 6), sf=d["sf"])
    b.set_rates(np.stack([d["ptransE"]] * 3), np.stack([d["ptransD"]] * 3))
    b.init_shape(0, "K", [24, 90])
    b.init_shape(1, "T", [30, 40, 90])
    b.init_points(2, *read_shape_points(str(tmp_path / "p.xyz")))
    for r in range(3):
        assert np.array_equal(b.state(r), refs[r]), r
    b.close()


def test_mulskips_e_sicsf(oracle_lib, tmp_path):
    """mulskips.e with InitSt E (SetSiCSF, a stacking fault off the diamond
    sites, run on the explicit-neighbour engine at the start.dat's
    PtransZig = 1): the initial frame equals the oracle's, and the run of
    4000 events writes its second frame."""
    from test_shape_points import sicsf_startdat
    L = 120
    d = tmp_path / "sicsf"
    d.mkdir()
    sicsf_startdat(d / "start.dat", 60, 24, 24)
    out = []
    for line in (d / "start.dat").read_text().splitlines():
        if "! IterMax" in line:
            line = "4000 ! IterMax"
        elif "! OutMolMol" in line:
            line = "4000 ! OutMolMol"
        out.append(line)
    (d / "start.dat").write_text("\n".join(out) + "\n")
    o = oracle_lib.Oracle(str(d / "start.dat"), L, L, L)
    o.init()
    o.write_frame(str(tmp_path / "ora"), 0.0, 0)
    o.close()
    r = subprocess.run([EXE], cwd=d, env=dict(os.environ, MULSKIPS_BOX=f"{L} {L} {L}"), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert (d / "I00000000.xyz").read_text() == (tmp_path / "ora.xyz").read_text()
    assert int((d / "I00000001.xyz").read_text().splitlines()[0].split()[-1]) >= 4000
