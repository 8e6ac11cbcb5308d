"""Drop-in boundary on the CPU: start.dat written by mulskips_gb300.setuprun
matches, record by record, the one the reference's own
pymulskips.setuprun.run_mulskips writes for the same process object; the
reader agrees with the oracle's parser; setup_mulskips_src leaves the
make.log line the reference checks."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

def first_tokens(path):
    out = []
    for line in open(path):
        toks = line.split("!")[0].split()
        out.append(toks)
    return out


def test_startdat_matches_reference_writer(tmp_path):
    """tests/golden/refwriter/start.dat was written by the reference's
    pymulskips.setuprun.run_mulskips(setup_only=True) for the same process
    object and arguments (tests/golden/make_fixtures.py)."""
    from mulskips_gb300.setuprun import PlainSi, run_mulskips

    class PVD(PlainSi):
        pass

    run_mulskips(runpath=str(tmp_path / "ours"), Simulation="FS", mp=PVD(T=1100.0), PtransZig=1.0,
                 ExitStrategy="Iter", OutMolMol=1000, IterMax=100000, Seed_box=[120, 120, 120], RunType="R",
                 IDUM=5, setup_only=True)
    a = first_tokens(os.path.join(GOLDEN, "refwriter", "start.dat"))
    b = first_tokens(tmp_path / "ours" / "start.dat")
    assert a == b


def test_reader_agrees_with_oracle(oracle_lib):
    from mulskips_gb300.startdat import parse_startdat
    for case in ("Si-SL", "surface"):
        p = os.path.join(GOLDEN, case, "start.dat")
        d = parse_startdat(p)
        o = oracle_lib.Oracle(p, 480, 480, 480)
        pE, pD = o.rates()
        o.close()
        assert np.array_equal(pE, d["ptransE"]) and np.array_equal(pD, d["ptransD"])


def test_setup_src_writes_box_and_make_log(tmp_path):
    from mulskips_gb300.setuprun import setup_mulskips_src
    (tmp_path / "mulskips.e").write_text("")
    assert setup_mulskips_src(str(tmp_path), 240, 240, 480)
    assert open(tmp_path / "mulskips_box.dat").read().split() == ["240", "240", "480"]
    assert "Compilation terminated" in open(tmp_path / "make.log").read()
    with pytest.raises(ValueError):
        setup_mulskips_src(str(tmp_path), 100, 240, 480)


@pytest.mark.parametrize("name", ["cvd", "in_sige", "la"])
def test_startdat_layouts_match_reference_writer(tmp_path, name):
    """The writer's other layouts against the reference's own
    run_mulskips(setup_only=True) output for the same process objects
    (tests/golden/refwriter/<name>.dat, tests/golden/make_fixtures.py):
    coverage rates, a SiGe geometry run with its Ge fraction and checkpoint,
    the LA block.  File names are compared by base name (the reference writes
    them under the caller's $PWD)."""
    import sys
    sys.path.insert(0, GOLDEN)
    import make_fixtures
    import process_stubs
    from mulskips_gb300.setuprun import run_mulskips
    kw = dict(make_fixtures.REF_WRITER_CASES[name])
    kw["mp"] = getattr(process_stubs, kw["mp"])()
    run_mulskips(runpath=str(tmp_path / "ours"), setup_only=True, **kw)

    def norm(path):
        return [[os.path.basename(t) if "/" in t else t for t in toks] for toks in first_tokens(path)]

    assert norm(os.path.join(GOLDEN, "refwriter", name + ".dat")) == norm(tmp_path / "ours" / "start.dat")


def test_sh_startdat_round_trip_and_oracle(tmp_path, oracle_lib):
    """write_startdat with InitSt SH and PtransZig < 1 (the config-2 input):
    the reader gives back the point file, PtransZig and the rates, and the
    oracle builds the same lattice from it as the library's point list says
    (every point's occupancy and species)."""
    from mulskips_gb300.shapes import faceted_slab_points
    from mulskips_gb300.startdat import parse_startdat, read_shape_points, write_startdat
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    D = np.full((3, 3), 0.25)
    for s in range(2):
        for n1 in range(4):
            for n2 in range(4 - n1):
                if n1 + n2:
                    E[s, n1, n2] = 1e13 * np.exp(-(0.4 + 0.05 * (n1 + 2 * n2 + s)) / (8.617e-5 * 1600.0))
    xyz, sp = faceted_slab_points(120, 60, 24)
    pts = tmp_path / "slab.xyz"
    with open(pts, "w") as fh:
        fh.write(f"{len(xyz)}\nslab\n")
        fh.write("".join(f"{'Si' if s == 1 else 'C'} {x} {y} {z}\n" for (x, y, z), s in zip(xyz.tolist(), sp)))
    p = tmp_path / "start.dat"
    write_startdat(str(p), E, D, ncrystal=2, list_crystal=(14, 6), init_st="SH", points=str(pts), run_type="R",
                   seed=3, sf=0.385833, ptrans_zig=0.5362)
    d = parse_startdat(str(p))
    assert d["init_st"] == "SH" and d["ptrans_zig"] == 0.5362
    assert np.allclose(d["ptransE"][:2, :, :, 0, 0, 0, 0], E[:2, :, :, 0, 0, 0, 0])
    assert np.allclose(d["ptransD"][:2], D[:2])
    assert d["cadfilename"] == str(pts)
    rxyz, rsp = read_shape_points(d["cadfilename"])
    assert np.array_equal(np.asarray(rxyz), xyz) and np.array_equal(np.asarray(rsp), sp)
    o = oracle_lib.Oracle(str(p), 120, 120, 120)
    o.init()
    lc = o.lattcoo()
    o.close()
    inner = (xyz[:, 2] > 3) & (xyz[:, 2] < 116)
    v = lc[xyz[inner, 2], xyz[inner, 1], xyz[inner, 0]]
    assert ((v >> 23) & 1).all()
    assert np.array_equal((v >> 27) & 7, sp[inner])
    with pytest.raises(ValueError):
        write_startdat(str(p), E, D, ncrystal=2, list_crystal=(14, 6), init_st="FS", points=str(pts))


def test_faceted_slab_points_refuses_bad_geometry():
    from mulskips_gb300.shapes import faceted_slab_points
    for L, h, P in ((130, 60, 24), (120, 60, 25), (120, 60, 48 * 5), (120, 10, 24), (120, 110, 24)):
        with pytest.raises(ValueError):
            faceted_slab_points(L, h, P)
