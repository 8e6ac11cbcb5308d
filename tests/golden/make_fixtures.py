"""Generate the golden fixtures under tests/golden/ from the MulSKIPS reference.

Run once where the reference checkout is present, with its path given as the
first argument or in MULSKIPS_REF (python make_fixtures.py <reference dir>).
The outputs are committed; the tests read only the committed files, never the
reference itself.

Fixtures written:
  numberslist.txt        the 1000 test-mode uniforms of
                         mulskips-source/mcevent/PickTreeEvent.f:77-1076
                         (RunType 'T'), one literal per line, as written
  <case>/start.dat       regression-tests/input-and-references-files/start-<case>.dat
  <case>/I00000000.xyz.gz, I00000001.xyz.gz, log.txt
                         the reference's own regression outputs for that case
  LA/start.dat, I0000000{0,1}.xyz.gz, log.txt
                         the reference's LA regression case, and its inputs from
                         LA-input.tar.gz in compact form: LA/geo_layers.npy
                         (LattGeo id of each layer z; the file is uniform per
                         layer, checked here) and LA/temp_sub.npz (TempStat at
                         the grid points with x, y, z multiples of 3, int16,
                         index [z/3, y/3, x/3])
  CAD/start.dat, I0000000{0,1}.xyz.gz, log.txt
                         the reference's CAD regression case (InitSt IN, one
                         coverage species), and its geometry from
                         CAD-input.tar.gz as CAD/geo.npz: the LattGeo id of
                         every site, int8 [z, y, x]; each line of the file is
                         one layer and, as Fortran's list-directed READ does,
                         only its first LenX*LenY values are kept (line 168
                         carries one value more)
  refwriter/start.dat    start.dat written by the reference's
                         pymulskips.setuprun.run_mulskips (setup_only) for the
                         plain Si(001) process object of mulskips_gb300.setuprun
  refwriter/{cvd,in_sige,la}.dat
                         the same writer for the process objects of
                         process_stubs.py (REF_WRITER_CASES below)
  analysis.json          the reference's post-processing on its own frames:
                         pymulskips.analyze.get_surface_height of every
                         golden I0000000{0,1}.xyz (default and a second set
                         of bin_size / surface_roughness), and
                         analyze_growth_rate ('finitediff' and 'polyfit',
                         Nexclude 2) of the synthetic frame series of
                         growth_series() below
"""
import gzip
import os
import re
import shutil
import sys

REF = None     # the reference checkout, set by main()
RT = None
HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["Si-SL", "surface", "cube", "cube-zigzag", "sphere", "inverted-pyramid", "finfet", "CVD-Si-SiH2"]


def numbers_list():
    src = open(os.path.join(REF, "mulskips-source", "mcevent", "PickTreeEvent.f")).read()
    body = src[src.index("numbers = (/"):src.index("/)", src.index("numbers = (/"))]
    vals = re.findall(r"[-+]?\d+\.\d+E[-+]\d+", body)
    assert len(vals) == 1000, len(vals)
    with open(os.path.join(HERE, "numberslist.txt"), "w") as f:
        f.write("\n".join(vals) + "\n")


def cases():
    for case in CASES:
        d = os.path.join(HERE, case)
        os.makedirs(d, exist_ok=True)
        shutil.copyfile(os.path.join(RT, f"start-{case}.dat"), os.path.join(d, "start.dat"))
        shutil.copyfile(os.path.join(RT, f"log-{case}.txt"), os.path.join(d, "log.txt"))
        for fr in ("I00000000", "I00000001"):
            with open(os.path.join(RT, f"{fr}-{case}.xyz"), "rb") as fi, \
                    gzip.GzipFile(os.path.join(d, f"{fr}.xyz.gz"), "wb", compresslevel=9, mtime=0) as fo:
                fo.write(fi.read())


def la_case(lx=480, ly=240, lz=240):
    import io
    import tarfile
    import numpy as np
    d = os.path.join(HERE, "LA")
    os.makedirs(d, exist_ok=True)
    shutil.copyfile(os.path.join(RT, "start-LA.dat"), os.path.join(d, "start.dat"))
    shutil.copyfile(os.path.join(RT, "log-LA.txt"), os.path.join(d, "log.txt"))
    for fr in ("I00000000", "I00000001"):
        with open(os.path.join(RT, f"{fr}-LA.xyz"), "rb") as fi, \
                gzip.GzipFile(os.path.join(d, f"{fr}.xyz.gz"), "wb", compresslevel=9, mtime=0) as fo:
            fo.write(fi.read())
    with tarfile.open(os.path.join(RT, "LA-input.tar.gz")) as tf:
        geo = np.loadtxt(io.TextIOWrapper(tf.extractfile(f"LattGeo.{lx}x{ly}x{lz}.dat")))
        tmp = np.loadtxt(io.TextIOWrapper(tf.extractfile(f"TempStat.{lx}x{ly}x{lz}.dat")))
    geo = geo.reshape(lz, ly, lx)
    assert (geo == geo[:, :1, :1]).all(), "LattGeo is not uniform per layer"
    np.save(os.path.join(d, "geo_layers.npy"), geo[:, 0, 0].astype(np.int8))
    tmp = tmp.reshape(lz, ly, lx)
    assert (tmp == np.rint(tmp)).all()
    np.savez_compressed(os.path.join(d, "temp_sub.npz"), t=tmp[::3, ::3, ::3].astype(np.int16))


def cad_case(lx=480, ly=240, lz=240):
    import io
    import tarfile
    import numpy as np
    d = os.path.join(HERE, "CAD")
    os.makedirs(d, exist_ok=True)
    shutil.copyfile(os.path.join(RT, "start-CAD.dat"), os.path.join(d, "start.dat"))
    shutil.copyfile(os.path.join(RT, "log-CAD.txt"), os.path.join(d, "log.txt"))
    for fr in ("I00000000", "I00000001"):
        with open(os.path.join(RT, f"{fr}-CAD.xyz"), "rb") as fi, \
                gzip.GzipFile(os.path.join(d, f"{fr}.xyz.gz"), "wb", compresslevel=9, mtime=0) as fo:
            fo.write(fi.read())
    rows = []
    with tarfile.open(os.path.join(RT, "CAD-input.tar.gz")) as tf:
        for line in io.TextIOWrapper(tf.extractfile(f"LattGeo.{lx}x{ly}x{lz}.withzeros.dat")):
            vals = line.split()
            assert len(vals) >= lx * ly
            rows.append(np.array(vals[:lx * ly], dtype=np.int8))
    assert len(rows) == lz
    np.savez_compressed(os.path.join(d, "geo.npz"), g=np.stack(rows).reshape(lz, ly, lx))


def reference_writer():
    import sys
    import tempfile
    import warnings
    sys.path.insert(0, REF)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import pymulskips.setuprun as ref_setup
    from mulskips_gb300.setuprun import PlainSi

    class PVD(PlainSi):    # the reference dispatches on the class name
        pass

    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        try:
            ref_setup.run_mulskips(execpath=tmp, runpath=os.path.join(tmp, "ref"), Simulation="FS",
                                   mp=PVD(T=1100.0), PtransZig=1.0, ExitStrategy="Iter", OutMolMol=1000,
                                   IterMax=100000, Seed_box=[120, 120, 120], RunType="R", IDUM=5,
                                   setup_only=True)
        finally:
            os.chdir(cwd)
        d = os.path.join(HERE, "refwriter")
        os.makedirs(d, exist_ok=True)
        shutil.copyfile(os.path.join(tmp, "ref", "start.dat"), os.path.join(d, "start.dat"))
    # the other layouts of the writer: coverage species (CVD), a SiGe crystal
    # with a geometry file (IN), and the LA block (file names are written
    # under $PWD, kept here as PWD/<name>; the tests compare base names)
    sys.path.insert(0, HERE)
    import process_stubs as ps
    for name, kw in REF_WRITER_CASES.items():
        kw = dict(kw)
        kw["mp"] = getattr(ps, kw["mp"])()
        with tempfile.TemporaryDirectory() as tmp:
            try:
                ref_setup.run_mulskips(execpath=tmp, runpath=os.path.join(tmp, "ref"), setup_only=True, **kw)
            finally:
                os.chdir(cwd)
            txt = open(os.path.join(tmp, "ref", "start.dat")).read()
        pwd = os.environ.get("PWD", cwd)
        with open(os.path.join(HERE, "refwriter", name + ".dat"), "w") as f:
            f.write(txt.replace(pwd + "/", "PWD/"))


# run_mulskips arguments of the extra writer fixtures (mp names a class of
# process_stubs.py)
REF_WRITER_CASES = {
    "cvd": dict(Simulation="FS", mp="CVD", ExitStrategy="Time", TotTime=3.0, OutTime=1.0,
                Seed_box=[48, 48, 48], RunType="R", IDUM=7),
    "in_sige": dict(Simulation="IN", mp="PVD", ExitStrategy="Iter", OutMolMol=1000, IterMax=4000,
                    cadfilename="geo.dat", RunType="T", IDUM=9, SaveFinalState=True, restartfilename="final.dat"),
    "la": dict(Simulation="LA", mp="PhaseChange", ExitStrategy="Time", TotTime=1e-8, OutTime=1e-9,
               cadfilename="LattGeo.dat", tempfilename="TempStat.dat", LenVac=10.0, LenNuc=20.0,
               initialState="inhomogeneous", LenSiGe=0.0, SaveCoo=True, coofilename="LattStat.dat",
               restartfilename="restart.dat", RunType="R", IDUM=3),
}


def growth_series(frame_lines, k):
    """Frame k of a synthetic growth series built from the lines of one
    golden frame: every z shifted by 0.9 k + 0.3 sin(k) A, at time
    10 k + k^2 / 7 s.  Returns (time, lines)."""
    import math
    t = 10.0 * k + k * k / 7.0
    dz = 0.9 * k + 0.3 * math.sin(k)
    out = []
    for line in frame_lines:
        sym, x, y, z = line.split()[:4]
        out.append(f"{sym} {x} {y} {float(z) + dz:.5f}")
    return t, out


def analysis():
    import glob as globmod
    import json
    import tempfile
    import types
    import warnings
    sys.path.insert(0, REF)
    # analyze_growth_rate imports matplotlib.pyplot before its work even with
    # plotting=False; this checkout has no matplotlib, so a module without
    # content stands in (nothing of it is called)
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", mpl.pyplot)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import pymulskips.analyze as ref_an
    out = {"surface_height": {}, "surface_height_b3_r10": {}, "growth": {}}
    cases = sorted(c for c in os.listdir(HERE) if os.path.exists(os.path.join(HERE, c, "I00000000.xyz.gz")))
    with tempfile.TemporaryDirectory() as tmp:
        for case in cases:
            for fr in ("I00000000", "I00000001"):
                p = os.path.join(tmp, f"{case}-{fr}.xyz")
                with gzip.open(os.path.join(HERE, case, fr + ".xyz.gz"), "rb") as fi, open(p, "wb") as fo:
                    fo.write(fi.read())
                key = f"{case}/{fr}"
                out["surface_height"][key] = ref_an.get_surface_height(p)
                out["surface_height_b3_r10"][key] = ref_an.get_surface_height(p, bin_size=3.0, surface_roughness=10.0)
        # growth series from the Si-SL final frame; the reference globs the
        # frames unsorted, so the series is handed over in time order
        with gzip.open(os.path.join(HERE, "Si-SL", "I00000001.xyz.gz"), "rt") as f:
            lines = f.read().splitlines()
        hdr, box, body = lines[0].split(), lines[1], lines[2:]
        run = os.path.join(tmp, "series")
        os.makedirs(run)
        for k in range(9):
            t, fl = growth_series(body, k)
            with open(os.path.join(run, f"I{k:08d}.xyz"), "w") as f:
                f.write(f" {hdr[0]} angstroem KMC-time: {t!r} Iter: {k}\n{box}\n" + "\n".join(fl) + "\n")
        orig = globmod.glob
        globmod.glob = lambda pat, *a, **kw: sorted(orig(pat, *a, **kw))
        try:
            for m in ("finitediff", "polyfit"):
                gr, h = ref_an.analyze_growth_rate(run, method=m, plotting=False, return_surf_height=True)
                out["growth"][m] = {"rate": gr, "heights": [float(v) for v in h]}
        finally:
            globmod.glob = orig
    with open(os.path.join(HERE, "analysis.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


def main(argv):
    global REF, RT
    REF = argv[1] if len(argv) > 1 else os.environ.get("MULSKIPS_REF")
    if not REF or not os.path.isdir(os.path.join(REF, "mulskips-source")):
        raise SystemExit("usage: make_fixtures.py <MulSKIPS reference checkout> (or set MULSKIPS_REF)")
    RT = os.path.join(REF, "regression-tests", "input-and-references-files")
    numbers_list()
    cases()
    la_case()
    cad_case()
    reference_writer()
    analysis()


if __name__ == "__main__":
    main(sys.argv)
