"""InitSt SH (SetShape.f, a lattice from a point-list file), on the CPU.

The oracle restates SetShape.f list by list (32-site shell scan, FIND_NN,
reciprocity checks, ad-void pass).  No regression case of the reference uses
SH, so it is pinned against the pinned flat initializers: the point list of
the Si(001) (SetSi) and 3C-SiC(001) (SetSiC3C) lattices of the reference's
Si-SL and surface cases gives back the same occupancy, species, walls and
coordinations (the first list entries follow SetShape's own scan order).
The library's one-byte initializer (mks_shapes::set_points, compiled for the
host by a helper) then builds byte-identical lattices to the oracle's, on
those lists and on a 3C-SiC slab carrying a {111}-faceted pyramid, and
refuses the same undefined inputs."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from mulskips_gb300.engine import coordination

HELPER_SRC = os.path.join(ROOT, "tests", "native", "shape_check.cpp")
NUMBERS = os.path.join(GOLDEN, "numberslist.txt")
# bond directions d of a site (a, b, z1) by the parity of z1: (da, db, dz)
OFF = np.array([[[0, 0, 1], [0, -1, -1], [-1, -1, 1], [-1, 0, -1]],
                [[1, 1, -1], [1, 0, 1], [0, 0, -1], [0, 1, 1]]])


@pytest.fixture(scope="module")
def helper(tmp_path_factory, oracle_lib):
    exe = str(tmp_path_factory.mktemp("native") / "shape_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", exe, HELPER_SRC,
                    os.path.join(ROOT, "oracle", "mks_oracle.c"), "-lm"], check=True)
    return exe


def write_points(path, xyz, sym):
    with open(path, "w") as f:
        f.write(f"{len(xyz)}\nshape\n")
        for (x, y, z), s in zip(xyz, sym):
            f.write(f"{s} {x} {y} {z}\n")


def sh_startdat(src_lines, path, points):
    """A start.dat equal to src_lines with InitSt SH and the point file."""
    out = []
    for i, l in enumerate(src_lines):
        if i == 2:
            out += ["SH ! Initstat", points]
        elif i == 3:
            continue
        else:
            out.append(l)
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def lattice_points(o, zmax):
    """Occupied diamond sites of an oracle lattice below zmax, with symbols."""
    lc = o.lattcoo()
    z, y, x = np.nonzero(((lc >> 23) & 1) != 0)
    x1, y1, z1 = x // 3, y // 3, z // 3
    dia = (x % 3 == 0) & (y % 3 == 0) & (z % 3 == 0) & (x1 % 2 == y1 % 2) & (x1 % 2 == z1 % 2)
    dia &= np.isin((x1 + y1 + z1) % 4, [0, 3]) & (z < zmax)
    x, y, z = x[dia], y[dia], z[dia]
    sp = (lc[z, y, x] >> 27) & 7
    return np.stack([x, y, z], 1), np.where(sp == 2, "C", "Si")


def run_helper(helper, startdat, points, side):
    r = subprocess.run([helper, startdat, NUMBERS, points, str(side), str(side), str(side)],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=900)
    return r.returncode, r.stdout


@pytest.mark.parametrize("case", ["Si-SL", "surface"])
def test_oracle_sh_matches_flat_initializers(oracle_lib, tmp_path, case):
    src = os.path.join(GOLDEN, case, "start.dat")
    o = oracle_lib.Oracle(src, 480, 480, 480)
    o.init()
    ref, _ = oracle_lib.compact_state(o)
    xyz, sym = lattice_points(o, 474)
    o.close()
    write_points(tmp_path / "p.xyz", xyz, sym)
    sh_startdat(open(src).read().splitlines(), tmp_path / "start.dat", str(tmp_path / "p.xyz"))
    o = oracle_lib.Oracle(str(tmp_path / "start.dat"), 480, 480, 480)
    o.init()
    mine, off = oracle_lib.compact_state(o)
    counts = o.counts()
    o.close()
    assert off == 0
    # the walls of SetSi above z = 473 are not in the list; SetSiC3C's atoms
    # at z <= 3 become SetShape walls
    keep = np.ones(ref.shape, bool)
    keep[474 // 3:] = False
    if case == "surface":
        keep[:2] = False
    a = np.where(ref == 0x80, 0x80, ref & 0x1F)
    b = np.where(mine == 0x80, 0x80, mine & 0x1F)
    assert np.array_equal(a[keep], b[keep])
    assert counts["mc"] == 6400


@pytest.mark.parametrize("case", ["Si-SL", "surface"])
def test_library_sh_equals_oracle_flat_lists(helper, oracle_lib, tmp_path, case):
    src = os.path.join(GOLDEN, case, "start.dat")
    o = oracle_lib.Oracle(src, 480, 480, 480)
    o.init()
    xyz, sym = lattice_points(o, 474)
    o.close()
    write_points(tmp_path / "p.xyz", xyz, sym)
    sh_startdat(open(src).read().splitlines(), tmp_path / "start.dat", str(tmp_path / "p.xyz"))
    rc, out = run_helper(helper, str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), 480)
    assert rc == 0 and "mismatch 0" in out, out


def pyramid_points(L, h_slab, h_pyr, sic=True):
    """A 3C slab over z = 6..h_slab with a square pyramid of {111} facets
    (z <= h_slab + h_pyr - |x - L/2| - |y - L/2|) on it, walls at z = 0, 3
    and at the top two layers; atoms with fewer than two neighbours removed
    until none is left.  Returns (xyz, symbols) of the points and (xyz,
    sublattice-1 flags) of the empty sites with exactly one neighbour."""
    NA = NB = L // 6
    NZ = L // 3 + 1
    z1, b, a = np.meshgrid(np.arange(NZ), np.arange(NB), np.arange(NA), indexing="ij")
    valid = ((a + b + (z1 >> 1)) & 1) == 0
    x, y, z = 3 * (2 * a + (z1 & 1)), 3 * (2 * b + (z1 & 1)), 3 * z1
    wall = valid & ((z <= 3) | (z >= L - 4))
    top = h_slab + h_pyr - np.abs(x - L // 2) - np.abs(y - L // 2)
    atom = valid & (z >= 6) & ((z <= h_slab) | (z <= top))
    while True:
        occ = atom | wall
        cnt = np.zeros(occ.shape, int)
        for par in (0, 1):
            for d in range(4):
                da, db, dz = OFF[par][d]
                sh = np.roll(np.roll(occ, -da, axis=2), -db, axis=1)
                shz = np.zeros_like(sh)
                if dz == 1:
                    shz[:-1] = sh[1:]
                else:
                    shz[1:] = sh[:-1]
                cnt[par::2] += shz[par::2]
        weak = atom & (cnt < 2)
        if not weak.any():
            break
        atom &= ~weak
    pts = wall | atom
    kind = ((x // 3 + y // 3 + z // 3) % 4 == 0)
    sym = np.where(kind | (not sic), "Si", "C")
    sel = np.nonzero(pts)
    lone = np.nonzero(valid & ~pts & (cnt == 1) & (z >= 6) & (z <= L - 8))
    return (np.stack([x[sel], y[sel], z[sel]], 1), sym[sel], np.stack([x[lone], y[lone], z[lone]], 1),
            kind[lone])


def sic_startdat(path, points, L):
    from mulskips_gb300.startdat import write_startdat
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    D = np.full((3, 3), 0.5)
    for s in range(2):
        for n1 in range(4):
            for n2 in range(4 - n1):
                if n1 + n2:
                    E[s, n1, n2] = 1e13 * np.exp(-0.6 * (n1 + n2) / (8.617e-5 * 1600.0))
    write_startdat(path, E, D, ncrystal=2, list_crystal=(14, 6), init_st="F", len1=L // 2, run_type="T")
    sh_startdat(open(path).read().splitlines(), path, points)


def test_library_sh_equals_oracle_pyramid(helper, oracle_lib, tmp_path):
    L = 240
    xyz, sym, _, _ = pyramid_points(L, 60, 54)
    # an off-site wall point away from every atom is taken and ignored
    xyz = np.vstack([xyz, [[1, 1, 1]]])
    sym = np.append(sym, "Si")
    write_points(tmp_path / "p.xyz", xyz, sym)
    sic_startdat(str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), L)
    rc, out = run_helper(helper, str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), L)
    assert rc == 0 and "mismatch 0" in out, out
    o = oracle_lib.Oracle(str(tmp_path / "start.dat"), L, L, L)
    o.init()
    st, _ = oracle_lib.compact_state(o)
    o.close()
    # the facets hold 2- and 3-coordinated atoms; first entries vary with the scan
    co = coordination(st)
    occ = (st & 3) != 0
    assert ((co == 2) & occ).sum() > 100 and ((co == 3) & occ).sum() > 100
    assert len(np.unique((st[occ & (co <= 3)] >> 5) & 3)) > 1


def test_faceted_slab_points_equal_oracle(helper, oracle_lib, tmp_path):
    """mulskips_gb300.shapes.faceted_slab_points (the {111}-faceted 3C-SiC
    slab of the config-2 bench line): the library's SetShape equals the
    oracle's, and the surface is {111} facets: its atoms hold three bonds
    (one dangling bond each, as on a {111} plane), two only on the pyramid
    apexes and ridges, none one."""
    from mulskips_gb300.shapes import faceted_slab_points
    L, h, P = 240, 120, 60
    xyz, sp = faceted_slab_points(L, h, P)
    write_points(tmp_path / "p.xyz", xyz, np.where(sp == 1, "Si", "C"))
    sic_startdat(str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), L)
    rc, out = run_helper(helper, str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), L)
    assert rc == 0 and "mismatch 0" in out, out
    o = oracle_lib.Oracle(str(tmp_path / "start.dat"), L, L, L)
    o.init()
    st, _ = oracle_lib.compact_state(o)
    o.close()
    co = coordination(st)
    occ = (st & 3) != 0
    assert occ.sum() == ((xyz[:, 2] > 3) & (xyz[:, 2] < L - 4)).sum()
    # periodic pyramids: 16 apexes at h + P/2, valleys at h - P/2
    z = xyz[(xyz[:, 2] > 3) & (xyz[:, 2] < L - 4), 2]
    assert h + P // 2 - 6 <= z.max() <= h + P // 2
    n2, n3 = ((co == 2) & occ).sum(), ((co == 3) & occ).sum()
    assert n3 > 1000 and n2 < n3 / 20, (n2, n3)
    assert not (occ & (co == 1)).any()


def test_undefined_inputs_refused_by_both(helper, tmp_path):
    L = 240
    xyz, sym, lone, lone_kind = pyramid_points(L, 60, 30)
    assert len(lone) > 0
    # an atom bonded once: the reference runs FIND_NN on a zero second neighbour
    xyz1 = np.vstack([xyz, lone[:1]])
    write_points(tmp_path / "p.xyz", xyz1, np.append(sym, "Si" if lone_kind[0] else "C"))
    sic_startdat(str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), L)
    rc, out = run_helper(helper, str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), L)
    assert "product: an atom with fewer than two neighbours" in out and "oracle: ok" not in out, out
    # an off-site wall point in the 32-site shell of the atom at (6, 0, 6): a
    # fifth neighbour for the reference, refused by the library
    xyz3 = np.vstack([xyz, [[5, 1, 1]]])
    write_points(tmp_path / "p.xyz", xyz3, np.append(sym, "Si"))
    rc, out = run_helper(helper, str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), L)
    assert "product: an atom next to an off-site wall point" in out and "oracle: ok" not in out, out
    # an atom off the diamond sites: the one-byte lattice refuses it
    xyz2 = np.vstack([xyz, [[1, 1, 30]]])
    write_points(tmp_path / "p.xyz", xyz2, np.append(sym, "Si"))
    rc, out = run_helper(helper, str(tmp_path / "start.dat"), str(tmp_path / "p.xyz"), L)
    assert "product: an atom off the diamond sites" in out, out


# InitSt, (Len1, Len2, Len3) in a 240^3 box: the variants of the reference's
# shaped initializers (MS/main.f:224-278) besides those its regression cases
# pin (cube, sphere, inverted-pyramid, finfet), which are covered again here
SHAPES = [("C", (60, 72, 48)), ("S", (96, 0, 0)), ("SS", (96, 0, 0)), ("I", (24, 90, 0)),
          ("D", (24, 90, 0)), ("Z", (24, 90, 0)), ("J", (24, 90, 0)), ("K", (24, 90, 0)),
          ("L", (24, 90, 0)), ("T", (30, 40, 90)), ("Fw", (130, 170, 0)), ("Fa", (130, 170, 75))]


@pytest.mark.parametrize("kind,lens", SHAPES, ids=[k for k, _ in SHAPES])
def test_library_shapes_equal_oracle(helper, tmp_path, kind, lens):
    """The one-byte shaped initializers (mks_shapes::build_shape, the code
    behind mks_init_shape) against the oracle's list-based restatements, every
    site byte, 3C-SiC rates."""
    from mulskips_gb300.startdat import write_startdat
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    for s in range(2):
        for n1 in range(4):
            for n2 in range(4 - n1):
                if n1 + n2:
                    E[s, n1, n2] = 1e13 * np.exp(-0.6 * (n1 + n2) / (8.617e-5 * 1600.0))
    p = str(tmp_path / "start.dat")
    write_startdat(p, E, np.full((3, 3), 0.5), ncrystal=2, list_crystal=(14, 6), init_st=kind, len1=lens[0],
                   lens=lens[1:], run_type="T")
    r = subprocess.run([helper, p, NUMBERS, "@" + kind, "240", "240", "240", *[str(v) for v in lens]],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=900)
    assert r.returncode == 0 and "mismatch 0" in r.stdout, r.stdout


def test_oracle_ss_is_the_pinned_sphere_in_si(oracle_lib, tmp_path):
    """SetNCSpSi (InitSt SS) against the sphere regression case (SetNCSp,
    pinned byte for byte): the same sites, coordinations and first list
    entries, every atom Si."""
    src = os.path.join(GOLDEN, "sphere", "start.dat")
    lines = open(src).read().splitlines()
    assert lines[2].split()[0] == "S"
    lines[2] = "SS ! Initstat"
    (tmp_path / "ss.dat").write_text("\n".join(lines) + "\n")
    o = oracle_lib.Oracle(src, 480, 480, 480)
    o.init()
    ref, _ = oracle_lib.compact_state(o)
    o.close()
    o = oracle_lib.Oracle(str(tmp_path / "ss.dat"), 480, 480, 480)
    o.init()
    ss, _ = oracle_lib.compact_state(o)
    o.close()
    occ = (ref & 3) != 0
    assert occ.sum() > 1000
    assert np.array_equal(ref & 0xFC, ss & 0xFC)
    assert np.array_equal(occ, (ss & 3) != 0) and ((ss[occ] & 3) == 1).all()


def test_oracle_fw_is_the_pinned_setsi_slab_in_sic(oracle_lib, tmp_path):
    """SetSiC3Cww (InitSt Fw) against SetSi (FS, pinned by the Si-SL case) on
    the surface case's start.dat: below the wall block the same walls, sites,
    coordinations and first list entries, the species of the 3C sublattices;
    from Lenww up to LenZ-7 every diamond site a wall."""
    src = os.path.join(GOLDEN, "surface", "start.dat")
    lines = open(src).read().splitlines()
    out = {}
    for kind, lens in (("FS", "120 120 120"), ("Fw", "120 240 0")):
        l2 = list(lines)
        l2[2], l2[3] = f"{kind} ! Initstat", f"{lens} ! Len1 Len2 Len3"
        (tmp_path / f"{kind}.dat").write_text("\n".join(l2) + "\n")
        o = oracle_lib.Oracle(str(tmp_path / f"{kind}.dat"), 480, 480, 480)
        o.init()
        out[kind], _ = oracle_lib.compact_state(o)
        o.close()
    fs, fw = out["FS"], out["Fw"]
    below = slice(0, 240 // 3)
    assert np.array_equal(fs[below] & 0xFC, fw[below] & 0xFC)
    occ = (fw[below] & 3) != 0
    assert occ.sum() > 1000 and set(np.unique(fw[below][occ] & 3)) == {1, 2}
    nz, nb, na = fw.shape
    z1, b, a = np.meshgrid(np.arange(nz), np.arange(nb), np.arange(na), indexing="ij")
    site = ((a + b + (z1 >> 1)) & 1) == 0
    block = site & (3 * z1 >= 240) & (3 * z1 <= 480 - 7)
    assert (fw[block] == 0x80).all()


def test_oracle_variant_species_rules(oracle_lib, tmp_path):
    """The inverted-pyramid variants share one geometry: SetInvPwOnlyCorSi
    (L) is SetInvPwOnlySiorC (K) with the two species swapped, SetInvPC (D)
    is SetInvPSi (Z) with C in place of Si."""
    from mulskips_gb300.startdat import write_startdat
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    for s in range(2):
        for n1 in range(4):
            for n2 in range(4 - n1):
                if n1 + n2:
                    E[s, n1, n2] = 1e13 * np.exp(-0.6 * (n1 + n2) / (8.617e-5 * 1600.0))
    st = {}
    for kind in "KLDZ":
        p = str(tmp_path / f"{kind}.dat")
        write_startdat(p, E, np.full((3, 3), 0.5), ncrystal=2, list_crystal=(14, 6), init_st=kind, len1=24,
                       lens=(90, 0), run_type="T")
        o = oracle_lib.Oracle(p, 240, 240, 240)
        o.init()
        st[kind], _ = oracle_lib.compact_state(o)
        o.close()
    occ = (st["K"] & 3) != 0
    assert occ.sum() > 1000
    swapped = st["K"].copy()
    swapped[occ] = (st["K"][occ] & 0xFC) | (3 - (st["K"][occ] & 3))
    assert np.array_equal(swapped, st["L"])
    assert np.array_equal(st["Z"] & 0xFC, st["D"] & 0xFC)
    assert ((st["Z"][occ] & 3) == 1).all() and ((st["D"][occ] & 3) == 2).all()
    assert np.array_equal(occ, (st["D"] & 3) != 0)


@pytest.fixture(scope="module")
def sicsf_lib(tmp_path_factory):
    import ctypes
    so = str(tmp_path_factory.mktemp("native") / "sicsf_check.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(ROOT, "tests", "native", "sicsf_check.cpp")], check=True)
    L = ctypes.CDLL(so)
    L.sicsf_build.restype = ctypes.c_longlong
    return L


def sicsf_startdat(path, len1, len2, len3, pzig="1.0"):
    """The cube-zigzag start.dat with InitSt E and the given Len1 Len2 Len3
    (SetSiCSF's slab height and the fault's vertex (Len2, Len3, Len1 -
    Len2), main.f:267-272)."""
    lines = open(os.path.join(GOLDEN, "cube-zigzag", "start.dat")).read().splitlines()
    lines[2] = "E ! Initstat"
    lines[3] = f"{len1} {len2} {len3} ! Len1 Len2 Len3"
    lines = [l.replace("0.8 ! PtransZig", f"{pzig} ! PtransZig") for l in lines]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def sicsf_library(lib, L, len1, len2, len3):
    import ctypes
    cap = 4 * L * L * L // 27 + 1024
    lc = np.zeros((L + 1, L, L), np.int32)
    xyz = np.zeros((cap, 3), np.int32)
    nn = np.zeros((cap, 4, 3), np.int32)
    kind = np.zeros(cap, np.int32)
    msg = ctypes.create_string_buffer(256)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    n = lib.sicsf_build(L, L, L, len1, len2, len3, len1 - len2, p(lc), p(xyz), p(nn), p(kind), ctypes.c_longlong(cap),
                        msg, 256)
    return n, msg.value.decode(), lc, xyz[:max(n, 0)], nn[:max(n, 0)], kind[:max(n, 0)]


@pytest.mark.parametrize("lens", [(60, 24, 24), (96, 36, 12), (84, 24, 48)])
def test_sicsf_equals_oracle(sicsf_lib, oracle_lib, tmp_path, lens):
    """InitSt E (SetSiCSF, a triangular triple stacking fault in 3C-SiC):
    the library's host builder (mulskips_gb300/csrc/sicsf.h) gives the
    oracle's LattCoo word for word and its ListAdAtom and ListAtom entry for
    entry, in order, NextN order included (a 120^3 box, three vertices)."""
    L = 120
    sicsf_startdat(tmp_path / "start.dat", *lens)
    o = oracle_lib.Oracle(str(tmp_path / "start.dat"), L, L, L)
    o.init()
    ref_lc = o.lattcoo()
    ref = oracle_lib.list_entries(o)
    o.close()
    n, msg, lc, xyz, nn, kind = sicsf_library(sicsf_lib, L, *lens)
    assert n >= 0, msg
    assert np.array_equal(lc, ref_lc[:L + 1])
    assert (ref["kind"] == 3).sum() == 0
    assert n == len(ref["kind"])
    assert np.array_equal(kind, ref["kind"]) and np.array_equal(xyz, ref["xyz"]) and np.array_equal(nn, ref["nn"])
    z, y, x = np.nonzero(((lc >> 23) & 1) == 1)
    assert ((x % 3 != 0) | (y % 3 != 0) | (z % 3 != 0)).sum() > 10      # the fault's atoms are off the sub-grid


def test_sicsf_refuses_what_the_reference_stops_on(sicsf_lib, oracle_lib, tmp_path):
    L = 120
    for lens, text in (((60, 27, 24), "wrong Site"), ((60, 108, 24), "SF dimension")):
        n, msg, *_ = sicsf_library(sicsf_lib, L, *lens)
        assert n < 0 and text in msg, msg
        sicsf_startdat(tmp_path / "start.dat", *lens)
        o = oracle_lib.Oracle(str(tmp_path / "start.dat"), L, L, L)
        with pytest.raises(Exception):
            o.init()
        o.close()
