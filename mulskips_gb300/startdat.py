"""start.dat reader/writer — the input format of the reference program.

The reader follows the positional list-directed READs of
mulskips-source/main.f:83-212 and mulskips-source/mcevent/SetProbability.f:21-143
(each READ starts a new record and takes its items from the front of it; the
rest of the record, including '!' comments, is ignored).  The writer follows
pymulskips/setuprun.py:292-389 (print_file_input).
"""
import itertools
import math

import numpy as np

KB_EV = 0.00008617330350

# maxElines of SetProbability.f:47-75, indexed [NCov][NCrystal]
MAX_E_LINES = {(1, 0): 3, (2, 0): 18, (3, 0): 57, (1, 1): 9, (2, 1): 50, (3, 1): 150, (1, 2): 19, (2, 2): 100,
               (3, 2): 288, (1, 3): 34, (2, 3): 172, (3, 3): 480}


class _Records:
    def __init__(self, path):
        self.lines = open(path).read().splitlines()
        self.i = 0

    def line(self):
        if self.i >= len(self.lines):
            raise ValueError("start.dat: unexpected end of file")
        s = self.lines[self.i]
        self.i += 1
        return s

    def items(self, n):
        out = []
        toks = self.line().replace(",", " ").split()
        while len(out) < n:
            if not toks:
                toks = self.line().replace(",", " ").split()
                continue
            out.append(toks.pop(0))
        return out


def _real(s):
    return float(s.replace("d", "e").replace("D", "e"))


def parse_startdat(path):
    r = _Records(path)
    d = {}
    nc, ncov = (int(x) for x in r.items(2))
    d["ncrystal"], d["ncov"] = nc, ncov
    if not 1 <= nc <= 3 or not 0 <= ncov <= 3:
        raise ValueError("NCrystal must be 1..3 and NCov 0..3")
    d["list_crystal"] = [int(x) for x in r.items(nc)]
    d["list_cov"] = [int(x) for x in r.items(ncov)] if ncov else []
    d["init_st"] = r.items(1)[0][:2]
    st = d["init_st"]
    if st == "FF":
        d["len"] = [int(x) for x in r.items(4)]
    elif st == "ST":
        it = r.items(6)
        d["len"] = [int(x) for x in it[:3]]
        d["angle"], d["Ttop"], d["Tbottom"] = (_real(x) for x in it[3:])
    elif st in ("IN", "SH"):
        d["cadfilename"] = r.line().strip()
    elif st == "LA":
        d["cadfilename"] = r.line().strip()
        d["tempfilename"] = r.line().strip()
        d["Tm"] = _real(r.items(1)[0])
        d["P0"] = _real(r.items(1)[0])
        d["sigma"] = _real(r.items(1)[0])
        d["Tflex"] = _real(r.items(1)[0])
        d["LenVac"] = _real(r.items(1)[0])
        d["LenNuc"] = _real(r.items(1)[0])
        d["Homogeneous"] = r.items(1)[0][:2]
    else:
        d["len"] = [int(x) for x in r.items(3)]
    lc = d["list_crystal"]
    if lc[:2] == [14, 32] and (nc == 2 or (nc == 3 and lc[2] == 5)):
        d["alloyfraction"] = _real(r.items(1)[0])
    d["ptrans_zig"] = _real(r.items(1)[0])
    d["sf"] = _real(r.items(1)[0])
    d["exit_strategy"] = r.items(1)[0][:4]
    if d["exit_strategy"] == "Iter":
        d["max_iter"] = int(r.items(1)[0])
        d["out_molmol"] = int(r.items(1)[0])
    elif d["exit_strategy"] == "Time":
        d["max_time"] = _real(r.items(1)[0])
        d["out_time"] = _real(r.items(1)[0])
    d["run_type"] = r.items(1)[0][:2]
    d["idum"] = int(r.items(1)[0])
    d["save_final_state"] = r.items(1)[0][:2]
    if d["save_final_state"] == "T":
        d["restartfilename"] = r.line().strip()
    d["save_coo"] = r.items(1)[0][:2]
    if d["save_coo"] == "T":
        d["coofilename"] = r.line().strip()
    pE = np.zeros((3, 4, 4, 4, 4, 4, 4))
    pD = np.zeros((3, 3))
    pAbs = np.zeros((3, 4))
    pDes = np.zeros((3, 4))
    for _ in range(MAX_E_LINES[(nc, ncov)]):
        s, el, v = r.items(3)
        s, el = int(s), int(el)
        if not 1 <= s <= nc:
            raise ValueError("1st index in evap prob must be <= NCrystal")
        idx = [0] * 6
        for j in range(1, nc + 1):
            idx[j - 1] = (el // 10 ** (nc + ncov - j)) % 10
        for j in range(nc + 1, nc + ncov + 1):
            idx[3 + j - nc - 1] = (el // 10 ** (nc + ncov - j)) % 10
        pE[(s - 1, *idx)] = _real(v)
    for _ in range(nc * 3):
        s, el, v = r.items(3)
        pD[int(s) - 1, int(el) - 1] = _real(v)
    for _ in range(ncov * 3):
        s, el, v = r.items(3)
        pAbs[int(s) - nc - 1, int(el)] = _real(v)
    for _ in range(ncov * 3):
        s, el, v = r.items(3)
        pDes[int(s) - nc - 1, int(el)] = _real(v)
    d["ptransE"], d["ptransD"], d["ptransAbs"], d["ptransDes"] = pE, pD, pAbs, pDes
    return d


def read_shape_points(path):
    """The point-list file of InitSt SH (SetShape.f:52-79): NFilled, one
    skipped record, then NFilled records `sym x y z`.  Returns (xyz [n, 3]
    int32, species [n] int8): 1 for 'Si', 2 for 'C' or 'Ge', 0 for any other
    symbol (sym is read as two characters)."""
    with open(path) as f:
        n = int(f.readline().replace(",", " ").split()[0])
        f.readline()
        xyz = np.zeros((n, 3), dtype=np.int32)
        sp = np.zeros(n, dtype=np.int8)
        i = 0
        while i < n:
            t = f.readline()
            if not t:
                raise ValueError("shape file: fewer than NFilled records")
            t = t.replace(",", " ").split()
            if len(t) < 4:
                raise ValueError("shape file: short record")
            sym = t[0][:2]
            sp[i] = 1 if sym == "Si" else (2 if sym in ("C", "Ge") else 0)
            xyz[i] = [int(t[1]), int(t[2]), int(t[3])]
            i += 1
    return xyz, sp


def write_plain_si_startdat(path, T=1100.0, e_bond=0.6, nu=1e13, flux=0.5, len1=120, max_iter=1000000,
                            out_molmol=None, run_type="R", seed=1, sf=5.43 / 12, lens=(120, 120)):
    """start.dat of the plain Si(001) model (InitSt FS, NCrystal 1): PTransE(1,n)
    = nu*exp(-n*e_bond/kT), PTransD(1,n) = flux."""
    e = [nu * math.exp(-n * e_bond / (KB_EV * T)) for n in (1, 2, 3)]
    out_molmol = out_molmol or max_iter
    lines = ["1 0 ! NCrystal, NCov", "14 ! Atomic numbers of crystal species", "FS ! Initstat",
             f"{len1} {lens[0]} {lens[1]} ! Len1 Len2 Len3", "1.0 ! PtransZig",
             f"{sf:.15f} ! KMC_sf", "Iter ! ExitStrategy", f"{max_iter} ! IterMax",
             f"{out_molmol} ! OutMolMol", f"{run_type} ! RunType", f"{seed} ! Random seed",
             "F ! Save final state", "F ! Save final Coor"]
    lines += [f"1 {n} {e[n - 1]!r} ! PtransE[1,{n}]" for n in (1, 2, 3)]
    lines += [f"1 {n} {flux!r} ! PtransD[1,{n}]" for n in (1, 2, 3)]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_startdat(path, ptransE, ptransD, ncrystal=1, list_crystal=(14,), init_st="FS", len1=120,
                   max_iter=1000000, out_molmol=None, run_type="R", seed=1, sf=5.43 / 12, lens=(120, 120),
                   alloy_fraction=0.0, ptrans_zig=1.0, points=None):
    """start.dat for NCrystal 1..3 species without coverage (main.f:83-212
    grammar): every PTransE(s, n_1..n_NCrystal) entry with 1 <= sum n <= 3 and
    the 3 PTransD entries of each species, from arrays in the engine layout
    (ptransE (3,4,4,4,4,4,4), ptransD (3,3)).  Si/Ge lists carry the alloy
    fraction record that main.f reads after the box sizes.  InitSt SH takes
    the point file's path (`points`) on the line where the others read the
    box sizes (main.f:224-278)."""
    E = np.asarray(ptransE, dtype=np.float64).reshape(3, 4, 4, 4, 4, 4, 4)
    D = np.asarray(ptransD, dtype=np.float64).reshape(3, 3)
    out_molmol = out_molmol or max_iter
    lc = " ".join(str(int(z)) for z in list_crystal[:ncrystal])
    if (init_st == "SH") != (points is not None):
        raise ValueError("InitSt SH needs a point file, and only SH takes one")
    lines = [f"{ncrystal} 0 ! NCrystal, NCov", f"{lc} ! Atomic numbers of crystal species",
             f"{init_st} ! Initstat", points if points is not None else f"{len1} {lens[0]} {lens[1]} ! Len1 Len2 Len3"]
    if ncrystal >= 2 and tuple(list_crystal[:2]) == (14, 32):
        lines.append(f"{float(alloy_fraction)!r} ! alloy fraction")
    lines += [f"{float(ptrans_zig)!r} ! PtransZig", f"{sf:.15f} ! KMC_sf", "Iter ! ExitStrategy", f"{max_iter} ! IterMax",
              f"{out_molmol} ! OutMolMol", f"{run_type} ! RunType", f"{seed} ! Random seed",
              "F ! Save final state", "F ! Save final Coor"]
    for s in range(ncrystal):
        for n in itertools.product(range(4), repeat=ncrystal):
            if not 1 <= sum(n) <= 3:
                continue
            idx = tuple(n) + (0,) * (3 - ncrystal)
            code = "".join(str(d) for d in n)
            lines.append(f"{s + 1} {code} {float(E[(s,) + idx + (0, 0, 0)])!r} ! PtransE")
    for s in range(ncrystal):
        for n in (1, 2, 3):
            lines.append(f"{s + 1} {n} {float(D[s, n - 1])!r} ! PtransD")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
