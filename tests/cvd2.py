"""A CVD input with two coverage species (imported by the tests): the
reference's CVD-Si-SiH2 start.dat (Si(001), H coverage) with Cl added as a
second coverage species.  NCrystal = 1, NCov = 2, so the evaporation block
has 19 entries keyed (n1, c1, c2) (SetProbability.f:47-100: the digits of
elind are the crystal then the coverage counts).  Rates: an atom's
evaporation is the H-covered rate of the reference case at c1 + c2 covered
neighbours, times 1.3 per Cl neighbour; Cl absorbs at half and desorbs at
three times the H rates."""
import os

from conftest import GOLDEN

CVD = os.path.join(GOLDEN, "CVD-Si-SiH2", "start.dat")


def two_coverage_startdat(path, run_type="T", seed=9117116, tot_time=None):
    from mulskips_gb300.startdat import parse_startdat
    src = open(CVD).read().splitlines()
    d = parse_startdat(CVD)
    E = d["ptransE"]
    out = ["1 2 ! NCrystal, NCov", "14 ! Atomic numbers of crystal species",
           "1 17 ! Atomic numbers of coverage species"]
    out += src[3:8]
    t = src[8] if tot_time is None else f"{tot_time!r} ! TotTime"
    o = src[9] if tot_time is None else f"{tot_time!r} ! OutTime"
    out += [t, o, f"{run_type} ! RunType", f"{seed} ! Random seed", "F ! Save final state", "F ! Save final Coor"]
    for n1 in (1, 2, 3):
        for c1 in range(0, 5 - n1):
            for c2 in range(0, 5 - n1 - c1):
                v = float(E[0, n1, 0, 0, c1 + c2, 0, 0]) * 1.3 ** c2
                out.append(f"1 {n1}{c1}{c2} {v!r}")
    for k in (1, 2, 3):
        out.append(f"1 {k} {float(d['ptransD'][0, k - 1])!r}")
    for sp, f in ((2, 1.0), (3, 0.5)):
        for k in (1, 2, 3):
            out.append(f"{sp} {k} {float(d['ptransAbs'][0, k]) * f!r}")
    for sp, f in ((2, 1.0), (3, 3.0)):
        for k in (1, 2, 3):
            out.append(f"{sp} {k} {float(d['ptransDes'][0, k]) * f!r}")
    open(path, "w").write("\n".join(out) + "\n")
    return path
