"""InitSt ST of the oracle: SetTrenchSi + rates interpolated per site from a
probability table (SetProbabilityFromField.f, InterpProbFromField.f,
Get_Prob.f:77-91).  No reference output exercises ST, so the checks are
internal: with every table row alike (power-of-two rates, so the
interpolation is exact) a temperature gradient must give the same run as a
fixed temperature; with distinct rows the rate of every listed site must be
the reference's integer-weighted interpolation at the site's temperature."""
import os

import numpy as np
from mulskips_gb300.engine import coordination


def write_st(d, ttop, tbottom, rows, run_type="T", iters=20000, seed=9117116, box=(480, 480, 480),
             lens=(60, 60, 120, 70.0)):
    """start.dat + table file of a Si trench; rows: [(T, (E1, E2, E3), (D1, D2, D3))]."""
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "table.dat"), "w") as f:
        f.write(f"{len(rows)}\n6\n")
        for T, E, D in rows:
            f.write(f"{T}\n")
            for n, e in enumerate(E, 1):
                f.write(f"1 {n} {e!r}\n")
            for n, v in enumerate(D, 1):
                f.write(f"1 {n} {v!r}\n")
    lines = ["1 0 ! NCrystal, NCov", "14 ! species", "ST ! InitSt",
             f"{lens[0]} {lens[1]} {lens[2]} {lens[3]} {ttop} {tbottom} ! Len1 Len2 Len3 angle Ttop Tbottom",
             "1.0 ! PtransZig", "0.4525 ! KMC_sf", "Iter ! ExitStrategy", f"{iters} ! IterMax",
             f"{iters} ! OutMolMol", f"{run_type} ! RunType", f"{seed} ! Random seed", "F ! Save final state",
             "F ! Save final Coor", "table.dat"]
    p = os.path.join(d, "start.dat")
    open(p, "w").write("\n".join(lines) + "\n")
    return p


def test_gradient_with_equal_rows_equals_fixed_temperature(oracle_lib, tmp_path):
    rows = [(T, (4096.0, 64.0, 1.0), (0.5, 0.5, 0.5)) for T in (900, 1000, 1200, 1300)]
    frames = []
    for tag, (tt, tb) in (("fixed", (1100.0, 1100.0)), ("grad", (1250.0, 950.0))):
        p = write_st(str(tmp_path / tag), tt, tb, rows)
        o = oracle_lib.Oracle(p, 480, 480, 480)
        o.init()
        o.run(20000)
        b = str(tmp_path / tag / "f")
        o.write_frame(b, o.time, o.iter)
        frames.append(open(b + ".xyz").read())
        o.close()
    assert frames[0] == frames[1]
    assert int(frames[0].split()[0]) > 1000


def test_site_rates_are_the_interpolated_tables(oracle_lib, tmp_path):
    rows = [(1000, (3.0e4, 7.0e2, 11.0), (0.3, 0.7, 1.3)),
            (1100, (5.0e4, 9.5e2, 17.0), (0.4, 0.9, 1.1)),
            (1250, (9.0e4, 2.1e3, 41.0), (0.6, 1.2, 1.9))]
    tt, tb = 1250.0, 1000.0
    p = write_st(str(tmp_path / "st"), tt, tb, rows, run_type="R")
    o = oracle_lib.Oracle(p, 480, 480, 480, numbers=None)
    o.init()
    st, _ = oracle_lib.compact_state(o)
    lc = o.lattcoo()
    Ts = np.array([r[0] for r in rows])

    def interp(t, col):
        vals = np.array(col, dtype=np.float64)
        k = np.nonzero(Ts == t)[0]
        if k.size:
            return vals[k[0]]
        iu = int(np.nonzero(Ts > t)[0][np.argmin(Ts[Ts > t] - t)])
        wl, wu = Ts[iu] - t, t - Ts[iu - 1]
        return (float(wl) * vals[iu - 1] + float(wu) * vals[iu]) / float(wl + wu)

    checked = 0
    for z1, b, a in zip(*np.nonzero((st != 0) & (st != 0x80))):
        s = int(st[z1, b, a])
        co, sp = int(coordination(np.uint8(s))), s & 3
        if (sp and co > 3) or (not sp and (co == 0 or co == 4)):
            continue
        x, y, z = 3 * (2 * a + (z1 & 1)), 3 * (2 * b + (z1 & 1)), 3 * z1
        which, _, ie, prob = o.site_info(int(x), int(y), int(z))
        if which != 1:
            continue
        t = int((lc[z, y, x] >> 9) & 8191)
        if sp:
            exp = interp(t, [r[1][co - 1] for r in rows])
        elif co == 1 and s >> 7:
            continue                                   # the 1e-6 dummy rate
        else:
            exp = interp(t, [r[2][co - 1] for r in rows]) + 0.0 + 0.0
        assert prob == exp, (x, y, z, t, co, sp, prob, exp)
        checked += 1
    o.close()
    assert checked > 500
