"""Confidence bands of the statistical parity tests (imported by them).

A test compares k observables of n1 GPU replicas with those of n2 seeds of
the serial oracle.  For each observable the difference of the two sample
means must lie inside the two-sided Welch t band at level 1 - 0.05 / k
(Bonferroni correction over the k observables of the test), so that the test
as a whole holds with 95 % confidence when both samplers have the same
distribution.  Seeds are fixed, so each test is deterministic."""
import json
import math
import os

import numpy as np

FAMILY_ALPHA = 0.05


def welch_band(x, y, k=1, alpha=FAMILY_ALPHA):
    """(difference of means x - y, band half-width, t quantile) at the
    per-observable level 1 - alpha / k."""
    from scipy import stats
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    vx, vy = x.var(ddof=1) / len(x), y.var(ddof=1) / len(y)
    se = math.sqrt(vx + vy)
    if se == 0.0:
        return float(x.mean() - y.mean()), 0.0, float("inf")
    dof = (vx + vy) ** 2 / (vx * vx / (len(x) - 1) + vy * vy / (len(y) - 1))
    q = float(stats.t.ppf(1.0 - alpha / (2.0 * k), dof))
    return float(x.mean() - y.mean()), q * se, q


class Family:
    """The k observables of one test: add() each, then check() them all."""

    def __init__(self, title, k, extra=None):
        self.title, self.k, self.rows, self.extra = title, k, [], extra

    def add(self, name, gpu, ref):
        d, hw, q = welch_band(gpu, ref, self.k)
        self.rows.append((name, np.mean(gpu), np.std(gpu, ddof=1), np.mean(ref), np.std(ref, ddof=1), d, hw, q,
                          len(gpu), len(ref)))

    def report(self):
        out = [f"{self.title}: 95 % family band, Bonferroni over {self.k} observables"]
        for name, mg, sg, mr, sr, d, hw, q, ng, nr in self.rows:
            rel = f" ({100 * d / mr:+.2f} % of ref)" if mr else ""
            out.append(f"  {name}: gpu {mg:.6g} +- {sg:.3g} (n={ng})  serial {mr:.6g} +- {sr:.3g} (n={nr})  "
                       f"diff {d:.4g}{rel}  band +-{hw:.4g} (t={q:.3f})")
        return "\n".join(out)

    def record(self):
        """Append the family's rows to the JSON-lines file named by
        MKS_STATS_OUT, if set (a record of the measured bands)."""
        path = os.environ.get("MKS_STATS_OUT")
        if not path:
            return
        rows = [{"observable": r[0], "gpu_mean": float(r[1]), "gpu_sd": float(r[2]), "ref_mean": float(r[3]),
                 "ref_sd": float(r[4]), "diff": float(r[5]), "band": float(r[6]), "t": float(r[7]),
                 "n_gpu": int(r[8]), "n_ref": int(r[9])} for r in self.rows]
        rec = {"test": os.environ.get("PYTEST_CURRENT_TEST", "").split(" ")[0], "family": self.title, "k": self.k,
               "rows": rows}
        if self.extra:
            rec.update(self.extra)
        with open(path, "a") as f:
            f.write(json.dumps(rec) + "\n")

    def check(self):
        assert len(self.rows) == self.k, "every observable of the family must be compared"
        print("\n" + self.report())
        self.record()
        bad = [r[0] for r in self.rows if not abs(r[5]) <= r[6]]
        assert not bad, f"outside the band: {bad}\n{self.report()}"
