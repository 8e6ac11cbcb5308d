"""LA barrier tables of the SiGe model and their theta-derivatives (CPU).

The tables are written out entry by entry as pymulskips' PhaseChange states
them (pymulskips/process.py:1029-1047 evaporation, 1101-1109 deposition) and
compared with the bond-sum form of mulskips_gb300.la.sige_barriers."""
import itertools

import numpy as np
import pytest

from mulskips_gb300 import la


def reference_tables(Ed2, delta, alpha=0.063, beta=0.085):
    E0 = np.zeros((2, 4, 4))
    s, g = Ed2
    E0[0, 1, 0] = 1 * s
    E0[0, 0, 1] = (1 - alpha) * 1 * (s + g) / 2
    E0[0, 1, 1] = (1 - alpha) * 2 * (3 * s + g) / 4
    E0[0, 2, 0] = 2 * s
    E0[0, 0, 2] = (1 - alpha) * 2 * (s + g) / 2
    E0[0, 2, 1] = (1 - alpha) * 3 * (5 * s + g) / 6
    E0[0, 1, 2] = (1 - alpha) * 3 * (2 * s + g) / 3
    E0[0, 3, 0] = 3 * s
    E0[0, 0, 3] = (1 - alpha) * 3 * (s + g) / 2
    E0[1, 1, 0] = (1 + 2 * beta) * 1 * (g + s) / 2
    E0[1, 0, 1] = 1 * g
    E0[1, 1, 1] = (1 + beta) * 2 * (3 * g + s) / 4
    E0[1, 2, 0] = (1 + 2.5 * beta) * 2 * (g + s) / 2
    E0[1, 0, 2] = 2 * g
    E0[1, 2, 1] = (1 + beta) * 3 * (2 * g + s) / 3
    E0[1, 1, 2] = (1 + beta) * 3 * (5 * g + s) / 6
    E0[1, 3, 0] = (1 + 4 * beta) * 3 * (g + s) / 2
    E0[1, 0, 3] = 3 * g
    D0 = np.zeros((2, 3))
    for k in (0, 1):
        D0[k] = [2 * (Ed2[k] - delta[k]), 2 * Ed2[k], 2 * (Ed2[k] + delta[k])]
    return E0, D0


@pytest.mark.parametrize("theta", [la.THETA_REF, (0.5, 2.5, 0.1, 0.3), (1.7, 0.8, 0.05, 0.0)])
def test_tables_match_phasechange(theta):
    E, dE, Ed, dEd = la.sige_barriers(theta)
    E0, D0 = reference_tables(theta[:2], theta[2:])
    np.testing.assert_allclose(E[:2, :, :, 0, 0, 0, 0], E0, rtol=1e-14, atol=0)
    np.testing.assert_allclose(Ed[:2], D0, rtol=1e-14, atol=0)
    # nothing outside the (Si, Ge) census and no third species
    mask = np.zeros(E.shape, dtype=bool)
    mask[:2, :, :, 0, 0, 0, 0] = True
    assert not E[~mask].any() and not Ed[2].any()


def test_derivatives_central_differences():
    th = np.array(la.THETA_REF)
    E, dE, Ed, dEd = la.sige_barriers(th)
    h = 1e-6
    for j in range(4):
        e = np.zeros(4)
        e[j] = h
        Ep, _, Dp, _ = la.sige_barriers(th + e)
        Em, _, Dm, _ = la.sige_barriers(th - e)
        np.testing.assert_allclose((Ep - Em) / (2 * h), dE[..., j], atol=1e-8)
        np.testing.assert_allclose((Dp - Dm) / (2 * h), dEd[..., j], atol=1e-8)


def test_tables_linear_in_theta():
    # every barrier is linear in theta: E(theta) = dE . theta
    th = np.array([0.7, 1.1, 0.2, 0.05])
    E, dE, Ed, dEd = la.sige_barriers(th)
    np.testing.assert_allclose(dE @ th, E, atol=1e-14)
    np.testing.assert_allclose(dEd @ th, Ed, atol=1e-14)


def test_max_rate_bound():
    th = la.THETA_REF
    mat = la.Material()
    E, _, Ed, _ = la.sige_barriers(th)
    r = la.max_rate(th, mat, 1800.0)
    kb = la.KB_EV
    for s, ns, ng in itertools.product((0, 1), range(4), range(4)):
        e = E[s, ns, ng, 0, 0, 0, 0]
        if e:
            assert mat.P0[s] * np.exp(-e / (kb * 1800.0)) <= r * (1 + 1e-12)
    for s, n in itertools.product((0, 1), range(3)):
        assert mat.P0[s] * np.exp(-Ed[s, n] / (kb * mat.Tm[s])) <= r * (1 + 1e-12)


def test_la_params_struct():
    p = la.la_params(la.Material(), la.Pulse(), zsurf=141.0, score=True)
    assert p.P0[0] == pytest.approx(1e13) and p.P0[2] == 0.0
    assert p.Tm[1] == pytest.approx(1210.0) and p.sigma[0] == pytest.approx(300.0)
    assert p.t0 == pytest.approx(100e-9) and p.L_nm == pytest.approx(200.0) and p.score == 1


def test_census_index_enumeration():
    seen = []
    for t in (1, 2, 3):
        for n1 in range(t, -1, -1):
            for n2 in range(t - n1, -1, -1):
                seen.append(la.census_index(n1, n2, t - n1 - n2))
    assert seen == list(range(la.NCENSUS))


def test_class_rates_and_share():
    mat = la.Material()
    r = la.class_rates(la.THETA_REF, mat, 1750.0)
    kb = la.KB_EV
    # Si atom with two Si (or wall) neighbours, Ge atom with two Ge neighbours
    si2 = la.CLS_OCC0 + la.census_index(2, 0, 0)
    ge2 = la.CLS_OCC0 + la.NCENSUS + la.census_index(0, 2, 0)
    assert r[si2] == pytest.approx(1e13 * np.exp(-1.8 / (kb * 1750.0)), rel=1e-12)
    assert r[ge2] == pytest.approx(1e13 * np.exp(-1.3 / (kb * 1750.0)), rel=1e-12)
    assert r[la.CLS_C1D] == 1e-8 and r[la.CLS_ISO] == 0.0
    hist = np.zeros((2, la.NCLASS), dtype=np.int64)
    hist[0, si2] = 1000
    hist[0, ge2] = 1
    hist[1, ge2] = 1000
    hist[:, la.CLS_ISO] = 10 ** 6
    np.testing.assert_allclose(la.share_rate(hist, r), [r[si2], r[ge2]])
