"""Laser-anneal (LA) melt / regrowth of SiGe with barrier gradients.

The rate law is the LA branch of the reference's Get_Prob
(mulskips-source/mcevent/Get_Prob.f:127-149,
mulskips-source-LaserAnnealing/mcevent/Get_Prob.f:127-152):

* melting of an atom of species s:  P0(s) exp(-E / kB T)
* solidification of s on a liquid site of coordination n:
  0.5 P0(s) xliq(s) exp(-Ed(s, n) / kB Tm(s)) (1 + erf((T - Tflex(s)) / A(s)))

with the barriers E, Ed of the SiGe parametrisation of pymulskips'
PhaseChange (pymulskips/process.py:1006-1120).  The four parameters theta =
(Ed2_Si, Ed2_Ge, delta_Si, delta_Ge) are differentiated: every replica
accumulates on the GPU the likelihood-ratio score

    S_j = sum_events d log k / d theta_j - int sum_sites d k / d theta_j dt

in FP64, and `Batch.lr_grad` turns scores and per-replica values f into the
gradient of E[f] (the backward step).  `RegrowthVelocity` wraps forward
(simulate, measure the regrowth velocity) and backward (score reduction) as a
torch.autograd.Function.

The temperature field is prescribed: T(z, t) = Tb + Ta exp(-((t - t0)/w)^2)
exp(-depth / L), depth below the initial surface, in integer K, per layer, at
each window's midpoint.  Liquid = molten (empty) sites below the initial
surface: a species' liquid is the atoms of it that melted.
"""
import math
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .engine import Batch, KB_EV

THETA_NAMES = ("Ed2_Si", "Ed2_Ge", "delta_Si", "delta_Ge")
# reference calibration of the SiGe examples
# (examples/ex4-LA-SiGe/*/MulSKIPS_LA_sockets.py: Ed2, delta = 0.03 Ed2)
THETA_REF = (0.90, 0.65, 0.027, 0.0195)

# SiGe_X evaporation energetics, pymulskips/process.py:1027-1052
ALPHA = 0.063          # Si atom with Ge neighbours: (1 - alpha) x bond sum
BETA = 0.085           # Ge atom with Si neighbours: (1 + k beta) x bond sum
GE_ALL_SI_K = {1: 2.0, 2: 2.5, 3: 4.0}   # k for a Ge atom whose neighbours are all Si


def sige_barriers(theta):
    """Barrier tables of the SiGe_X model and their derivatives.

    Returns (E, dE, Ed, dEd): E the PTransE table (3,4,4,4,4,4,4) in eV,
    indexed [species][n_Si][n_Ge][n_3][cov...] like start.dat (species 0 = Si,
    1 = Ge), dE = dE/dtheta (..., 4); Ed the PTransD table (3, 3) (species,
    coordination 1..3) and dEd (3, 3, 4).

    Evaporation (process.py:1029-1047): the barrier of an atom is its bond
    sum, a like bond counting Ed2 of the species and a Si-Ge bond the mean of
    the two, scaled by (1 - alpha) for a Si atom with any Ge neighbour and by
    (1 + k beta) for a Ge atom with any Si neighbour (k = 1 with mixed
    neighbours, 2 / 2.5 / 4 for 1 / 2 / 3 Si neighbours only).
    Solidification (process.py:1101-1109): Ed(s, n) = 2 (Ed2_s + (n - 2) delta_s).
    """
    th = np.asarray(theta, dtype=np.float64).reshape(4)
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    dE = np.zeros(E.shape + (4,))
    for s in (0, 1):
        for ns in range(4):
            for ng in range(4):
                n = ns + ng
                if n < 1 or n > 3:
                    continue
                # bond sum as coefficients of (Ed2_Si, Ed2_Ge)
                if s == 0:
                    c = np.array([ns + 0.5 * ng, 0.5 * ng])
                    fac = (1.0 - ALPHA) if ng > 0 else 1.0
                else:
                    c = np.array([0.5 * ns, ng + 0.5 * ns])
                    if ns == 0:
                        fac = 1.0
                    elif ng == 0:
                        fac = 1.0 + GE_ALL_SI_K[ns] * BETA
                    else:
                        fac = 1.0 + BETA
                E[s, ns, ng, 0, 0, 0, 0] = fac * (c[0] * th[0] + c[1] * th[1])
                dE[s, ns, ng, 0, 0, 0, 0, 0] = fac * c[0]
                dE[s, ns, ng, 0, 0, 0, 0, 1] = fac * c[1]
    Ed = np.zeros((3, 3))
    dEd = np.zeros((3, 3, 4))
    for s in (0, 1):
        for n in (1, 2, 3):
            Ed[s, n - 1] = 2.0 * (th[s] + (n - 2) * th[2 + s])
            dEd[s, n - 1, s] = 2.0
            dEd[s, n - 1, 2 + s] = 2.0 * (n - 2)
    return E, dE, Ed, dEd


@dataclass
class Material:
    """Per-species constants of the LA rate law (species Si, Ge).  Tm, A and
    Tflex follow pymulskips/process.py:926 and the SiGe examples; P0 is the
    attempt frequency nu."""
    P0: tuple = (1e13, 1e13)
    Tm: tuple = (1688.0, 1210.0)
    Tflex: tuple = (1110.0, 900.0)
    A: tuple = (300.0, 210.0)


@dataclass
class Pulse:
    """T(z, t) = Tb + Ta exp(-((t - t0)/w)^2) exp(-depth / L)."""
    Tb: float = 300.0
    Ta: float = 1500.0
    t0: float = 100e-9
    w: float = 40e-9
    L_nm: float = 200.0


def la_params(mat, pulse, zsurf, score=True):
    p = N.MksLaParams()
    for s in range(3):
        k = min(s, len(mat.P0) - 1)
        p.P0[s] = mat.P0[k] if s < len(mat.P0) else 0.0
        p.Tm[s] = mat.Tm[k]
        p.Tflex[s] = mat.Tflex[k]
        p.sigma[s] = mat.A[k]
    p.Tb, p.Ta, p.t0, p.w, p.L_nm = pulse.Tb, pulse.Ta, pulse.t0, pulse.w, pulse.L_nm
    p.zsurf = float(zsurf)
    p.score = 1 if score else 0
    p.liquid_weighting = 1
    return p


def max_rate(theta, mat, T_peak):
    """Largest single-site rate the law can reach at temperature T_peak (the
    bound that sets the window length)."""
    E, _, Ed, _ = sige_barriers(theta)
    r = 0.0
    for s in (0, 1):
        e = E[s][E[s] != 0]
        if e.size:
            r = max(r, mat.P0[s] * math.exp(-float(e.min()) / (KB_EV * T_peak)))
        d = Ed[s][Ed[s] != 0]
        if d.size:
            r = max(r, mat.P0[s] * math.exp(-float(d.min()) / (KB_EV * mat.Tm[s])))
    return r


# rate classes of the engine (mulskips_gb300/csrc/lattice.cuh)
CLS_C1, CLS_C1D, CLS_C2, CLS_C3, CLS_ISO, CLS_OCC0, NCENSUS, CLS_C1I, NCLASS = 1, 2, 3, 4, 5, 6, 19, 63, 64


def census_index(n1, n2, n3):
    """Index of the neighbour census (n1, n2, n3), 1 <= sum <= 3, ordered by
    total, then n1 and n2 descending (the engine's enumeration)."""
    t = n1 + n2 + n3
    k = {1: 0, 2: 3, 3: 9}[t]
    for a in range(t, n1, -1):
        k += t - a + 1
    return k + (t - n1) - n2


def class_rates(theta, mat, T, xliq=(1.0, 1.0, 1.0)):
    """Rate of one site of every engine class under the LA law at
    temperature T (liquid fractions xliq for the solidification classes)."""
    E, _, Ed, _ = sige_barriers(theta)
    return class_rates_tables(E, Ed, mat, T, xliq)


def class_rates_tables(E, Ed, mat, T, xliq=(1.0, 1.0, 1.0)):
    """class_rates for barrier tables E (PTransE layout) and Ed (3, 3)."""
    E = np.asarray(E, dtype=np.float64).reshape(3, 4, 4, 4, 4, 4, 4)
    Ed = np.asarray(Ed, dtype=np.float64).reshape(3, 3)
    r = np.zeros(NCLASS)
    for sp in range(min(3, len(mat.P0))):
        for n1 in range(4):
            for n2 in range(4 - n1):
                for n3 in range(4 - n1 - n2):
                    if n1 + n2 + n3 == 0:
                        continue
                    e = E[sp, n1, n2, n3, 0, 0, 0]
                    if e:
                        r[CLS_OCC0 + sp * NCENSUS + census_index(n1, n2, n3)] = \
                            mat.P0[sp] * math.exp(-e / (KB_EV * T))
    for co, cls in ((1, CLS_C1), (2, CLS_C2), (3, CLS_C3)):
        for sp in range(min(3, len(mat.P0))):
            d = Ed[sp, co - 1]
            if d:
                r[cls] += 0.5 * mat.P0[sp] * xliq[sp] * math.exp(-d / (KB_EV * mat.Tm[sp])) * \
                    (1.0 + math.erf((T - mat.Tflex[sp]) / mat.A[sp]))
    r[CLS_C1D] = 1e-8      # Get_Prob.f:183
    r[CLS_C1I] = 1e-6      # Get_Prob_Ini.f:104, dummies written by an initializer
    return r


def share_rate(hist, rates):
    """Rate of the class carrying the largest share of the total rate (the
    isolated-atom and dummy classes left out), per replica."""
    w = hist.astype(np.float64) * rates[None, :]
    w[:, CLS_ISO] = 0.0
    w[:, CLS_C1D] = 0.0
    w[:, CLS_C1I] = 0.0
    return rates[np.argmax(w, axis=1)]


@dataclass
class Anneal:
    """A batch of SiGe LA replicas: box (LenX, LenY, LenZ) grid units, slab
    height len1, Ge fraction x_ge, one seed per replica."""
    n: int
    box: tuple = (768, 768, 3072)
    len1: int = 2880
    x_ge: float = 0.2
    seed: int = 4
    mat: Material = field(default_factory=Material)
    pulse: Pulse = field(default_factory=Pulse)
    f_tau: float = 0.3
    sf: float = 5.43 / 12
    tau_rule: str = "share"     # "share": dominant class; "max": fastest class

    def __post_init__(self):
        self.batch = Batch([self.box] * self.n, [self.seed * 1000003 + i for i in range(self.n)], ncrystal=2,
                           list_crystal=(14, 32), sf=self.sf)
        self.zsurf = self.len1 - (self.len1 % 24) - 3          # top atom layer (grid units)
        self.area = (self.box[0] // 6) * (self.box[1] // 6) // 2   # sites per layer
        self.layer_nm = 3 * self.sf / 10.0
        self.t = 0.0

    def start(self, theta, score=True, tau=None):
        """Fresh slabs, barrier tables for theta, clock at 0, scores at 0.
        tau: window length; default f_tau / (largest rate at the peak
        temperature)."""
        E, dE, Ed, dEd = sige_barriers(theta)
        self.theta = np.asarray(theta, dtype=np.float64)
        b = self.batch
        b.set_rates(np.broadcast_to(E, (self.n,) + E.shape), np.broadcast_to(Ed, (self.n, 3, 3)))
        b.init_alloy(self.len1, self.x_ge, self.seed)
        p = la_params(self.mat, self.pulse, self.zsurf, score)
        b.set_la(p, np.broadcast_to(dE, (self.n,) + dE.shape) if score else None,
                 np.broadcast_to(dEd, (self.n,) + dEd.shape) if score else None)
        self.tau_fixed = tau
        self.t = 0.0
        self.c0 = b.la_counts()[0].sum(axis=1)

    def tau_at(self, ta, tb):
        """Window length for [ta, tb] at the hottest surface temperature the
        pulse reaches in that interval: f_tau over the rate of the class
        carrying the largest share of the current event sites' total rate
        (rule "share", the accuracy rule of the plain model), or over the
        fastest rate the law allows (rule "max"); one length for the batch."""
        p = self.pulse
        tc = min(max(p.t0, ta), tb)
        T_max = p.Tb + p.Ta * math.exp(-((tc - p.t0) / p.w) ** 2)
        if self.tau_rule == "max":
            return self.f_tau / max_rate(self.theta, self.mat, T_max)
        r = share_rate(self.batch.class_histogram(), class_rates(self.theta, self.mat, T_max))
        return self.f_tau / float(np.max(r))

    def advance(self, t_end, segment=1e-9, on_segment=None):
        """Run every replica to time t_end in segments, each cut into a
        multiple of 8 windows no longer than its tau (the fixed tau given to
        start, else tau_at of the segment) and ending exactly at the segment
        end.  A segment is `segment` long, or 8 windows when those are
        longer (cold stretches of the pulse).  on_segment() is called after
        each segment."""
        ev = 0
        while self.t < t_end * (1.0 - 1e-12):
            if self.tau_fixed:
                te, tau0 = (min(t_end, self.t + segment) if on_segment else t_end), self.tau_fixed
            else:
                te = min(t_end, self.t + segment)
                tau0 = self.tau_at(self.t, te)
                if 8.0 * tau0 > te - self.t and te < t_end:
                    te = min(t_end, self.t + 8.0 * tau0)
                    tau0 = min(tau0, self.tau_at(self.t, te))
            dt = te - self.t
            nw = max(8, int(math.ceil(dt / tau0 / 8.0 - 1e-9)) * 8)
            tau = dt / nw
            ev += self.batch.run(tau, nw, 0, self.t + dt - 0.5 * tau)
            self.t = te
            if on_segment:
                on_segment()
        return ev

    def crystal(self):
        """Crystal atoms per replica (n,)."""
        return self.batch.la_counts()[0].sum(axis=1)

    def velocity(self, t1, t2, causal=False):
        """Regrowth velocity (m/s) per replica between t1 and t2: crystal
        atoms gained / sites per layer x layer thickness / (t2 - t1).  With
        causal, each segment's share of it is passed to the engine's causal
        LR accumulation as the segment ends (batch.lr_result() then gives
        the gradient of the mean velocity)."""
        scale = self.layer_nm * 1e-9 / (self.area * (t2 - t1))
        self.advance(t1)
        n1 = self.crystal()
        if causal:                                  # start() cleared the sums
            last = [n1]

            def step():
                c = self.crystal()
                self.batch.lr_accumulate((c - last[0]).astype(np.float64) * scale)
                last[0] = c

            self.advance(t2, on_segment=step)
        else:
            self.advance(t2)
        n2 = self.crystal()
        self.last_v = (n2 - n1).astype(np.float64) * scale
        return self.last_v


def regrowth_velocity_lr(sim, theta, t1, t2):
    """Mean regrowth velocity over the replicas and its LR gradient (the
    causal form: each segment's velocity increment weighted by the score of
    the path before it)."""
    sim.start(theta, score=True)
    v = sim.velocity(t1, t2, causal=True)
    g, se = sim.batch.lr_result()
    return v, g, se


def _autograd_function():
    import torch

    class RegrowthVelocity(torch.autograd.Function):
        """v(theta) = mean regrowth velocity of an `Anneal` batch between t1
        and t2; backward returns the likelihood-ratio gradient."""

        @staticmethod
        def forward(ctx, theta, sim, t1, t2):
            th = theta.detach().cpu().double().numpy()
            sim.start(th, score=True)
            v = sim.velocity(t1, t2, causal=True)
            g, se = sim.batch.lr_result()
            sim.last_grad = (g, se)
            ctx.save_for_backward(torch.as_tensor(g, dtype=theta.dtype, device=theta.device))
            ctx.se = se
            return torch.as_tensor(float(v.mean()), dtype=theta.dtype, device=theta.device)

        @staticmethod
        def backward(ctx, gout):
            (g,) = ctx.saved_tensors
            return gout * g, None, None, None

    return RegrowthVelocity


_RV = None


def regrowth_velocity(theta, sim, t1, t2):
    """torch entry point: differentiable mean regrowth velocity."""
    global _RV
    if _RV is None:
        _RV = _autograd_function()
    return _RV.apply(theta, sim, t1, t2)
