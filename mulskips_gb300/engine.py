"""Python face of the GB300 KMC engine (a thin layer over the C ABI).

`Lattice` is one KMC system (the plain path, `mks_*`); `Batch` holds many
independent replicas advanced together (`mks_batch_*`).  Both keep their
state on the GPU; the methods copy in and out through host buffers.
"""
import ctypes as C
import math

import numpy as np

from . import _native as N

KB_EV = 0.00008617330350  # Boltzmann constant in eV/K, mulskips-source/mcevent/Get_Prob.f:70


def coordination(st):
    """Coordination of every site of a compact state (numpy uint8 array in
    the layout of mks_get_state): bits 2-4, where the value 5 of an
    initializer's dummy coor-1 site (Get_Prob_Ini's rate) reads as 1."""
    st = np.asarray(st, dtype=np.uint8)
    return (st >> 2) & (7 ^ (st & 4))


def arrhenius_tables(T, e_bond=0.6, nu=1e13, flux=0.5, ncrystal=1):
    """PTransE / PTransD arrays of the plain Si(001) model: evaporation rate
    nu*exp(-n*e_bond/kT) for an atom with n bonded neighbours (n = 1..3) and a
    deposition rate `flux` on every empty site with >= 1 bonded neighbour."""
    pE = np.zeros((3, 4, 4, 4, 4, 4, 4), dtype=np.float64)
    pD = np.zeros((3, 3), dtype=np.float64)
    for n in (1, 2, 3):
        pE[0, n, 0, 0, 0, 0, 0] = nu * math.exp(-n * e_bond / (KB_EV * T))
        pD[0, n - 1] = flux
    return pE, pD


def _cfg(lenx, leny, lenz, ncrystal, list_crystal, ptrans_zig, sf, seed, list_cov=()):
    c = N.MksConfig()
    c.lenx, c.leny, c.lenz = int(lenx), int(leny), int(lenz)
    c.ncrystal, c.ncov = int(ncrystal), len(list_cov)
    lc = list(list_crystal) + [0] * (3 - len(list_crystal))
    lv = list(list_cov) + [0] * (3 - len(list_cov))
    for i in range(3):
        c.list_crystal[i] = int(lc[i])
        c.list_cov[i] = int(lv[i])
    c.ptrans_zig = float(ptrans_zig)
    c.sf = float(sf)
    c.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return c


def _site_rates(h, rep, xyz):
    p = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
    n = p.shape[0]
    cls = np.zeros(max(n, 1), dtype=np.int32)
    rate = np.zeros(max(n, 1), dtype=np.float32)
    N.check(N.lib().mks_site_rates(h, int(rep), N.ptr(p), n, N.ptr(cls), N.ptr(rate)))
    return cls[:n], rate[:n]


class Lattice:
    """One KMC system on the GPU.  list_cov: atomic number of the coverage
    species (at most one; e.g. (1,) for H in CVD)."""

    def __init__(self, lenx, leny, lenz, ncrystal=1, list_crystal=(14,), ptrans_zig=1.0, sf=5.43 / 12,
                 seed=1, list_cov=(), explicit_nn=False):
        """explicit_nn: run the explicit-neighbour engine even at PtransZig = 1
        (the engine of PtransZig < 1; needed for atoms off the diamond sites,
        InitSt 'E')."""
        self.dims = (int(lenx), int(leny), int(lenz))
        self.na, self.nb, self.nz = lenx // 6, leny // 6, lenz // 3 + 1
        h = C.c_void_p()
        cfg = _cfg(lenx, leny, lenz, ncrystal, list_crystal, ptrans_zig, sf, seed, list_cov)
        cfg.explicit_nn = 1 if explicit_nn else 0
        N.check(N.lib().mks_create(C.byref(cfg), C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            N.lib().mks_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_rates(self, ptransE, ptransD):
        e = np.ascontiguousarray(ptransE, dtype=np.float64).reshape(-1)
        d = np.ascontiguousarray(ptransD, dtype=np.float64).reshape(-1)
        assert e.size == 3 * 4096 and d.size == 9
        N.check(N.lib().mks_set_rates(self._h, N.ptr(e), N.ptr(d)))

    def set_coverage_rates(self, ptransAbs, ptransDes):
        """PtransAbs / PtransDes as 3x3 [coverage species][coor-1]."""
        a = np.ascontiguousarray(ptransAbs, dtype=np.float64).reshape(-1)
        d = np.ascontiguousarray(ptransDes, dtype=np.float64).reshape(-1)
        assert a.size == 9 and d.size == 9
        N.check(N.lib().mks_set_coverage_rates(self._h, N.ptr(a), N.ptr(d)))

    def init_flat(self, kind="S", len1=120):
        N.check(N.lib().mks_init_flat(self._h, kind.encode()[:1], int(len1)))

    def init_shape(self, init_st, lens, params=None):
        """The reference's shaped lattices: 'C' (SetNC), 'S' (SetNCSp), 'SS'
        (SetNCSpSi), 'I' (SetInvPOff) and its variants 'D', 'Z', 'J', 'K', 'L',
        'T' (SetTrench), 'Fw' / 'Fa' (SetSiC3Cww / SetSiC3Cwwaperture), 'FF'
        (SetSiFINFET), 'ST' (SetTrenchSi, params = angle, Ttop, Tbottom), 'E'
        (SetSiCSF, a stacking fault off the diamond sites: a handle made with
        ptrans_zig < 1 or explicit_nn=True, rates set first)."""
        l = np.zeros(4, dtype=np.int32)
        l[:len(lens)] = lens
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
        N.check(N.lib().mks_init_shape(self._h, init_st.encode(), N.ptr(l), None if p is None else N.ptr(p)))

    def init_cad(self, geo):
        """SetCAD (InitSt IN) from the LattGeo id of every grid point, [z, y, x]."""
        g = np.ascontiguousarray(geo, dtype=np.int8)
        assert g.size == self.dims[0] * self.dims[1] * self.dims[2]
        N.check(N.lib().mks_batch_init_cad(self._h, 0, N.ptr(g)))

    def init_points(self, xyz, species):
        """SetShape (InitSt SH) from grid points xyz [n, 3] with species 1 (Si)
        or 2 (C / Ge); startdat.read_shape_points reads the reference's file."""
        p = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        sp = np.ascontiguousarray(species, dtype=np.int8).reshape(-1)
        assert sp.size == p.shape[0]
        N.check(N.lib().mks_init_points(self._h, N.ptr(p), N.ptr(sp), int(sp.size)))

    def replay(self, events):
        ev = np.ascontiguousarray(events, dtype=N.EVENT_DTYPE)
        N.check(N.lib().mks_replay(self._h, N.ptr(ev), int(ev.size)))

    def run(self, tau, max_windows, max_events=0, max_time=0.0):
        ne = C.c_int64()
        t = C.c_double()
        N.check(N.lib().mks_run(self._h, float(tau), int(max_windows), int(max_events), float(max_time),
                                C.byref(ne), C.byref(t)))
        return ne.value, t.value

    def state(self):
        n = N.lib().mks_state_size(self._h)
        a = np.empty(n, dtype=np.uint8)
        N.check(N.lib().mks_get_state(self._h, N.ptr(a), n))
        return a.reshape(self.nz, self.nb, self.na)

    def set_state(self, st):
        a = np.ascontiguousarray(st, dtype=np.uint8).reshape(-1)
        N.check(N.lib().mks_set_state(self._h, N.ptr(a), a.size))

    def set_state_ptr(self, addr, n):
        """Upload from a raw host address (e.g. a pinned buffer)."""
        N.check(N.lib().mks_set_state(self._h, C.c_void_p(addr), int(n)))

    def clock(self):
        """(simulated time, windows run, accepted events) of the lattice."""
        t, w, e = C.c_double(), C.c_int64(), C.c_int64()
        N.check(N.lib().mks_get_clock(self._h, 0, C.byref(t), C.byref(w), C.byref(e)))
        return t.value, w.value, e.value

    def set_clock(self, time, window, events):
        N.check(N.lib().mks_set_clock(self._h, 0, float(time), int(window), int(events)))

    def prefetch_state_ptr(self, addr, n):
        """Start copying a compact state from (pinned) host memory into the
        second device buffer; it becomes the lattice at swap_state()."""
        N.check(N.lib().mks_prefetch_state(self._h, C.c_void_p(addr), int(n)))

    def swap_state(self):
        N.check(N.lib().mks_swap_state(self._h))

    def get_state_ptr(self, addr, n):
        N.check(N.lib().mks_get_state(self._h, C.c_void_p(addr), int(n)))

    def frame_sites_ptr(self, kind, addr, cap):
        """Compact-state indices of the sites listed in an output frame (kind 0:
        atoms with coordination <= 3, kind 1: voids), in the reference's z, y,
        x order, written to device-visible host memory at addr (cap entries);
        returns their number."""
        n = C.c_int64()
        N.check(N.lib().mks_frame_sites(self._h, int(kind), C.c_void_p(addr), int(cap), C.byref(n)))
        return n.value

    def class_histogram(self):
        h = np.zeros(N.MKS_NCLASS, dtype=np.int64)
        N.check(N.lib().mks_class_histogram(self._h, N.ptr(h), N.MKS_NCLASS))
        return h

    def site_rates(self, xyz):
        """(class, FP32 rate) of the sites at grid points xyz [n, 3] (the
        tree-leaf rates of the reference's MC particles)."""
        return _site_rates(self._h, 0, xyz)

    def write_frame(self, base, time, it):
        """The frame files <base>.xyz, _d, _v (and _w for SiC) of the
        current lattice; returns the SiC NumAtWrong count (0 otherwise)."""
        w = C.c_int64()
        N.check(N.lib().mks_write_frame(self._h, str(base).encode(), float(time), int(it), C.byref(w)))
        return w.value

    def observables(self):
        o = N.MksObservables()
        N.check(N.lib().mks_get_observables(self._h, C.byref(o)))
        return o.as_dict()

    def status(self):
        s = N.MksStatus()
        N.check(N.lib().mks_get_status(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def lattcoo(self):
        lx, ly, lz = self.dims
        a = np.empty((lz + 1, ly, lx), dtype=np.int32)
        N.check(N.lib().mks_get_lattice(self._h, N.ptr(a)))
        return a

    def load_lattcoo(self, arr):
        a = np.ascontiguousarray(arr, dtype=np.int32)
        lx, ly, lz = self.dims
        assert a.size == lx * ly * (lz + 1)
        N.check(N.lib().mks_load_lattice(self._h, N.ptr(a)))

    def load_lists(self, lattcoo, xyz, nn, event=None, rate=None):
        """Arm-chair stacking (ptrans_zig < 1): the full reference state, LattCoo
        [z, y, x] and the list entries (grid points xyz (n, 3), NextN nn
        (n, 4, 3)), rated as an initializer rates them, or with the given
        event codes (0 none, 1 deposition, 2 dummy, 4 evaporation) and rates."""
        a = np.ascontiguousarray(lattcoo, dtype=np.int32)
        lx, ly, lz = self.dims
        assert a.size == lx * ly * (lz + 1)
        p = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        q = np.ascontiguousarray(nn, dtype=np.int32).reshape(-1, 4, 3)
        assert len(p) == len(q)
        e = r = None
        if event is not None:
            e = np.ascontiguousarray(event, dtype=np.int32).reshape(-1)
            r = np.ascontiguousarray(rate, dtype=np.float32).reshape(-1)
            assert e.size == len(p) and r.size == len(p)
        N.check(N.lib().mks_load_lists(self._h, N.ptr(a), len(p), N.ptr(p), N.ptr(q),
                                       None if e is None else N.ptr(e), None if r is None else N.ptr(r)))

    def lists(self):
        """Arm-chair stacking: every listed site as a dict of xyz (n, 3), nn
        (n, 4, 3), kind (1 with an event, 2 bulk atom, 3 void), event (1
        deposition, 2 dummy, 4 evaporation, 5 isolated atom) and rate."""
        n = C.c_int64()
        N.check(N.lib().mks_get_lists(self._h, 0, None, None, None, None, None, C.byref(n)))
        m = max(n.value, 1)
        out = {"xyz": np.zeros((m, 3), np.int32), "nn": np.zeros((m, 4, 3), np.int32),
               "kind": np.zeros(m, np.int32), "event": np.zeros(m, np.int32), "rate": np.zeros(m, np.float32)}
        N.check(N.lib().mks_get_lists(self._h, m, *(N.ptr(out[k]) for k in ("xyz", "nn", "kind", "event", "rate")),
                                      C.byref(n)))
        return {k: v[:n.value] for k, v in out.items()}

    def set_tiling(self, width):
        N.check(N.lib().mks_set_tiling(self._h, int(width)))

    def tiling(self):
        return N.lib().mks_get_tiling(self._h)

    def set_colours(self, ncolour):
        """Tile colouring: 0 brick (3 colours) where it fits, 3 brick for all,
        4 square grid (4 colours) for all."""
        N.check(N.lib().mks_set_colours(self._h, int(ncolour)))

    def colours(self):
        return N.lib().mks_get_colours(self._h)

    def set_schedule(self, persistent):
        N.check(N.lib().mks_set_schedule(self._h, 1 if persistent else 0))

    def suggest_tau(self, f=0.3):
        t = np.zeros(1)
        N.check(N.lib().mks_suggest_tau(self._h, float(f), N.ptr(t)))
        return float(t[0])

    def run_stats(self):
        k, g, p = C.c_int64(), C.c_int64(), C.c_int64()
        ms = C.c_double()
        N.check(N.lib().mks_last_run_stats(self._h, C.byref(k), C.byref(g), C.byref(ms), C.byref(p)))
        return {"kernel_launches": k.value, "graph_launches": g.value, "kernel_ms": ms.value,
                "phase_launches": p.value}


class Batch:
    """Independent replicas of uneven boxes advanced together."""

    def __init__(self, boxes, seeds, ncrystal=1, list_crystal=(14,), sf=5.43 / 12, list_cov=()):
        cfgs = (N.MksConfig * len(boxes))()
        for i, (b, s) in enumerate(zip(boxes, seeds)):
            cfgs[i] = _cfg(b[0], b[1], b[2], ncrystal, list_crystal, 1.0, sf, s, list_cov)
        h = C.c_void_p()
        N.check(N.lib().mks_batch_create(cfgs, len(boxes), C.byref(h)))
        self._h = h
        self.n = len(boxes)
        self.boxes = [tuple(int(v) for v in b) for b in boxes]

    def close(self):
        if self._h:
            N.lib().mks_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_rates(self, ptransE, ptransD):
        e = np.ascontiguousarray(ptransE, dtype=np.float64).reshape(-1)
        d = np.ascontiguousarray(ptransD, dtype=np.float64).reshape(-1)
        assert e.size == self.n * 3 * 4096 and d.size == self.n * 9
        N.check(N.lib().mks_batch_set_rates(self._h, N.ptr(e), N.ptr(d)))

    def set_coverage_rates(self, ptransAbs, ptransDes):
        """Per replica PtransAbs / PtransDes, n x 3 x 3."""
        a = np.ascontiguousarray(ptransAbs, dtype=np.float64).reshape(-1)
        d = np.ascontiguousarray(ptransDes, dtype=np.float64).reshape(-1)
        assert a.size == self.n * 9 and d.size == self.n * 9
        N.check(N.lib().mks_batch_set_coverage_rates(self._h, N.ptr(a), N.ptr(d)))

    def init_flat(self, kind, len1):
        l1 = np.ascontiguousarray(len1, dtype=np.int32)
        N.check(N.lib().mks_batch_init_flat(self._h, kind.encode()[:1], N.ptr(l1)))

    def run(self, tau, max_windows, max_events_each=0, max_time_each=0.0):
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(tau, dtype=np.float64), (self.n,)))
        ne = C.c_int64()
        N.check(N.lib().mks_batch_run(self._h, N.ptr(t), int(max_windows), int(max_events_each),
                                      float(max_time_each), C.byref(ne)))
        return ne.value

    def suggest_tau(self, f=0.3):
        t = np.zeros(self.n)
        N.check(N.lib().mks_suggest_tau(self._h, float(f), N.ptr(t)))
        return t

    def observables(self):
        o = (N.MksObservables * self.n)()
        N.check(N.lib().mks_batch_observables(self._h, o))
        return [x.as_dict() for x in o]

    def set_tiling(self, width):
        N.check(N.lib().mks_set_tiling(self._h, int(width)))

    def tiling(self):
        return N.lib().mks_get_tiling(self._h)

    def set_tilings(self, widths):
        """Tile width of each replica (mks_batch_set_tiling)."""
        w = np.ascontiguousarray(widths, dtype=np.int32).reshape(-1)
        assert w.size == self.n
        N.check(N.lib().mks_batch_set_tiling(self._h, N.ptr(w)))

    def tilings(self):
        w = np.zeros(self.n, dtype=np.int32)
        N.check(N.lib().mks_batch_get_tiling(self._h, N.ptr(w)))
        return w

    def set_colours(self, ncolour):
        """Tile colouring: 0 brick (3 colours) where it fits, 3 brick for all,
        4 square grid (4 colours) for all."""
        N.check(N.lib().mks_set_colours(self._h, int(ncolour)))

    def colours(self):
        return N.lib().mks_get_colours(self._h)

    def set_schedule(self, persistent):
        N.check(N.lib().mks_set_schedule(self._h, 1 if persistent else 0))

    def run_stats(self):
        k, g, p = C.c_int64(), C.c_int64(), C.c_int64()
        ms = C.c_double()
        N.check(N.lib().mks_last_run_stats(self._h, C.byref(k), C.byref(g), C.byref(ms), C.byref(p)))
        return {"kernel_launches": k.value, "graph_launches": g.value, "kernel_ms": ms.value,
                "phase_launches": p.value}

    def class_histogram(self):
        """(n, MKS_NCLASS) event sites per rate class of every replica."""
        h = np.zeros((self.n, N.MKS_NCLASS), dtype=np.int64)
        N.check(N.lib().mks_batch_class_histogram(self._h, N.ptr(h), N.MKS_NCLASS))
        return h

    def site_rates(self, rep, xyz):
        """(class, FP32 rate) of replica rep's sites at grid points xyz [n, 3]."""
        return _site_rates(self._h, rep, xyz)

    def load_lattice(self, rep, lattcoo):
        """Replica rep from a LattCoo(0:LenX-1,0:LenY-1,0:LenZ) array (x fastest)."""
        lc = np.ascontiguousarray(lattcoo, dtype=np.int32)
        N.check(N.lib().mks_batch_load_lattice(self._h, int(rep), N.ptr(lc)))

    def state(self, rep):
        """The compact one-byte state of replica rep, [z1, b, a]."""
        lx, ly, lz = self.boxes[rep]
        a = np.empty((lz // 3 + 1, ly // 6, lx // 6), dtype=np.uint8)
        N.check(N.lib().mks_batch_get_state(self._h, int(rep), N.ptr(a), a.size))
        return a

    def init_shape(self, rep, init_st, lens, params=None):
        """Replica rep by one of the reference's shaped initializers
        (Lattice.init_shape lists them)."""
        l = np.zeros(4, dtype=np.int32)
        l[:len(lens)] = lens
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
        N.check(N.lib().mks_batch_init_shape(self._h, int(rep), init_st.encode(), N.ptr(l),
                                             None if p is None else N.ptr(p)))

    def init_cad(self, rep, geo, alloy=0.0, seed=0):
        """Replica rep by SetCAD (InitSt IN) from the LattGeo id of every grid
        point, [z, y, x]; with alloy > 0 species 2 is drawn on each Si site."""
        g = np.ascontiguousarray(geo, dtype=np.int8)
        if alloy > 0.0:
            N.check(N.lib().mks_batch_init_cad_alloy(self._h, int(rep), N.ptr(g), float(alloy),
                                                     int(seed) & 0xFFFFFFFFFFFFFFFF))
        else:
            N.check(N.lib().mks_batch_init_cad(self._h, int(rep), N.ptr(g)))

    def init_points(self, rep, xyz, species):
        """Replica rep by SetShape (InitSt SH) from grid points xyz [n, 3] with
        species 1 (Si) or 2 (C / Ge)."""
        p = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        sp = np.ascontiguousarray(species, dtype=np.int8).reshape(-1)
        assert sp.size == p.shape[0]
        N.check(N.lib().mks_batch_init_points(self._h, int(rep), N.ptr(p), N.ptr(sp), int(sp.size)))

    def load_temperature(self, rep, lattcoo):
        """Static LA temperatures of replica rep from the LattCoo T bits."""
        lc = np.ascontiguousarray(lattcoo, dtype=np.int32)
        N.check(N.lib().mks_batch_load_temperature(self._h, int(rep), N.ptr(lc)))

    # ---- in-process LA coupling: the FEM <-> KMC socket messages ----
    def set_field(self, rep, field):
        """Temperature field (K) of replica rep as the reference's SENDFIELD
        message: field[z, x + LenX*y] (shape (LenZ, LenX*LenY)), or that
        array flattened with z fastest; 10 marks a wall (temperature kept)."""
        f = np.asarray(field, dtype=np.int32)
        if f.ndim == 2:
            f = f.T                      # [z, j] -> memory order z fastest
        f = np.ascontiguousarray(f).reshape(-1)
        N.check(N.lib().mks_batch_set_field(self._h, int(rep), N.ptr(f)))

    def set_tabulated(self, temps, ptransE, ptransD):
        """Rates interpolated per site from tables at temperatures temps (InitSt
        ST): temps (n, ntemp) increasing, ptransE (n, ntemp, 3, 4, 4, 4, 4, 4, 4),
        ptransD (n, ntemp, 3, 3); the temperature fields must be loaded."""
        t = np.ascontiguousarray(temps, dtype=np.int32).reshape(self.n, -1)
        nt = t.shape[1]
        e = np.ascontiguousarray(ptransE, dtype=np.float64).reshape(-1)
        d = np.ascontiguousarray(ptransD, dtype=np.float64).reshape(-1)
        assert e.size == self.n * nt * 3 * 4096 and d.size == self.n * nt * 9
        N.check(N.lib().mks_batch_set_tabulated(self._h, nt, N.ptr(t), N.ptr(e), N.ptr(d)))

    def get_phases(self, rep=0):
        """(coo, species) of replica rep as the reference's GETPHASES / GETXGE
        messages: arrays [z, x + LenX*y] of shape (LenZ, LenX*LenY) (views
        of buffers with z fastest)."""
        lx, ly, lz = self.boxes[rep]
        c = np.empty(lz * lx * ly, dtype=np.int32)
        d = np.empty(lz * lx * ly, dtype=np.int32)
        N.check(N.lib().mks_batch_get_phases(self._h, int(rep), N.ptr(c), N.ptr(d)))
        return c.reshape(lx * ly, lz).T, d.reshape(lx * ly, lz).T

    def lattcoo(self):
        """LattCoo(0:LenX-1, 0:LenY-1, 0:LenZ) of a one-replica batch."""
        assert self.n == 1
        lx, ly, lz = self.boxes[0]
        a = np.empty((lz + 1, ly, lx), dtype=np.int32)
        N.check(N.lib().mks_get_lattice(self._h, N.ptr(a)))
        return a

    # ---- laser anneal (LA) mode ----
    def init_alloy(self, len1, x, seed):
        """SetSi-like slabs with species 2 substituted at fraction x[i]."""
        l1 = np.ascontiguousarray(np.broadcast_to(np.asarray(len1, dtype=np.int32), (self.n,)))
        xs = np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (self.n,)))
        N.check(N.lib().mks_batch_init_alloy(self._h, N.ptr(l1), N.ptr(xs), int(seed) & 0xFFFFFFFFFFFFFFFF))

    def set_la(self, params, dptransE=None, dptransD=None):
        """params: one MksLaParams per replica (or one for all)."""
        if isinstance(params, N.MksLaParams):
            params = [params] * self.n
        arr = (N.MksLaParams * self.n)(*params)
        de = None if dptransE is None else np.ascontiguousarray(dptransE, dtype=np.float64).reshape(-1)
        dd = None if dptransD is None else np.ascontiguousarray(dptransD, dtype=np.float64).reshape(-1)
        if de is not None:
            assert de.size == self.n * 3 * 4096 * 4 and dd is not None and dd.size == self.n * 9 * 4
        N.check(N.lib().mks_batch_set_la(self._h, arr, None if de is None else N.ptr(de),
                                         None if dd is None else N.ptr(dd)))
        self._la_keep = (de, dd)

    def score(self, reset=False):
        out = np.zeros((self.n, 4))
        N.check(N.lib().mks_batch_get_score(self._h, N.ptr(out), 1 if reset else 0))
        return out

    def la_counts(self):
        """(crystal atoms per species (n, 3), liquid fractions in use (n, 3))."""
        c = np.zeros((self.n, 3), dtype=np.int64)
        x = np.zeros((self.n, 3))
        N.check(N.lib().mks_batch_la_counts(self._h, N.ptr(c), N.ptr(x)))
        return c, x

    def lr_accumulate(self, df):
        """Causal LR step: df, one increment of the observable per replica
        over the segment just run, weighted by the score so far (GPU)."""
        d = np.ascontiguousarray(df, dtype=np.float64).reshape(-1)
        assert d.size == self.n
        N.check(N.lib().mks_batch_lr_accumulate(self._h, N.ptr(d)))

    def lr_result(self, reset=True):
        """(gradient, standard error) of the causal sums of lr_accumulate."""
        g, se = np.zeros(4), np.zeros(4)
        N.check(N.lib().mks_batch_lr_result(self._h, 1 if reset else 0, N.ptr(g), N.ptr(se)))
        return g, se

    def lr_grad(self, f, baseline=True):
        """Likelihood-ratio gradient of E[f] (one f per replica) and its
        standard error, computed on the GPU from the accumulated scores."""
        fv = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        assert fv.size == self.n
        g, se = np.zeros(4), np.zeros(4)
        N.check(N.lib().mks_batch_lr_grad(self._h, N.ptr(fv), 1 if baseline else 0, N.ptr(g), N.ptr(se)))
        return g, se
