"""ctypes wrapper of the oracle library (oracle/_build/libmks_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, as the checker.  The product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libmks_oracle.so")
NUMBERS = os.path.join(os.path.dirname(HERE), "tests", "golden", "numberslist.txt")

EVENT_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("itrans", "i1"), ("arm", "i1"),
                        ("pad", "<i2")])

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.ora_create.restype = C.c_void_p
        L.ora_create.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.ora_destroy.argtypes = [C.c_void_p]
        L.ora_last_error.restype = C.c_char_p
        L.ora_init.argtypes = [C.c_void_p]
        L.ora_run.argtypes = [C.c_void_p, C.c_int64, C.c_char_p]
        L.ora_main.argtypes = [C.c_void_p, C.c_char_p]
        L.ora_run_until.argtypes = [C.c_void_p, C.c_double]
        L.ora_trace_enable.argtypes = [C.c_void_p, C.c_int]
        L.ora_trace_len.restype = C.c_int64
        L.ora_trace_len.argtypes = [C.c_void_p]
        L.ora_trace.restype = C.c_void_p
        L.ora_trace.argtypes = [C.c_void_p]
        L.ora_trace_clear.argtypes = [C.c_void_p]
        L.ora_iter.restype = C.c_int64
        L.ora_iter.argtypes = [C.c_void_p]
        L.ora_time.restype = C.c_double
        L.ora_time.argtypes = [C.c_void_p]
        L.ora_total_rate.restype = C.c_double
        L.ora_total_rate.argtypes = [C.c_void_p]
        L.ora_counts.argtypes = [C.c_void_p, C.c_void_p]
        L.ora_get_lattcoo.argtypes = [C.c_void_p, C.c_void_p]
        L.ora_site_info.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ora_write_xyz.argtypes = [C.c_void_p, C.c_char_p]
        L.ora_write_frame.argtypes = [C.c_void_p, C.c_char_p, C.c_double, C.c_int64]
        L.ora_get_rates.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.ora_get_cov_rates.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.ora_ncov.argtypes = [C.c_void_p]
        L.ora_ran3_sequence.argtypes = [C.c_int, C.c_int, C.c_void_p]
        L.ora_mc_classes.restype = C.c_int64
        L.ora_mc_classes.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        L.ora_mc_sites.restype = C.c_int64
        L.ora_mc_sites.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        L.ora_list_entries.restype = C.c_int64
        L.ora_list_entries.argtypes = [C.c_void_p] * 6 + [C.c_int64]
        L.ora_compact_state.restype = C.c_int64
        L.ora_compact_state.argtypes = [C.c_void_p, C.c_void_p]
        L.ora_set_la_input.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.ora_set_geometry.argtypes = [C.c_void_p, C.c_void_p]
        L.ora_la_alloy.argtypes = [C.c_void_p, C.c_double, C.c_uint64]
        L.ora_la_set.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_uint64]
        L.ora_la_run_until.argtypes = [C.c_void_p, C.c_double]
        L.ora_la_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


class OraLa(C.Structure):
    """ora_la_t of mks_oracle.h."""
    _fields_ = [("P0", C.c_double * 3), ("Tm", C.c_double * 3), ("Tflex", C.c_double * 3),
                ("sigma", C.c_double * 3), ("Tb", C.c_double), ("Ta", C.c_double), ("t0", C.c_double),
                ("w", C.c_double), ("L_nm", C.c_double), ("zsurf", C.c_double), ("tau", C.c_double),
                ("phase", C.c_int)]


class Oracle:
    def __init__(self, startdat, lenx, leny, lenz, numbers=NUMBERS, num_mc_max=0):
        self.dims = (lenx, leny, lenz)
        h = lib().ora_create(startdat.encode(), numbers.encode() if numbers else None, lenx, leny, lenz,
                             num_mc_max)
        if not h:
            raise RuntimeError(lib().ora_last_error().decode())
        self._h = h

    def close(self):
        if self._h:
            lib().ora_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def init(self):
        if lib().ora_init(self._h):
            raise RuntimeError(lib().ora_last_error().decode())

    def run(self, n, outdir=None):
        r = lib().ora_run(self._h, int(n), outdir.encode() if outdir else None)
        if r < 0:
            raise RuntimeError(lib().ora_last_error().decode())
        return r

    def run_until(self, tmax):
        r = lib().ora_run_until(self._h, float(tmax))
        if r < 0:
            raise RuntimeError(lib().ora_last_error().decode())
        return r

    def set_geometry(self, geo):
        """InitSt IN input (see ora_set_geometry): LattGeo id of every grid point, [z, y, x]."""
        g = np.ascontiguousarray(geo, dtype=np.int8)
        self._geo = g
        if lib().ora_set_geometry(self._h, g.ctypes.data_as(C.c_void_p)):
            raise RuntimeError(lib().ora_last_error().decode())

    def set_la_input(self, geo, tsub):
        """InitSt LA input (see ora_set_la_input): layer ids and 3-grid temperatures."""
        self._la_in = (np.ascontiguousarray(geo, dtype=np.int8), np.ascontiguousarray(tsub, dtype=np.int16))
        if lib().ora_set_la_input(self._h, *(a.ctypes.data_as(C.c_void_p) for a in self._la_in)):
            raise RuntimeError(lib().ora_last_error().decode())

    # ---- per-species LA law with liquid fractions and FP64 score ----
    def la_alloy(self, x, seed):
        if lib().ora_la_alloy(self._h, float(x), int(seed) & 0xFFFFFFFFFFFFFFFF):
            raise RuntimeError(lib().ora_last_error().decode())

    def la_set(self, params, E, dE, D, dD, seed):
        self._la_keep = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) if a is not None else None
                         for a in (E, dE, D, dD)]
        k = self._la_keep
        r = lib().ora_la_set(self._h, C.byref(params), *(None if a is None else a.ctypes.data_as(C.c_void_p)
                                                         for a in k), int(seed) & 0xFFFFFFFFFFFFFFFF)
        if r:
            raise RuntimeError(lib().ora_last_error().decode())

    def la_run_until(self, t):
        r = lib().ora_la_run_until(self._h, float(t))
        if r < 0:
            raise RuntimeError(lib().ora_last_error().decode())
        return r

    def la_state(self):
        sc = np.zeros(4)
        cr = np.zeros(3, dtype=np.int64)
        xl = np.zeros(3)
        ev = C.c_int64()
        lib().ora_la_state(self._h, sc.ctypes.data_as(C.c_void_p), cr.ctypes.data_as(C.c_void_p),
                           xl.ctypes.data_as(C.c_void_p), C.byref(ev))
        return {"score": sc, "crystal": cr, "xliq": xl, "events": ev.value}

    def atoms(self):
        st, _ = compact_state(self)
        sp = st & 3
        if lib().ora_ncov(self._h):           # species value 3 marks a covered empty site
            return int(np.count_nonzero((sp == 1) | (sp == 2)))
        return int(np.count_nonzero(sp != 0))

    def trace_enable(self, on=True):
        lib().ora_trace_enable(self._h, 1 if on else 0)

    def trace(self, clear=True):
        n = lib().ora_trace_len(self._h)
        p = lib().ora_trace(self._h)
        if n == 0:
            out = np.zeros(0, dtype=EVENT_DTYPE)
        else:
            buf = (C.c_char * (n * EVENT_DTYPE.itemsize)).from_address(p)
            out = np.frombuffer(bytes(buf), dtype=EVENT_DTYPE).copy()
        if clear:
            lib().ora_trace_clear(self._h)
        return out

    @property
    def time(self):
        return lib().ora_time(self._h)

    @property
    def iter(self):
        return lib().ora_iter(self._h)

    @property
    def total_rate(self):
        return lib().ora_total_rate(self._h)

    def counts(self):
        a = np.zeros(3, dtype=np.int32)
        lib().ora_counts(self._h, a.ctypes.data_as(C.c_void_p))
        return {"bulk": int(a[0]), "voids": int(a[1]), "mc": int(a[2])}

    def lattcoo(self):
        lx, ly, lz = self.dims
        a = np.empty((lz + 1, ly, lx), dtype=np.int32)
        lib().ora_get_lattcoo(self._h, a.ctypes.data_as(C.c_void_p))
        return a

    def site_info(self, x, y, z):
        nn = np.zeros(12, dtype=np.int32)
        ie = C.c_int32()
        pr = C.c_double()
        which = lib().ora_site_info(self._h, x, y, z, nn.ctypes.data_as(C.c_void_p), C.byref(ie), C.byref(pr))
        return which, nn.reshape(4, 3), ie.value, pr.value

    def write_xyz(self, path):
        if lib().ora_write_xyz(self._h, path.encode()):
            raise RuntimeError(lib().ora_last_error().decode())

    def write_frame(self, base, time, it):
        """<base>.xyz, _d, _v, _w as WriteMolMolXYZFile writes them."""
        if lib().ora_write_frame(self._h, base.encode(), float(time), int(it)):
            raise RuntimeError(lib().ora_last_error().decode())

    def rates(self):
        e = np.zeros(3 * 4096)
        d = np.zeros(9)
        lib().ora_get_rates(self._h, e.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p))
        return e.reshape(3, 4, 4, 4, 4, 4, 4), d.reshape(3, 3)

    def cov_rates(self):
        """PtransAbs, PtransDes as 3x3 [coverage species][coor-1]."""
        a = np.zeros(9)
        d = np.zeros(9)
        lib().ora_get_cov_rates(self._h, a.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p))
        return a.reshape(3, 3), d.reshape(3, 3)


def ran3_sequence(idum, n):
    out = np.zeros(n)
    lib().ora_ran3_sequence(int(idum), int(n), out.ctypes.data_as(C.c_void_p))
    return out


def compact_state(o):
    """The oracle state as one byte per diamond site, in the GPU engine's
    layout (mulskips_gb300/csrc/lattice.cuh).  Returns (state, offgrid)."""
    lx, ly, lz = o.dims
    out = np.zeros((lz // 3 + 1, ly // 6, lx // 6), dtype=np.uint8)
    r = lib().ora_compact_state(o._h, out.ctypes.data_as(C.c_void_p))
    if r < 0:
        raise AssertionError("a list entry of the oracle is not a bond direction")
    return out, int(r)


def mc_classes(o):
    """(class, rate) of every MC particle of the oracle, GPU class enumeration."""
    n = o.counts()["mc"]
    cls = np.zeros(max(n, 1), dtype=np.int32)
    rate = np.zeros(max(n, 1), dtype=np.float64)
    m = lib().ora_mc_classes(o._h, cls.ctypes.data_as(C.c_void_p), rate.ctypes.data_as(C.c_void_p), n)
    return cls[:m], rate[:m]


def mc_sites(o):
    """Grid coordinates (n, 3) of the MC particles, in the order of mc_classes."""
    n = o.counts()["mc"]
    xyz = np.zeros((max(n, 1), 3), dtype=np.int32)
    m = lib().ora_mc_sites(o._h, xyz.ctypes.data_as(C.c_void_p), n)
    return xyz[:m]


def list_entries(o):
    """Every list entry of the oracle (ListAdAtom, ListAtom, ListVoid, each in
    its order): dict of xyz (n, 3), nn (n, 4, 3), kind (1 MC, 2 bulk, 3 void),
    ind_event and prob (MC particles only)."""
    c = o.counts()
    n = c["bulk"] + c["voids"] + c["mc"]
    xyz = np.zeros((max(n, 1), 3), dtype=np.int32)
    nn = np.zeros((max(n, 1), 4, 3), dtype=np.int32)
    kind = np.zeros(max(n, 1), dtype=np.int32)
    ie = np.zeros(max(n, 1), dtype=np.int32)
    pr = np.zeros(max(n, 1), dtype=np.float64)
    m = lib().ora_list_entries(o._h, *(a.ctypes.data_as(C.c_void_p) for a in (xyz, nn, kind, ie, pr)), n)
    assert m == n
    return {"xyz": xyz[:n], "nn": nn[:n], "kind": kind[:n], "ind_event": ie[:n], "prob": pr[:n]}


def rate_of_site(o, x, y, z):
    """(list kind, Ind_Event, rate) of the site, from the oracle's lists."""
    which, _, ie, pr = o.site_info(x, y, z)
    return which, ie, pr


def la_replica(args):
    """One oracle LA replica (for a spawn process pool): SiGe slab of Ge
    fraction x in a (lx, ly, lz) box, barrier tables E/dE/D/dD, LA parameters
    `la` (dict of OraLa fields); returns the crystal counts and FP64 scores at
    each time of `marks`."""
    import tempfile
    (startdat_text, dims, x, alloy_seed, la, E, dE, D, dD, seed, marks) = args
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "start.dat")
        with open(p, "w") as f:
            f.write(startdat_text)
        o = Oracle(p, *dims, numbers=None)
        o.init()
        o.la_alloy(x, alloy_seed)
        prm = OraLa()
        for k, v in la.items():
            if isinstance(v, (list, tuple)):
                for i, vi in enumerate(v):
                    getattr(prm, k)[i] = vi
            else:
                setattr(prm, k, v)
        o.la_set(prm, E, dE, D, dD, seed)
        out = []
        for t in marks:
            rc = o.la_run_until(t)
            st = o.la_state()
            out.append((st["crystal"].copy(), st["score"].copy(), st["events"], rc))
        o.close()
    return out


def la_regression_replica(args):
    """One oracle run of the LA regression input with RunType R (for a spawn
    pool): atoms (occupied non-wall sites) at each time of `marks`."""
    import tempfile
    startdat_text, dims, geo, tsub, marks = args
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "start.dat")
        with open(p, "w") as f:
            f.write(startdat_text)
        o = Oracle(p, *dims, numbers=None)
        o.set_la_input(geo, tsub)
        o.init()
        out = []
        for t in marks:
            r = o.run_until(t)
            out.append((o.atoms(), o.iter, r))
        o.close()
    return out
