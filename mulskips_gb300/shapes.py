"""Point lists for InitSt SH (SetShape, `mulskips-source/initial/SetShape.f:50-80`:
one `symbol x y z` line per occupied grid point) that the reference has no
initializer for.

faceted_slab_points builds a 3C (zincblende) slab whose whole top surface is
{111} facets: a periodic array of square pyramids z = h + P/2 - |dx| - |dy|
(dx, dy the offsets from the nearest pyramid axis, period P), i.e. the
planes +-x +-y + z = const.  The reference cannot start from a flat (111)
surface in its cubic, x/y-periodic box (every initializer of `main.f:224-278`
is (001)-oriented), so a surface made only of {111} facets is the form a
(111) substrate takes here.  Diamond sites are enumerated in the compact
coordinates of the one-byte lattice: layer z1 = z / 3, columns a, b with x =
3 (2 a + (z1 & 1)), y = 3 (2 b + (z1 & 1)), a site where (a + b + z1 / 2) is
even.  Walls fill z <= 3 and z >= L - 4 (the reference's wall layers);
atoms with fewer than two occupied neighbours are removed until none is
left, as a stable SetShape input needs."""
import numpy as np

# neighbour offsets (da, db, dz1) of a site on an even (row 0) and an odd
# (row 1) layer: the four bonds of the diamond lattice in compact coordinates
NEIGHBOURS = np.array([[[0, 0, 1], [0, -1, -1], [-1, -1, 1], [-1, 0, -1]],
                       [[1, 1, -1], [1, 0, 1], [0, 0, -1], [0, 1, 1]]])


def _neighbour_counts(occ):
    """Occupied bonded neighbours of every compact site (periodic in a, b)."""
    cnt = np.zeros(occ.shape, np.int8)
    for par in (0, 1):
        for da, db, dz in NEIGHBOURS[par]:
            sh = np.roll(occ, (-db, -da), axis=(1, 2))
            shz = np.zeros_like(sh)
            if dz == 1:
                shz[:-1] = sh[1:]
            else:
                shz[1:] = sh[:-1]
            cnt[par::2] += shz[par::2]
    return cnt


def faceted_slab_points(L, h_slab, period, sic=True):
    """(xyz [n, 3] int32 grid points, species [n] int8: 1 Si, 2 C) of a
    {111}-faceted slab in an L^3 box: pyramids of period `period` grid units
    (L a multiple of it) with their valleys at z = h_slab - period / 2 and
    apexes at h_slab + period / 2, over a bulk from z = 6.  With sic the two
    fcc sublattices hold Si and C (x/3 + y/3 + z/3 = 0 mod 4 is Si), else
    every atom is Si.  Wall points carry species 1 (SetShape does not read
    it)."""
    if L % 12 or L % period or period % 12:
        raise ValueError("L and the period must be multiples of 12, L a multiple of the period")
    if not (6 + period // 2 < h_slab < L - 8 - period // 2):
        raise ValueError("the slab must clear both walls")
    NA = NB = L // 6
    NZ = L // 3 + 1
    z1 = np.arange(NZ, dtype=np.int32)[:, None, None]
    b = np.arange(NB, dtype=np.int32)[None, :, None]
    a = np.arange(NA, dtype=np.int32)[None, None, :]
    valid = ((a + b + (z1 >> 1)) & 1) == 0
    x = 3 * (2 * a + (z1 & 1))
    y = 3 * (2 * b + (z1 & 1))
    z = 3 * z1
    half = period // 2
    top = h_slab + half - np.abs(x % period - half) - np.abs(y % period - half)
    wall = valid & ((z <= 3) | (z >= L - 4))
    atom = valid & (z >= 6) & (z <= top)
    while True:
        weak = atom & (_neighbour_counts(atom | wall) < 2)
        if not weak.any():
            break
        atom &= ~weak
    pts = wall | atom
    sel = np.nonzero(pts)
    xs = np.broadcast_to(x, pts.shape)[sel]
    ys = np.broadcast_to(y, pts.shape)[sel]
    zs = np.broadcast_to(z, pts.shape)[sel]
    si = (xs // 3 + ys // 3 + zs // 3) % 4 == 0
    species = np.where(si | (not sic) | (zs <= 3) | (zs >= L - 4), 1, 2).astype(np.int8)
    return np.stack([xs, ys, zs], 1).astype(np.int32), species
