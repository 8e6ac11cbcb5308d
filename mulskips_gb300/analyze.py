"""Trajectory observables of a run, computed the reference's way.

The reference measures growth on its output frames (pymulskips/analyze.py):
`get_surface_height` (:124-207) takes the z coordinates of every line of an
I*.xyz frame, finds the most populated 5 A slice of the box, averages the z
values in it, then averages again over +-20 A around that mean;
`analyze_growth_rate` (:209-416) turns the heights of a time series of frames
into a rate in micron/hour by central finite differences ('finitediff', the
default) or a straight-line fit ('polyfit'), leaving Nexclude frames out at
each end.  This module restates both on the compact lattice (one byte per
diamond site, the layout of mks_get_state), where the lines of a frame are
the covered sites, the atoms of coordination <= 3 and the voids
(WriteMolMolXYZFile.f:171-222), and adds the column-height statistics of
mks_get_observables (mean height and RMS roughness of the top atom of each
(a, b) column).  Results agree with the reference's functions on its own
frames (tests/golden/analysis.json, written by tests/golden/make_fixtures.py).
"""
import numpy as np

from .engine import coordination

WALL = 0x80


def frame_z(st, sf, cov=False):
    """z coordinates (A) of the lines of the I*.xyz frame of compact state st
    ([z1, b, a] uint8) in the reference's order: the grid scan (covered sites
    and atoms of coordination <= 3, WriteMolMolXYZFile.f:171-215), then the
    voids (:216-222; the reference lists those in its ListVoid order, which
    only changes the last bits of a sum)."""
    st = np.asarray(st, dtype=np.uint8)
    nz = st.shape[0]
    sp = st & 3
    co = coordination(st)
    notwall = st != WALL
    covered = (sp == 3) & notwall if cov else np.zeros(st.shape, bool)
    atom = (sp != 0) & ~covered & notwall
    listed = covered | (atom & (co <= 3))
    void = (st != 0) & notwall & (co == 4) & ((sp == 0) | covered)
    zg = (3.0 * sf) * np.arange(nz, dtype=np.float64)
    per_layer = listed.reshape(nz, -1).sum(axis=1)
    per_layer_void = void.reshape(nz, -1).sum(axis=1)
    return np.concatenate([np.repeat(zg, per_layer), np.repeat(zg, per_layer_void)])


def _seq_mean(vals):
    """Mean by one running sum in order, as the reference's loop forms it."""
    s = 0.0
    for v in vals.tolist():
        s = s + v
    return s / float(len(vals))


def surface_height(z, zl, bin_size=5.0, surface_roughness=20.0):
    """get_surface_height (pymulskips/analyze.py:124-207) of the z values of
    one frame (A) in a box of height zl (A, the third 'periodic' length)."""
    z = np.asarray(z, dtype=np.float64)
    if len(z) == 0:
        raise ValueError("empty frame")
    if np.all(z == z[0]) or (z.max() - z.min()) < bin_size:
        # this branch divides the built-in sum() (compensated since Python
        # 3.12), the others a running sum
        return sum(z.tolist()) / len(z)
    databins = int(zl / bin_size)
    hist, _ = np.histogram(z, bins=databins, range=(0.0, zl))
    k = int(np.flatnonzero(hist == hist.max())[0])
    # the slice is taken as bin_size * k, not at the histogram's own edges
    z_min = float(bin_size * k)
    z_max = float(z_min + bin_size)
    if z_max < z.min():
        z_min += bin_size
        z_max += bin_size
    z_ave = _seq_mean(z[(z > z_min) & (z < z_max)])
    z_min = z_ave - surface_roughness
    z_max = z_ave + surface_roughness
    return _seq_mean(z[(z > z_min) & (z < z_max)])


def growth_rate(times, heights, method="finitediff", n_exclude=2):
    """Growth rate (micron/hour) of surface heights (A) at times (s), as
    analyze_growth_rate's get_growth_rate (pymulskips/analyze.py:296-367):
    'finitediff' averages one-sided end and central inner differences over
    the frames [n_exclude:-n_exclude]; 'polyfit' fits a line to those frames.
    Returns (per-frame rates, average)."""
    t = np.asarray(times, dtype=np.float64)
    h = np.asarray(heights, dtype=np.float64)
    conv = 3600 * 1e-4
    if method == "finitediff":
        gr = [(h[1] - h[0]) / (t[1] - t[0]) * conv]
        for i in range(1, len(t) - 1):
            gr.append((h[i + 1] - h[i - 1]) / (t[i + 1] - t[i - 1]) * conv)
        gr.append((h[-1] - h[-2]) / (t[-1] - t[-2]) * conv)
        return gr, float(np.mean(np.array(gr[n_exclude:-n_exclude])))
    if method == "polyfit":
        x = t[n_exclude:-n_exclude]
        y = h[n_exclude:-n_exclude]
        c = np.polynomial.polynomial.polyfit(x, y, 1)
        ave = c[1] * conv
        return list(np.ones(len(t)) * ave), float(ave)
    raise ValueError(f"method {method}")


def column_heights(st):
    """Height (grid units, 3 z1) of the top atom of every (a, b) column of
    compact state st, -1 for an empty column; walls are not atoms."""
    st = np.asarray(st, dtype=np.uint8)
    nz = st.shape[0]
    atom = ((st & 3) != 0) & (st != WALL)
    has = atom.any(axis=0)
    top = nz - 1 - np.argmax(atom[::-1], axis=0)
    return np.where(has, 3 * top, -1)


def height_stats(st):
    """(mean height, RMS roughness) of the columns holding atoms, grid units,
    as mks_get_observables defines them."""
    h = column_heights(st)
    h = h[h >= 0].astype(np.float64)
    if h.size == 0:
        return 0.0, 0.0
    m = h.mean()
    return float(m), float(np.sqrt(max(0.0, (h * h).mean() - m * m)))


def state_observables(st, cov=False):
    """Counts and column statistics of compact state st as mks_get_observables
    defines them: atoms, atoms per species, covered sites (coverage mode;
    covered2 those of the second coverage species, bit 7 of a covered byte),
    mean height and RMS roughness of the columns (grid units)."""
    st = np.asarray(st, dtype=np.uint8)
    sp = st & 3
    notwall = st != WALL
    covered = (sp == 3) & notwall if cov else np.zeros(st.shape, bool)
    atom = (sp != 0) & notwall & ~covered
    m, r = height_stats(np.where(covered, 0, st).astype(np.uint8))
    return {"atoms": int(atom.sum()), "species": [int(((sp == s) & atom).sum()) for s in (1, 2, 3)],
            "covered": int(covered.sum()), "covered2": int((covered & ((st & 0x80) != 0)).sum()),
            "mean_height": m, "rms_roughness": r}
