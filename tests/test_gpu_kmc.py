"""Synchronous-sublattice KMC on the GPU: lattice invariants after runs
(coordination bytes equal the bonded-neighbour count of the occupancy, class
histogram consistent), clock and event accounting, batching."""
import numpy as np
import pytest
from mulskips_gb300.engine import coordination

pytestmark = pytest.mark.gpu

NB_OFF = [[(0, 0, 1), (0, -1, -1), (-1, -1, 1), (-1, 0, -1)],
          [(1, 1, -1), (1, 0, 1), (0, 0, -1), (0, 1, 1)]]


def check_invariants(st):
    """Coordination of atoms = occupied neighbours incl. walls; of tracked
    empty sites = occupied non-wall neighbours (the reference's bookkeeping,
    deposition.f / Evaporation.f)."""
    nz, nb, na = st.shape
    wall = st == 0x80
    occ = ((st & 3) != 0) & ~wall
    co = coordination(st)
    z = np.arange(nz)[:, None, None]
    n_occ = np.zeros(st.shape, np.int32)
    n_wall = np.zeros(st.shape, np.int32)
    for par in (0, 1):
        for (da, db, dz) in NB_OFF[par]:
            o2 = np.zeros_like(occ)
            w2 = np.zeros_like(wall)
            src = np.roll(np.roll(occ, -da, axis=2), -db, axis=1)
            srcw = np.roll(np.roll(wall, -da, axis=2), -db, axis=1)
            if dz > 0:
                o2[:-dz] = src[dz:]
                w2[:-dz] = srcw[dz:]
            else:
                o2[-dz:] = src[:dz]
                w2[-dz:] = srcw[:dz]
            m = (z % 2 == par)
            n_occ += np.where(m, o2, 0)
            n_wall += np.where(m, w2, 0)
    valid = ((np.arange(na)[None, None, :] + np.arange(nb)[None, :, None] + (z >> 1)) & 1) == 0
    atoms = occ & valid
    assert np.array_equal(co[atoms], (n_occ + n_wall)[atoms]), "atom coordination inconsistent"
    tracked = (~occ) & (~wall) & (st != 0) & valid
    assert np.array_equal(co[tracked], n_occ[tracked]), "empty-site coordination inconsistent"
    # every empty site touching an atom is tracked
    untracked = (st == 0) & valid & (n_occ > 0)
    assert not untracked.any(), "empty site next to an atom is not tracked"
    return int(atoms.sum())


def test_sublattice_run_invariants():
    from mulskips_gb300 import Lattice, arrhenius_tables
    pE, pD = arrhenius_tables(1100.0)
    with Lattice(480, 480, 480, seed=7) as lat:
        lat.set_rates(pE, pD)
        lat.init_flat("S", 240)
        n0 = check_invariants(lat.state())
        tau = 2e-8
        ev, t = lat.run(tau, 16)
        assert ev > 0
        assert abs(t - 16 * tau) < 1e-15
        n1 = check_invariants(lat.state())
        assert n1 < n0          # T = 1100 K etches
        obs = lat.observables()
        assert obs["events"] == ev and obs["atoms"] == n1
        h = lat.class_histogram()
        assert h[1:].sum() == obs["mc_sites"]
        st = lat.status()
        assert st["error"] == 0


def test_growth_regime_invariants():
    """Low temperature: deposition wins and the film grows."""
    from mulskips_gb300 import Lattice, arrhenius_tables
    pE, pD = arrhenius_tables(400.0, flux=5.0)
    with Lattice(480, 480, 480, seed=3) as lat:
        lat.set_rates(pE, pD)
        lat.init_flat("S", 120)
        n0 = check_invariants(lat.state())
        ev, t = lat.run(0.01, 40)
        n1 = check_invariants(lat.state())
        assert ev > 1000 and n1 > n0


def test_batch_uneven_replicas():
    from mulskips_gb300 import Batch, arrhenius_tables
    sides = [16, 24, 40]
    boxes = [(12 * s, 12 * s, 12 * s) for s in sides]
    b = Batch(boxes, seeds=[11, 12, 13])
    pEs, pDs = zip(*[arrhenius_tables(T) for T in (1000.0, 1100.0, 1200.0)])
    b.set_rates(np.stack(pEs), np.stack(pDs))
    b.init_flat("S", [12 * s // 2 for s in sides])
    ev = b.run(1e-8, 8)
    obs = b.observables()
    assert ev == sum(o["events"] for o in obs) and all(o["events"] > 0 for o in obs)
    b.close()


def test_unsupported_config_is_rejected():
    """Configurations outside the engine fail at creation with an error code:
    arm-chair stacking in a batch or with a coverage species, three coverage
    species, two with NCrystal = 2, a box side that is not a multiple of 12."""
    import ctypes as C
    from mulskips_gb300 import Lattice
    from mulskips_gb300 import _native as N
    from mulskips_gb300._native import MksError
    from mulskips_gb300.engine import _cfg
    with pytest.raises(MksError):
        Lattice(100, 480, 480)
    with pytest.raises(MksError):
        Lattice(480, 480, 480, ptrans_zig=0.8, list_cov=(1,))
    with pytest.raises(MksError):
        Lattice(480, 480, 480, list_cov=(1, 17, 9))
    with pytest.raises(MksError):
        Lattice(480, 480, 480, ncrystal=2, list_crystal=(14, 6), list_cov=(1, 17))
    cfgs = (N.MksConfig * 2)(*[_cfg(480, 480, 480, 1, (14,), 0.8, 5.43 / 12, s) for s in (1, 2)])
    h = C.c_void_p()
    with pytest.raises(MksError):
        N.check(N.lib().mks_batch_create(cfgs, 2, C.byref(h)))
    with Lattice(480, 480, 480, ptrans_zig=0.8) as lat:      # arm-chair stacking: a supported mode
        assert lat.dims == (480, 480, 480)


@pytest.mark.parametrize("colours", [3, 4])
def test_persistent_schedule_equals_per_colour_launches(colours):
    """The persistent kernel (each tile waits only for its neighbours: 6 on
    the three-colour brick tiling, 8 on the four-colour grid) and one launch
    per colour phase give the same lattice bit for bit."""
    from mulskips_gb300 import Lattice, arrhenius_tables
    pE, pD = arrhenius_tables(1100.0)
    states = []
    for persistent in (0, 1):
        with Lattice(480, 480, 480, seed=21) as lat:
            lat.set_colours(colours)
            assert lat.colours() == colours
            lat.set_schedule(persistent)
            lat.set_rates(pE, pD)
            lat.init_flat("S", 240)
            ev, t = lat.run(1e-8, 40)
            states.append((lat.state(), ev))
    assert states[0][1] == states[1][1] and states[0][1] > 0
    assert np.array_equal(states[0][0], states[1][0])


def test_batch_mixes_tilings():
    """A batch whose small replicas cannot take the brick tiling runs them on
    the four-colour grid and the others on the brick; both schedules agree."""
    from mulskips_gb300 import Batch, arrhenius_tables
    pE, pD = arrhenius_tables(1100.0)
    boxes = [(192, 192, 192), (480, 480, 480), (288, 288, 288)]
    states = []
    for persistent in (0, 1):
        b = Batch(boxes, seeds=[5, 6, 7])
        b.set_tiling(8)
        assert b.colours() == 4                    # the 32-site rows take the grid
        b.set_schedule(persistent)
        b.set_rates(np.stack([pE] * 3), np.stack([pD] * 3))
        b.init_flat("S", [96, 240, 144])
        ev = b.run(1e-8, 24)
        states.append(([b.state(r) for r in range(3)], ev))
        b.close()
    assert states[0][1] == states[1][1] > 0
    for r in range(3):
        assert np.array_equal(states[0][0][r], states[1][0][r])
        check_invariants(states[1][0][r])


def test_batch_widths_per_replica():
    """mks_batch_set_tiling: each replica of a batch cut at its own width;
    the persistent and per-colour schedules agree and the lattices stay
    consistent."""
    from mulskips_gb300 import Batch, arrhenius_tables
    pE, pD = arrhenius_tables(1100.0)
    boxes = [(288, 288, 288), (480, 480, 480), (384, 384, 384)]
    states = []
    for persistent in (0, 1):
        b = Batch(boxes, seeds=[15, 16, 17])
        b.set_tilings([4, 8, 6])
        assert list(b.tilings()) == [4, 8, 6] and b.tiling() == 8
        b.set_schedule(persistent)
        b.set_rates(np.stack([pE] * 3), np.stack([pD] * 3))
        b.init_flat("S", [144, 240, 192])
        ev = b.run(1e-8, 24)
        states.append(([b.state(r) for r in range(3)], ev, [o["events"] for o in b.observables()]))
        b.close()
    assert states[0][1] == states[1][1] > 0 and min(states[1][2]) > 0
    for r in range(3):
        assert np.array_equal(states[0][0][r], states[1][0][r])
        check_invariants(states[1][0][r])


@pytest.mark.parametrize("width,colours", [(4, 4), (6, 3), (6, 4), (8, 3), (8, 4)])
def test_tile_widths_keep_invariants(width, colours):
    from mulskips_gb300 import Lattice, arrhenius_tables
    pE, pD = arrhenius_tables(1100.0)
    with Lattice(480, 480, 480, seed=4) as lat:
        lat.set_tiling(width)
        lat.set_colours(colours)
        assert lat.colours() == colours
        lat.set_rates(pE, pD)
        lat.init_flat("S", 240)
        ev, _ = lat.run(2e-8, 24)
        assert ev > 0
        check_invariants(lat.state())


def test_prefetched_state_swaps_in():
    """mks_prefetch_state copies the next lattice while the current one runs;
    after mks_swap_state the engine holds exactly the prefetched bytes, and
    runs from them as from mks_set_state."""
    torch = pytest.importorskip("torch")
    from mulskips_gb300 import Lattice, arrhenius_tables
    pE, pD = arrhenius_tables(1100.0)
    lat = Lattice(480, 480, 480, seed=3)
    lat.set_rates(pE, pD)
    lat.init_flat("S", 120)
    base = lat.state().copy()
    lat.run(2e-9, 8)
    later = lat.state().copy()
    assert not np.array_equal(base, later)
    pinned = torch.empty(base.size, dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = base.reshape(-1)
    lat.prefetch_state_ptr(pinned.data_ptr(), base.size)
    lat.run(2e-9, 8)                        # runs on `later` while the copy is in flight
    lat.swap_state()
    assert np.array_equal(lat.state(), base)
    lat.run(2e-9, 8)
    a = lat.state().copy()
    ref = Lattice(480, 480, 480, seed=3)
    ref.set_rates(pE, pD)
    ref.set_state(base)
    ref.run(2e-9, 8)
    check_invariants(a)
    assert abs(int(((a & 3) != 0).sum()) - int(((ref.state() & 3) != 0).sum())) < 2000
    lat.close()
    ref.close()
