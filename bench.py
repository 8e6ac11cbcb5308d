#!/usr/bin/env python
"""Benchmark: accepted KMC events/s of the plain Si(001) model on one GB300.

Workload (one step = one pass of the KMC hot path over the lattice):
  plain Si(001), 256 conventional cells per side (3072^3 super-lattice grid,
  134M diamond sites), substrate filling the box (Len1 = 3000 grid units),
  walls as SetSi, PtransE(1,n) = 1e13 exp(-0.6 n eV / kT), PtransD(1,n) = 0.5,
  T cycling over {1000, 1100, 1200} K by step; 256 sublattice windows per step,
  each tau = 0.3 / r* long (r* the rate of the class carrying the largest
  share, the accuracy-matched window).  The lattice (268 MB) is larger than
  L2, and L2 is flushed before each timed step.

`value`: events / device time of the KMC kernels (CUDA events on the
engine's stream), inputs resident.  `e2e`: the same through the C ABI with
host buffers, timed on the host: the lattice uploaded from pinned memory,
the windows, then the step's result as the reference writes it (the frame's
site list and the observables) read back.
Side lines (not the headline): `batched` (512 small replicas), `la_gradient`
(the SiGe laser-anneal gradient), `cvd` (Si(001) + H, one coverage
species, with the serial oracle's events/s on the reference's 480^3 case) and
`stacking` (3C-SiC with arm-chair stacking, PtransZig < 1, on the
explicit-neighbour engine).
`--impl reference`: the reference CPU path (the oracle restatement; the
Fortran reference has no compiler here) on all host cores.
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import shutil
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TEMPS = (1000.0, 1100.0, 1200.0)
BOX = 3072
LEN1 = 3000
ACCURATE_F = 0.3      # tau = 0.3 / r*: inside the 95 % band of the serial etch rate
WINDOWS_PER_STEP = 256
BATCH_WINDOWS_PER_STEP = 64   # the small batched replicas would etch to their walls in longer steps
ALGO_BYTES_PER_EVENT = 28   # uint8 reads of site+4NN+12NNN occupancy, 5 coordinations; 6 writes
METRIC = "accepted KMC events/s (plain Si(001) 256^3 cells)"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index=0):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.index = index

    def __enter__(self):
        if shutil.which("nvidia-smi"):
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except OSError:
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(r[1]) for r in rows)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": float(rows[0][2]), "reasons": sorted(reasons),
                "samples": len(rows)}


# ---------------------------------------------------------------- CPU side
def _oracle_sample(args):
    """One bounded sample of the same model on the CPU oracle: a 480^3 box with
    a Len1=360 Si(001) slab at temperature T, run until the slab is gone."""
    T, seed = args
    from oracle import ora
    from mulskips_gb300.startdat import write_plain_si_startdat
    d = tempfile.mkdtemp()
    p = os.path.join(d, "start.dat")
    write_plain_si_startdat(p, T=T, len1=360, max_iter=100000000, seed=seed)
    o = ora.Oracle(p, 480, 480, 480, numbers=None)
    o.init()
    atoms0, mc0 = o.atoms(), o.counts()["mc"]
    t0 = time.perf_counter()
    o.run(100000000)
    dt = time.perf_counter() - t0
    n = o.iter - 1
    o.close()
    shutil.rmtree(d, ignore_errors=True)
    return n, dt, atoms0, mc0


# the serial reference's selection: a sum tree of 2^20 - 1 nodes (Levels = 20,
# AllocateArrays.f:30-43), descended with one uniform per level
# (PickTreeEvent.f:41-55)
TREE_LEVELS = 20


def cpu_baseline(seconds=10.0, cores=1):
    """Events/s of the oracle on `cores` processes (one seed each), the total
    events, runs, and the sample's slab state (mean initial atoms and MC sites
    of a run)."""
    from oracle import ora
    ora.build()
    ctx = mp.get_context("spawn")
    ev = 0
    busy = 0.0
    k = 0
    atoms0 = mc0 = 0
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        while time.perf_counter() - t0 < seconds:
            jobs = [(TEMPS[(k + i) % 3], 1000 + k + i) for i in range(cores)]
            k += cores
            res = pool.map(_oracle_sample, jobs)
            ev += sum(r[0] for r in res)
            busy += max(r[1] for r in res)
            atoms0 += sum(r[2] for r in res)
            mc0 += sum(r[3] for r in res)
    return ev / busy, ev, k, {"initial_atoms": atoms0 / k, "initial_mc_sites": mc0 / k,
                              "tree_levels": TREE_LEVELS, "uniforms_per_pick": TREE_LEVELS - 1}


def reduce_over_ranks(dist, wall, count, device="cpu"):
    """Whole-job figures of a timed region: the slowest rank's time and the
    units all ranks processed (value = count / wall).  dist is
    torch.distributed (initialised) or None for one process."""
    if dist is None:
        return wall, float(count)
    import torch
    t = torch.tensor([wall, float(count)], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = t.clone()
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return mx[0].item(), sm[1].item()


# ---------------------------------------------------------------- GPU side
def gb300(args, rank, world):
    import numpy as np
    import torch
    from mulskips_gb300 import Lattice, arrhenius_tables

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    from mulskips_gb300.autotune import choose_width
    tables = [arrhenius_tables(T) for T in TEMPS]
    lat = Lattice(BOX, BOX, BOX, sf=5.43 / 12, seed=1 + rank)

    lat.init_flat("S", LEN1)
    lat.set_rates(*tables[1])
    width = choose_width(lat, lat.suggest_tau(ACCURATE_F), widths=(6, 8), windows=64)
    taus = []

    def step(k):
        pE, pD = tables[k % 3]
        lat.set_rates(pE, pD)
        tau = lat.suggest_tau(ACCURATE_F)
        taus.append(tau)
        ev, _ = lat.run(tau, WINDOWS_PER_STEP)
        st = lat.run_stats()
        return ev, st

    # L2 flush between timed steps: the lattice is larger than L2 but the
    # surface band a step works on is not
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    for k in range(args.warmup):
        step(k)
    barrier()
    events = 0
    dev_ms = 0.0
    launches = 0
    phases = 0
    with Clocks(dev) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ev, st = step(args.warmup + k)
            events += ev
            dev_ms += st["kernel_ms"]
            launches += st["kernel_launches"]
            phases += st["phase_launches"]
        barrier()
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    dev_ms_max, events_all = reduce_over_ranks(dist, dev_ms, events, "cuda")
    value = events_all / (dev_ms_max / 1e3)

    # end to end through the C ABI with pinned host buffers
    pE, pD = tables[0]
    lat.set_rates(pE, pD)
    lat.init_flat("S", LEN1)
    n = lat.state().size
    host_in = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    frame_cap = 16 << 20
    host_frame = torch.empty(frame_cap, dtype=torch.int32, pin_memory=True)
    host_in.numpy()[:] = lat.state().reshape(-1)
    e2e_events = 0
    frame_bytes = 0
    barrier()
    t0 = time.perf_counter()
    # double-buffered input: step k+1's lattice is copied while step k's
    # result is read back (a copy during the windows would evict their L2
    # working set)
    lat.prefetch_state_ptr(host_in.data_ptr(), n)
    for k in range(args.steps):
        pE, pD = tables[k % 3]
        lat.set_rates(pE, pD)
        lat.swap_state()
        ev, _ = lat.run(taus[k % len(taus)], WINDOWS_PER_STEP)
        if k + 1 < args.steps:
            lat.prefetch_state_ptr(host_in.data_ptr(), n)
        # the step's result, as the reference writes it: the frame's site
        # list (I*.xyz atoms) and the observables
        frame_bytes += 4 * lat.frame_sites_ptr(0, host_frame.data_ptr(), frame_cap)
        obs = lat.observables()
        e2e_events += ev
    barrier()
    e2e_wall = time.perf_counter() - t0
    lat.close()
    e2e_wall, e2e_events = reduce_over_ranks(dist, e2e_wall, e2e_events, "cuda")
    e2e = e2e_events / e2e_wall

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_kind = peaks()
    # dominant kernel: the sublattice phase kernel; per-launch averages
    per_launch_events = events / max(phases, 1)
    per_launch_s = (dev_ms / 1e3) / max(phases, 1)
    achieved = per_launch_events * ALGO_BYTES_PER_EVENT / per_launch_s / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "sl_persistent_traffic.json")
    if os.path.exists(tp):
        try:
            tj = json.load(open(tp))
            traffic = tj.get("dram_bytes_per_launch", None)
        except Exception:
            traffic = None
    batched = batched_bench(args) if not args.no_batched else None
    la_grad = la_gradient_bench() if not args.no_batched else None
    cvd = cvd_bench() if not args.no_batched else None
    stacking = stacking_bench() if not args.no_batched else None
    config2 = config2_bench() if not args.no_batched else None
    base_v, base_ev, base_runs, base_slab = cpu_baseline(seconds=args.cpu_seconds, cores=1)
    all_cores = os.cpu_count() or 1
    all_v, _, _, _ = cpu_baseline(seconds=args.cpu_seconds, cores=all_cores)
    if batched:
        batched["batched_over_plain_3072cube"] = batched["value"] / value
        batched["batched_over_cpu_all_cores"] = batched["value"] / all_v
    accuracy = bench_accuracy(width)
    line = {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "plain Si(001) KMC, 256^3 cells (3072^3 grid, 134M sites), Len1=3000 slab, "
                               "T cycling 1000/1100/1200 K by step, F=0.5 ML/s, E=0.6 eV/bond, nu=1e13, "
                               f"{WINDOWS_PER_STEP} sublattice windows per step of tau = {ACCURATE_F}/k(n=2) "
                               "(the accuracy-matched window; config 1 states 1e-4 s, longer than the slab's life)",
                   "box_grid": BOX, "len1": LEN1, "tau_s": taus[:3], "tile_width": width,
                   "temperatures_K": list(TEMPS),
                   "events_per_step": events / args.steps,
                   "l2": "lattice 268 MB > 129 MB L2; 256 MB write flushes L2 before each timed step",
                   "parallelism": f"replicas x{world}" if world > 1 else "single replica"},
        "e2e": {"value": e2e, "unit": "events/s", "h2d_bytes_per_step": n + 2 * 8 * 4096 * 3,
                "d2h_bytes_per_step": int(frame_bytes / max(1, args.steps)) + 3 * 8 * 64,
                "path": "C ABI: set_rates, lattice upload from pinned memory (double-buffered: the next step's "
                        "copy overlaps this step's read-back), the windows, frame site list (I*.xyz atoms) and "
                        "observables back"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "note": f"28 B/event algorithmic x events per k_sl_persistent launch ({WINDOWS_PER_STEP} windows) / mean "
                             f"launch time; traffic: ncu dram bytes of one such launch; "
                             f"peak {peak_kind}"},
        "cpu_baseline": {"value": base_v, "unit": "events/s", "cores": 1, "kind": "port",
                         "sample": f"oracle (serial C restatement) on {base_runs} runs of the same model in a "
                                   f"480^3 box, Len1=360 slab etched to the walls, T cycling 1000/1100/1200 K, "
                                   f"{base_ev} events",
                         "slab": base_slab},
        "cpu_all_cores": {"value": all_v, "unit": "events/s", "cores": all_cores,
                          "sample": "the cpu_baseline sample, one oracle process per core"},
        "accuracy": accuracy,
        "clocks": clocks,
        "wall_s_timed": wall,
        "batched": batched,
        "la_gradient": la_grad,
        "cvd": cvd,
        "stacking": stacking,
        "config2": config2,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def bench_accuracy(width):
    """The growth-rate error at this benchmark's window rule (f = 0.3) and
    tile width, as the statistical parity test measured it on GB300 on the
    same model in a 480^3 box at the benchmark's three temperatures (32 GPU
    replicas against 32 serial seeds, 95 % family band): the cases of
    profiles/etch_accuracy_480cube.json (written from that test's record) at
    this run's width and f."""
    p = os.path.join(ROOT, "profiles", "etch_accuracy_480cube.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    tag = f"width {width} colours 3 k2*tau=0.265"
    cases = [f for f in d["families"] if tag in f["case"]]
    return {"source": d["source"], "band": d["band"], "bench_tile_width": width, "bench_f": ACCURATE_F,
            "cases": [{"case": f["case"], "growth_rate": f["observables"]["growth rate um/h"],
                       "atoms": f["observables"]["atoms"]} for f in cases]}


def batched_bench(args):
    """Config 3: 512 independent Si(001) replicas, box side ~U{16..96} cells,
    T ~ U(900, 1300) K, F ~ logU(0.05, 5) ML/s, seed 1000+i, in one persistent
    launch per block of windows; tau per replica and tile width autotuned:
    the window factor f by the pilot tuner (autotune.choose_f: 16 replicas
    of the model at 1100 K, 0.5 ML/s in 480^3 boxes, each f of the ladder
    against the shortest), one width for the batch by a timed trial, then one
    per group of box sizes by coordinate descent.
    Also one replica of the median size run alone (the plain single-replica
    path) for the batched/plain ratio."""
    import numpy as np
    from mulskips_gb300 import Batch, Lattice, arrhenius_tables
    from mulskips_gb300.autotune import choose_f, choose_width, choose_widths, size_groups
    pE, pD = arrhenius_tables(1100.0, flux=0.5)

    def pilot(f):
        p = Batch([(480, 480, 480)] * 16, seeds=[300 + s for s in range(16)])
        p.set_rates(np.stack([pE] * 16), np.stack([pD] * 16))
        p.init_flat("S", [120] * 16)
        return p

    f, pilots = choose_f(pilot, 4e-7)
    rng = np.random.default_rng(3)
    n = 512
    sides = rng.integers(16, 97, n)
    temps = rng.uniform(900.0, 1300.0, n)
    flux = 10.0 ** rng.uniform(math.log10(0.05), math.log10(5.0), n)
    boxes = [(12 * int(s), 12 * int(s), 12 * int(s)) for s in sides]
    len1 = [max(48, (6 * int(s)) // 24 * 24) for s in sides]
    tabs = [arrhenius_tables(float(temps[i]), flux=float(flux[i])) for i in range(n)]
    b = Batch(boxes, seeds=[1000 + i for i in range(n)])
    b.set_rates(np.stack([t[0] for t in tabs]), np.stack([t[1] for t in tabs]))
    b.init_flat("S", len1)
    tau = b.suggest_tau(f)
    width = choose_width(b, tau, restore=False)
    # then one width per group of box sizes, starting from the batch's best
    groups = size_groups(sides)
    widths, trials = choose_widths(b, b.suggest_tau(f), groups)
    by_group = [{"side_cells": [int(sides[g].min()), int(sides[g].max())], "replicas": int(len(g)),
                 "tile_width": int(widths[g[0]])} for g in groups]
    tau = b.suggest_tau(f)
    b.run(tau, 8)
    ev = 0
    ms = 0.0
    for _ in range(args.steps):
        ev += b.run(tau, BATCH_WINDOWS_PER_STEP)
        ms += b.run_stats()["kernel_ms"]
    b.close()
    med = int(np.median(sides))
    one = Lattice(12 * med, 12 * med, 12 * med, seed=7)
    one.set_rates(*arrhenius_tables(1100.0, flux=0.5))
    one.init_flat("S", max(48, (6 * med) // 24 * 24))
    t1 = one.suggest_tau(f)
    one.set_tiling(width)
    one.run(t1, 8)
    ev1, _ = one.run(t1, BATCH_WINDOWS_PER_STEP * args.steps)
    ms1 = one.run_stats()["kernel_ms"]
    one.close()
    v = ev / (ms / 1e3)
    v1 = ev1 / (ms1 / 1e3)
    return {"value": v, "unit": "events/s", "replicas": n, "events": ev, "windows": BATCH_WINDOWS_PER_STEP * args.steps,
            "tile_width": width, "tile_width_by_size_group": by_group, "width_trials": trials,
            "single_replica_value": v1, "single_replica_side_cells": med,
            "batched_over_single": v / v1,
            "f": f, "f_pilots": pilots,
            "workload": "512 Si(001) replicas, side ~U{16..96} cells, T~U(900,1300) K, F~logU(0.05,5), "
                        f"seed 1000+i, tau = {f}/r* per replica (f from the pilot tuner)"}


def cvd_bench(windows=4096, oracle_events=3000000):
    """CVD of Si(001) under one coverage species (H) with the rates of the
    reference's CVD-Si-SiH2 case, on a 3072 x 3072 x 240 grid (Len1 = 48 slab,
    41x the reference's 480^2 surface), window factor f = 0.3: events/s of one
    mks_run call over `windows` windows after a 256-window warm-up (wall time
    of the synchronous call), against the serial oracle on the reference's own
    480^3 case (RunType R)."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300.startdat import parse_startdat
    from oracle import ora
    path = os.path.join(ROOT, "tests", "golden", "CVD-Si-SiH2", "start.dat")
    d = parse_startdat(path)
    lat = Lattice(3072, 3072, 240, sf=d["sf"], list_cov=d["list_cov"], seed=5)
    lat.set_rates(d["ptransE"], d["ptransD"])
    lat.set_coverage_rates(d["ptransAbs"][:, 1:], d["ptransDes"][:, 1:])
    lat.init_flat("S", 48)
    tau = lat.suggest_tau(ACCURATE_F)
    lat.run(tau, 256)
    e0 = lat.observables()["events"]
    t0 = time.perf_counter()
    lat.run(tau, windows)
    wall = time.perf_counter() - t0
    obs = lat.observables()
    lat.close()
    ev = obs["events"] - e0
    txt = open(path).read().replace("T ! RunType", "R ! RunType")
    tmp = tempfile.mkdtemp()
    p = os.path.join(tmp, "start.dat")
    open(p, "w").write(txt)
    o = ora.Oracle(p, 480, 480, 480, numbers=None)
    o.init()
    c0 = time.perf_counter()
    o.run(oracle_events)
    cdt = time.perf_counter() - c0
    n = o.iter - 1
    o.close()
    shutil.rmtree(tmp, ignore_errors=True)
    return {"value": ev / wall, "unit": "events/s", "events": int(ev), "windows": windows, "tau_s": tau,
            "covered_sites": int(obs["covered"]), "atoms": int(obs["atoms"]),
            "oracle_events_per_s": n / cdt, "oracle_events": int(n),
            "workload": "Si(001) + H CVD, rates of the reference's CVD-Si-SiH2 case, 3072x3072x240 grid, "
                        "Len1=48, f=0.3; oracle: the reference's 480^3 case, serial, 1 core"}


PZIG_1600K = 1.0 / (1.0 + math.exp(-0.02 / (0.00008617330350 * 1600.0)))   # 0.5362


def stacking_bench(side=1536, cube=960, warm_blocks=24, windows=1024, oracle_events=2000000):
    """Config 2 (3C-SiC with stacking faults): arm-chair stacking on the
    explicit-neighbour engine.  A 3C-SiC parallelepiped (SetNC, `cube` grid
    units a side, 80 cells) in a 128^3-cell box (1536^3 grid), the SiC rates
    of the reference's cube-zigzag case, PtransZig = 1 / (1 + exp(-0.02 eV /
    kT)) at 1600 K (a 0.02 eV preference for cubic stacking on ties).  The
    config's own rates (barriers U(0.4, 0.9) eV at 1600 K) evaporate every
    atom far faster than a flux of 1 ML/s deposits, so nothing would grow or
    stack; the cube-zigzag rates grow the crystal and form stacking faults.
    Window factor f = 0.01 (two species), re-suggested for each of the
    warm-up's blocks of 64 windows while the fast C adatoms of the initial
    faces evaporate; then events/s over `windows` windows at the largest
    suggestion of the warm-up's second half, the steady value (a single fast
    site -- an adatom of rate ~300/s against deposition at 1e-3/s per site --
    makes the suggestion 3e-5 s for as long as it lives, which can be most
    of the warm-up), wall time of the synchronous call, with the
    non-epitaxial bulk count (_d.xyz); against the serial oracle on the
    reference's 480^3 cube-zigzag case (RunType R, one core)."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300.autotune import accurate_f
    from mulskips_gb300.startdat import parse_startdat
    from oracle import ora
    path = os.path.join(ROOT, "tests", "golden", "cube-zigzag", "start.dat")
    d = parse_startdat(path)
    f = accurate_f(2)
    lat = Lattice(side, side, side, ncrystal=2, list_crystal=d["list_crystal"], sf=d["sf"], ptrans_zig=PZIG_1600K,
                  seed=11)
    lat.set_rates(d["ptransE"], d["ptransD"])
    lat.init_shape("C", [cube, cube, cube])
    taus = []
    for _ in range(warm_blocks):
        taus.append(lat.suggest_tau(f))
        lat.run(taus[-1], 64)
    tau = float(max(taus[warm_blocks // 2:]))
    t0 = time.perf_counter()
    n, tsim = lat.run(tau, windows)
    wall = time.perf_counter() - t0
    obs = lat.observables()
    lat.close()
    txt = open(path).read().replace("T   ! R = production run", "R   ! R = production run")
    tmp = tempfile.mkdtemp()
    p = os.path.join(tmp, "start.dat")
    open(p, "w").write(txt)
    o = ora.Oracle(p, 480, 480, 480, numbers=None)
    o.init()
    c0 = time.perf_counter()
    o.run(oracle_events)
    cdt = time.perf_counter() - c0
    m = o.iter - 1
    o.close()
    shutil.rmtree(tmp, ignore_errors=True)
    return {"value": n / wall, "unit": "events/s", "events": int(n), "windows": windows, "tau_s": tau,
            "sim_time_s": tsim, "atoms": int(obs["atoms"]), "nonepitaxial_bulk": int(obs["nonepitaxial"]),
            "ptrans_zig": PZIG_1600K, "oracle_events_per_s": m / cdt, "oracle_events": int(m),
            "workload": f"3C-SiC parallelepiped (SetNC, {cube} grid units a side) in a {side}^3 grid (128^3 cells), "
                        "rates of the reference's cube-zigzag case, PtransZig 0.5362 (0.02 eV at 1600 K), f = 0.01; "
                        "oracle: the reference's 480^3 cube-zigzag case, serial, 1 core"}


def config2_tables(seed=2, T=1600.0):
    """Config 2's rate tables: per-species flux F_s ~ U(0.1, 1.0) ML/s as
    PtransD(s, n) for n = 1..3, and the 18 evaporation entries of
    SetProbability.f:49-50 (species Si, C x the neighbour census (n_Si, n_C),
    1 <= n_Si + n_C <= 3) with barriers E ~ U(0.4, 0.9) eV and prefactor 1e13
    s^-1 at T, drawn from numpy's PCG64 with `seed`.  Returns (PtransE,
    PtransD, F, barriers)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    F = rng.uniform(0.1, 1.0, 2)
    Eb = rng.uniform(0.4, 0.9, (2, 9))
    E = np.zeros((3, 4, 4, 4, 4, 4, 4))
    D = np.zeros((3, 3))
    for s in range(2):
        D[s, :] = F[s]
        j = 0
        for n1 in range(4):
            for n2 in range(4 - n1):
                if n1 + n2:
                    E[s, n1, n2] = 1e13 * math.exp(-Eb[s, j] / (0.00008617330350 * T))
                    j += 1
    return E, D, F, Eb


def config2_oracle(E, D, sf, events, side=480, h_slab=400, period=96):
    """The serial oracle (RunType R, one core) on config 2's model in a 480^3
    box: the same rates and PtransZig on a {111}-faceted slab of the same
    form, `events` events (fewer than half its atoms, so the etch front stays
    clear of the bottom wall).  Returns (events/s, events)."""
    from mulskips_gb300.shapes import faceted_slab_points
    from mulskips_gb300.startdat import write_startdat
    from oracle import ora
    xyz, sp = faceted_slab_points(side, h_slab, period)
    assert events < 0.5 * int(((xyz[:, 2] > 3) & (xyz[:, 2] < side - 4)).sum())
    tmp = tempfile.mkdtemp()
    try:
        pts = os.path.join(tmp, "slab.xyz")
        with open(pts, "w") as fh:
            fh.write(f"{len(xyz)}\nslab\n")
            fh.write("".join(f"{'Si' if s == 1 else 'C'} {x} {y} {z}\n" for (x, y, z), s in zip(xyz.tolist(), sp)))
        p = os.path.join(tmp, "start.dat")
        write_startdat(p, E, D, ncrystal=2, list_crystal=(14, 6), init_st="SH", points=pts, run_type="R",
                       seed=7, sf=sf, ptrans_zig=PZIG_1600K, max_iter=10 ** 9)
        o = ora.Oracle(p, side, side, side, numbers=None)
        o.init()
        c0 = time.perf_counter()
        o.run(events)
        cdt = time.perf_counter() - c0
        m = o.iter - 1
        o.close()
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return m / cdt, m


def config2_bench(side=1536, h_slab=768, period=192, warm_blocks=8, windows=1024, oracle_events=200000):
    """Config 2 as stated: 3C-SiC (Si, C) in a 128^3-cell box (1536^3 grid)
    on a slab whose surface is {111} facets only (an SH point list of square
    pyramids of period 192 grid units, mulskips_gb300.shapes), per-species
    fluxes U(0.1, 1.0) ML/s and 18 evaporation barriers U(0.4, 0.9) eV with
    a 1e13 prefactor at 1600 K (table seed 2), PtransZig = 0.5362, on the
    explicit-neighbour engine.  These rates evaporate a surface atom at
    1e10-1e11 s^-1 against a deposition of at most 1 s^-1 per site, so the
    slab etches (the atoms lost and the etch rate are in the line); an
    arm-chair choice needs a deposition next to a single bond and is rare.
    Window factor f = 0.01 (two species), re-suggested per block of 64
    warm-up windows; then events/s over `windows` windows at the largest
    suggestion of the warm-up's second half, wall time of the synchronous
    call."""
    from mulskips_gb300 import Lattice
    from mulskips_gb300.autotune import accurate_f
    from mulskips_gb300.shapes import faceted_slab_points
    from mulskips_gb300.startdat import parse_startdat
    sf = parse_startdat(os.path.join(ROOT, "tests", "golden", "cube-zigzag", "start.dat"))["sf"]
    E, D, F, Eb = config2_tables()
    xyz, sp = faceted_slab_points(side, h_slab, period)
    f = accurate_f(2)
    lat = Lattice(side, side, side, ncrystal=2, list_crystal=(14, 6), sf=sf, ptrans_zig=PZIG_1600K, seed=13)
    lat.set_rates(E, D)
    lat.init_points(xyz, sp)
    a0 = lat.observables()["atoms"]
    taus = []
    t_warm = 0.0
    for _ in range(warm_blocks):
        taus.append(lat.suggest_tau(f))
        _, t_warm = lat.run(taus[-1], 64)
    tau = float(max(taus[warm_blocks // 2:]))
    a1 = lat.observables()["atoms"]
    t0 = time.perf_counter()
    n, tsim = lat.run(tau, windows)
    wall = time.perf_counter() - t0
    obs = lat.observables()
    lat.close()
    ov, om = config2_oracle(E, D, sf, oracle_events)
    return {"value": n / wall, "unit": "events/s", "events": int(n), "windows": windows, "tau_s": tau,
            "oracle_events_per_s": ov, "oracle_events": int(om),
            "atoms_initial": int(a0), "atoms_before": int(a1), "atoms_after": int(obs["atoms"]),
            "etch_atoms_per_s": (int(a1) - int(obs["atoms"])) / (tsim - t_warm),
            "nonepitaxial_bulk": int(obs["nonepitaxial"]), "ptrans_zig": PZIG_1600K,
            "flux_ml_per_s": [float(v) for v in F], "barriers_eV": Eb.round(4).tolist(),
            "workload": f"3C-SiC slab with {{111}} facets only (SH point list, pyramids of period {period}, valleys "
                        f"at z = {h_slab - period // 2}, apexes at {h_slab + period // 2}) in a {side}^3 grid, "
                        "fluxes U(0.1,1) ML/s, 18 barriers U(0.4,0.9) eV, nu 1e13, 1600 K, table seed 2, "
                        "PtransZig 0.5362, f = 0.01; oracle: the same model on a slab of the same form in a "
                        "480^3 box, serial, 1 core"}


def la_gradient_bench():
    """Config 4: 128 SiGe replicas (64x64x256 cells, Ge 0.2) under the laser
    pulse T = 300 + 1500 exp(-((t-100 ns)/40 ns)^2) exp(-z/200 nm) K, melting
    and regrowth with the LA rate law, the FP64 likelihood-ratio score of the
    four barrier parameters; the mean regrowth velocity between 115 and
    145 ns and its gradient from the backward kernel.  Wall time of the whole
    forward + backward (device work and the host loop of segments)."""
    from mulskips_gb300 import la
    sim = la.Anneal(n=128)
    t0 = time.perf_counter()
    v, g, se = la.regrowth_velocity_lr(sim, la.THETA_REF, 115e-9, 145e-9)
    wall = time.perf_counter() - t0
    ev = sum(o["events"] for o in sim.batch.observables())
    sim.batch.close()
    return {"events_per_s": ev / wall, "events": int(ev), "wall_s": wall, "replicas": 128,
            "regrowth_velocity_m_per_s": float(v.mean()), "velocity_sd": float(v.std(ddof=1)),
            "theta": dict(zip(la.THETA_NAMES, la.THETA_REF)),
            "grad_m_per_s_per_eV": dict(zip(la.THETA_NAMES, map(float, g))),
            "grad_se": dict(zip(la.THETA_NAMES, map(float, se)))}


def reference(args, rank, world):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    samples = []
    for _ in range(args.warmup):
        pass
    total_ev = 0
    total_t = 0.0
    slab = None
    for k in range(args.steps):
        v, ev, runs, slab = cpu_baseline(seconds=args.cpu_seconds, cores=cores)
        samples.append(v)
        total_ev += ev
        total_t += ev / v
    value = total_ev / total_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "plain Si(001) KMC, same rates; bounded CPU sample: 480^3 box, Len1=360 slab "
                               "etched to the walls, T cycling 1000/1100/1200 K, one oracle process per core"},
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": cores, "kind": "port",
                         "sample": "serial C restatement of the reference (no Fortran compiler for the "
                                   "reference itself), one independent seed per core",
                         "slab": slab},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--only", choices=["stacking", "config2", "batched", "cvd", "la"], default=None,
                    help="run one side line alone and print it (e.g. for a profile of its kernel)")
    ap.add_argument("--stacking-side", type=int, default=1536)
    ap.add_argument("--stacking-cube", type=int, default=960)
    ap.add_argument("--stacking-windows", type=int, default=1024)
    args = ap.parse_args()
    if args.only == "stacking":
        print(json.dumps(stacking_bench(side=args.stacking_side, cube=args.stacking_cube,
                                        windows=args.stacking_windows, oracle_events=200000)))
        return
    if args.only:
        line = {"batched": lambda: batched_bench(args), "cvd": lambda: cvd_bench(oracle_events=200000),
                "config2": config2_bench,
                "la": la_gradient_bench}[args.only]()
        print(json.dumps(line))
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.gpus == 1 else 1)))
    if args.impl == "reference":
        reference(args, rank, world)
    else:
        gb300(args, rank, world)


if __name__ == "__main__":
    main()
