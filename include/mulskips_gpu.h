/*
 * mulskips_gpu.h — C ABI of the GB300 KMC engine (libmulskips_gpu.so).
 *
 * The reference MulSKIPS program is one serial Fortran executable whose KMC
 * state lives in module globals (mulskips-source/modules/defsystem.f) and whose
 * hot loop is mulskips-source/main.f:304-371.  It has no library interface;
 * the only precedent for a C ABI in the project is the ISO_C_BINDING socket
 * layer (mulskips-source-LaserAnnealing/sockets/fsockets.f:45-62).  The entry
 * points below replace the reference's internal calls one to one, so that a
 * Fortran or C++ host (mulskips.e) or the Python wrapper can drive the GPU:
 *
 *   mks_create / mks_destroy     module state + AllocateArrays
 *                                (defsystem.f:49-68, AllocateArrays.f:24-45)
 *   mks_set_rates                SetProbability (SetProbability.f:21-143)
 *   mks_set_coverage_rates       its PtransAbs / PtransDes part (:121-140),
 *                                with IndexEvent_Abs (Get_Prob.f:22-52),
 *                                absorption.f and desorption.f
 *   mks_init_flat                SetSi / SetSiC3C (SetSi.f:25-221,
 *                                SetSiC3C.f:25-199), main.f:237-239,224-226
 *   mks_init_shape               the shaped initializers of main.f:224-278
 *                                (SetNC, SetNCSp(Si), SetInvPOff and its
 *                                variants, SetTrench(Si), SetSiC3Cww(aperture),
 *                                SetSiFINFET)
 *   mks_batch_init_cad(_la,      SetCAD (SetCAD.f:80-341) for InitSt IN, with
 *     _alloy)                    SetT and the molten nucleus for LA
 *   mks_init_points              SetShape (SetShape.f:25-436, InitSt SH)
 *   mks_load_lattice             continuation / CAD load of LattCoo
 *                                (SetCAD.f:54-79,301-418)
 *   mks_write_frame              WriteMolMolXYZFile.f:22-406
 *   mks_get_lattice              LattCoo dump (main.f:385-403)
 *   mks_run                      the KMC loop main.f:304-371 (PickTreeEvent,
 *                                Deposition, Evaporation, Get_Prob, UpdateTree)
 *   mks_replay                   Deposition.f / Evaporation.f applied to a
 *                                given event sequence (no selection)
 *   mks_class_histogram          the per-class view of the rate tree Tree(:)
 *   mks_site_rates               the tree leaves: ListAdAtom ProbTrans
 *                                (Get_Prob.f:54-331, Get_Prob_Ini.f:23-161)
 *   mks_get_observables          the scans of WriteMolMolXYZFile.f:77-119 and
 *                                pymulskips/analyze.py:124-207
 *
 * All pointers are host memory owned by the caller; data is copied in/out.
 * Every function returns 0 on success or one of the MKS_ERR_* codes; the
 * reference STOPs the process on the same conditions (UpdateTree.f:38-48,
 * Add.f:37-45, Erase.f:41-50, Get_Prob.f:293-298).  mks_last_error() gives
 * the message of the last failure on the calling thread.
 *
 * One handle holds a batch of independent replicas (1 for a plain run) on one
 * GPU, with one CUDA stream.  Handles are not thread-safe; several handles
 * may live in one process.
 *
 * Arm-chair stacking.  With PtransZig < 1 (a single-replica handle, NCov = 0)
 * a deposition on a coor-1 site may take the hexagonal (arm-chair) position
 * of IF_Arm_Choice.f:21-56, whose atoms lie off the diamond sub-grid
 * (FIND_SN.f:67).  Such a handle runs the explicit-neighbour engine: one
 * LattCoo word and one LattInd word per grid point and the NextN list of
 * every listed site, as the reference stores them (defsystem.f:49,87-91,
 * defdertype.f:25-45).  The initializers build the lattice as usual; it is
 * expanded at the first call that runs or reads it.  mks_replay, mks_run,
 * mks_get_lattice, mks_get_observables (nonepitaxial: the non-epitaxial bulk
 * atoms of the reference's _d.xyz, WriteMolMolXYZFile.f:120-160),
 * mks_write_frame, mks_get_status, mks_get_clock and mks_suggest_tau work
 * on it; the compact-lattice calls (mks_get_state, mks_class_histogram,
 * mks_site_rates, mks_frame_sites, mks_replay_noalloc, mks_set_clock) return
 * MKS_ERR_UNSUPPORTED once it is expanded.
 */
#ifndef MULSKIPS_GPU_H
#define MULSKIPS_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MKS_OK 0
#define MKS_ERR_ARG 1          /* bad argument or unsupported box size        */
#define MKS_ERR_CUDA 2         /* CUDA runtime failure / no device            */
#define MKS_ERR_INVARIANT 3    /* lattice state contradicts the model         */
#define MKS_ERR_CAPACITY 4     /* a tile held more surface sites than fit     */
#define MKS_ERR_UNSUPPORTED 5  /* feature outside the engine (e.g. PtransZig<1) */
#define MKS_ERR_TIMEOUT 6      /* a bounded device wait gave up               */

#define MKS_NCLASS 64          /* rate classes, see mks_class_histogram       */

typedef struct mks_handle mks_handle;

/* One replica's setup (the scalar part of start.dat, main.f:83-212). */
typedef struct {
    int32_t lenx, leny, lenz;      /* LenX, LenY, LenZ; LenX, LenY multiples of 12, LenZ of 3 */
    int32_t ncrystal, ncov;        /* NCrystal (1..3), NCov (0; 1 with NCrystal <= 2; 2 with NCrystal = 1) */
    int32_t list_crystal[3];       /* atomic numbers (ListCrystal)               */
    double ptrans_zig;             /* PtransZig; < 1 selects arm-chair stacking (see below) */
    double sf;                     /* super-lattice parameter in Angstrom        */
    uint64_t seed;                 /* IDUM / replica seed                        */
    int32_t list_cov[3];           /* coverage atomic numbers (ListCov, main.f:91) */
    int32_t explicit_nn;           /* 1: the explicit-neighbour engine even at PtransZig = 1,
                                      for lattices with atoms off the diamond sites (InitSt E);
                                      0 (the default): that engine only when PtransZig < 1 */
} mks_config;

/* One applied event (the trace format of the oracle and of mks_replay). */
typedef struct {
    int32_t x, y, z;               /* grid coordinates of the event site         */
    int8_t itrans;                 /* 1..3 deposition of that species, 4 evaporation,
                                      5 desorption, 6 / 7 absorption of coverage species 1 / 2 */
    int8_t arm;                    /* arm-chair stacking choice of a tie (IF_Arm_Choice.f:44-51) */
    int16_t pad;
} mks_event;

typedef struct {
    int64_t events;                /* accepted events since creation             */
    double time;                   /* simulated time (FP64 clock)                */
    int64_t atoms;                 /* occupied non-wall sites                    */
    int64_t undercoord;            /* atoms with coordination <= 3 (xyz count)   */
    int64_t mc_sites;              /* sites with an event (NumAdAtom)            */
    int64_t voids;                 /* empty sites with coordination 4            */
    int64_t species[3];            /* atoms per species                          */
    double mean_height;            /* mean top-atom height, grid units           */
    double rms_roughness;          /* RMS of the column heights, grid units      */
    double total_rate;             /* sum of all event rates (FP64)              */
    int64_t nonepitaxial;          /* off-lattice bulk atoms (stacking faults)   */
    int64_t covered;               /* empty sites carrying the coverage species (NumCovTotal) */
} mks_observables;

typedef struct {
    int32_t error;                 /* last device error code (0 = none)          */
    int32_t pending_tiles;         /* tiles left unfinished by a window          */
    int64_t fallback_tiles;        /* tiles run from global memory               */
    int64_t windows;               /* sublattice windows completed               */
    int32_t active;                /* 1 while the replica still runs             */
    int32_t stop_reason;           /* 0 running, 1 few MC sites, 2 max events, 3 max time,
                                      4 regrown (LA mode) */
} mks_status;

/* ---- plain (single-replica) interface ---- */
int mks_create(const mks_config *cfg, mks_handle **out);
void mks_destroy(mks_handle *h);
const char *mks_version(void);
int mks_last_error(char *buf, int32_t len);

/* ptransE: 3*4^6 doubles indexed [s][n1][n2][n3][c1][c2][c3] (the PTransE
 * array of defsystem.f:63-64); ptransD: 3x3 doubles [s][coor-1].          */
int mks_set_rates(mks_handle *h, const double *ptransE, const double *ptransD);
/* Coverage species (NCov = 1 with NCrystal <= 2, or NCov = 2 with NCrystal
 * = 1): ptransAbs, ptransDes are 3x3 doubles [coverage species][coor-1]
 * (PtransAbs / PtransDes, SetProbability.f:121-140; rows past NCov must be
 * zero).  An empty site of coordination n then carries deposition +
 * absorption at sum_s PtransD(s,n) + sum_i PtransAbs(i,n) (Get_Prob.f:
 * 155-204), the species absorbed drawn past the deposition share by the
 * cumulative PtransAbs (IndexEvent_Abs, :22-52); a site covered by species i
 * desorbs at PtransDes(i,n) (:93-118); an atom's evaporation key counts its
 * covered neighbours of each species (PE(NSiC,n1,n2,0,c1,c2,0), :309-312).
 * mks_replay takes itrans 5 for a desorption and 5+i for an absorption of
 * species i (main.f:346-356).  Replaces IndexEvent_Abs / absorption.f /
 * desorption.f.                                                           */
int mks_set_coverage_rates(mks_handle *h, const double *ptransAbs, const double *ptransDes);
/* kind 'S' = SetSi (InitSt FS), 'C' = SetSiC3C (InitSt F); len1 is the slab
 * height, rounded down to a multiple of 24 as main.f:226,238 does.         */
int mks_init_flat(mks_handle *h, char kind, int32_t len1);
/* LattCoo(0:LenX-1,0:LenY-1,0:LenZ), x fastest (Fortran order).           */
int mks_load_lattice(mks_handle *h, const int32_t *lattcoo);
int mks_get_lattice(mks_handle *h, int32_t *lattcoo);
/* Arm-chair stacking handles only (PtransZig < 1): load the full reference
 * state -- LattCoo(0:LenX-1, 0:LenY-1, 0:LenZ) (x fastest) and n list
 * entries (ListAdAtom, ListAtom and ListVoid; grid point xyz[3i..3i+2] and
 * NextN nn[12i..12i+11], defdertype.f:25-45).  With event and rate NULL
 * every entry is rated as Get_Prob_Ini does (an unsupported coor-1 site at
 * 1e-6, Get_Prob_Ini.f:102-104); with both given, entry i keeps event code
 * event[i] (0 none, 1 deposition, 2 dummy deposition, 4 evaporation) and
 * rate[i] -- the ProbTrans of a saved ListAdAtom, which the reference does
 * not recompute when only a site's second neighbours change -- except that
 * an atom without reciprocal neighbours is the isolated atom of
 * Get_Prob.f:300-306.  Continuation from a saved state (main.f:385-403
 * writes LattCoo; the lists follow).                                       */
int mks_load_lists(mks_handle *h, const int32_t *lattcoo, int64_t n, const int32_t *xyz, const int32_t *nn,
                   const int32_t *event, const float *rate);
/* Arm-chair stacking handles only: every listed site, with its grid point
 * (xyz, 3 per site), NextN (nn, 12 per site), kind (1 with an event, the
 * ListAdAtom entries; 2 a bulk atom, ListAtom; 3 a void, ListVoid), event
 * (1 deposition, 2 dummy deposition, 4 evaporation, 5 isolated atom) and FP32
 * rate (the ProbTrans of the tree leaf; 0 for an isolated atom, whose rate is
 * 1e5 x the total, Get_Prob.f:305).  *n gets the count; the arrays (all
 * non-NULL) are written when cap >= *n.                                   */
int mks_get_lists(mks_handle *h, int64_t cap, int32_t *xyz, int32_t *nn, int32_t *kind, int32_t *event, float *rate,
                  int64_t *n);
/* Compact state: one byte per diamond site (a, b, z1) at index
 * (z1 * (LenY/6) + b) * (LenX/6) + a (bits 0-1 species, 2-4 coordination,
 * 5-6 first list entry, 7 dummy flag; 0x80 a wall; coordination field 5 with
 * the dummy flag: a coor-1 site still at Get_Prob_Ini's dummy rate 1e-6,
 * Get_Prob_Ini.f:102-104); n >= mks_state_size().                        */
int64_t mks_state_size(mks_handle *h);
int mks_get_state(mks_handle *h, uint8_t *st, int64_t n);
/* The compact state of replica rep, NZ*NB*NA bytes (NA = LenX/6, NB = LenY/6,
 * NZ = LenZ/3 + 1), in the layout of mks_get_state.                     */
int mks_batch_get_state(mks_handle *h, int32_t rep, uint8_t *st, int64_t n);
/* Upload compact state bytes (same layout); the per-tile bands are rebuilt. */
int mks_set_state(mks_handle *h, const uint8_t *st, int64_t n);
/* Double-buffered input: mks_prefetch_state starts copying a compact state
 * (layout of mks_get_state; pinned host memory makes it asynchronous) into a
 * second device buffer on its own stream, overlapping the work in flight;
 * mks_swap_state makes it the lattice once the copy is done (ordered on the
 * engine's stream) and rescans the tiles.  No counterpart in the reference
 * (the Fortran program has one in-memory lattice).                        */
int mks_prefetch_state(mks_handle *h, const uint8_t *st, int64_t n);
int mks_swap_state(mks_handle *h);
int mks_replay(mks_handle *h, const mks_event *trace, int64_t n);
/* mks_replay without any device allocation: no counterpart in the reference
 * (the Fortran program has no device memory at all).  For callers that may
 * not call cudaMalloc -- e.g. a host that has handed its whole memory budget
 * to the lattice, or that runs this step under a stream-ordered memory pool it
 * must not grow.  The trace is staged in one fixed 1 MiB + 256 B device array
 * owned by the library, so n may be at most MKS_REPLAY_NOALLOC_MAX events per
 * call (longer traces are rejected with MKS_ERR_ARG; split them).  The array
 * is shared by every call and every handle on a device: calls that overlap on
 * the GPU (several handles or threads at once) race and must be serialized.
 * Each call starts by clearing the array's progress counter, and the array
 * keeps the last call's trace afterwards.  mks_create / mks_batch_create look
 * up the array's device address once, with the handle's device current, and
 * keep it in the handle.                                                  */
#define MKS_REPLAY_NOALLOC_MAX 65536
int mks_replay_noalloc(mks_handle *h, const mks_event *trace, int64_t n);
/* Synchronous-sublattice KMC: windows of length tau (s); stops after
 * max_windows windows, or once max_events / max_time is reached (checked per
 * window), or when fewer than 21 surface sites remain (main.f:307-310).    */
int mks_run(mks_handle *h, double tau, int64_t max_windows, int64_t max_events,
            double max_time, int64_t *events_done, double *time_out);
/* Event sites per rate class (nclass >= MKS_NCLASS): 1 empty coor-1, 2 its
 * dummy (1e-8, Get_Prob.f:183), 3 coor-2, 4 coor-3, 5 isolated atom, 6..62
 * atoms by species and census (PTransE key), 63 the dummy an initializer
 * wrote (1e-6, Get_Prob_Ini.f:104); coverage mode: 6..8 covered sites,
 * 9..58 atoms by species, census and covered neighbours.                  */
int mks_class_histogram(mks_handle *h, int64_t *hist, int32_t nclass);
/* Rate class and FP32 rate of n sites of replica rep given by grid
 * coordinates xyz[3n] (AtomXYZ of ListAdAtom, defdertype.f:32-37): the
 * ProbTrans of the reference's tree leaves (Get_Prob.f:54-331,
 * Get_Prob_Ini.f:23-161).  Class 0 for a site without an event, -1 for a
 * grid point that is not a diamond site; isolated atoms (class 5, rate
 * 1e5 x Tree(1), Get_Prob.f:305) report rate 0.                           */
int mks_site_rates(mks_handle *h, int32_t rep, const int32_t *xyz, int64_t n, int32_t *cls, float *rate);
/* Sites listed in an output frame, as compact-state indices in the
 * reference's z, y, x scan order (WriteMolMolXYZFile.f:171-260): kind 0 the
 * atoms with coordination <= 3 and, with a coverage species, the covered
 * sites (the H / Cl lines, :176-178), kind 1 the voids (covered or not).
 * *n gets the count; the indices are written when idx is non-NULL and
 * cap >= *n.                                                               */
int mks_frame_sites(mks_handle *h, int32_t kind, uint32_t *idx, int64_t cap, int64_t *n);
/* The output frame files of WriteMolMolXYZFile.f:22-406 for the current
 * lattice: <base>.xyz (atoms of coordination <= 3 and covered sites in the
 * z, y, x scan, then the voids), <base>_d.xyz (non-epitaxial bulk: none with
 * cubic stacking), <base>_v.xyz (voids; for SiC labelled by their neighbours'
 * species, :216-260) and, for SiC, <base>_w.xyz (bulk atoms with three
 * neighbours of the right species once those with none have been counted as
 * swapped, :264-398; the reference's swap-and-restore of LattCoo, which
 * gives every swapped site the type of the last one, is not applied to the
 * run).  Voids follow the scan order, not the reference's ListVoid order.
 * *num_at_wrong (may be NULL) gets the SiC NumAtWrong count, else 0.       */
int mks_write_frame(mks_handle *h, const char *base, double time, int64_t iter, int64_t *num_at_wrong);
int mks_get_observables(mks_handle *h, mks_observables *obs);
int mks_get_status(mks_handle *h, mks_status *st);

/* ---- batched replicas ---- */
/* n replicas of uneven boxes, each with its own rates and seed, advanced
 * together; tau per replica.  Replica i uses rates ptransE + i*3*4096 and
 * ptransD + i*9.                                                           */
int mks_batch_create(const mks_config *cfgs, int32_t n, mks_handle **out);
int mks_batch_set_rates(mks_handle *h, const double *ptransE, const double *ptransD);
/* mks_set_coverage_rates per replica: replica i uses ptransAbs + i*9 and
 * ptransDes + i*9.                                                         */
int mks_batch_set_coverage_rates(mks_handle *h, const double *ptransAbs, const double *ptransDes);
int mks_batch_init_flat(mks_handle *h, char kind, const int32_t *len1);
int mks_batch_run(mks_handle *h, const double *tau, int64_t max_windows,
                  int64_t max_events_each, double max_time_each, int64_t *events_total);
int mks_batch_observables(mks_handle *h, mks_observables *obs /* n entries */);
/* Class histogram of every replica (n * nclass, nclass >= 64), the
 * per-replica view of mks_class_histogram.                               */
int mks_batch_class_histogram(mks_handle *h, int64_t *hist, int32_t nclass);
int32_t mks_batch_size(mks_handle *h);

/* Tile width (sites, 4..8) of the sublattice decomposition; the default
 * is 8.  Re-partitions every replica (no counterpart in the reference, whose
 * loop is serial; the tile shape is one of the autotuner's knobs).         */
int mks_set_tiling(mks_handle *h, int32_t width);
int32_t mks_get_tiling(mks_handle *h);
/* Tile width per replica (n entries, 4..8 each): replicas of a batch may be
 * cut at different widths (the autotuner picks one per group of replica
 * sizes); mks_get_tiling then gives the largest.                          */
int mks_batch_set_tiling(mks_handle *h, const int32_t *widths);
int mks_batch_get_tiling(mks_handle *h, int32_t *widths);
/* Colouring of the sublattice tiles (no counterpart in the reference, whose
 * loop is serial).  0 (the default): every replica whose tiles can be at
 * least 6 sites wide at the current width takes the brick tiling -- rows of
 * tiles with the odd rows shifted by half a tile, three colours, 3 phases
 * and 6 neighbours per tile per window -- and the others the square grid of
 * four colours (4 phases, 8 neighbours); 3: the brick tiling for every
 * replica (MKS_ERR_ARG if one cannot take it); 4: the square grid for all.
 * mks_get_colours gives the largest colour count in use.                 */
int mks_set_colours(mks_handle *h, int32_t ncolour);
int32_t mks_get_colours(mks_handle *h);
/* Schedule of the sublattice windows: 1 (default) one persistent kernel in
 * which each tile waits only for its eight neighbours, 0 one launch per
 * colour phase.  Both give the same lattice for the same seed.           */
int mks_set_schedule(mks_handle *h, int32_t persistent);
/* Replica clock: simulated time, windows run (the counter the random draws
 * are keyed on) and accepted events.  Saving them with mks_get_state and
 * restoring both into a handle with the same seed continues a run bit for bit
 * (the reference's RunType C resume re-seeds its generator instead).      */
int mks_get_clock(mks_handle *h, int32_t rep, double *time, int64_t *window, int64_t *events);
int mks_set_clock(mks_handle *h, int32_t rep, double time, int64_t window, int64_t events);
/* Failure injection for tests: tile `tile` (-1: none) never publishes its
 * progress in the persistent schedule, so its neighbours' bounded waits
 * (spin_limit_cycles, default about 2 s) run out and the run returns
 * MKS_ERR_TIMEOUT with the context intact.  No counterpart in the reference. */
int mks_debug_hold_tile(mks_handle *h, int32_t tile, int64_t spin_limit_cycles);

/* Window length per replica (n entries): tau = f / r*, r* the rate of the
 * class carrying the largest share of the replica's total rate.  Validated
 * against the serial reference: f = 0.3 for one species (plain Si), f = 0.03
 * for two (3C-SiC rates).  No counterpart in the reference, whose loop is
 * serial.                                                                */
int mks_suggest_tau(mks_handle *h, double f, double *tau);

/* ---- laser-anneal rate law and barrier gradients ---- */
/* LA mode (mulskips-source/mcevent/Get_Prob.f:127-149 and
 * mulskips-source-LaserAnnealing/mcevent/Get_Prob.f:127-152): after this
 * call the PTransE / PTransD tables given to mks_batch_set_rates are barriers
 * in eV.  Melting of an atom: P0(s) exp(-E / kB T); solidification of species
 * s on a liquid site of coordination n: 0.5 P0(s) xliq(s) exp(-Ed(s,n) / kB
 * Tm(s)) (1 + erf((T - Tflex(s)) / sigma(s))), xliq(s) the fraction of the
 * molten atoms that are of species s (CountLiquid / SUM(CountLiquid),
 * LaserAnnealing main.f:637; the atoms present at this call count as solid),
 * refreshed every 8 windows.  A replica stops (stop reason 4) once it holds
 * more atoms than at this call (LaserAnnealing main.f:714-723).  T is the prescribed field
 * T(z,t) = Tb + Ta exp(-((t-t0)/w)^2) exp(-depth/L), depth = max(0, (zsurf -
 * z) sf / 10) nm, in integer K, evaluated per layer at each window's midpoint.
 * With score != 0 each replica accumulates (FP64) the likelihood-ratio score
 * sum_events d log k / d theta - int d R_tot / d theta dt for four
 * parameters theta, given dptransE (n*3*4096*4, d PTransE / d theta in the
 * PTransE layout) and dptransD (n*9*4).  No counterpart in the reference
 * (which has no derivatives); exponential waiting times are used.          */
typedef struct {
    float P0[3], Tm[3], Tflex[3], sigma[3];
    float Tb, Ta, t0, w;
    float L_nm, zsurf;
    int32_t score;
    int32_t liquid_weighting;  /* 1: LaserAnnealing law (liquid fractions, vacuum
                                  above zsurf, stop rule); 0: the law of
                                  mulskips-source/mcevent/Get_Prob.f:127-149 */
} mks_la_params;
int mks_batch_set_la(mks_handle *h, const mks_la_params *p, const double *dptransE, const double *dptransD);
int mks_batch_get_score(mks_handle *h, double *score, int32_t reset);
/* LA mode: crystal atoms per species (n*3) and the liquid fractions in use
 * (n*3, may be NULL).  Replaces the CountCrystal / CountLiquid report of
 * LaserAnnealing inpout/WriteMolMolSource.f:44-49.                        */
int mks_batch_la_counts(mks_handle *h, int64_t *crystal, double *xliq);
/* Backward step of the score: from one value f[i] per replica (host, n) the
 * likelihood-ratio gradient of E[f], grad[j] = mean_i (f_i - b_i) S_ij with
 * S the FP64 scores accumulated since the last reset and b_i the mean of the
 * other replicas' f (use_baseline != 0) or 0; se[j] (may be NULL) is its
 * standard error.  No counterpart in the reference.                      */
int mks_batch_lr_grad(mks_handle *h, const double *f, int32_t use_baseline, double *grad, double *se);
/* Causal form of the same gradient for an observable that is a sum of
 * increments over segments of the run, f = sum_k df_k (e.g. crystal atoms
 * gained per segment): after each segment the host passes df (one value per
 * replica) and the engine adds (df_i - b_i) S_i to replica i's FP64 sums,
 * S_i the score of its path so far and b_i the leave-one-out mean of df.
 * An increment is weighted only by the score of the path before it (the
 * later score has zero mean given that past), which lowers the variance.
 * mks_batch_lr_result gives the mean of the sums over the replicas and its
 * standard error (grad[4], se[4]) and clears the sums with reset != 0, as
 * mks_batch_set_la does.  No counterpart in the reference.               */
int mks_batch_lr_accumulate(mks_handle *h, const double *df);
int mks_batch_lr_result(mks_handle *h, int32_t reset, double *grad, double *se);
/* Static per-site temperatures for LA mode, from the T bits (9..21) of a
 * LattCoo array (SetT, mulskips-source/initial/SetT.f:25-50), replacing T(z,t)
 * for replica rep.  Call before mks_batch_set_la.                          */
int mks_batch_load_temperature(mks_handle *h, int32_t rep, const int32_t *lattcoo);
/* In-process LA coupling: the arrays of the reference's FEM <-> KMC socket
 * messages (LaserAnnealing main.f:160-345), int32 at every grid point in the
 * message layout, index z + LenZ * (x + LenX * y) (the Fortran arrays
 * b / c / d(LenZ, LenX*LenY)).
 * mks_batch_set_field replaces SENDFIELD + SetT (initial/SetT.f:34-48): the
 * temperature (K) of each site for LA mode; 10 marks a wall and keeps the
 * site's previous temperature.  It may be called between runs (after
 * mks_batch_set_la too).
 * mks_batch_get_phases replaces GETPHASES / GETXGE (main.f:796-817): coo gets
 * the coordination of every occupied site, species its ListCrystal index,
 * both 10 on walls and 0 elsewhere; grid points off the diamond sub-grid get
 * 10 in layers whose diamond sites are all walls, else 0 (pymulskips reads
 * the values 1..4 only, pymulskips/io.py:1013-1066).  Either pointer may be
 * NULL.                                                                    */
int mks_batch_set_field(mks_handle *h, int32_t rep, const int32_t *field);
/* The reference's shaped initial lattices (main.f:240-278), built in place
 * of replica rep's lattice: init_st "C" SetNC (lens = Len1, Len2, Len3),
 * "S" SetNCSp (Len1), "SS" SetNCSpSi (Len1), "I" SetInvPOff (Len1, Len2, as
 * main.f:245-246 passes them) and its variants "D" SetInvPC, "Z" SetInvPSi,
 * "J" SetInvPwAPB, "K" SetInvPwOnlySiorC, "L" SetInvPwOnlyCorSi (Len1,
 * Len2), "T" SetTrench (Len1, Len2, Len3), "Fw" SetSiC3Cww (Len1, Len2) and
 * "Fa" SetSiC3Cwwaperture (Len1, Len2, Len3; these two and "FF" round each
 * length down to a multiple of 24), "FF" SetSiFINFET (Len1..Len4), "ST"
 * SetTrenchSi (Len1, Len2, Len3; params = angle in degrees, Ttop, Tbottom in
 * K; also loads the temperature field T(z) for mks_batch_set_tabulated), "E"
 * SetSiCSF (Len1, Len2, Len3: a 3C-SiC slab up to Len1 with a triangular
 * triple stacking fault whose vertex is (Len2, Len3, Len1 - Len2), as
 * main.f:267-272 passes it; its atoms lie off the diamond sites, so only a
 * handle on the explicit-neighbour engine takes it -- PtransZig < 1 or
 * mks_config.explicit_nn = 1 -- and the rates must be set first).
 * Same result as the reference's routines including their closing
 * coordination passes.                                                      */
int mks_batch_init_shape(mks_handle *h, int32_t rep, const char *init_st, const int32_t *lens, const double *params);
int mks_init_shape(mks_handle *h, const char *init_st, const int32_t *lens, const double *params);
/* SetCAD for InitSt IN (SetCAD.f:80-341): geo holds the LattGeo id of every
 * grid point, int8 [z][y][x] (LenZ*LenY*LenX; 1 Si, 10 wall, 0 empty; the
 * layers z <= 3 and >= LenZ-4 are walls whatever they hold).  NCrystal = 1. */
int mks_batch_init_cad(mks_handle *h, int32_t rep, const int8_t *geo);
/* SetCAD for InitSt IN with the alloy fraction of a SiGe start.dat
 * (SetCAD.f:215-222): each Si site takes species 2 with probability x.  The
 * reference draws with the compiler's RAND(); here a generator seeded by
 * seed.  NCrystal >= 2 when x > 0.                                        */
int mks_batch_init_cad_alloy(mks_handle *h, int32_t rep, const int8_t *geo, double x, uint64_t seed);
/* SetShape for InitSt SH (SetShape.f:25-436): n grid points xyz[3*i..3*i+2]
 * = (x, y, z), 0 <= x < LenX, 0 <= y < LenY, 0 <= z <= LenZ, with
 * species[i] 1 (Si) or 2 (C / Ge); the points of the reference's point-list
 * file (sym x y z records).  Points with z <= 3 or z >= LenZ-4 are walls
 * (their species is not read), every other one an atom on a diamond site.
 * The coordinations, MC / bulk split and first list entries are those of
 * SetShape.f's shell scan and ad-void pass.  MKS_ERR_UNSUPPORTED for the
 * inputs the reference leaves undefined (an atom with fewer than two
 * neighbours, a reciprocity check reaching a wall, a vacancy with four MC
 * neighbours) and for an atom off the diamond sites or next to an off-site
 * wall point.                                                              */
int mks_batch_init_points(mks_handle *h, int32_t rep, const int32_t *xyz, const int8_t *species, int64_t n);
int mks_init_points(mks_handle *h, const int32_t *xyz, const int8_t *species, int64_t n);
/* The same for InitSt LA (SetCAD.f:166-212, fresh start): homogeneous 1
 * keeps the Si sites at z <= LenZ - INT((LenVac + LenNuc)/sf), 0 those
 * outside the nucleus ball of radius LenNuc/sf around (LenX/2, LenY/2,
 * LenZ - INT(LenVac/sf)); lengths in Angstrom.  -1 is InitSt IN.          */
int mks_batch_init_cad_la(mks_handle *h, int32_t rep, const int8_t *geo, int32_t homogeneous, double len_vac,
                          double len_nuc);
/* Tabulated rates instead of fixed tables (InitSt ST: SetProbabilityFromField.f,
 * InterpProbFromField.f, Get_Prob.f:77-91): each site's rates are the
 * PtransE / PtransD tables at its own temperature, linear in T between the
 * ntemp (<= 32) tabulated temperatures (the reference's integer-weighted
 * interpolation) and clamped outside them.  Replica i uses temps + i*ntemp
 * (increasing), ptransE + (i*ntemp + k)*3*4096 and ptransD + (i*ntemp + k)*9
 * for row k.  The temperatures are the replica's static field
 * (mks_batch_load_temperature or mks_batch_set_field, loaded first).  Every
 * class rate and deposition sum must not decrease with T (the kernel bounds a
 * tile's rates at its hottest layer and thins).  NCov = 0.  Switches the
 * replicas to the per-site-temperature kernels, like mks_batch_set_la.     */
int mks_batch_set_tabulated(mks_handle *h, int32_t ntemp, const int32_t *temps, const double *ptransE,
                            const double *ptransD);
int mks_batch_get_phases(mks_handle *h, int32_t rep, int32_t *coo, int32_t *species);
/* mks_load_lattice for replica rep of a batch.                            */
int mks_batch_load_lattice(mks_handle *h, int32_t rep, const int32_t *lattcoo);
/* SetSi-like slab with species 2 substituted on each atom with probability
 * x[i] (SetSiGex.f places Ge with the compiler's RAND(); here Philox).     */
int mks_batch_init_alloy(mks_handle *h, const int32_t *len1, const double *x, uint64_t seed);

/* Launch statistics of the last mks_run / mks_batch_run: kernel launches,
 * graph launches, and the device time (ms) of the sublattice kernels
 * measured with CUDA events on the engine's stream.                        */
int mks_last_run_stats(mks_handle *h, int64_t *kernel_launches, int64_t *graph_launches,
                       double *kernel_ms, int64_t *phase_launches);

#ifdef __cplusplus
}
#endif
#endif
