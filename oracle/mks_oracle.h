/*
 * mks_oracle.h — serial CPU restatement of the MulSKIPS KMC event loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle for the GPU engine in
 * mulskips_gb300/.  Only tests/, __graft_entry__.smoke() and the cpu_baseline
 * leg of bench.py may load it.  The product never calls it.
 *
 * It restates, function by function, the reference Fortran program
 * (mulskips-source/main.f and mulskips-source/mcevent/, lattice/, initial/,
 * inpout/) on the same dense super-lattice grid (LattCoo/LattInd int32 bit
 * fields), with the same ran3 generator, the same 1000-value test-mode list,
 * the same binary sum-tree and the same list bookkeeping, so that a given
 * start.dat produces the same event sequence and the same output frames.
 * Parity is pinned against the reference's own regression fixtures
 * (regression-tests/input-and-references-files, cases Si-SL and surface).
 */
#ifndef MKS_ORACLE_H
#define MKS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora ora_t;

/* One applied KMC event, as the GPU replay consumes it. */
typedef struct {
    int32_t x, y, z;   /* super-lattice grid coordinates of the event site   */
    int8_t  itrans;    /* 1..3 deposition of that species, 4 evaporation,
                          5 desorption, >=6 absorption                      */
    int8_t  arm;       /* 1 if a coor-1 deposition chose arm-chair stacking  */
    int16_t pad;
} ora_event_t;

/* Create an oracle from a start.dat file (reference format).  `numbers_path`
 * is the 1000-value test-mode uniform list (needed for RunType 'T'); may be
 * NULL otherwise.  `num_mc_max` <= 0 keeps the reference's 500000.
 * Returns NULL on error (message in ora_last_error()).                     */
ora_t *ora_create(const char *startdat_path, const char *numbers_path,
                  int lenx, int leny, int lenz, int num_mc_max);
void ora_destroy(ora_t *o);
const char *ora_last_error(void);

/* Run the initializer named by InitSt (FS, F, Fw, Fa, C, S, SS, I, D, Z, J, K, L,
 * T, ST, FF, IN, LA, SH; the point-list file of SH is read from the path named
 * in start.dat).  0 on success. */
int ora_init(ora_t *o);

/* Input of InitSt 'LA' (SetT + SetCAD, fresh start, NCrystal 1), used by
 * ora_init: `geo` holds the LattGeo id of each layer z = 0..LenZ-1 (1 Si,
 * 10 wall/air; the geometry must be uniform per layer), `tsub` the TempStat
 * temperature (K) of the grid points with x, y, z multiples of 3, index
 * ((z/3)*(LenY/3) + y/3)*(LenX/3) + x/3.  Copied.  0 on success. */
int ora_set_la_input(ora_t *o, const int8_t *geo, const int16_t *tsub);
/* InitSt IN input: the LattGeo id of every site (1 = Si, 10 = wall, 0 =
 * empty), int8 [z][y][x], LENZ*LENY*LENX values (SetCAD.f:155-236). */
int ora_set_geometry(ora_t *o, const int8_t *geo);
/* Advance up to n events (stops early on the reference's exit conditions).
 * Returns 0 ok, 1 "few MC particles" stop, 2 exit condition reached,
 * <0 error.  Writes output frames into `outdir` when non-NULL.             */
int ora_run(ora_t *o, int64_t n, const char *outdir);

/* Advance until the clock passes tmax (or an exit condition); returns as
 * ora_run.  No output frames. */
int ora_run_until(ora_t *o, double tmax);

/* Run the whole program like mulskips.e in directory `outdir`. */
int ora_main(ora_t *o, const char *outdir);

/* Trace recording. */
void ora_trace_enable(ora_t *o, int on);
int64_t ora_trace_len(const ora_t *o);
const ora_event_t *ora_trace(const ora_t *o);
void ora_trace_clear(ora_t *o);

/* State access. */
int64_t ora_iter(const ora_t *o);          /* Iter (next event number) */
double ora_time(const ora_t *o);
double ora_total_rate(const ora_t *o);     /* Tree(1)                  */
int ora_counts(const ora_t *o, int32_t out[3]);   /* NumAtoms, NumVoids, NumAdAtom */
void ora_dims(const ora_t *o, int32_t out[3]);
/* Copy LattCoo(0:LenX-1,0:LenY-1,0:LenZ) (x fastest) into out. */
void ora_get_lattcoo(const ora_t *o, int32_t *out);
/* Per-site list data of the site at (x,y,z): which list (0 none, 1 MC,
 * 2 bulk, 3 void), the 4 listed neighbours (12 ints), Ind_Event and rate.  */
int ora_site_info(const ora_t *o, int x, int y, int z, int32_t nn[12],
                  int32_t *ind_event, double *prob);
/* Write the xyz frame exactly as WriteMolMolXYZFile would. */
int ora_write_xyz(ora_t *o, const char *path);
int ora_write_frame(ora_t *o, const char *base, double time, int64_t iter);

/* The state as one byte per diamond site, in the GPU engine's layout
 * (mulskips_gb300/csrc/lattice.cuh): out[(z1*LenY/6 + b)*LenX/6 + a] =
 * species | coor<<2 | first-list-entry direction<<5 | dummy<<7, 0x80 wall; a
 * dummy coor-1 site still at Get_Prob_Ini's rate 1e-6 has coordination
 * field 5 (the engine's init-time dummy).
 * Returns the number of non-wall points off the diamond sub-grid (arm-chair
 * sites, which that layout cannot hold), or -1 if a list entry is not a bond. */
int64_t ora_compact_state(const ora_t *o, uint8_t *out);

/* Rate class of every listed MC particle, in the GPU engine's enumeration
 * (0 none, 1 empty coor-1, 2 empty coor-1 with the dummy rate, 3 coor-2,
 * 4 coor-3, 5 isolated atom, 6 + (species-1)*19 + census index for atoms,
 * 63 coor-1 dummy at Get_Prob_Ini's rate),
 * derived from the oracle's own lists and reciprocity checks.  Writes up to
 * n (class, rate) pairs and returns NumAdAtom.                              */
int64_t ora_mc_classes(const ora_t *o, int32_t *cls, double *rate, int64_t n);
/* Grid coordinates (x, y, z) of the MC particles in the same list order,
 * up to n of them; returns NumAdAtom.                                      */
int64_t ora_mc_sites(const ora_t *o, int32_t *xyz, int64_t n);
int64_t ora_list_entries(const ora_t *o, int32_t *xyz, int32_t *nn, int32_t *kind, int32_t *ind_event,
                         double *prob, int64_t n);

/* Export the rate tables parsed from start.dat. */
void ora_get_rates(const ora_t *o, double ptransE[3 * 4096], double ptransD[9]);
int ora_ncov(const ora_t *o);
/* PtransAbs / PtransDes as [coverage species][coor-1]. */
void ora_get_cov_rates(const ora_t *o, double ptransAbs[9], double ptransDes[9]);
/* ---- per-species LA law with liquid fractions and LR score ----
 * (LaserAnnealing variant: LA/mcevent/Get_Prob.f:127-152, LA/main.f:637,
 * 676-723).  Prescribed T(z,t) = Tb + Ta exp(-((t_mid-t0)/w)^2)
 * exp(-max(0, (zsurf - z) sf/10 nm)/L), t_mid the midpoint of the window of
 * length tau holding t; liquid fractions refreshed every `phase` windows.
 * The clock of ora_la_run_until is exponential (CTMC) and the FP64 score of
 * theta is accumulated; see mks_oracle.c.                                  */
typedef struct {
    double P0[3], Tm[3], Tflex[3], sigma[3];
    double Tb, Ta, t0, w, L_nm, zsurf;
    double tau;
    int phase;
} ora_la_t;
/* Substitute species 2 on every atom with probability x (after ora_init). */
int ora_la_alloy(ora_t *o, double x, uint64_t seed);
/* Switch to LA mode: PTransE (3*4096, PTransE(s,n1,n2,n3,c1,c2,c3) layout,
 * barriers in eV), its theta-derivatives (3*4096*4, may be NULL), PTransD (9)
 * and derivatives (9*4, may be NULL); the atoms present count as crystal. */
int ora_la_set(ora_t *o, const ora_la_t *p, const double *ptransE, const double *dptransE,
               const double *ptransD, const double *dptransD, uint64_t seed);
/* Advance to t_end (a window boundary).  Returns 0, 4 (more atoms than at
 * ora_la_set), 1 (<= 20 MC particles) or < 0 on error. */
int ora_la_run_until(ora_t *o, double t_end);
void ora_la_state(const ora_t *o, double score[4], int64_t crystal[3], double xliq[3], int64_t *events);
/* Raw ran3 for testing: seed then draw n values. */
void ora_ran3_sequence(int idum, int n, double *out);

#ifdef __cplusplus
}
#endif
#endif
